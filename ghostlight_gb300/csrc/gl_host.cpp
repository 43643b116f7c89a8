// gl_host.cpp — host builders of the flare path (compiled -ffp-contract=off so
// float arithmetic is the reference host build's, operation for operation).
//
//   * lens packing into SurfRec + per-wavelength IOR slices
//   * ghost-pair enumeration            (ghost.cpp:17-31)
//   * entrance-pupil mask and grid       (aperture_sampler.h:49-223)
//   * spectral table + 3x3 correction    (spectral.cpp:317-459)
//   * filter estimators for the re-check (ghost.cpp:34-102)
#include "gl_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "gl_colorimetry.inc"

namespace gl {

thread_local std::string g_last_error;
thread_local int g_last_launches = 0;

int fail(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

static bool rot_identity(const float* m)
{
    const float eps = 1e-6f;
    return (fabsf(m[0] - 1.f) < eps && fabsf(m[1]) < eps && fabsf(m[2]) < eps &&
            fabsf(m[3]) < eps && fabsf(m[4] - 1.f) < eps && fabsf(m[5]) < eps &&
            fabsf(m[6]) < eps && fabsf(m[7]) < eps && fabsf(m[8] - 1.f) < eps);
}

int pack_lens(const gl_surface* in, int n, SurfRec* out, int tables, bool may_upload)
{
    if (in == nullptr || n <= 0) return fail(GL_ERR_INVALID, "lens has no surfaces");
    if (n > kMaxSurfaces) return fail(GL_ERR_INVALID, "lens has more than 64 surfaces");
    for (int i = 0; i < n; ++i)
    {
        const gl_surface& g = in[i];
        SurfRec& r = out[i];
        std::memset(&r, 0, sizeof(r));
        if (g.aperture_shape < GL_APERTURE_CIRCLE || g.aperture_shape > GL_APERTURE_IMAGE)
            return fail(GL_ERR_INVALID, "unknown aperture shape " + std::to_string(g.aperture_shape));
        if (g.coating_model < GL_COATING_SIMPLE || g.coating_model > GL_COATING_ARTIST)
            return fail(GL_ERR_INVALID, "unknown coating model " + std::to_string(g.coating_model));
        if (g.aperture_shape == GL_APERTURE_POLYGON && g.aperture_blades < 3)
            return fail(GL_ERR_INVALID, "polygon aperture needs >= 3 blades");
        r.z = g.z;
        r.radius = g.radius;
        r.semi_ap = g.semi_aperture;
        r.aspect = g.aperture_aspect;
        r.rot_rad = g.aperture_rotation_rad;
        r.shape = (g.aperture_shape == GL_APERTURE_POLYGON) ? 1 : (g.aperture_shape == GL_APERTURE_IMAGE ? 2 : 0);
        r.blades = (g.aperture_shape == GL_APERTURE_IMAGE) ? 0 : g.aperture_blades;
        if (g.aperture_shape == GL_APERTURE_IMAGE && g.aperture_blades != 0)
        {
            // aperture_blades names the bitmap in the store; 0 = not loaded
            const float* px = nullptr;
            int disc = 0;
            int rc = coating_table_address(g.aperture_blades, kStoreImage, tables, may_upload, &px, &r.img_w,
                                           &r.img_h, &disc, &r.img_semi);
            if (rc) return rc;
            const uint64_t a = (uint64_t)(uintptr_t)px;
            r.img_lo = (uint32_t)a;
            r.img_hi = (uint32_t)(a >> 32);
        }
        if (r.shape == 1)
        {
            // check_aperture (trace_core.h:159-166) evaluates these per hit;
            // the same float operations once here give the same values.
            r.sector = 2.0f * kPi / (float)g.aperture_blades;
            r.apothem = g.semi_aperture * cosf(0.5f * r.sector);
            r.blade = make_blade_profile(g.aperture_blades, g.aperture_rotation_rad, g.aperture_curvature,
                                         g.aperture_twist, g.aperture_notch_rad, g.aperture_notch_angle_rad);
        }
        r.conic = g.conic_k;
        r.dec_x = g.decenter_x;
        r.dec_y = g.decenter_y;
        r.inv_r = (fabsf(g.radius) > 0.0f) ? 1.0f / g.radius : 0.0f;
        for (int k = 0; k < 9; ++k) r.rot[k] = g.rot[k];
        int nt = g.n_asphere_terms;
        if (nt < 0) nt = 0;
        if (nt > 8) nt = 8;
        for (int k = 0; k < 8; ++k) r.asph[k] = g.asphere_terms[k];
        r.n_asph = nt;
        r.form = g.form;
        r.cyl_axis = g.cyl_axis;
        r.flags = (g.is_active ? SF_ACTIVE : 0) | (g.is_stop ? SF_STOP : 0) |
                  ((g.decenter_x != 0.0f || g.decenter_y != 0.0f || !rot_identity(g.rot)) ? SF_TRANSFORMED : 0);
        r.coating = g.coating_model;
        r.ar_layers = g.ar_layers;
        if (g.coating_model >= GL_COATING_SPECTRAL && g.coating_model <= GL_COATING_SPECTRAL_ANGULAR)
        {
            // ar_layers names the table; 0 = none (bare Fresnel)
            r.ar_layers = 0;
            if (g.ar_layers != 0)
            {
                const float* t = nullptr;
                int rc = coating_table_address(g.ar_layers, g.coating_model, tables, may_upload, &t, &r.tab_n0,
                                               &r.tab_n1, &r.tab_discard, &r.tab_ref_ior);
                if (rc) return rc;
                const uint64_t a = (uint64_t)(uintptr_t)t;
                r.tab_lo = (uint32_t)a;
                r.tab_hi = (uint32_t)(a >> 32);
            }
        }
        r.tint_r = g.tint_r; r.tint_g = g.tint_g; r.tint_b = g.tint_b; r.tint_s = g.tint_strength;
        r.g_sigma = g.gauss_sigma; r.g_bg = g.gauss_background; r.g_peak = g.gauss_peak;
        r.g_dx = g.gauss_decenter_x; r.g_dy = g.gauss_decenter_y;
    }
    return GL_OK;
}

// dispersion_ior / sellmeier_n / Surface::ior_at (fresnel.h:27-63, optical_system.h:230)
float ior_at(const gl_surface& s, float lam)
{
    if (s.disp_model == GL_DISP_SELLMEIER)
    {
        float l = lam * 1e-3f;
        float l2 = l * l;
        float n2 = 1.0f;
        n2 += s.sellmeier_B[0] * l2 / (l2 - s.sellmeier_C[0]);
        n2 += s.sellmeier_B[1] * l2 / (l2 - s.sellmeier_C[1]);
        n2 += s.sellmeier_B[2] * l2 / (l2 - s.sellmeier_C[2]);
        return (n2 > 0.0f) ? sqrtf(n2) : 1.0f;
    }
    const float n_d = s.ior, V_d = s.abbe_v;
    if (V_d < 0.1f || n_d <= 1.0001f) return n_d;
    const float lF = 486.13f, lC = 656.27f, ld = 587.56f;
    float dn = (n_d - 1.0f) / V_d;
    float iF = 1.0f / (lF * lF), iC = 1.0f / (lC * lC), id = 1.0f / (ld * ld);
    float B = dn / (iF - iC);
    float A = n_d - B * id;
    return A + B / (lam * lam);
}

// Per-wavelength IOR slices, ghost_render.cu:809-823.
void build_ior_tables(const gl_surface* s, int n, const float* lambdas, int n_lam,
                      float* at, float* bf)
{
    for (int li = 0; li < n_lam; ++li)
    {
        float last = 1.0f;
        for (int k = 0; k < n; ++k)
        {
            at[li * n + k] = ior_at(s[k], lambdas[li]);
            bf[li * n + k] = last;
            if (s[k].is_active) last = at[li * n + k];
        }
    }
}

float ior_before_nd(const gl_surface* s, int idx)
{
    for (int k = idx - 1; k >= 0; --k)
        if (s[k].is_active) return s[k].ior;
    return 1.0f;
}

// ---- pupil mask (aperture_sampler.h:49-133) ------------------------------
PupilMask resolve_pupil_mask(const gl_surface* surfs, int n, int blades_override, float rotation_deg)
{
    int n_blades = 0;
    float rot_rad = 0.0f, aspect = 1.0f;
    BladeProfile blade = make_blade_profile(0, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f);
    for (int i = 0; i < n; ++i)
    {
        if (!surfs[i].is_stop) continue;
        aspect = surfs[i].aperture_aspect;
        if (surfs[i].aperture_shape == GL_APERTURE_POLYGON && surfs[i].aperture_blades >= 3)
        {
            n_blades = surfs[i].aperture_blades;
            rot_rad = surfs[i].aperture_rotation_rad;
            blade = make_blade_profile(n_blades, rot_rad, surfs[i].aperture_curvature, surfs[i].aperture_twist,
                                       surfs[i].aperture_notch_rad, surfs[i].aperture_notch_angle_rad);
        }
        break;
    }
    if (blades_override > 0)
    {
        // a plain n-gon by definition: the stop's blade shape is dropped
        n_blades = blades_override;
        rot_rad = rotation_deg * (kPi / 180.0f);
        blade = make_blade_profile(0, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f);
    }
    PupilMask m;
    m.blade = blade;
    m.aspect = aspect;
    m.n_blades = n_blades;
    m.rot_rad = rot_rad;
    const bool poly = n_blades >= 3;
    m.apothem = poly ? cosf(kPi / n_blades) : 1.0f;
    m.sector = poly ? (2.0f * kPi / n_blades) : 1.0f;
    return m;
}

bool pupil_contains(const PupilMask& m, float u, float v)
{
    const float ux = u / m.aspect;
    const float r2 = ux * ux + v * v;
    if (r2 > 1.0f) return false;
    if (m.n_blades >= 3)
    {
        if (m.blade.deformed) return sqrtf(r2) <= blade_radius_at(m.blade, atan2f(v, ux));
        float angle = atan2f(v, ux) - m.rot_rad;
        float sector = fmodf(angle, m.sector);
        if (sector < 0.0f) sector += m.sector;
        if (sqrtf(r2) * cosf(sector - m.sector * 0.5f) > m.apothem) return false;
    }
    return true;
}

static uint32_t wang_hash(uint32_t s)
{
    s = (s ^ 61u) ^ (s >> 16u);
    s *= 9u;
    s ^= s >> 4u;
    s *= 0x27d4eb2du;
    s ^= s >> 15u;
    return s;
}

static float radical_inverse2(uint32_t n)
{
    n = (n << 16u) | (n >> 16u);
    n = ((n & 0x00ff00ffu) << 8u) | ((n & 0xff00ff00u) >> 8u);
    n = ((n & 0x0f0f0f0fu) << 4u) | ((n & 0xf0f0f0f0u) >> 4u);
    n = ((n & 0x33333333u) << 2u) | ((n & 0xccccccccu) >> 2u);
    n = ((n & 0x55555555u) << 1u) | ((n & 0xaaaaaaaau) >> 1u);
    return (float)n * (1.0f / 4294967296.0f);
}

static float radical_inverse3(uint32_t n)
{
    float r = 0.0f, f = 1.0f / 3.0f;
    while (n > 0) { r += (n % 3u) * f; n /= 3u; f /= 3.0f; }
    return r;
}

int build_aperture_samples(const gl_surface* surfs, int n, const gl_sampler_params& p,
                           std::vector<gl_pupil_sample>& out)
{
    out.clear();
    const PupilMask mask = resolve_pupil_mask(surfs, n, p.blades_override, p.rotation_deg);
    const int N = p.ray_grid;
    if (N <= 0) return GL_OK;
    if (N > 4096) return fail(GL_ERR_INVALID, "ray_grid above 4096");
    const uint32_t seed_offset = (uint32_t)p.jitter_seed * 1000003u;
    out.reserve((size_t)N * N);
    for (int k = 0; k < N * N; ++k)
    {
        const int gx = k % N, gy = k / N;
        float u, v;
        if (p.pupil_jitter == 2)
        {
            u = radical_inverse2((uint32_t)k) * 2.0f - 1.0f;
            v = radical_inverse3((uint32_t)k) * 2.0f - 1.0f;
        }
        else
        {
            float ju = (p.pupil_jitter == 1) ? wang_hash((uint32_t)k + seed_offset) / 4294967296.0f : 0.5f;
            float jv = (p.pupil_jitter == 1)
                           ? wang_hash((uint32_t)k + (uint32_t)(N * N) + seed_offset) / 4294967296.0f
                           : 0.5f;
            u = ((gx + ju) / N) * 2.0f - 1.0f;
            v = ((gy + jv) / N) * 2.0f - 1.0f;
        }
        if (pupil_contains(mask, u, v)) out.push_back({u, v});
    }
    return GL_OK;
}

// ---- spectral (spectral.cpp:113-459) -------------------------------------
static void cie_interpolate(float lam, float* sr, float* sg, float* sb)
{
    const int count = GL_CIE_COUNT;
    if (lam < GL_CIE_WL[0] || lam > GL_CIE_WL[count - 1]) { *sr = *sg = *sb = 0.0f; return; }
    int lo = 0, hi = count - 2;
    while (lo < hi)
    {
        int mid = (lo + hi) / 2;
        if (GL_CIE_WL[mid + 1] < lam) lo = mid + 1; else hi = mid;
    }
    const float w0 = GL_CIE_WL[lo], w1 = GL_CIE_WL[lo + 1];
    const float t = (lam - w0) / (w1 - w0);
    *sr = GL_CIE_X[lo] + t * (GL_CIE_X[lo + 1] - GL_CIE_X[lo]);
    *sg = GL_CIE_Y[lo] + t * (GL_CIE_Y[lo + 1] - GL_CIE_Y[lo]);
    *sb = GL_CIE_Z[lo] + t * (GL_CIE_Z[lo + 1] - GL_CIE_Z[lo]);
}

int output_matrix(int cs, const float* custom, float M[9])
{
    if (cs >= 0 && cs <= 4) { std::memcpy(M, GL_OUTPUT_MATRICES[cs], 9 * sizeof(float)); return GL_OK; }
    if (cs == GL_CS_CUSTOM)
    {
        if (custom) std::memcpy(M, custom, 9 * sizeof(float));
        else for (int k = 0; k < 9; ++k) M[k] = (k % 4 == 0) ? 1.0f : 0.0f;
        return GL_OK;
    }
    return fail(GL_ERR_INVALID, "unknown output colour space");
}

int input_matrix(int cs, const float* custom, float M[9])
{
    if (cs >= 0 && cs <= 1) { std::memcpy(M, GL_INPUT_MATRICES[cs], 9 * sizeof(float)); return GL_OK; }
    if (cs == GL_CS_INPUT_CUSTOM)
    {
        if (custom) std::memcpy(M, custom, 9 * sizeof(float));
        else for (int k = 0; k < 9; ++k) M[k] = (k % 4 == 0) ? 1.0f : 0.0f;
        return GL_OK;
    }
    return fail(GL_ERR_INVALID, "unknown input colour space");
}

// The CIE 1931 sensor's matrix_to_xyz is the identity; its products are
// written out so the float operations match spectral.cpp:341-348.
std::vector<gl_spectral_sample> spectral_table(int n, float lmin, float lmax, const float M[9])
{
    std::vector<gl_spectral_sample> t((size_t)n);
    const float delta = (lmax - lmin) / n;
    const float I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    for (int i = 0; i < n; ++i)
    {
        float lam = lmin + (i + 0.5f) * delta;
        t[i].lambda = lam;
        float sr, sg, sb;
        cie_interpolate(lam, &sr, &sg, &sb);
        float xr = I[0] * sr + I[1] * sg + I[2] * sb;
        float xg = I[3] * sr + I[4] * sg + I[5] * sb;
        float xb = I[6] * sr + I[7] * sg + I[8] * sb;
        t[i].cmf_r = M[0] * xr + M[1] * xg + M[2] * xb;
        t[i].cmf_g = M[3] * xr + M[4] * xg + M[5] * xb;
        t[i].cmf_b = M[6] * xr + M[7] * xg + M[8] * xb;
    }
    float sum_g = 0.0f;
    for (int i = 0; i < n; ++i) sum_g += t[i].cmf_g * delta;
    if (sum_g > 1e-9f)
    {
        float inv = 1.0f / sum_g;
        for (auto& s : t) { s.cmf_r *= inv; s.cmf_g *= inv; s.cmf_b *= inv; }
    }
    return t;
}

static void gram(const std::vector<gl_spectral_sample>& t, float O[3][3])
{
    for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) O[a][b] = 0.0f;
    for (const auto& s : t)
    {
        const float c[3] = {s.cmf_r, s.cmf_g, s.cmf_b};
        for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) O[a][b] += c[a] * c[b];
    }
}

static void m3mul_host(const float A[3][3], const float B[3][3], float D[3][3])
{
    float tmp[3][3] = {};
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            for (int k = 0; k < 3; ++k) tmp[r][c] += A[r][k] * B[k][c];
    std::memcpy(D, tmp, sizeof(tmp));
}

static void m3inv_host(const float m[3][3], float inv[3][3])
{
    const float det = m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) -
                      m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                      m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]);
    if (std::fabs(det) < 1e-20f)
    {
        for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) inv[r][c] = (r == c) ? 1.0f : 0.0f;
        return;
    }
    const float id = 1.0f / det;
    inv[0][0] = (m[1][1] * m[2][2] - m[1][2] * m[2][1]) * id;
    inv[0][1] = -(m[0][1] * m[2][2] - m[0][2] * m[2][1]) * id;
    inv[0][2] = (m[0][1] * m[1][2] - m[0][2] * m[1][1]) * id;
    inv[1][0] = -(m[1][0] * m[2][2] - m[1][2] * m[2][0]) * id;
    inv[1][1] = (m[0][0] * m[2][2] - m[0][2] * m[2][0]) * id;
    inv[1][2] = -(m[0][0] * m[1][2] - m[0][2] * m[1][0]) * id;
    inv[2][0] = (m[1][0] * m[2][1] - m[1][1] * m[2][0]) * id;
    inv[2][1] = -(m[0][0] * m[2][1] - m[0][1] * m[2][0]) * id;
    inv[2][2] = (m[0][0] * m[1][1] - m[0][1] * m[1][0]) * id;
}

// compute_spectral_correction, spectral.cpp:419-459 (300-sample dense
// reference, 16-sample brightness anchor).
void spectral_correction(const std::vector<gl_spectral_sample>& tn, float lmin, float lmax,
                         const float M[9], float C[9])
{
    float On[3][3], Od[3][3], Oa[3][3];
    gram(tn, On);
    gram(spectral_table(300, lmin, lmax, M), Od);
    gram(spectral_table(16, lmin, lmax, M), Oa);
    const float bn = On[1][0] + On[1][1] + On[1][2];
    const float bd = Od[1][0] + Od[1][1] + Od[1][2];
    const float ba = Oa[1][0] + Oa[1][1] + Oa[1][2];
    if (!(bn > 1e-20f) || !(bd > 1e-20f))
    {
        for (int k = 0; k < 9; ++k) C[k] = (k % 4 == 0) ? 1.0f : 0.0f;
        return;
    }
    float Onh[3][3], Odh[3][3];
    const float ibn = 1.0f / bn, ibd = 1.0f / bd;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) { Onh[a][b] = On[a][b] * ibn; Odh[a][b] = Od[a][b] * ibd; }
    float Oni[3][3], Cc[3][3];
    m3inv_host(Onh, Oni);
    m3mul_host(Odh, Oni, Cc);
    const float s = ba / bn;
    for (int a = 0; a < 3; ++a) for (int b = 0; b < 3; ++b) C[3 * a + b] = Cc[a][b] * s;
}

// ---- filter estimators on the host (ghost.cpp:34-102) --------------------
static const float kProbeLambdas[3] = {650.0f, 550.0f, 450.0f};

float host_intensity_estimate(const gl_surface* s, const SurfRec* recs, int n, int a, int b)
{
    std::vector<float> at(n), bf(n);
    float total = 0.0f;
    for (int ch = 0; ch < 3; ++ch)
    {
        build_ior_tables(s, n, &kProbeLambdas[ch], 1, at.data(), bf.data());
        TraceOut r = trace_ghost(recs, n, at.data(), bf.data(), v3(0.0f, 0.0f, s[0].z - kSpawnOffset),
                                 v3(0.0f, 0.0f, 1.0f), kProbeLambdas[ch], a, b);
        if (r.status == 0) total += r.w;
    }
    return total / 3.0f;
}

void host_filter_probe(const gl_surface* s, const SurfRec* recs, int n, int a, int b, FilterProbe* out)
{
    std::vector<float> at(n), bf(n);
    const float start_z = s[0].z - kSpawnOffset, front_R = s[0].semi_aperture;
    for (int ch = 0; ch < 3; ++ch)
    {
        build_ior_tables(s, n, &kProbeLambdas[ch], 1, at.data(), bf.data());
        TraceOut r = trace_ghost(recs, n, at.data(), bf.data(), v3(0.0f, 0.0f, start_z), v3(0.0f, 0.0f, 1.0f),
                                 kProbeLambdas[ch], a, b);
        out->w[ch] = r.w;
        out->wok[ch] = r.status == 0;
    }
    build_ior_tables(s, n, &kProbeLambdas[1], 1, at.data(), bf.data());
    out->mnx = 1e30f; out->mxx = -1e30f; out->mny = 1e30f; out->mxy = -1e30f;
    out->valid = 0;
    for (int k = 0; k < 64; ++k)
    {
        const float u = ((k % 8 + 0.5f) / 8) * 2.0f - 1.0f;
        const float v = ((k / 8 + 0.5f) / 8) * 2.0f - 1.0f;
        if (u * u + v * v > 1.0f) continue;
        TraceOut r = trace_ghost(recs, n, at.data(), bf.data(), v3(u * front_R, v * front_R, start_z),
                                 v3(0.0f, 0.0f, 1.0f), kProbeLambdas[1], a, b);
        if (r.status != 0) continue;
        out->mnx = std::min(out->mnx, r.x); out->mxx = std::max(out->mxx, r.x);
        out->mny = std::min(out->mny, r.y); out->mxy = std::max(out->mxy, r.y);
        ++out->valid;
    }
}

float host_spread_boost(const gl_surface* s, const SurfRec* recs, int n, int a, int b,
                        float hw, float hh, float max_boost)
{
    const int G = 8;
    std::vector<float> at(n), bf(n);
    build_ior_tables(s, n, &kProbeLambdas[1], 1, at.data(), bf.data());
    const float front_R = s[0].semi_aperture, start_z = s[0].z - kSpawnOffset;
    float mnx = 1e30f, mxx = -1e30f, mny = 1e30f, mxy = -1e30f;
    int valid = 0;
    for (int gy = 0; gy < G; ++gy)
        for (int gx = 0; gx < G; ++gx)
        {
            float u = ((gx + 0.5f) / G) * 2.0f - 1.0f;
            float v = ((gy + 0.5f) / G) * 2.0f - 1.0f;
            if (u * u + v * v > 1.0f) continue;
            TraceOut r = trace_ghost(recs, n, at.data(), bf.data(), v3(u * front_R, v * front_R, start_z),
                                     v3(0.0f, 0.0f, 1.0f), kProbeLambdas[1], a, b);
            if (r.status != 0) continue;
            mnx = std::min(mnx, r.x); mxx = std::max(mxx, r.x);
            mny = std::min(mny, r.y); mxy = std::max(mxy, r.y);
            ++valid;
        }
    if (valid < 2) return 1.0f;
    float gw = std::max(mxx - mnx, 0.01f), gh = std::max(mxy - mny, 0.01f);
    float area = (gw * gh) / ((2.0f * hw) * (2.0f * hh));
    return std::clamp(area, 1.0f, max_boost);
}

}  // namespace gl

// ===========================================================================
// C-ABI: host builders
// ===========================================================================
using namespace gl;

extern "C" {

const char* gl_last_error(void) { return g_last_error.c_str(); }
int gl_version(void) { return 100; }
int gl_last_launch_count(void) { return g_last_launches; }

int gl_finalize_z(gl_surface* s, int n)
{
    if (!s || n <= 0) return fail(GL_ERR_INVALID, "finalize: lens has no surfaces");
    float total = 0.0f;
    for (int i = 0; i < n; ++i) total += s[i].thickness;
    float z = -total;
    for (int i = 0; i < n; ++i) { s[i].z = z; z += s[i].thickness; }
    return GL_OK;
}

// PupilMask::contains (aperture_sampler.h:63-82) at host points, host float
// arithmetic; aspect_one rasterises the stop round as the starburst does.
int gl_pupil_contains(const gl_surface* surfaces, int n, int blades_override, float rotation_deg, int aspect_one,
                      const float* uv, int n_pts, uint8_t* out)
{
    if (!surfaces || n <= 0 || n_pts < 0 || (n_pts > 0 && (!uv || !out)))
        return fail(GL_ERR_INVALID, "pupil_contains: bad arguments");
    PupilMask m = resolve_pupil_mask(surfaces, n, blades_override, rotation_deg);
    if (aspect_one) m.aspect = 1.0f;
    for (int k = 0; k < n_pts; ++k) out[k] = pupil_contains(m, uv[2 * k], uv[2 * k + 1]) ? 1 : 0;
    return GL_OK;
}

// Boundary radius (normalised; 1 = blade tip) of a bladed stop's silhouette
// at angles theta: ApertureProfile::radius_at of make_aperture_profile
// (aperture_profile.h:192-196, 285-358), host float arithmetic.
int gl_blade_radius(int blades, float rotation_rad, float curvature, float twist, float notch_rad,
                    float notch_angle_rad, const float* theta, int n, float* out)
{
    if (blades < 3 || n < 0 || (n > 0 && (!theta || !out)))
        return fail(GL_ERR_INVALID, "blade_radius: needs >= 3 blades and n angles");
    const BladeProfile b = make_blade_profile(blades, rotation_rad, curvature, twist, notch_rad, notch_angle_rad);
    for (int i = 0; i < n; ++i)
    {
        if (b.deformed)
        {
            out[i] = blade_radius_at(b, theta[i]);
        }
        else
        {
            // the regular polygon, as check_aperture evaluates it (trace_core.h:159-166)
            float off = fmodf(theta[i] - rotation_rad, b.sigma);
            if (off < 0.0f) off += b.sigma;
            off -= 0.5f * b.sigma;
            out[i] = cosf(0.5f * b.sigma) / cosf(off);
        }
    }
    return GL_OK;
}

// Element rotation of the lens-file loader (make_rotation,
// optical_system.cpp:185-199): R = Ry(tilt_y) Rx(tilt_x) Rz(roll), row-major,
// float arithmetic with the C library's float cosine and sine.
int gl_euler_rotation(float tilt_x_deg, float tilt_y_deg, float roll_deg, float* out)
{
    if (!out) return fail(GL_ERR_INVALID, "euler_rotation: null output");
    const float kPi = 3.14159265358979323846f;
    const float tx = tilt_x_deg * (kPi / 180.0f);
    const float ty = tilt_y_deg * (kPi / 180.0f);
    const float rz = roll_deg * (kPi / 180.0f);
    const float cx = std::cos(tx), sx = std::sin(tx);
    const float cy = std::cos(ty), sy = std::sin(ty);
    const float cz = std::cos(rz), sz = std::sin(rz);
    out[0] = cy * cz + sy * sx * sz;  out[1] = -cy * sz + sy * sx * cz;  out[2] = sy * cx;
    out[3] = cx * sz;                 out[4] = cx * cz;                  out[5] = -sx;
    out[6] = -sy * cz + cy * sx * sz; out[7] = sy * sz + cy * sx * cz;   out[8] = cy * cx;
    return GL_OK;
}

int gl_enumerate_ghost_pairs(const gl_surface* s, int n, gl_ghost_pair* out, int cap, int* n_out)
{
    if (!s || n <= 0 || !n_out) return fail(GL_ERR_INVALID, "enumerate_ghost_pairs: bad arguments");
    int k = 0;
    for (int a = 0; a < n; ++a)
    {
        if (!s[a].is_active) continue;
        for (int b = a + 1; b < n; ++b)
        {
            if (!s[b].is_active) continue;
            if (out && k < cap) out[k] = {a, b};
            ++k;
        }
    }
    *n_out = k;
    return (out && k > cap) ? fail(GL_ERR_INVALID, "enumerate_ghost_pairs: capacity too small") : GL_OK;
}

int gl_build_aperture_samples(const gl_surface* s, int n, const gl_sampler_params* p,
                              gl_pupil_sample* out, int cap, int* n_out)
{
    if (!s || n <= 0 || !p || !n_out) return fail(GL_ERR_INVALID, "build_aperture_samples: bad arguments");
    std::vector<gl_pupil_sample> v;
    int rc = build_aperture_samples(s, n, *p, v);
    if (rc) return rc;
    *n_out = (int)v.size();
    if (out)
    {
        if ((int)v.size() > cap) return fail(GL_ERR_INVALID, "build_aperture_samples: capacity too small");
        std::memcpy(out, v.data(), v.size() * sizeof(gl_pupil_sample));
    }
    return GL_OK;
}

int gl_build_spectral_table(int n, int output_cs, const float* custom, gl_spectral_sample* out,
                            float* corr)
{
    if (n < 1 || !out) return fail(GL_ERR_INVALID, "build_spectral_table: bad arguments");
    if (corr) for (int k = 0; k < 9; ++k) corr[k] = (k % 4 == 0) ? 1.0f : 0.0f;
    if (n == 3)
    {
        // Fixed RGB preview wavelengths with identity weights (ghost_render.cu:781-788).
        out[0] = {650.0f, 1.0f, 0.0f, 0.0f};
        out[1] = {550.0f, 0.0f, 1.0f, 0.0f};
        out[2] = {450.0f, 0.0f, 0.0f, 1.0f};
        return GL_OK;
    }
    float M[9];
    int rc = output_matrix(output_cs, custom, M);
    if (rc) return rc;
    std::vector<gl_spectral_sample> t = spectral_table(n, 400.0f, 700.0f, M);
    std::memcpy(out, t.data(), t.size() * sizeof(gl_spectral_sample));
    if (corr) spectral_correction(t, 400.0f, 700.0f, M, corr);
    return GL_OK;
}

int gl_color_matrices(int input_cs, const float* custom_in, int output_cs, const float* custom_out,
                      float* m_in9, float* m_out9)
{
    if (!m_in9 || !m_out9) return fail(GL_ERR_INVALID, "color_matrices: bad arguments");
    int rc = input_matrix(input_cs, custom_in, m_in9);
    if (rc) return rc;
    return output_matrix(output_cs, custom_out, m_out9);
}

}  // extern "C"
