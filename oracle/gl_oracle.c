/*
 * gl_oracle.c — CPU oracle of the flare path.  TEST INFRASTRUCTURE ONLY: only
 * tests/, __graft_entry__.smoke() and bench.py's cpu_baseline leg load it, as
 * the parity reference; the product never does.
 *
 * gl_oracle_impl.h restates the reference trace (JaydenB/ghostlight
 * ghostlight/src/trace.cpp, trace_core.h, fresnel.h) and is instantiated for
 * float (the reference host arithmetic: filter decisions, per-ray pins) and
 * double (the FP64 oracle the GPU images are measured against).  This file
 * adds the host mirror of the ghost kernel's main path (ghost_render.cu:
 * 280-463), the pair filter (ghost.cpp:17-138) and the pupil sampler
 * (aperture_sampler.h:49-223).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

#include "ghostlight_gb300.h"

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

static int orc_rot_identity(const float* m)
{
    const float eps = 1e-6f;
    return (fabsf(m[0] - 1.f) < eps && fabsf(m[1]) < eps && fabsf(m[2]) < eps &&
            fabsf(m[3]) < eps && fabsf(m[4] - 1.f) < eps && fabsf(m[5]) < eps &&
            fabsf(m[6]) < eps && fabsf(m[7]) < eps && fabsf(m[8] - 1.f) < eps);
}

/* ---- authored blade silhouette -----------------------------------------
 * ApertureProfile / make_aperture_profile, aperture_profile.h:82-358: each
 * half blade edge a conic arc in u = 1/r through the waist and the tip, the
 * notch a chord across the tip.  The derived block is built in float, as the
 * reference does; the boundary radius is evaluated in the instantiation's
 * scalar type (impl: blade_radius). */
typedef struct {
    int blades, deformed, facets;
    float rotation, sigma, half, r_w, phi_w, u_w, u_rise, qR, qL, p, beta, eA, eB;
} orc_blade;

static float orc_bclamp(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }

static float orc_blade_u_edge(const orc_blade* b, float phi)
{
    const float psi = phi - b->phi_w;
    const float sh = sinf(0.5f * psi);
    return b->u_w - b->u_rise * (sh * sh) * ((psi >= 0.0f) ? b->qR : b->qL);
}

static int orc_blade_authored(const gl_surface* s)
{
    return s->aperture_curvature != 0.0f || s->aperture_twist != 0.0f || s->aperture_notch_rad != 0.0f;
}

static orc_blade orc_make_blade(const gl_surface* s)
{
    const float pi = (float)M_PI;
    orc_blade b;
    memset(&b, 0, sizeof(b));
    b.blades = s->aperture_blades;
    const float curv = orc_bclamp(s->aperture_curvature, -1.0f, 1.0f);
    const float twist = orc_bclamp(s->aperture_twist, -1.0f, 1.0f);
    const float notch = orc_bclamp(s->aperture_notch_rad, -(float)(M_PI / 4.0), (float)(M_PI / 4.0));
    const float rake = orc_bclamp(s->aperture_notch_angle_rad, 0.0f, (float)(M_PI / 4.0));
    b.rotation = s->aperture_rotation_rad;
    b.sigma = 2.0f * pi / (float)b.blades;
    b.half = 0.5f * b.sigma;
    b.deformed = !(curv == 0.0f && twist == 0.0f && notch == 0.0f);
    const float a = cosf(b.half);
    b.r_w = (curv >= 0.0f) ? (a + curv * (1.0f - a)) : (a * (1.0f + curv * 0.55f));
    const float lim = fmaxf(0.0f, b.half - 4.0f * (float)(M_PI / 180.0));
    b.phi_w = orc_bclamp(twist * b.half, -lim, lim);
    const float dR = b.half - b.phi_w, dL = b.half + b.phi_w;
    b.u_w = 1.0f / b.r_w;
    b.u_rise = b.u_w - 1.0f;
    const float sR = sinf(0.5f * dR), sL = sinf(0.5f * dL);
    b.qR = 1.0f / (sR * sR);
    b.qL = 1.0f / (sL * sL);
    const float e = (fabsf(notch) / (45.0f * (float)(M_PI / 180.0))) * 0.45f * b.half;
    const float sk = orc_bclamp(rake / (float)(M_PI / 4.0), 0.0f, 1.0f);
    float eA = fminf(e * (1.0f + sk), 0.90f * b.half);
    float eB = e * (1.0f - sk);
    if (notch < 0.0f) { const float t = eA; eA = eB; eB = t; }
    if (e > 1e-9f && b.r_w < 1.0f && (eA + eB) > 1e-9f)
    {
        const float pa = b.half - eA, pb = b.half + eB;
        const float ra = 1.0f / orc_blade_u_edge(&b, pa);
        const float rb = 1.0f / orc_blade_u_edge(&b, -b.half + eB);
        const float ax = ra * cosf(pa), ay = ra * sinf(pa);
        const float bx = rb * cosf(pb), by = rb * sinf(pb);
        const float dx = bx - ax, dy = by - ay;
        const float dl = sqrtf(dx * dx + dy * dy);
        if (dl >= 1e-9f)
        {
            float nx = dy / dl, ny = -dx / dl;
            if (ax * nx + ay * ny < 0.0f) { nx = -nx; ny = -ny; }
            const float p = ax * nx + ay * ny;
            if (p > 1e-6f) { b.facets = 1; b.p = p; b.beta = atan2f(ny, nx); b.eA = eA; b.eB = eB; }
        }
    }
    return b;
}

/* ---- coating tables ------------------------------------------------------
 * OpticalSystem::coating_tables (optical_system.h:288-295) keyed by the id a
 * table-coated surface carries in ar_layers: the test registers each table
 * under the id the product's store gave it.  Layout per entry: axis0[n0]
 * (nm or degrees), axis1[n1] (SPECTRAL_ANGULAR angles), r (n0 or n0*n1,
 * wavelength-major). */
#define ORC_MAX_TABLES 256
typedef struct { int model, n0, n1, discard; float ref_ior; float* data; } orc_table;
static orc_table orc_tables[ORC_MAX_TABLES];

int orc_coating_register(int id, int model, int n0, int n1, const float* data, float ref_ior, int discard)
{
    if (id < 1 || id >= ORC_MAX_TABLES || n0 < 1 || n1 < 0) return -1;
    const size_t len = (size_t)n0 + (size_t)n1 + (n1 ? (size_t)n0 * n1 : (size_t)n0);
    float* d = (float*)malloc(len * sizeof(float));
    if (!d) return -1;
    memcpy(d, data, len * sizeof(float));
    free(orc_tables[id].data);
    orc_tables[id].model = model; orc_tables[id].n0 = n0; orc_tables[id].n1 = n1;
    orc_tables[id].discard = discard; orc_tables[id].ref_ior = ref_ior; orc_tables[id].data = d;
    return 0;
}

/* ApertureImage (optical_system.h:262-269) under the id a GL_APERTURE_IMAGE
 * surface carries in aperture_blades: w x h luminance, the boundary radius in
 * ref_ior. */
int orc_image_register(int id, int w, int h, const float* pixels, float semi_diameter)
{
    if (id < 1 || id >= ORC_MAX_TABLES || w < 1 || h < 1) return -1;
    float* d = (float*)malloc((size_t)w * h * sizeof(float));
    if (!d) return -1;
    memcpy(d, pixels, (size_t)w * h * sizeof(float));
    free(orc_tables[id].data);
    orc_tables[id].model = 100; orc_tables[id].n0 = w; orc_tables[id].n1 = h;
    orc_tables[id].discard = 0; orc_tables[id].ref_ior = semi_diameter; orc_tables[id].data = d;
    return 0;
}

static const orc_table* orc_coating_find(int id)
{
    if (id < 1 || id >= ORC_MAX_TABLES || !orc_tables[id].data) return NULL;
    return &orc_tables[id];
}

/* ---- float instantiation ------------------------------------------------ */
#define R float
#define SFX(x) x##_f32
#define SQRT sqrtf
#define ASIN asinf
#define COS cosf
#define SIN sinf
#define ATAN2 atan2f
#define FMOD fmodf
#define FABS fabsf
#define EXP expf
#define FLOOR floorf
#define FMIN fminf
#define FMAX fmaxf
#include "gl_oracle_impl.h"
#undef R
#undef SFX
#undef SQRT
#undef ASIN
#undef COS
#undef SIN
#undef ATAN2
#undef FMOD
#undef FABS
#undef EXP
#undef FLOOR
#undef FMIN
#undef FMAX

/* ---- double instantiation ----------------------------------------------- */
#define R double
#define SFX(x) x##_f64
#define SQRT sqrt
#define ASIN asin
#define COS cos
#define SIN sin
#define ATAN2 atan2
#define FMOD fmod
#define FABS fabs
#define EXP exp
#define FLOOR floor
#define FMIN fmin
#define FMAX fmax
#include "gl_oracle_impl.h"
#undef R
#undef SFX

/* rays: n x 7 floats (o, d, lambda); out: n x 5 doubles (x, y, z, w, status).
 * b < 0 traces a primary ray. */
int orc_trace(const gl_surface* S, int N, int a, int b, const float* rays, int n_rays,
              int fp64, double* out)
{
    for (int i = 0; i < n_rays; ++i)
    {
        const float* r = rays + 7 * (size_t)i;
        double* q = out + 5 * (size_t)i;
        if (fp64)
        {
            v3_f64 o = mk_f64(r[0], r[1], r[2]), d = mk_f64(r[3], r[4], r[5]);
            result_f64 t = (b < 0) ? trace_primary_f64(S, N, o, d, r[6])
                                   : trace_ghost_f64(S, N, o, d, r[6], a, b);
            q[0] = t.x; q[1] = t.y; q[2] = t.z; q[3] = t.w; q[4] = t.status;
        }
        else
        {
            v3_f32 o = mk_f32(r[0], r[1], r[2]), d = mk_f32(r[3], r[4], r[5]);
            result_f32 t = (b < 0) ? trace_primary_f32(S, N, o, d, r[6])
                                   : trace_ghost_f32(S, N, o, d, r[6], a, b);
            q[0] = t.x; q[1] = t.y; q[2] = t.z; q[3] = t.w; q[4] = t.status;
        }
    }
    return 0;
}

/* enumerate_ghost_pairs, ghost.cpp:17-31 */
int orc_enumerate(const gl_surface* S, int N, int* out_ab, int cap)
{
    int k = 0;
    for (int a = 0; a < N; ++a)
    {
        if (!S[a].is_active) continue;
        for (int b = a + 1; b < N; ++b)
        {
            if (!S[b].is_active) continue;
            if (k < cap) { out_ab[2 * k] = a; out_ab[2 * k + 1] = b; }
            ++k;
        }
    }
    return k;
}

static float ior_before_nd(const gl_surface* S, int idx)
{
    for (int k = idx - 1; k >= 0; --k)
        if (S[k].is_active) return S[k].ior;
    return 1.0f;
}

/* filter_ghost_pairs, ghost.cpp:105-138, in the reference's float arithmetic */
int orc_filter(const gl_surface* S, int N, float hw, float hh, float min_int, int normalize,
               float max_boost, int* out_ab, float* out_boost, float* out_fp, int cap)
{
    static const float lams[3] = {650.0f, 550.0f, 450.0f};
    const float start_z = S[0].z - 20.0f;
    const float front_R = S[0].semi_aperture;
    int kept = 0;
    for (int a = 0; a < N; ++a)
    {
        if (!S[a].is_active) continue;
        for (int b = a + 1; b < N; ++b)
        {
            if (!S[b].is_active) continue;
            if (fabsf(ior_before_nd(S, a) - S[a].ior) < 0.001f ||
                fabsf(ior_before_nd(S, b) - S[b].ior) < 0.001f) continue;
            float total = 0.0f;
            for (int ch = 0; ch < 3; ++ch)
            {
                result_f32 r = trace_ghost_f32(S, N, mk_f32(0, 0, start_z), mk_f32(0, 0, 1), lams[ch], a, b);
                if (r.status == GL_TRACE_OK) total += r.w;
            }
            float est = total / 3.0f;
            if (est < min_int) continue;
            float boost = 1.0f, fpw = 0.0f, fph = 0.0f;
            {
                float mnx = 1e30f, mxx = -1e30f, mny = 1e30f, mxy = -1e30f;
                int valid = 0;
                for (int gy = 0; gy < 8; ++gy)
                    for (int gx = 0; gx < 8; ++gx)
                    {
                        float u = ((gx + 0.5f) / 8) * 2.0f - 1.0f;
                        float v = ((gy + 0.5f) / 8) * 2.0f - 1.0f;
                        if (u * u + v * v > 1.0f) continue;
                        result_f32 r = trace_ghost_f32(S, N, mk_f32(u * front_R, v * front_R, start_z),
                                                       mk_f32(0, 0, 1), 550.0f, a, b);
                        if (r.status != GL_TRACE_OK) continue;
                        mnx = r.x < mnx ? r.x : mnx; mxx = r.x > mxx ? r.x : mxx;
                        mny = r.y < mny ? r.y : mny; mxy = r.y > mxy ? r.y : mxy;
                        ++valid;
                    }
                if (valid >= 2) { fpw = mxx - mnx; fph = mxy - mny; }
                if (normalize && valid >= 2)
                {
                    float gw = (mxx - mnx) > 0.01f ? (mxx - mnx) : 0.01f;
                    float gh = (mxy - mny) > 0.01f ? (mxy - mny) : 0.01f;
                    float area = (gw * gh) / ((2.0f * hw) * (2.0f * hh));
                    boost = (area < 1.0f) ? 1.0f : (max_boost < area ? max_boost : area);
                }
            }
            if (kept < cap)
            {
                out_ab[2 * kept] = a; out_ab[2 * kept + 1] = b; out_boost[kept] = boost;
                if (out_fp) { out_fp[2 * kept] = fpw; out_fp[2 * kept + 1] = fph; }
            }
            ++kept;
        }
    }
    return kept;
}

/* PupilMask::contains + build_aperture_samples, aperture_sampler.h:49-223
 * (plain polygon stop or blades override). */
static uint32_t orc_wang(uint32_t s)
{
    s = (s ^ 61u) ^ (s >> 16u);
    s *= 9u; s ^= s >> 4u; s *= 0x27d4eb2du; s ^= s >> 15u;
    return s;
}
static float orc_halton2(uint32_t n)
{
    n = (n << 16u) | (n >> 16u);
    n = ((n & 0x00ff00ffu) << 8u) | ((n & 0xff00ff00u) >> 8u);
    n = ((n & 0x0f0f0f0fu) << 4u) | ((n & 0xf0f0f0f0u) >> 4u);
    n = ((n & 0x33333333u) << 2u) | ((n & 0xccccccccu) >> 2u);
    n = ((n & 0x55555555u) << 1u) | ((n & 0xaaaaaaaau) >> 1u);
    return (float)n * (1.0f / 4294967296.0f);
}
static float orc_halton3(uint32_t n)
{
    float r = 0.0f, f = 1.0f / 3.0f;
    while (n > 0) { r += (n % 3u) * f; n /= 3u; f /= 3.0f; }
    return r;
}

/* Boundary radius of a stop's blade silhouette (normalised, float) at
 * angles theta[0..n): the profile of an authored stop, the plain n-gon's
 * otherwise. */
int orc_blade_radius(const gl_surface* stop, const float* theta, int n, float* out)
{
    if (!stop || stop->aperture_shape != GL_APERTURE_POLYGON || stop->aperture_blades < 3) return -1;
    orc_blade b = orc_make_blade(stop);
    for (int i = 0; i < n; ++i) out[i] = blade_radius_f32(&b, theta[i]);
    return 0;
}

int orc_aperture_samples(const gl_surface* S, int N, int grid, int jitter, int seed,
                         int blades_override, float rotation_deg, float* out_uv, int cap)
{
    int nb = 0; float rot = 0.0f, aspect = 1.0f;
    int deformed = 0;
    orc_blade blade;
    memset(&blade, 0, sizeof(blade));
    for (int i = 0; i < N; ++i)
    {
        if (!S[i].is_stop) continue;
        aspect = S[i].aperture_aspect;
        if (S[i].aperture_shape == GL_APERTURE_POLYGON && S[i].aperture_blades >= 3)
        {
            nb = S[i].aperture_blades; rot = S[i].aperture_rotation_rad;
            if (orc_blade_authored(&S[i])) { blade = orc_make_blade(&S[i]); deformed = blade.deformed; }
        }
        break;
    }
    if (blades_override > 0) { nb = blades_override; rot = rotation_deg * ((float)M_PI / 180.0f); deformed = 0; }
    const int poly = nb >= 3;
    const float apothem = poly ? cosf((float)M_PI / nb) : 1.0f;
    const float sector = poly ? (2.0f * (float)M_PI / nb) : 1.0f;
    const uint32_t so = (uint32_t)seed * 1000003u;
    int k_out = 0;
    for (int k = 0; k < grid * grid; ++k)
    {
        const int gx = k % grid, gy = k / grid;
        float u, v;
        if (jitter == 2) { u = orc_halton2((uint32_t)k) * 2.0f - 1.0f; v = orc_halton3((uint32_t)k) * 2.0f - 1.0f; }
        else
        {
            float ju = (jitter == 1) ? orc_wang((uint32_t)k + so) / 4294967296.0f : 0.5f;
            float jv = (jitter == 1) ? orc_wang((uint32_t)k + (uint32_t)(grid * grid) + so) / 4294967296.0f : 0.5f;
            u = ((gx + ju) / grid) * 2.0f - 1.0f;
            v = ((gy + jv) / grid) * 2.0f - 1.0f;
        }
        const float ux = u / aspect, r2 = ux * ux + v * v;
        if (r2 > 1.0f) continue;
        if (poly && deformed)
        {
            if (!(sqrtf(r2) <= blade_radius_f32(&blade, atan2f(v, ux)))) continue;
        }
        else if (poly)
        {
            float ang = atan2f(v, ux) - rot;
            float sec = fmodf(ang, sector);
            if (sec < 0.0f) sec += sector;
            if (sqrtf(r2) * cosf(sec - sector * 0.5f) > apothem) continue;
        }
        if (k_out < cap) { out_uv[2 * k_out] = u; out_uv[2 * k_out + 1] = v; }
        ++k_out;
    }
    return k_out;
}

/* PupilMask::contains (aperture_sampler.h:63-82) of the lens's stop at the
 * points uv[2k], uv[2k+1] -> out[k]; aspect_one forces the ellipse round. */
int orc_pupil_contains(const gl_surface* S, int N, int blades_override, float rotation_deg, int aspect_one,
                       const float* uv, int n_pts, unsigned char* out)
{
    int nb = 0; float rot = 0.0f, aspect = 1.0f;
    int deformed = 0;
    orc_blade blade;
    memset(&blade, 0, sizeof(blade));
    for (int i = 0; i < N; ++i)
    {
        if (!S[i].is_stop) continue;
        aspect = S[i].aperture_aspect;
        if (S[i].aperture_shape == GL_APERTURE_POLYGON && S[i].aperture_blades >= 3)
        {
            nb = S[i].aperture_blades; rot = S[i].aperture_rotation_rad;
            if (orc_blade_authored(&S[i])) { blade = orc_make_blade(&S[i]); deformed = blade.deformed; }
        }
        break;
    }
    if (blades_override > 0) { nb = blades_override; rot = rotation_deg * ((float)M_PI / 180.0f); deformed = 0; }
    if (aspect_one) aspect = 1.0f;
    const int poly = nb >= 3;
    const float apothem = poly ? cosf((float)M_PI / nb) : 1.0f;
    const float sector = poly ? (2.0f * (float)M_PI / nb) : 1.0f;
    for (int k = 0; k < n_pts; ++k)
    {
        const float u = uv[2 * k], v = uv[2 * k + 1];
        const float ux = u / aspect, r2 = ux * ux + v * v;
        int in = r2 <= 1.0f;
        if (in && poly && deformed) in = sqrtf(r2) <= blade_radius_f32(&blade, atan2f(v, ux));
        else if (in && poly)
        {
            float ang = atan2f(v, ux) - rot;
            float sec = fmodf(ang, sector);
            if (sec < 0.0f) sec += sector;
            in = !(sqrtf(r2) * cosf(sec - sector * 0.5f) > apothem);
        }
        out[k] = (unsigned char)in;
    }
    return 0;
}

/* Host mirror of the ghost kernel's full-pupil main path
 * (ghost_render.cu:280-463): per pair, source, pupil sample and wavelength,
 * trace and splat bilinearly.  pair_grid / grid_offsets select each pair's
 * pupil grid (one shared grid when pair_grid is NULL).  fp64 selects the
 * double instantiation.  out: 3 planes of W*H doubles. */
int orc_render(const gl_surface* S, int N, const int* pairs_ab, const float* boosts,
               const int* pair_grid, int n_pairs, const float* src5, int n_src,
               const float* grid_uv, const int* grid_offsets, const float* spec4, int n_spec,
               float hw, float hh, int W, int H, float gain, int fp64, int n_threads, double* out)
{
    const size_t npx = (size_t)W * H;
    if (n_threads > 0) omp_set_num_threads(n_threads);
    int nt = omp_get_max_threads();
    double* acc = (double*)calloc((size_t)nt * 3 * npx, sizeof(double));
    if (!acc) return -1;
    const float front_R = S[0].semi_aperture, start_z = S[0].z - 20.0f;
    for (int pi = 0; pi < n_pairs; ++pi)
    {
        const int g = pair_grid ? pair_grid[pi] : 0;
        const int g0 = grid_offsets[g], ng = grid_offsets[g + 1] - g0;
        if (ng <= 0) continue;
        const int a = pairs_ab[2 * pi], b = pairs_ab[2 * pi + 1];
        const long long n_work = (long long)n_src * ng;
        #pragma omp parallel for schedule(dynamic, 64)
        for (long long wi = 0; wi < n_work; ++wi)
        {
            double* img = acc + (size_t)omp_get_thread_num() * 3 * npx;
            const int si = (int)(wi / ng), gi = (int)(wi % ng);
            const float* sr = src5 + 5 * si;
            const float u = grid_uv[2 * (g0 + gi)], v = grid_uv[2 * (g0 + gi) + 1];
            if (fp64)
            {
                const double bx = tan((double)sr[0]), by = tan((double)sr[1]);
                const double w_ray = 1.0 / ng;
                v3_f64 d = normalized_f64(mk_f64(bx, by, 1.0));
                v3_f64 o = mk_f64(u * (double)front_R - 20.0 * bx, v * (double)front_R - 20.0 * by,
                                  (double)S[0].z - 20.0);
                for (int li = 0; li < n_spec; ++li)
                {
                    const float* sp = spec4 + 4 * li;
                    result_f64 r = trace_ghost_f64(S, N, o, d, sp[0], a, b);
                    if (r.status != GL_TRACE_OK || !isfinite(r.x) || !isfinite(r.y)) continue;
                    double base = r.w * w_ray * gain * boosts[pi];
                    if (base < 1e-14) continue;
                    double px = (r.x / (2.0 * hw) + 0.5) * W, py = (r.y / (2.0 * hh) + 0.5) * H;
                    if (!isfinite(px) || !isfinite(py)) continue;
                    px = fmax(-2.0e9, fmin(2.0e9, px)); py = fmax(-2.0e9, fmin(2.0e9, py));
                    double P = sr[2] * (double)sp[1] + sr[3] * (double)sp[2] + sr[4] * (double)sp[3];
                    double power = P * base;
                    splat_f64(img, W, H, px, py, power * sp[1], power * sp[2], power * sp[3]);
                }
            }
            else
            {
                const float bx = tanf(sr[0]), by = tanf(sr[1]);
                const float w_ray = 1.0f / (float)ng;
                v3_f32 d = normalized_f32(mk_f32(bx, by, 1.0f));
                v3_f32 o = mk_f32(u * front_R + (-20.0f * bx), v * front_R + (-20.0f * by), start_z);
                for (int li = 0; li < n_spec; ++li)
                {
                    const float* sp = spec4 + 4 * li;
                    result_f32 r = trace_ghost_f32(S, N, o, d, sp[0], a, b);
                    if (r.status != GL_TRACE_OK || !isfinite(r.x) || !isfinite(r.y)) continue;
                    float base = r.w * w_ray * gain * boosts[pi];
                    if (base < 1e-14f) continue;
                    float px = (r.x / (2.0f * hw) + 0.5f) * (float)W, py = (r.y / (2.0f * hh) + 0.5f) * (float)H;
                    if (!isfinite(px) || !isfinite(py)) continue;
                    px = fmaxf(-2.0e9f, fminf(2.0e9f, px)); py = fmaxf(-2.0e9f, fminf(2.0e9f, py));
                    float P = sr[2] * sp[1] + sr[3] * sp[2] + sr[4] * sp[3];
                    float power = P * base;
                    splat_f32(img, W, H, px, py, power * sp[1], power * sp[2], power * sp[3]);
                }
            }
        }
    }
    memset(out, 0, 3 * npx * sizeof(double));
    for (int t = 0; t < nt; ++t)
        for (size_t i = 0; i < 3 * npx; ++i) out[i] += acc[(size_t)t * 3 * npx + i];
    free(acc);
    return nt;
}
