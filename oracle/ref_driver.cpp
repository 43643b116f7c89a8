// ref_driver.cpp — C wrapper around the reference's own CPU code for the
// flare path (JaydenB/ghostlight, ghostlight/src).  TEST INFRASTRUCTURE ONLY:
// built by oracle/build.py into oracle/_ref/ from the reference sources where
// they lie, it is used to pin the oracle and to generate golden vectors, and as
// the CPU baseline when it is present.  Never shipped, never on the product
// path.
//
// The render harness at ref_render_ghosts_cpu mirrors the main path of the
// reference's ghost_kernel (ghostlight/src/ghost_render.cu:280-463, full pupil,
// no concentration) on the host: per pair, source, pupil sample and wavelength
// it calls the reference's trace_ghost_ray (trace.cpp:171) and splats the
// bilinear taps exactly as the kernel does (ghost_render.cu:423-463).
#include "optical_system.h"
#include "trace.h"
#include "ghost.h"
#include "aperture_sampler.h"
#include "spectral.h"
#include "lens_calibration.h"
#include "source_map.h"
#include "spawn_plane.h"

#include "ghostlight_gb300.h"

#include <cmath>
#include <cstring>
#include <map>
#include <vector>
#include <omp.h>

namespace {

// Coating tables by the id a table-coated flat record carries in ar_layers
// (the test registers each one with ref_coating_register); make_lens puts
// them into OpticalSystem::coating_tables the way the reference's own
// setters do (bind_geometry.cpp:412-513).
struct RefTable { int model, n0, n1, discard; float ref_ior; std::vector<float> data; };
std::map<int, RefTable> g_ref_tables;
// bitmap apertures by the id an IMAGE record carries in aperture_blades
struct RefImage { int w, h; float semi; std::vector<float> px; };
std::map<int, RefImage> g_ref_images;

void to_ref(const gl_surface& g, Surface& s)
{
    s = Surface{};
    s.radius = g.radius; s.thickness = g.thickness; s.ior = g.ior; s.abbe_v = g.abbe_v;
    s.semi_aperture = g.semi_aperture; s.z = g.z;
    s.is_stop = g.is_stop != 0; s.is_active = g.is_active != 0;
    s.aperture_shape = g.aperture_shape; s.aperture_blades = g.aperture_blades;
    s.aperture_rotation_rad = g.aperture_rotation_rad; s.aperture_aspect = g.aperture_aspect;
    s.aperture_curvature = g.aperture_curvature; s.aperture_twist = g.aperture_twist;
    s.aperture_notch_rad = g.aperture_notch_rad; s.aperture_notch_angle_rad = g.aperture_notch_angle_rad;
    s.decenter_x = g.decenter_x; s.decenter_y = g.decenter_y;
    for (int k = 0; k < 9; ++k) s.rot[k] = g.rot[k];
    s.form = g.form; s.conic_k = g.conic_k;
    for (int k = 0; k < 8; ++k) s.asphere_terms[k] = g.asphere_terms[k];
    s.n_asphere_terms = g.n_asphere_terms; s.cyl_axis = g.cyl_axis;
    s.disp_model = g.disp_model;
    for (int k = 0; k < 3; ++k) { s.sellmeier_B[k] = g.sellmeier_B[k]; s.sellmeier_C[k] = g.sellmeier_C[k]; }
    s.coating.model = (CoatingModel)g.coating_model;
    s.coating.ar_layers = g.ar_layers;
    s.coating.tint_r = g.tint_r; s.coating.tint_g = g.tint_g; s.coating.tint_b = g.tint_b;
    s.coating.tint_strength = g.tint_strength;
    s.coating.gauss_sigma = g.gauss_sigma; s.coating.gauss_background = g.gauss_background;
    s.coating.gauss_peak = g.gauss_peak;
    s.coating.gauss_decenter_x = g.gauss_decenter_x; s.coating.gauss_decenter_y = g.gauss_decenter_y;
    s.refresh_aperture_profile();
}

void from_ref(const Surface& s, gl_surface& g)
{
    std::memset(&g, 0, sizeof(g));
    g.radius = s.radius; g.thickness = s.thickness; g.ior = s.ior; g.abbe_v = s.abbe_v;
    g.semi_aperture = s.semi_aperture; g.z = s.z;
    g.is_stop = s.is_stop; g.is_active = s.is_active;
    g.aperture_shape = s.aperture_shape; g.aperture_blades = s.aperture_blades;
    g.aperture_rotation_rad = s.aperture_rotation_rad; g.aperture_aspect = s.aperture_aspect;
    g.aperture_curvature = s.aperture_curvature; g.aperture_twist = s.aperture_twist;
    g.aperture_notch_rad = s.aperture_notch_rad; g.aperture_notch_angle_rad = s.aperture_notch_angle_rad;
    g.decenter_x = s.decenter_x; g.decenter_y = s.decenter_y;
    for (int k = 0; k < 9; ++k) g.rot[k] = s.rot[k];
    g.form = s.form; g.conic_k = s.conic_k;
    for (int k = 0; k < 8; ++k) g.asphere_terms[k] = s.asphere_terms[k];
    g.n_asphere_terms = s.n_asphere_terms; g.cyl_axis = s.cyl_axis;
    g.disp_model = s.disp_model;
    for (int k = 0; k < 3; ++k) { g.sellmeier_B[k] = s.sellmeier_B[k]; g.sellmeier_C[k] = s.sellmeier_C[k]; }
    g.coating_model = (int)s.coating.model; g.ar_layers = s.coating.ar_layers;
    g.tint_r = s.coating.tint_r; g.tint_g = s.coating.tint_g; g.tint_b = s.coating.tint_b;
    g.tint_strength = s.coating.tint_strength;
    g.gauss_sigma = s.coating.gauss_sigma; g.gauss_background = s.coating.gauss_background;
    g.gauss_peak = s.coating.gauss_peak;
    g.gauss_decenter_x = s.coating.gauss_decenter_x; g.gauss_decenter_y = s.coating.gauss_decenter_y;
}

// Build an OpticalSystem from the flat table.  z is taken verbatim (the caller
// already laid it out); finalize() is not re-run so the two sides trace the
// same numbers.
OpticalSystem* make_lens(const gl_surface* surfs, int n)
{
    OpticalSystem* L = new OpticalSystem();
    L->surfaces.resize(n);
    for (int i = 0; i < n; ++i) to_ref(surfs[i], L->surfaces[i]);
    L->surface_ids.resize(n);
    L->aperture_images.resize(n);
    L->coating_tables.resize(n);
    for (int i = 0; i < n; ++i)
    {
        const int m = surfs[i].coating_model;
        if (m < 1 || m > 3) continue;
        Coating& c = L->surfaces[i].coating;
        c.ar_layers = 0;
        auto it = g_ref_tables.find(surfs[i].ar_layers);
        if (it == g_ref_tables.end() || it->second.model != m) continue;
        const RefTable& t = it->second;
        CoatingTables& ct = L->coating_tables[i];
        if (m == 3)
        {
            ct.sa_wavelengths.assign(t.data.begin(), t.data.begin() + t.n0);
            ct.sa_angles.assign(t.data.begin() + t.n0, t.data.begin() + t.n0 + t.n1);
            ct.sa_r.assign(t.data.begin() + t.n0 + t.n1, t.data.end());
        }
        else
        {
            for (int k = 0; k < t.n0; ++k) ct.table.push_back({t.data[k], t.data[t.n0 + k]});
        }
        c.out_of_range_discard = t.discard != 0;
        c.angle_ref_ior = t.ref_ior;
    }
    for (int i = 0; i < n; ++i)
    {
        if (surfs[i].aperture_shape != (int)APERTURE_IMAGE) continue;
        L->surfaces[i].aperture_blades = 0;
        auto it = g_ref_images.find(surfs[i].aperture_blades);
        if (it == g_ref_images.end()) continue;
        ApertureImage& img = L->aperture_images[i];
        img.width = it->second.w;
        img.height = it->second.h;
        img.pixels = it->second.px;
        img.semi_diameter = it->second.semi;
        L->surfaces[i].aperture_semi_diameter = it->second.semi;
    }
    L->sync_coating_pointers();
    return L;
}

FlareConfig make_filter_cfg(float min_int, int normalize, float max_boost)
{
    FlareConfig c;
    c.min_ghost_intensity = min_int;
    c.ghost_normalize = normalize != 0;
    c.max_area_boost = max_boost;
    return c;
}

} // namespace

extern "C" {

int ref_sizeof_surface() { return (int)sizeof(gl_surface); }

int ref_image_register(int id, int w, int h, const float* px, float semi)
{
    g_ref_images[id] = RefImage{w, h, semi, std::vector<float>(px, px + (size_t)w * h)};
    return 0;
}

int ref_coating_register(int id, int model, int n0, int n1, const float* data, float ref_ior, int discard)
{
    RefTable t{model, n0, n1, discard, ref_ior, {}};
    const size_t len = (size_t)n0 + n1 + (n1 ? (size_t)n0 * n1 : (size_t)n0);
    t.data.assign(data, data + len);
    g_ref_tables[id] = std::move(t);
    return 0;
}

// OpticalSystem::bake_coating_layers on surface `index` of a flat table:
// out_wl[31], out_ang[18], out_r[31*18], *ref_ior.  Layers as
// gl_coating_bake_layers takes them.
int ref_bake_layers(const gl_surface* surfs, int n, int index, int n_layers, const float* thickness_nm,
                    const int* nk_count, const float* nk_lambda_um, const float* nk_n, const float* nk_k,
                    float* out_wl, float* out_ang, float* out_r, float* ref_ior)
{
    OpticalSystem* L = make_lens(surfs, n);
    int o = 0;
    for (int l = 0; l < n_layers; ++l)
    {
        CoatingLayerSpec spec;
        spec.thickness_nm = thickness_nm[l];
        for (int k = 0; k < nk_count[l]; ++k)
        {
            spec.nk_lambda_um.push_back(nk_lambda_um[o + k]);
            spec.nk_n.push_back(nk_n[o + k]);
            spec.nk_k.push_back(nk_k[o + k]);
        }
        o += nk_count[l];
        L->coating_tables[index].layers.push_back(spec);
    }
    std::string err;
    const bool ok = L->bake_coating_layers(index, &err);
    int rc = -1;
    const CoatingTables& t = L->coating_tables[index];
    if (ok && t.sa_wavelengths.size() == 31 && t.sa_angles.size() == 18)
    {
        std::memcpy(out_wl, t.sa_wavelengths.data(), 31 * 4);
        std::memcpy(out_ang, t.sa_angles.data(), 18 * 4);
        std::memcpy(out_r, t.sa_r.data(), 31 * 18 * 4);
        *ref_ior = L->surfaces[index].coating.angle_ref_ior;
        rc = 0;
    }
    delete L;
    return rc;
}

// The coating tables the reference loader gives surface `index` of a lens
// file: model, extents, discard flag and angle medium into meta
// (model, n0, n1, discard), ref_ior; the table as axis0 | axis1 | r into
// data (cap floats).  Returns the float count, or -1.
int ref_load_lens_coating(const char* path, int index, int* meta, float* ref_ior, float* data, int cap)
{
    OpticalSystem L;
    if (!L.load(path) || index < 0 || index >= L.num_surfaces()) return -1;
    const Coating& c = L.surfaces[index].coating;
    const CoatingTables& t = L.coating_tables[index];
    std::vector<float> d;
    int n0 = 0, n1 = 0;
    if (!t.table.empty())
    {
        n0 = (int)t.table.size();
        for (const auto& e : t.table) d.push_back(e.key);
        for (const auto& e : t.table) d.push_back(e.r);
    }
    else if (!t.sa_r.empty())
    {
        n0 = (int)t.sa_wavelengths.size();
        n1 = (int)t.sa_angles.size();
        d.insert(d.end(), t.sa_wavelengths.begin(), t.sa_wavelengths.end());
        d.insert(d.end(), t.sa_angles.begin(), t.sa_angles.end());
        d.insert(d.end(), t.sa_r.begin(), t.sa_r.end());
    }
    meta[0] = (int)c.model; meta[1] = n0; meta[2] = n1; meta[3] = c.out_of_range_discard ? 1 : 0;
    *ref_ior = c.angle_ref_ior;
    if (data) for (int k = 0; k < (int)d.size() && k < cap; ++k) data[k] = d[(size_t)k];
    return (int)d.size();
}

// Load a .lens file with the reference loader; returns the surface count, or
// -1 on failure.  out may be NULL to query the count.
int ref_load_lens(const char* path, gl_surface* out, int cap, float* focal_length)
{
    OpticalSystem L;
    if (!L.load(path)) return -1;
    const int n = L.num_surfaces();
    if (out) for (int i = 0; i < n && i < cap; ++i) from_ref(L.surfaces[i], out[i]);
    if (focal_length) *focal_length = L.focal_length;
    return n;
}

// OpticalSystem::finalize on a flat table (fills z).
int ref_finalize(gl_surface* surfs, int n)
{
    OpticalSystem L;
    L.surfaces.resize(n);
    for (int i = 0; i < n; ++i) to_ref(surfs[i], L.surfaces[i]);
    if (!L.finalize()) return -1;
    for (int i = 0; i < n; ++i) surfs[i].z = L.surfaces[i].z;
    return 0;
}

// rays: n x 7 (ox,oy,oz,dx,dy,dz,lambda); out: n x 5 (x,y,z,w,status).
// bounce_b < 0 traces a primary ray.
int ref_trace(const gl_surface* surfs, int n, int a, int b,
              const float* rays, int n_rays, float* out)
{
    OpticalSystem* L = make_lens(surfs, n);
    for (int i = 0; i < n_rays; ++i)
    {
        Ray r;
        r.origin = Vec3f(rays[7*i+0], rays[7*i+1], rays[7*i+2]);
        r.dir    = Vec3f(rays[7*i+3], rays[7*i+4], rays[7*i+5]);
        r.lambda = rays[7*i+6];
        TraceResult t = (b < 0) ? trace_primary_ray(r, *L) : trace_ghost_ray(r, *L, a, b);
        out[5*i+0] = t.position.x; out[5*i+1] = t.position.y; out[5*i+2] = t.position.z;
        out[5*i+3] = t.weight;     out[5*i+4] = (float)(int)t.status;
    }
    delete L;
    return 0;
}

int ref_enumerate(const gl_surface* surfs, int n, int* out_ab, int cap)
{
    OpticalSystem* L = make_lens(surfs, n);
    std::vector<GhostPair> p = enumerate_ghost_pairs(*L);
    delete L;
    for (size_t i = 0; i < p.size() && (int)i < cap; ++i) { out_ab[2*i] = p[i].surf_a; out_ab[2*i+1] = p[i].surf_b; }
    return (int)p.size();
}

int ref_filter(const gl_surface* surfs, int n, float hw, float hh,
               float min_int, int normalize, float max_boost,
               int* out_ab, float* out_boost, int cap)
{
    OpticalSystem* L = make_lens(surfs, n);
    std::vector<GhostPair> pairs; std::vector<float> boosts;
    filter_ghost_pairs(*L, hw, hh, make_filter_cfg(min_int, normalize, max_boost), pairs, boosts);
    delete L;
    for (size_t i = 0; i < pairs.size() && (int)i < cap; ++i)
    {
        out_ab[2*i] = pairs[i].surf_a; out_ab[2*i+1] = pairs[i].surf_b; out_boost[i] = boosts[i];
    }
    return (int)pairs.size();
}

int ref_aperture_samples(const gl_surface* surfs, int n, int ray_grid, int jitter,
                         int seed, int blades_override, float rotation_deg,
                         float* out_uv, int cap)
{
    OpticalSystem* L = make_lens(surfs, n);
    ApertureSamplerParams p;
    p.ray_grid = ray_grid; p.pupil_jitter = jitter; p.jitter_seed = seed;
    p.blades_override = blades_override; p.rotation_deg = rotation_deg;
    std::vector<ApertureSample> s = build_aperture_samples(*L, p);
    delete L;
    for (size_t i = 0; i < s.size() && (int)i < cap; ++i) { out_uv[2*i] = s[i].u; out_uv[2*i+1] = s[i].v; }
    return (int)s.size();
}

// out: n x 4 (lambda, cmf_r, cmf_g, cmf_b); corr: 9 floats (identity when
// correction is off or n == 3, matching ghost_render.cu:781-798).
int ref_spectral_table(int n, int output_cs, float* out, float* corr)
{
    std::vector<GPUSpectralSample> t;
    for (int k = 0; k < 9; ++k) corr[k] = (k % 4 == 0) ? 1.0f : 0.0f;
    if (n == 3)
    {
        t = {{650.0f, 1, 0, 0}, {550.0f, 0, 1, 0}, {450.0f, 0, 0, 1}};
    }
    else
    {
        const SensorProfile& prof = get_sensor_profile(SENSOR_CIE_1931);
        float M[3][3]; float custom[3][3] = {};
        resolve_output_matrix((OutputColorSpace)output_cs, custom, M);
        t = build_spectral_table(n, 400.0f, 700.0f, prof, M);
        float C[3][3];
        compute_spectral_correction(t, 400.0f, 700.0f, prof, M, C);
        for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) corr[3*r+c] = C[r][c];
    }
    for (int i = 0; i < (int)t.size(); ++i)
    {
        out[4*i+0] = t[i].lambda; out[4*i+1] = t[i].cmf_r;
        out[4*i+2] = t[i].cmf_g;  out[4*i+3] = t[i].cmf_b;
    }
    return (int)t.size();
}

// The built-in CIE 1931 2-degree observer table (spectral.cpp get_sensor_profile).
int ref_cie_profile(float* wl, float* x, float* y, float* z, int cap)
{
    const SensorProfile& p = get_sensor_profile(SENSOR_CIE_1931);
    for (int i = 0; i < p.count && i < cap; ++i)
    { wl[i] = p.wavelengths[i]; x[i] = p.sens_r[i]; y[i] = p.sens_g[i]; z[i] = p.sens_b[i]; }
    return p.count;
}

int ref_color_matrices(int input_cs, int output_cs, float* m_in, float* m_out)
{
    float custom[3][3] = {}; float A[3][3], B[3][3];
    resolve_input_matrix((InputColorSpace)input_cs, custom, A);
    resolve_output_matrix((OutputColorSpace)output_cs, custom, B);
    for (int r = 0; r < 3; ++r) for (int c = 0; c < 3; ++c) { m_in[3*r+c] = A[r][c]; m_out[3*r+c] = B[r][c]; }
    return 0;
}

// out (13 floats): sensor_half_w, sensor_half_h, max_half_angle_h, max_half_angle_v,
// image_circle_semi_w, image_circle_semi_h, focal_length_x, focal_length_y,
// entrance_pupil_semi_x, entrance_pupil_semi_y, f_number_x, f_number_y, pupil_area_frac
int ref_calibrate(const gl_surface* surfs, int n, float focal_length, float* out)
{
    OpticalSystem* L = make_lens(surfs, n);
    L->focal_length = focal_length;
    LensCalibration c = calibrate_lens(*L, 587.56f);
    delete L;
    const float v[13] = {c.sensor_half_w, c.sensor_half_h, c.max_half_angle_h, c.max_half_angle_v,
                         c.image_circle_semi_w, c.image_circle_semi_h, c.focal_length_x,
                         c.focal_length_y, c.entrance_pupil_semi_x, c.entrance_pupil_semi_y,
                         c.f_number_x, c.f_number_y, c.pupil_area_frac};
    for (int k = 0; k < 13; ++k) out[k] = v[k];
    return 0;
}

// Source-position solve (source_map.cpp:182) and its forward map at the
// solved angle (:456).  out: angle_x, angle_y, status, screen_x, screen_y.
int ref_solve_source(const gl_surface* surfs, int n, const float* calib13,
                     float ndc_x, float ndc_y, float eff_hw, float eff_hh, float* out)
{
    OpticalSystem* L = make_lens(surfs, n);
    LensCalibration c{};
    c.sensor_half_w = calib13[0]; c.sensor_half_h = calib13[1];
    c.max_half_angle_h = calib13[2]; c.max_half_angle_v = calib13[3];
    c.image_circle_semi_w = calib13[4]; c.image_circle_semi_h = calib13[5];
    c.focal_length_x = calib13[6]; c.focal_length_y = calib13[7];
    c.entrance_pupil_semi_x = calib13[8]; c.entrance_pupil_semi_y = calib13[9];
    c.f_number_x = calib13[10]; c.f_number_y = calib13[11]; c.pupil_area_frac = calib13[12];
    SourceMapSolve s = solve_source_angle(*L, c, ndc_x, ndc_y, eff_hw, eff_hh);
    float sx = 0, sy = 0;
    source_map_screen(s, s.angle_x, s.angle_y, &sx, &sy);
    delete L;
    out[0] = s.angle_x; out[1] = s.angle_y; out[2] = (float)(int)s.status;
    out[3] = sx; out[4] = sy;
    return 0;
}

// Host mirror of ghost_kernel's main path (ghost_render.cu:280-463): full
// pupil (no concentration), bilinear point splat.  out: 3 planes of W*H,
// accumulated in double then rounded.  Threads: OpenMP over (pair, sample).
int ref_render_ghosts_cpu(const gl_surface* surfs, int n,
                          const int* pairs_ab, const float* boosts, int n_pairs,
                          const float* sources5, int n_src,
                          const float* grid_uv, int n_grid,
                          const float* spec4, int n_spec,
                          float hw, float hh, int W, int H, float gain,
                          int n_threads, float* out_rgb)
{
    OpticalSystem* L = make_lens(surfs, n);
    const float front_R = L->surfaces[0].semi_aperture;
    const float start_z = L->surfaces[0].z - SPAWN_OFFSET;
    const float ray_weight = 1.0f / (float)n_grid;
    const size_t npx = (size_t)W * H;
    if (n_threads > 0) omp_set_num_threads(n_threads);
    int nt = 1;
    #pragma omp parallel
    {
        #pragma omp single
        nt = omp_get_num_threads();
    }
    std::vector<std::vector<double>> acc(nt, std::vector<double>(3 * npx, 0.0));
    const long long n_work = (long long)n_pairs * n_src * n_grid;
    #pragma omp parallel for schedule(dynamic, 256)
    for (long long wi = 0; wi < n_work; ++wi)
    {
        const int tid = omp_get_thread_num();
        double* img = acc[tid].data();
        const int gi  = (int)(wi % n_grid);
        const int ps  = (int)(wi / n_grid);
        const int pi  = ps / n_src, si = ps % n_src;
        const int a = pairs_ab[2*pi], b = pairs_ab[2*pi+1];
        const float* src = sources5 + 5 * si;
        const float u = grid_uv[2*gi], v = grid_uv[2*gi+1];
        const float bx = tanf(src[0]), by = tanf(src[1]);
        const Vec3f beam = Vec3f(bx, by, 1.0f).normalized();
        float sdx, sdy; spawn_shift(bx, by, sdx, sdy);
        for (int li = 0; li < n_spec; ++li)
        {
            Ray r;
            r.origin = Vec3f(u * front_R + sdx, v * front_R + sdy, start_z);
            r.dir = beam;
            r.lambda = spec4[4*li];
            TraceResult res = trace_ghost_ray(r, *L, a, b);
            if (res.status != TraceStatus::OK) continue;
            if (!std::isfinite(res.position.x) || !std::isfinite(res.position.y)) continue;
            float base = res.weight * ray_weight * gain * boosts[pi];
            if (base < 1e-14f) continue;
            float px = (res.position.x / (2.0f * hw) + 0.5f) * (float)W;
            float py = (res.position.y / (2.0f * hh) + 0.5f) * (float)H;
            if (!std::isfinite(px) || !std::isfinite(py)) continue;
            px = std::fmax(-2.0e9f, std::fmin(2.0e9f, px));
            py = std::fmax(-2.0e9f, std::fmin(2.0e9f, py));
            int x0 = (int)std::floor(px - 0.5f), y0 = (int)std::floor(py - 0.5f);
            float fx = (px - 0.5f) - (float)x0, fy = (py - 0.5f) - (float)y0;
            const float wt[4] = {(1.0f - fx) * (1.0f - fy), fx * (1.0f - fy),
                                 (1.0f - fx) * fy, fx * fy};
            const int ox[4] = {0, 1, 0, 1}, oy[4] = {0, 0, 1, 1};
            const float* sp = spec4 + 4 * li;
            float P = src[2] * sp[1] + src[3] * sp[2] + src[4] * sp[3];
            float power = P * base;
            float c[3] = {power * sp[1], power * sp[2], power * sp[3]};
            for (int k = 0; k < 4; ++k)
            {
                int xi = x0 + ox[k], yi = y0 + oy[k];
                if (xi < 0 || xi >= W || yi < 0 || yi >= H) continue;
                size_t pix = (size_t)yi * W + xi;
                for (int ch = 0; ch < 3; ++ch)
                    if (std::fabs(c[ch]) > 1e-14f) img[ch * npx + pix] += (double)(c[ch] * wt[k]);
            }
        }
    }
    for (size_t i = 0; i < 3 * npx; ++i)
    {
        double s = 0.0;
        for (int t = 0; t < nt; ++t) s += acc[t][i];
        out_rgb[i] = (float)s;
    }
    delete L;
    return nt;
}

} // extern "C"
