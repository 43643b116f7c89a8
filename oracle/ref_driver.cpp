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

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>
#include <omp.h>

#ifdef REF_GPU
#include "PointFlareRenderer.h"
#include "SourceFlareRenderer.h"
#include "render_config.h"
#include <cuda_runtime.h>
#endif

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

// ---------------------------------------------------------------------------
// One full frame of the ghost layer on the host, for the CPU reference arm.
// The reference has no CPU flare renderer, so this harness restates the host
// side of launch_ghost_render around the reference's own trace:
//  * the off-sensor cull of probe_cull_and_concentrate (ghost_render.cu:
//    976-1080, concentration off): pass 0 probes every pair with a 40^2
//    wang-jittered pupil grid (jitter seed 0x9E3779B9 * (pass + 1)) at every
//    wavelength against the sensor inflated by 1.25; passes 1-2 re-probe the
//    pairs still without an on-sensor landing; a pair none of them lands is
//    not rendered;
//  * the main path of ghost_kernel (ghost_render.cu:280-463) for every kept
//    pair over its own regular pupil grid (build_aperture_samples, no jitter)
//    with ray weight 1 / n_grid of that grid, splatted bilinearly;
//  * the colour correction of spectral_correct_kernel (:610-622).
// Threads: OpenMP over (pair, pupil sample); one float image per thread,
// summed at the end.  counts: {probe traces, render traces, kept pairs}.
// ---------------------------------------------------------------------------
namespace {

inline void splat_point(float* img, size_t npx, int W, int H, float hw, float hh,
                        const TraceResult& res, float base, const float* src, const float* sp)
{
    float px = (res.position.x / (2.0f * hw) + 0.5f) * (float)W;
    float py = (res.position.y / (2.0f * hh) + 0.5f) * (float)H;
    if (!std::isfinite(px) || !std::isfinite(py)) return;
    px = std::fmax(-2.0e9f, std::fmin(2.0e9f, px));
    py = std::fmax(-2.0e9f, std::fmin(2.0e9f, py));
    const int x0 = (int)std::floor(px - 0.5f), y0 = (int)std::floor(py - 0.5f);
    const float fx = (px - 0.5f) - (float)x0, fy = (py - 0.5f) - (float)y0;
    const float wt[4] = {(1.0f - fx) * (1.0f - fy), fx * (1.0f - fy), (1.0f - fx) * fy, fx * fy};
    const int ox[4] = {0, 1, 0, 1}, oy[4] = {0, 0, 1, 1};
    const float P = src[2] * sp[1] + src[3] * sp[2] + src[4] * sp[3];
    const float power = P * base;
    const float c[3] = {power * sp[1], power * sp[2], power * sp[3]};
    for (int k = 0; k < 4; ++k)
    {
        const int xi = x0 + ox[k], yi = y0 + oy[k];
        if (xi < 0 || xi >= W || yi < 0 || yi >= H) continue;
        const size_t pix = (size_t)yi * W + xi;
        for (int ch = 0; ch < 3; ++ch)
            if (std::fabs(c[ch]) > 1e-14f) img[ch * npx + pix] += c[ch] * wt[k];
    }
}

}  // namespace

extern "C" int ref_render_frame_cpu(const gl_surface* surfs, int n,
                                    const int* pairs_ab, const float* boosts, const int* pair_side, int n_pairs,
                                    const float* src5, const float* spec4, int n_spec, const float* corr9,
                                    float hw, float hh, int W, int H, float gain, int cull, int n_threads,
                                    float* out_rgb, long long* counts)
{
    OpticalSystem* L = make_lens(surfs, n);
    const float front_R = L->surfaces[0].semi_aperture;
    const float start_z = L->surfaces[0].z - SPAWN_OFFSET;
    const size_t npx = (size_t)W * H;
    if (n_threads > 0) omp_set_num_threads(n_threads);
    const float bx = tanf(src5[0]), by = tanf(src5[1]);
    const Vec3f beam = Vec3f(bx, by, 1.0f).normalized();
    float sdx, sdy; spawn_shift(bx, by, sdx, sdy);

    // pupil grids, one per distinct side
    std::map<int, std::vector<ApertureSample>> grids;
    for (int p = 0; p < n_pairs; ++p)
        if (!grids.count(pair_side[p]))
        {
            ApertureSamplerParams sp; sp.ray_grid = pair_side[p]; sp.pupil_jitter = 0; sp.jitter_seed = 0;
            grids[pair_side[p]] = build_aperture_samples(*L, sp);
        }

    // ---- off-sensor cull ----
    std::vector<char> keep(n_pairs, 1);
    long long probe_traces = 0;
    if (cull && n_pairs > 1 && n_spec != 3)
    {
        std::vector<char> cand(n_pairs, 1);
        const float mhw = hw * 1.25f, mhh = hh * 1.25f;
        for (int pass = 0; pass < 3; ++pass)
        {
            ApertureSamplerParams pp; pp.ray_grid = 40; pp.pupil_jitter = 1;
            pp.jitter_seed = (int)(0x9E3779B9u * (unsigned)(pass + 1));
            const std::vector<ApertureSample> probe = build_aperture_samples(*L, pp);
            const int np = (int)probe.size();
            if (np <= 0) { if (pass == 0) break; else continue; }
            std::vector<int> hit(n_pairs, 0);
            long long traces = 0;
            #pragma omp parallel for schedule(dynamic, 1) reduction(+:traces)
            for (int p = 0; p < n_pairs; ++p)
            {
                if (!cand[p]) continue;
                const int a = pairs_ab[2 * p], b = pairs_ab[2 * p + 1];
                int h = 0;
                for (int g = 0; g < np; ++g)
                    for (int li = 0; li < n_spec; ++li)
                    {
                        Ray r;
                        r.origin = Vec3f(probe[g].u * front_R + sdx, probe[g].v * front_R + sdy, start_z);
                        r.dir = beam; r.lambda = spec4[4 * li];
                        ++traces;
                        TraceResult res = trace_ghost_ray(r, *L, a, b);
                        if (res.status != TraceStatus::OK) continue;
                        if (!std::isfinite(res.position.x) || !std::isfinite(res.position.y)) continue;
                        const float spx = (res.position.x / (2.0f * mhw) + 0.5f) * (float)W;
                        const float spy = (res.position.y / (2.0f * mhh) + 0.5f) * (float)H;
                        if (std::isfinite(spx) && std::isfinite(spy) && spx >= 0.0f && spx < (float)W &&
                            spy >= 0.0f && spy < (float)H) ++h;
                    }
                hit[p] = h;
            }
            probe_traces += traces;
            int n_cand = 0;
            for (int p = 0; p < n_pairs; ++p)
                if (cand[p] && hit[p] > 0) cand[p] = 0;
                else if (cand[p]) ++n_cand;
            if (n_cand == 0) break;
        }
        for (int p = 0; p < n_pairs; ++p) keep[p] = cand[p] ? 0 : 1;
    }

    // ---- render: (pair, sample) work list over the kept pairs ----
    std::vector<long long> first(n_pairs + 1, 0);
    for (int p = 0; p < n_pairs; ++p)
        first[p + 1] = first[p] + (keep[p] ? (long long)grids[pair_side[p]].size() : 0);
    const long long n_work = first[n_pairs];
    std::vector<const std::vector<ApertureSample>*> gptr(n_pairs);
    for (int p = 0; p < n_pairs; ++p) gptr[p] = &grids[pair_side[p]];
    int nt = 1;
    #pragma omp parallel
    {
        #pragma omp single
        nt = omp_get_num_threads();
    }
    std::vector<std::vector<float>> acc(nt);
    long long render_traces = 0;
    #pragma omp parallel reduction(+:render_traces)
    {
        const int tid = omp_get_thread_num();
        acc[tid].assign(3 * npx, 0.0f);
        float* img = acc[tid].data();
        #pragma omp for schedule(dynamic, 512)
        for (long long wi = 0; wi < n_work; ++wi)
        {
            const int p = (int)(std::upper_bound(first.begin(), first.end(), wi) - first.begin()) - 1;
            const std::vector<ApertureSample>& g = *gptr[p];
            const ApertureSample& s = g[(size_t)(wi - first[p])];
            const float ray_weight = 1.0f / (float)g.size();
            const int a = pairs_ab[2 * p], b = pairs_ab[2 * p + 1];
            for (int li = 0; li < n_spec; ++li)
            {
                Ray r;
                r.origin = Vec3f(s.u * front_R + sdx, s.v * front_R + sdy, start_z);
                r.dir = beam; r.lambda = spec4[4 * li];
                ++render_traces;
                TraceResult res = trace_ghost_ray(r, *L, a, b);
                if (res.status != TraceStatus::OK) continue;
                if (!std::isfinite(res.position.x) || !std::isfinite(res.position.y)) continue;
                const float base = res.weight * ray_weight * gain * boosts[p];
                if (base < 1e-14f) continue;
                splat_point(img, npx, W, H, hw, hh, res, base, src5, spec4 + 4 * li);
            }
        }
    }
    // sum the thread images, then the colour correction
    #pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)npx; ++i)
    {
        float rgb[3];
        for (int ch = 0; ch < 3; ++ch)
        {
            float t = 0.0f;
            for (int k = 0; k < nt; ++k) t += acc[k][ch * npx + i];
            rgb[ch] = t;
        }
        for (int ch = 0; ch < 3; ++ch)
            out_rgb[ch * npx + i] = corr9 ? corr9[3 * ch] * rgb[0] + corr9[3 * ch + 1] * rgb[1] +
                                            corr9[3 * ch + 2] * rgb[2]
                                          : rgb[ch];
    }
    int kept = 0;
    for (int p = 0; p < n_pairs; ++p) kept += keep[p];
    if (counts) { counts[0] = probe_traces; counts[1] = render_traces; counts[2] = kept; }
    delete L;
    return nt;
}


// Landing extent of a ghost on the sensor (ghost_w, ghost_h; 0 when fewer than
// two probe rays land): the 8x8 on-axis probe at 550 nm of
// estimate_ghost_spread (ghost.cpp:53-102), traced with the reference's own
// trace_ghost_ray, for n_pairs pairs.
extern "C" int ref_ghost_footprints(const gl_surface* surfs, int n, const int* pairs_ab, int n_pairs,
                                    float* out_wh)
{
    OpticalSystem* L = make_lens(surfs, n);
    const float front_R = L->surfaces[0].semi_aperture;
    const float start_z = L->surfaces[0].z - SPAWN_OFFSET;
    for (int p = 0; p < n_pairs; ++p)
    {
        float mnx = 1e30f, mxx = -1e30f, mny = 1e30f, mxy = -1e30f;
        int valid = 0;
        for (int gy = 0; gy < 8; ++gy)
            for (int gx = 0; gx < 8; ++gx)
            {
                const float u = ((gx + 0.5f) / 8) * 2.0f - 1.0f;
                const float v = ((gy + 0.5f) / 8) * 2.0f - 1.0f;
                if (u * u + v * v > 1.0f) continue;
                Ray r;
                r.origin = Vec3f(u * front_R, v * front_R, start_z);
                r.dir = Vec3f(0, 0, 1);
                r.lambda = 550.0f;
                TraceResult res = trace_ghost_ray(r, *L, pairs_ab[2 * p], pairs_ab[2 * p + 1]);
                if (res.status != TraceStatus::OK) continue;
                mnx = std::min(mnx, res.position.x); mxx = std::max(mxx, res.position.x);
                mny = std::min(mny, res.position.y); mxy = std::max(mxy, res.position.y);
                ++valid;
            }
        out_wh[2 * p] = valid >= 2 ? mxx - mnx : 0.0f;
        out_wh[2 * p + 1] = valid >= 2 ? mxy - mny : 0.0f;
    }
    delete L;
    return 0;
}

#ifdef REF_GPU
// ---------------------------------------------------------------------------
// The reference's GPU renderer (render_point_flare / render_source_flare,
// PointFlareRenderer.cpp:11, SourceFlareRenderer.cpp:24) on a lens given as
// flat records.  Fields follow PointFlareConfig (render_config.h) by name.
// ---------------------------------------------------------------------------
struct RefGpuCfg {
    int ray_grid, spectral_samples, pupil_jitter, jitter_seed;
    float sensor_half_w, sensor_half_h, flare_gain, min_ghost_intensity;
    int cull_dead_pairs, concentrate_samples, adaptive_sample_budgets, aperture_blades;
    float source_x, source_y, source_r, source_g, source_b;
    int starburst, starburst_engine, starburst_grid, sb_spectral_samples;
    float pupil_fill, scale_trim;
    int spectral_correction, output_cs, use_survivor_mask, collect_stats;
    int veil, pad2;
    float veil_gain, veil_spread, veil_falloff;
};

extern "C" int refgpu_sizeof_cfg() { return (int)sizeof(RefGpuCfg); }

// calib13: the 13 calibration values (ref_calibrate order) or NULL to
// calibrate here.  offsets: n_offsets x 3 (render_source_flare) or NULL
// (render_point_flare).  out_ghost / out_star: 3 planes of W*H or NULL.
// ms: wall time of the render call (its own uploads, kernels and D2H).
// stats (8 doubles, or NULL; filled when collect_stats): the renderer's own
// GhostRenderStats ms_grid_build, ms_upload, ms_kernel, ms_download,
// ms_total, n_pairs, traces_total, traces_on_sensor.
// include_ab: n_include (a, b) pairs for GhostFilter INCLUDE (render_config.h:
// 51-62), or NULL for every filtered pair.
extern "C" int refgpu_render(const gl_surface* surfs, int n, float focal_length, const float* calib13,
                             const RefGpuCfg* g, const float* offsets, int n_offsets, int W, int H,
                             float* out_ghost, float* out_star, double* ms, double* stats,
                             const int* include_ab, int n_include, float* out_veil)
{
    OpticalSystem* L = make_lens(surfs, n);
    L->focal_length = focal_length;
    LensCalibration c{};
    if (calib13)
    {
        c.sensor_half_w = calib13[0]; c.sensor_half_h = calib13[1];
        c.max_half_angle_h = calib13[2]; c.max_half_angle_v = calib13[3];
        c.image_circle_semi_w = calib13[4]; c.image_circle_semi_h = calib13[5];
        c.focal_length_x = calib13[6]; c.focal_length_y = calib13[7];
        c.entrance_pupil_semi_x = calib13[8]; c.entrance_pupil_semi_y = calib13[9];
        c.f_number_x = calib13[10]; c.f_number_y = calib13[11]; c.pupil_area_frac = calib13[12];
    }
    else
        c = calibrate_lens(*L, 587.56f);
    PointFlareConfig cfg;
    cfg.ray_grid = g->ray_grid; cfg.spectral_samples = g->spectral_samples;
    cfg.pupil_jitter = g->pupil_jitter; cfg.jitter_seed = g->jitter_seed;
    cfg.sensor_half_w = g->sensor_half_w; cfg.sensor_half_h = g->sensor_half_h;
    cfg.flare_gain = g->flare_gain; cfg.min_ghost_intensity = g->min_ghost_intensity;
    cfg.cull_dead_pairs = g->cull_dead_pairs != 0; cfg.concentrate_samples = g->concentrate_samples != 0;
    cfg.adaptive_sample_budgets = g->adaptive_sample_budgets != 0;
    if (g->aperture_blades) cfg.aperture_blades = g->aperture_blades;
    cfg.source_x = g->source_x; cfg.source_y = g->source_y;
    cfg.source_r = g->source_r; cfg.source_g = g->source_g; cfg.source_b = g->source_b;
    cfg.spectral_correction = g->spectral_correction != 0;
    cfg.output_cs = (OutputColorSpace)g->output_cs;
    cfg.diffraction.starburst = g->starburst != 0;
    cfg.diffraction.starburst_engine = g->starburst_engine ? StarburstEngine::MDFT : StarburstEngine::SPRITE;
    cfg.diffraction.starburst_grid = g->starburst_grid;
    cfg.diffraction.spectral_samples = g->sb_spectral_samples;
    cfg.diffraction.pupil_fill = g->pupil_fill; cfg.diffraction.scale_trim = g->scale_trim;
    cfg.diffraction.use_survivor_mask = g->use_survivor_mask != 0;
    cfg.collect_stats = g->collect_stats != 0;
    cfg.diffraction.veil = g->veil != 0;
    if (g->veil)
    {
        cfg.diffraction.veil_gain = g->veil_gain;
        cfg.diffraction.veil_spread = g->veil_spread;
        cfg.diffraction.veil_falloff = g->veil_falloff;
    }
    if (include_ab && n_include > 0)
    {
        cfg.ghost_filter.mode = GhostFilter::Mode::INCLUDE;
        for (int i = 0; i < n_include; ++i) cfg.ghost_filter.pairs.emplace_back(include_ab[2 * i], include_ab[2 * i + 1]);
    }
    FlareBuffers out;
    const auto t0 = std::chrono::steady_clock::now();
    const bool ok = offsets ? render_source_flare(W, H, offsets, n_offsets, *L, c, cfg, out)
                            : render_point_flare(W, H, *L, c, cfg, out);
    const auto t1 = std::chrono::steady_clock::now();
    if (ms) *ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
    delete L;
    if (!ok) return -1;
    if (stats)
    {
        const GhostRenderStats& t = out.stats;
        const double v[8] = {t.ms_grid_build, t.ms_upload, t.ms_kernel, t.ms_download, t.ms_total,
                             (double)t.n_pairs, (double)t.traces_total, (double)t.traces_on_sensor};
        for (int k = 0; k < 8; ++k) stats[k] = out.has_stats ? v[k] : -1.0;
    }
    const size_t npx = (size_t)W * H;
    if (out_ghost)
    {
        const std::vector<float>* pl[3] = {&out.ghost_r, &out.ghost_g, &out.ghost_b};
        for (int k = 0; k < 3; ++k)
            for (size_t i = 0; i < npx; ++i) out_ghost[k * npx + i] = pl[k]->size() == npx ? (*pl[k])[i] : 0.0f;
    }
    if (out_veil)
    {
        const std::vector<float>* pl[3] = {&out.veil_r, &out.veil_g, &out.veil_b};
        for (int k = 0; k < 3; ++k)
            for (size_t i = 0; i < npx; ++i) out_veil[k * npx + i] = pl[k]->size() == npx ? (*pl[k])[i] : 0.0f;
    }
    if (out_star)
    {
        const std::vector<float>* pl[3] = {&out.starburst_r, &out.starburst_g, &out.starburst_b};
        for (int k = 0; k < 3; ++k)
            for (size_t i = 0; i < npx; ++i) out_star[k * npx + i] = pl[k]->size() == npx ? (*pl[k])[i] : 0.0f;
    }
    return 0;
}
#endif  // REF_GPU
