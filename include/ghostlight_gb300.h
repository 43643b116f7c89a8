/*
 * ghostlight_gb300.h — C-ABI of the GB300 flare hot path.
 *
 * Plain C: fixed-layout structs, raw pointers and sizes, int status codes.
 * Device pointers are CUDA global-memory addresses (for example a torch
 * tensor's data_ptr()); `stream` is a cudaStream_t passed as void*.
 * The library never frees caller memory.  Every entry point returns GL_OK (0)
 * or a negative GL_ERR_* code; gl_last_error() gives the message of the last
 * failure on the calling thread.
 *
 * Each declaration names the reference interface it replaces
 * (JaydenB/ghostlight, path within that project, file:line).
 */
#ifndef GHOSTLIGHT_GB300_H
#define GHOSTLIGHT_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define GL_OK                0
#define GL_ERR_INVALID      -1   /* bad argument (maps to ValueError)        */
#define GL_ERR_OOM          -2   /* device allocation failed                 */
#define GL_ERR_CUDA         -3   /* CUDA launch / runtime error              */
#define GL_ERR_TIMEOUT      -4   /* a bounded device wait gave up            */
#define GL_ERR_BUDGET       -5   /* request above the admission budget       */
#define GL_ERR_NO_DEVICE    -6   /* no CUDA device                           */
#define GL_ERR_UNSUPPORTED  -7   /* feature outside the implemented path     */

/* ---- enums (values match ghostlight/src/optical_system.h:54-97) ---------- */
#define GL_FORM_SPHERE        0
#define GL_FORM_ASPHERE       1
#define GL_FORM_CYLINDRICAL   2
#define GL_CYL_AXIS_X         0
#define GL_CYL_AXIS_Y         1
#define GL_APERTURE_CIRCLE    0
#define GL_APERTURE_POLYGON   1
#define GL_APERTURE_IMAGE     2
#define GL_DISP_AIR           0
#define GL_DISP_ABBE          1
#define GL_DISP_SELLMEIER     2
#define GL_COATING_SIMPLE     0
#define GL_COATING_SPECTRAL   1   /* ar_layers = gl_coating_table id   */
#define GL_COATING_ANGULAR    2   /* ar_layers = gl_coating_table id   */
#define GL_COATING_SPECTRAL_ANGULAR 3 /* ar_layers = gl_coating_table id */
#define GL_COATING_ATTENUATOR 4
#define GL_COATING_ARTIST     5

/* TraceStatus, ghostlight/src/trace_event.h:13-19 */
#define GL_TRACE_OK             0
#define GL_TRACE_VIGNETTED      1
#define GL_TRACE_TIR            2
#define GL_TRACE_MISSED_SURFACE 3
#define GL_TRACE_INVALID_INPUT  4

/* Output colour spaces, ghostlight/src/spectral.h:24-31 */
#define GL_CS_ACESCG      0
#define GL_CS_SRGB_LINEAR 1
#define GL_CS_P3_D65      2
#define GL_CS_P3_D60      3
#define GL_CS_XYZ         4
#define GL_CS_CUSTOM      5
/* Input colour spaces, ghostlight/src/spectral.h:18-22 */
#define GL_CS_INPUT_ACESCG      0
#define GL_CS_INPUT_SRGB_LINEAR 1
#define GL_CS_INPUT_CUSTOM      2

/* ---- data formats ------------------------------------------------------- */

/* One sequential surface.  Field meaning follows struct Surface,
 * ghostlight/src/optical_system.h:157-249 (the trace-facing subset: table and
 * image-backed coatings/apertures are not part of this path).  All fields are
 * 4 bytes so the layout is identical in C, C++, CUDA and ctypes. */
typedef struct gl_surface {
    float   radius;                 /* signed radius (mm), 0 = flat          */
    float   thickness;              /* axial gap to the next surface (mm)    */
    float   ior;                    /* n_d of the medium after the surface   */
    float   abbe_v;                 /* V_d of the medium after the surface   */
    float   semi_aperture;          /* clear semi-diameter (mm)              */
    float   z;                      /* world vertex z (mm); sensor at z = 0  */
    int32_t is_stop;
    int32_t is_active;
    int32_t aperture_shape;         /* GL_APERTURE_*                         */
    int32_t aperture_blades;
    float   aperture_rotation_rad;
    float   aperture_aspect;
    float   aperture_curvature;     /* blade shape; all 0 = plain polygon    */
    float   aperture_twist;
    float   aperture_notch_rad;
    float   aperture_notch_angle_rad;
    float   decenter_x, decenter_y;
    float   rot[9];                 /* row-major local->world rotation       */
    int32_t form;                   /* GL_FORM_*                             */
    float   conic_k;
    float   asphere_terms[8];       /* A4, A6, ... A18                       */
    int32_t n_asphere_terms;
    int32_t cyl_axis;               /* GL_CYL_AXIS_*                         */
    int32_t disp_model;             /* GL_DISP_*                             */
    float   sellmeier_B[3];
    float   sellmeier_C[3];         /* um^2                                  */
    int32_t coating_model;          /* GL_COATING_*                          */
    int32_t ar_layers;              /* SIMPLE: 0 bare, 1 MgF2, 2+ multi      */
    float   tint_r, tint_g, tint_b, tint_strength;        /* ARTIST          */
    float   gauss_sigma, gauss_background, gauss_peak;    /* ATTENUATOR      */
    float   gauss_decenter_x, gauss_decenter_y;
} gl_surface;

/* GPUSpectralSample, ghostlight/src/spectral.h:46-50 */
typedef struct gl_spectral_sample { float lambda, cmf_r, cmf_g, cmf_b; } gl_spectral_sample;
/* ApertureSample, ghostlight/src/aperture_sampler.h:21 */
typedef struct gl_pupil_sample { float u, v; } gl_pupil_sample;
/* GhostPair, ghostlight/src/ghost.h:12-16 */
typedef struct gl_ghost_pair { int32_t surf_a, surf_b; } gl_ghost_pair;
/* FlareSource, ghostlight/src/ghost.h:18-23 (angles in radians) */
typedef struct gl_flare_source { float angle_x, angle_y, r, g, b; } gl_flare_source;

/* ApertureSamplerParams, ghostlight/src/aperture_sampler.h:28-42 */
typedef struct gl_sampler_params {
    int32_t ray_grid;
    int32_t pupil_jitter;           /* 0 regular, 1 wang hash, 2 Halton      */
    int32_t jitter_seed;
    int32_t blades_override;        /* 0 = derive from the stop              */
    float   rotation_deg;
} gl_sampler_params;

/* The FlareConfig fields filter_ghost_pairs reads,
 * ghostlight/src/render_config.h:281-284 */
typedef struct gl_filter_params {
    float   min_ghost_intensity;
    int32_t ghost_normalize;
    float   max_area_boost;
} gl_filter_params;

/* ---- errors ------------------------------------------------------------- */
const char* gl_last_error(void);
int         gl_version(void);

/* ---- host builders (no GPU) -------------------------------------------- */

/* OpticalSystem::finalize, ghostlight/src/optical_system.cpp:1425 —
 * lays z so the chain ends at the sensor (z = 0). */
int gl_finalize_z(gl_surface* surfaces, int n);

/* ApertureProfile::radius_at (ghostlight/src/aperture_profile.h:192-196) of
 * make_aperture_profile (:285-358): the normalised boundary radius (1 = blade
 * tip) of a bladed stop at each angle theta[i] (radians, absolute), for the
 * authored curvature [-1, 1], twist [-1, 1], notch and notch angle (radians);
 * with none authored, the regular polygon.  Host float arithmetic. */
int gl_blade_radius(int blades, float rotation_rad, float curvature, float twist, float notch_rad,
                    float notch_angle_rad, const float* theta, int n, float* out);

/* ---- table-backed coatings ----------------------------------------------
 * OpticalSystem::coating_tables (ghostlight/src/optical_system.h:285-301) and
 * its Python setters set_coating_spectral_table / set_coating_angular_table /
 * set_coating_sa_table / set_coating_layers (bindings/python/src/
 * bind_geometry.cpp:412-590).  A table is an immutable entry of a
 * process-wide store, named by a positive id; a surface selects it with
 * coating_model = GL_COATING_SPECTRAL / ANGULAR / SPECTRAL_ANGULAR and
 * ar_layers = id (ar_layers = 0: no table, bare Fresnel as the reference's
 * null-table fallback, trace_core.h:657-660).  Identical content gives the
 * same id; entries live for the process.
 *
 * gl_coating_table_create: 1-D models take keys axis0[n0] (nm or degrees,
 * ascending) and r[n0], axis1 = NULL, n1 = 0; SPECTRAL_ANGULAR takes
 * wavelengths axis0[n0], angles axis1[n1] (both ascending) and
 * r[n0 * n1] wavelength-major.  angle_ref_ior: index of the medium the angle
 * axis is measured in (ignored by SPECTRAL); out_of_range_discard: a lookup
 * outside the table carries no energy instead of clamping. */
int gl_coating_table_create(int32_t model, const float* axis0, int32_t n0, const float* axis1, int32_t n1,
                            const float* r, float angle_ref_ior, int32_t out_of_range_discard, int32_t* out_id);
int gl_coating_table_info(int32_t id, int32_t* model, int32_t* n0, int32_t* n1, float* angle_ref_ior,
                          int32_t* out_of_range_discard);
int gl_coating_table_read(int32_t id, float* axis0, float* axis1, float* r);
/* Bitmap aperture (ApertureImage, ghostlight/src/optical_system.h:262-269;
 * sampled by sample_aperture_image, trace.cpp:31-48): width x height
 * row-major luminance in [0, 1] and the world radius of the image boundary
 * (aperture_semi_diameter).  A surface selects it with aperture_shape =
 * GL_APERTURE_IMAGE and aperture_blades = id (0: not loaded, the surface
 * passes every ray inside its clear aperture, as the reference does before
 * the pixels are decoded).  Same store as the coating tables:
 * gl_coating_table_info reports model 100, n0 = width, n1 = height,
 * angle_ref_ior = semi-diameter; gl_coating_table_read returns the pixels
 * in r. */
int gl_aperture_image_create(int32_t width, int32_t height, const float* pixels, float semi_diameter,
                             int32_t* out_id);
/* Copy a table to the current device ahead of an allocation-free render
 * (the other entry points copy it on first use). */
int gl_coating_table_prepare(int32_t id);
/* OpticalSystem::bake_coating_layers (ghostlight/src/optical_system.cpp:
 * 1483-1575): the thin-film stack of n_layers layers (thickness_nm[l]; n,k
 * samples at nk_lambda_um in um, nk_count[l] of them per layer, concatenated)
 * on surface `index`, baked on 400..700 nm x 0..85 degrees into a
 * SPECTRAL_ANGULAR table whose angle axis is the medium before the surface. */
int gl_coating_bake_layers(const gl_surface* surfaces, int32_t n, int32_t index, int32_t n_layers,
                           const float* thickness_nm, const int32_t* nk_count, const float* nk_lambda_um,
                           const float* nk_n, const float* nk_k, int32_t* out_id);

/* make_rotation, ghostlight/src/optical_system.cpp:185-199 — the element
 * rotation R = Ry(tilt_y) Rx(tilt_x) Rz(roll) of the lens-file loader
 * (row-major 3x3 into out[9]; float arithmetic, C library cosf/sinf). */
int gl_euler_rotation(float tilt_x_deg, float tilt_y_deg, float roll_deg, float* out);

/* enumerate_ghost_pairs, ghostlight/src/ghost.cpp:17-31 */
int gl_enumerate_ghost_pairs(const gl_surface* surfaces, int n,
                             gl_ghost_pair* out, int cap, int* n_out);

/* build_aperture_samples, ghostlight/src/aperture_sampler.h:180-223 */
int gl_build_aperture_samples(const gl_surface* surfaces, int n,
                              const gl_sampler_params* p,
                              gl_pupil_sample* out, int cap, int* n_out);

/* build_spectral_table + compute_spectral_correction,
 * ghostlight/src/spectral.cpp:317-369 and :419 (CIE 1931 sensor).
 * correction_out (9 floats, row-major) may be NULL. */
int gl_build_spectral_table(int n_samples, int output_cs,
                            const float* custom_xyz_to_output /* 9 or NULL */,
                            gl_spectral_sample* out, float* correction_out);

/* resolve_input_matrix / resolve_output_matrix, ghostlight/src/spectral.cpp:186,247 */
int gl_color_matrices(int input_cs, const float* custom_in, int output_cs,
                      const float* custom_out, float* m_in9, float* m_out9);

/* ---- device entry points ------------------------------------------------ */

/* filter_ghost_pairs, ghostlight/src/ghost.cpp:105-138 (+ the estimators at
 * :34-102).  The per-pair probe traces run as one device launch; decisions
 * whose device estimate lies within a guard band of the threshold are
 * re-evaluated on the host in the reference's own FP32 arithmetic, so the
 * surviving set and its order are the reference's.  Synchronous. */
int gl_filter_ghost_pairs(const gl_surface* surfaces, int n,
                          float sensor_half_w, float sensor_half_h,
                          const gl_filter_params* params,
                          gl_ghost_pair* out_pairs, float* out_boosts,
                          float* out_footprint_mm /* 2 per pair or NULL */,
                          int cap, int* n_out, int* n_rechecked);

/* trace_ghost_ray / trace_primary_ray, ghostlight/src/trace.cpp:171,243,
 * batched.  d_rays: n_rays x 7 floats (ox,oy,oz, dx,dy,dz, lambda_nm);
 * d_out: n_rays x 5 floats (x,y,z, weight, status).  bounce_b < 0 traces a
 * primary ray.  Synchronous on `stream`: the call waits for its copies and
 * the launch before it returns. */
int gl_trace_rays(const gl_surface* surfaces, int n,
                  int bounce_a, int bounce_b,
                  const float* d_rays, int n_rays, float* d_out, void* stream);

/* Allocation-free form of gl_trace_rays, for callers that may not allocate
 * device memory while they run (a plug-in whose host application owns the
 * device heap, a real-time thread, a host that reserved the whole device).
 * No counterpart in the reference.  Same arguments and results as
 * gl_trace_rays; the packed lens tables go to a fixed array inside the library
 * (at most 64 surfaces; larger lenses are rejected with GL_ERR_INVALID), so the
 * call allocates no device memory.  The array's device address is looked up
 * (cudaGetSymbolAddress, no allocation) on every call.  All calls share the
 * array; calls that overlap on the GPU race on it.  Synchronous on `stream`,
 * so it must not be called while `stream` is being captured into a CUDA
 * graph: it returns GL_ERR_INVALID then. */
int gl_trace_rays_noalloc(const gl_surface* surfaces, int n,
                          int bounce_a, int bounce_b,
                          const float* d_rays, int n_rays, float* d_out, void* stream);

/* Ghost render: the main scatter of launch_ghost_render,
 * ghostlight/src/ghost_render.cu:630-1442 (kernel :209-491, colour
 * correction :610-622).  All pairs x sources are traced by ONE persistent
 * launch (or, with plain_per_pair, one launch per pair — the reference's
 * per-ghost loop shape, ghost_render.cu:1544-1557, kept as a baseline).
 * pair_grid[i] selects which pupil grid pair i samples (adaptive grids);
 * grid_offsets has n_grids+1 entries into `samples`.
 * With cull_dead_pairs (and more than one pair, and not the three-sample
 * preview table) the frame first runs the reference's off-sensor probe —
 * three wang-jittered 40x40 pupil passes over every wavelength with the
 * frame inflated by 1.25 — on the device, and the render skips every pair no
 * probe ray landed for; there is no host round trip.  plain_per_pair renders
 * every pair (the reference's per-pair loop culls nothing, :1000).
 * Outputs are planar float32 W x H, overwritten.  Asynchronous. */
typedef struct gl_ghost_render_params {
    int32_t width, height;
    int32_t fmt_w, fmt_h, fmt_x0, fmt_y0;
    float   sensor_half_w, sensor_half_h;
    float   flare_gain;
    int32_t apply_correction;
    float   correction[9];
    int32_t plain_per_pair;          /* 1 = one launch per pair (baseline)  */
    int32_t splat_mode;              /* 0 = bilinear point splat (reference) */
    int32_t cull_dead_pairs;         /* off-sensor probe cull, ghost_render.cu:976-1238 */
    int32_t blades_override;         /* sampler override for the probe grids */
    float   rotation_deg;
} gl_ghost_render_params;

int gl_render_ghosts(const gl_surface* surfaces, int n_surfaces,
                     const gl_ghost_pair* pairs, const float* area_boosts,
                     const int32_t* pair_grid, int n_pairs,
                     const gl_flare_source* sources, int n_sources,
                     const gl_pupil_sample* samples, const int32_t* grid_offsets,
                     int n_grids,
                     const gl_spectral_sample* spec, int n_spec,
                     const gl_ghost_render_params* params,
                     float* d_out_r, float* d_out_g, float* d_out_b,
                     void* stream);

/* The same render split into a resident plan (all uploads, synchronous) and
 * an execute step that only enqueues kernels on `stream` (so it can be
 * captured in a CUDA graph and replayed).  Same arguments as
 * gl_render_ghosts.  A plan may be executed any number of times; executes
 * of one plan must not overlap on the device (they share its accumulator). */
typedef struct gl_ghost_plan gl_ghost_plan;
int gl_ghost_plan_create(const gl_surface* surfaces, int n_surfaces,
                         const gl_ghost_pair* pairs, const float* area_boosts,
                         const int32_t* pair_grid, int n_pairs,
                         const gl_flare_source* sources, int n_sources,
                         const gl_pupil_sample* samples, const int32_t* grid_offsets,
                         int n_grids,
                         const gl_spectral_sample* spec, int n_spec,
                         const gl_ghost_render_params* params, gl_ghost_plan** out);
int gl_ghost_plan_execute(gl_ghost_plan* plan, float* d_out_r, float* d_out_g,
                          float* d_out_b, void* stream);
/* rays = ray-wavelength traces per execute at most (render + probe passes);
 * n_items = 32-sample work items;
 * grid = CTAs of the persistent launch. */
int gl_ghost_plan_info(const gl_ghost_plan* plan, long long* rays, int* n_items, int* grid);
/* Launch shape of the batched render (the autotuner's knob; no counterpart in
 * the reference, whose launch shape is fixed at ghost_render.cu:1544):
 * items_per_warp = 0 -> persistent work queue over ctas_per_sm CTAs per SM
 * (0 = all resident); > 0 -> one-shot CTAs of that many 32-sample items per warp. */
int gl_ghost_plan_set_launch(gl_ghost_plan* plan, int items_per_warp, int ctas_per_sm);
/* Wavelength split of the render and probe work (the autotuner's other knob;
 * no counterpart in the reference): each 32-sample item becomes `chunks`
 * tasks over consecutive wavelength ranges, so the tasks left at the end of
 * the queue are shorter.  >= 1, clamped to n_spec; the default is about eight
 * wavelengths per task (31 -> 4, 16 -> 2, 8 -> 1). */
int gl_ghost_plan_set_lambda_split(gl_ghost_plan* plan, int chunks);
/* Ray-wavelength traces the last execute ran (render + cull probes; a probe
 * warp stops at its first on-sensor hit).  Synchronous. */
int gl_ghost_plan_traced(const gl_ghost_plan* plan, long long* out);
/* The pupil-sample order the batched render traces in: a stable sort along a
 * Morton curve over the pupil square, so the 32 samples of a warp are
 * neighbours.  Plans order their grids themselves; a grid ordered once by
 * this call (and cached by the caller) is only checked, not re-sorted.
 * (No counterpart in the reference, which traces in mask order.) */
int gl_morton_order(const gl_pupil_sample* in, int n, gl_pupil_sample* out);
/* The same count split into the render launch and the off-sensor probe
 * launch.  Synchronous.  (No counterpart in the reference.) */
/* collect_stats (render_config.h:33-35, ghost_render.cu:1357-1431): the
 * plan's items traced again without weights, splat or cull; out[3 i + k] =
 * pair i's {traces, traces that left the lens, traces landing in the frame}.
 * Synchronises the stream. */
int gl_ghost_plan_stats(gl_ghost_plan* plan, unsigned long long* out, void* stream);
int gl_ghost_plan_traced_split(const gl_ghost_plan* plan, long long* render, long long* probe);
/* Optional cudaEvent_t handles (NULL = none) that every later execute records
 * on its stream before the probe launch, before the render launch and after
 * the render launch, so a caller can time the render kernel alone with
 * cudaEventElapsedTime.  Inside a stream capture they become external
 * event-record nodes.  (No counterpart in the reference.) */
int gl_ghost_plan_set_timing(gl_ghost_plan* plan, void* ev_probe, void* ev_render, void* ev_end);
/* Per-pair probe hit counts of the last execute (0 = culled); all 1 when the
 * plan does not cull.  Synchronous. */
int gl_ghost_plan_pair_hits(const gl_ghost_plan* plan, int32_t* out, int n);
int gl_ghost_plan_destroy(gl_ghost_plan* plan);

/* ---- TEST-ONLY: tensor-core building block (tcgen05) ---------------------- */

/* Test hook, not part of the drop-in surface: no reference caller binds it.
 * C[M x N] (float32, row-major) = A[M x K] * B[N x K]^T with BF16 operands
 * (row-major, device) and FP32 accumulation in tensor memory: the TMA +
 * tcgen05 pipeline the matrix-DFT starburst is built on, exposed so it can
 * be checked against a library GEMM.  M, N multiples of 128, K of 64.
 * No counterpart in the reference (its starburst uses SIMT dot products,
 * mdft_render.cu:137-172).  Synchronous. */
int gl_gemm_bf16_tc(const void* d_a, const void* d_b, float* d_c, int M, int N, int K, void* stream);

/* Matrix-DFT starburst in field form (E = W_y A W_x^T, the field form of
 * mdft_render.cu's per-wavelength triple product): for each wavelength l,
 *   W_x[k][j] = exp(-2 pi i scale_x[l] (j - (n-1)/2)(k - center_x)),
 *   E_l = W_y A W_x^T  (K_out x K_out),  out_c += weights_rgb[3l+c] |E_l|^2.
 * form 0: three-term split-BF16 products on tcgen05 with FP32 accumulation;
 * form 1: TF32 tcgen05.  n and K_out multiples of 128.  The DFT matrices are
 * built once (phase reduced in FP64) and stay resident in the plan.  The
 * pupil amplitude is n x n float32 on the device; outputs are K_out x K_out
 * planar float32, overwritten.  Asynchronous; gl_mdft_plan_status reads the
 * device error word (non-zero = a bounded pipeline wait gave up). */
typedef struct gl_mdft_plan gl_mdft_plan;
int gl_mdft_plan_create(int n, int K_out, int n_lambda, const double* scale_x,
                        const double* scale_y, double center_x, double center_y,
                        const float* weights_rgb, int form, void* stream,
                        gl_mdft_plan** out);
int gl_mdft_plan_execute(gl_mdft_plan* plan, const float* d_pupil, float* d_out_r,
                         float* d_out_g, float* d_out_b, void* stream);
int gl_mdft_plan_status(gl_mdft_plan* plan, int* err_code);
int gl_mdft_plan_destroy(gl_mdft_plan* plan);
/* Rectangular output (Kx columns x Ky rows, multiples of 128); the square
 * create above is Kx = Ky = K_out. */
int gl_mdft_plan_create2(int n, int Kx, int Ky, int n_lambda, const double* scale_x,
                         const double* scale_y, double center_x, double center_y,
                         const float* weights_rgb, int form, void* stream, gl_mdft_plan** out);
/* Move the pattern's centre (output pixels, |c| < 12288): enqueues the
 * rebuild of the plan's DFT matrices on `stream` (graph-capturable), as the
 * reference rebuilds its phase matrices per source (mdft_render.cu:109-135). */
int gl_mdft_plan_set_center(gl_mdft_plan* plan, double center_x, double center_y, void* stream);
/* GEMM grid of the tcgen05 forms (0 = one CTA per SM); autotuner knob. */
int gl_mdft_plan_set_launch(gl_mdft_plan* plan, int ctas);
/* Output tile of the second GEMM (E = W_y T) of the tcgen05 forms, in
 * complex output columns per unit: 128 (default; N = 256 MMAs, two pipeline
 * stages) or 64 (N = 128 MMAs, three stages, twice the units, so a small
 * frame spreads over more SMs); the autotuner's tile-shape knob.  No
 * counterpart in the reference (its starburst contracts with SIMT dot
 * products, mdft_render.cu:137-172).  Results agree to float rounding. */
int gl_mdft_plan_set_tile(gl_mdft_plan* plan, int tile_n);
/* Restrict the next executes to wavelengths [lam_begin, lam_end) (0, -1:
 * all): a large pattern enqueued as several short wavelength ranges (each
 * accumulating) frees its CTAs' SMs between the ranges, so a serving loop's
 * smaller patterns are not held behind it. */
int gl_mdft_plan_set_lambda_range(gl_mdft_plan* plan, int lam_begin, int lam_end);
/* execute with accumulate != 0 adds into the output planes instead of
 * overwriting them (a starburst layered onto a ghost image). */
int gl_mdft_plan_execute2(gl_mdft_plan* plan, const float* d_pupil, float* d_out_r,
                          float* d_out_g, float* d_out_b, int accumulate, void* stream);
/* The reference's own matrix-DFT engine, mdft_starburst (mdft_render.cu:
 * 199-340): the exact pixel-box integral of the intensity through the
 * compact pupil autocorrelation C (Mc x Mc real, Mc = 2 mc + 1, padded with
 * zeros to n x n; gl_sprite_plan_autocorr builds it):
 *   W_x[k][j] = sinc(s_l (j - mc)) exp(-2 pi i s_l (j - mc)(k - center_x)),
 *   I_l = Re(W_y C W_x^T),  out_c += weights_rgb[3l+c] tint_c I_l,
 * s_l = pixel pitch / pattern period at wavelength l (the reference's
 * px / S_l), center = source pixel - 0.5 - window origin.  box = 1 selects
 * this form (Re E accumulated); box = 0 is the field form |E|^2 above;
 * red_center is the reduction index of zero lag (mc for the box form,
 * (n - 1) / 2 for the field form).  Same GEMMs, operand layout and forms as
 * gl_mdft_plan_create2. */
int gl_mdft_plan_create3(int n, int Kx, int Ky, int n_lambda, const double* scale_x,
                         const double* scale_y, double center_x, double center_y,
                         const float* weights_rgb, int form, int box, float red_center,
                         void* stream, gl_mdft_plan** out);
/* execute2 with the output placed in larger planes: plan pixel (l, k) ->
 * plane pixel (y0 + l, x0 + k) of out_w x out_h planes, for l < win_h,
 * k < win_w (the reference's clamped window around the source, :275-290);
 * tint_rgb (3 floats, NULL = 1) scales the weights for this launch (the
 * source colour).  accumulate = 0 clears the whole planes first. */
int gl_mdft_plan_execute3(gl_mdft_plan* plan, const float* d_pupil, float* d_out_r,
                          float* d_out_g, float* d_out_b, int accumulate, int out_w, int out_h,
                          int x0, int y0, int win_w, int win_h, const float* tint_rgb, void* stream);

/* Pupil amplitude of the lens's stop on an N x N grid, 4 x 4 supersampled
 * (build_pupil_kernel, starburst_render.cu:155-191, stop term only): grid
 * coordinate g in [-1, 1) maps to pupil coordinate g / pupil_fill; a
 * supersample counts when it lies inside the stop silhouette
 * (PupilMask::contains, aperture_sampler.h:63-82).  float N x N on the
 * device, asynchronous. */
int gl_build_pupil(const gl_surface* surfaces, int n_surfaces, int N, float pupil_fill,
                   int blades_override, float rotation_deg, float* d_out, void* stream);
/* gl_build_pupil with the rest of build_pupil_kernel's modifiers
 * (starburst_render.cu:155-191): aspect_one = 1 rasterises the stop round
 * (the starburst takes an anamorphic pupil's aspect in the per-axis pitch,
 * starburst_render.cu:738); d_env = the ME x ME cat's-eye envelope over pupil
 * [-1, 1]^2 (device; NULL = none), each inside supersample weighted by its
 * bilinear sample (sample_env :136). */
int gl_build_pupil2(const gl_surface* surfaces, int n_surfaces, int N, float pupil_fill, int blades_override,
                    float rotation_deg, int aspect_one, const float* d_env, int env_n, float* d_out, void* stream);
/* PupilMask::contains (aperture_sampler.h:63-82) of the lens's stop at host
 * points uv[2 k], uv[2 k + 1] -> out[k] (host float arithmetic). */
int gl_pupil_contains(const gl_surface* surfaces, int n, int blades_override, float rotation_deg, int aspect_one,
                      const float* uv, int n_pts, uint8_t* out);

/* PSF / veil image convolution: out_c = in_c (*) k ('same' size, kernel
 * centred, odd kw x kh, float32).  The reference has no such operation on
 * this path (its veil is an analytic glare-spread sprite splatted per source,
 * veil_render.cu:94-243); this is the flare path's image-space form.  FFT
 * route: zero-padded circular convolution of size P x Q = the smallest
 * 2^a 3^b sizes covering image + kernel - 1, two channels per complex
 * transform, three HBM passes; the kernel spectrum stays resident in the
 * plan.  Planes are W x H float32 on the device.  Asynchronous. */
typedef struct gl_conv_plan gl_conv_plan;
int gl_conv2d_plan_create(int width, int height, const float* h_kernel, int kw, int kh,
                          void* stream, gl_conv_plan** out);
int gl_conv2d_plan_execute(gl_conv_plan* plan, const float* d_in_r, const float* d_in_g,
                           const float* d_in_b, float* d_out_r, float* d_out_g,
                           float* d_out_b, void* stream);
/* The same with a second layer summed into the input on load (the flare
 * composite, ghosts + starburst, convolved without a separate add pass). */
int gl_conv2d_plan_execute2(gl_conv_plan* plan, const float* d_in_r, const float* d_in_g,
                            const float* d_in_b, const float* d_add_r, const float* d_add_g,
                            const float* d_add_b, float* d_out_r, float* d_out_g,
                            float* d_out_b, void* stream);
int gl_conv2d_plan_info(const gl_conv_plan* plan, int* P, int* Q);
int gl_conv2d_plan_destroy(gl_conv_plan* plan);

/* ---- SPRITE starburst engine ---------------------------------------------
 * The reference's default starburst engine, render_starburst's sprite path
 * (ghostlight/src/starburst_render.cu:969-1073; kernels psf_from_fft :202,
 * bake_sprite :255, downsample :283, splat_resample :316).
 *
 * gl_sprite_plan_create: N x N grid (power of two, 256..8192) and the
 * spectral table the bake integrates over (cmf already scaled as the caller
 * wants them: the reference premultiplies the sample spacing and white-
 * balances), lambda_ref the wavelength of the one FFT (550 nm).
 * gl_sprite_plan_bake: d_pupil = N x N real stop amplitude on the device
 * (gl_build_pupil); FFT, |.|^2 fftshifted, normalised to unit sum, baked over
 * wavelength and box-summed by ds (power of two <= N/8) into the M x M RGB
 * sprite, M = N / ds.  Stream-ordered, nothing read back.
 * gl_sprite_plan_splat: sources = n_src x {px, py, r, g, b} (host; buffer
 * pixels and colour), texel pitch sx_ds/sy_ds and pixel pitch px_mm_x/y (mm),
 * footprint half-extent rx/ry (pixels), gain; ADDS into the three planes.
 * gl_sprite_plan_read: copies of the PSF (N x N, |FFT|^2 before the 1/energy
 * scale) and the sprite (M x M x 3) into device buffers, and the
 * PSF energy (FP64) to the host. */
typedef struct gl_sprite_plan gl_sprite_plan;
int gl_sprite_plan_create(int N, const gl_spectral_sample* spec, int n_spec, float lambda_ref, gl_sprite_plan** out);
int gl_sprite_plan_bake(gl_sprite_plan* plan, const float* d_pupil, int ds, void* stream);
int gl_sprite_plan_splat(gl_sprite_plan* plan, const float* sources, int n_src, float sx_ds, float sy_ds,
                         float px_mm_x, float px_mm_y, int rx, int ry, float gain, float* d_out_r, float* d_out_g,
                         float* d_out_b, int width, int height, void* stream);
int gl_sprite_plan_read(gl_sprite_plan* plan, float* d_psf, float* d_sprite, double* energy, int* M, void* stream);
int gl_sprite_plan_destroy(gl_sprite_plan* plan);
/* The matrix-DFT engine's compact autocorrelation (mdft_render.cu:233-262):
 * G = FFT2(|FFT2(A)|^2) of the N x N pupil amplitude d_pupil, at the lags
 * |l| <= mc, scaled by 1 / (G[0][0] N^2) so the pattern sums to one texel
 * area per period: d_C[(ly + mc) ldc + (lx + mc)], rows x ldc floats, zeroed
 * first (the padding of the GEMM operand).  Four FFT passes on the plan's
 * buffers, the scale read on the device; invalidates the plan's sprite. */
int gl_sprite_plan_autocorr(gl_sprite_plan* plan, const float* d_pupil, int mc, float* d_C, int ldc, int rows,
                            void* stream);
/* The splat of one source (splat_resample_kernel, starburst_render.cu:316)
 * from a baked M x M x 3 sprite held by the caller (a copy read out with
 * gl_sprite_plan_read): the source is passed by value, so the call stages
 * nothing, allocates nothing and keeps no state; splats of one sprite on
 * several streams run side by side.  ADDS into the three planes. */
int gl_sprite_splat_source(const float* d_sprite, int M, float px, float py, float r, float g, float b,
                           float sx_ds, float sy_ds, float px_mm_x, float px_mm_y, int rx, int ry, float gain,
                           float* d_out_r, float* d_out_g, float* d_out_b, int width, int height, void* stream);

/* ---- Serving: resident lenses and stream-ordered requests -----------------
 * The reference renders one flare per blocking call under process-wide
 * mutexes (ghost_render.cu:504-511, entered from bind_renderers.cpp:85-134)
 * and has no serving layer; these calls are what a request loop over the
 * flare path binds instead.
 *
 * gl_lens: one lens kept in HBM across requests — packed surfaces, the
 * filtered ghost pairs (gl_filter_ghost_pairs output, order kept), the
 * off-sensor probe grids, and caches of IOR slices per wavelength set and of
 * pupil grids per ray_grid (filled on first use, or ahead by
 * gl_lens_prepare).  A lens must outlive every request created on it. */
typedef struct gl_lens gl_lens;
int gl_lens_create(const gl_surface* surfaces, int n_surfaces, const gl_ghost_pair* pairs,
                   const float* area_boosts, int n_pairs, int blades_override,
                   float rotation_deg, gl_lens** out);
int gl_lens_prepare(gl_lens* lens, int ray_grid, const gl_spectral_sample* spec, int n_spec);
int gl_lens_info(const gl_lens* lens, int* n_pairs, long long* device_bytes);
int gl_lens_destroy(gl_lens* lens);

/* gl_request: one ghost-layer render on a resident lens with one uniform
 * pupil grid (ray_grid^2, masked) for every pair — the computation of
 * launch_ghost_render (ghost_render.cu:630) for those inputs.  Its device
 * memory (accumulator, spectral table, counters) is one allocation from a
 * stream-ordered pool on `stream`; create / enqueue / destroy never
 * synchronise the device, so requests on different streams overlap.
 * items_per_warp = 0: persistent work queue over the whole GPU;
 * > 0: short CTAs of that many 32-sample items per warp, which the CTA
 * scheduler interleaves with other streams' work by stream priority.
 * destroy frees the memory in stream order after the enqueued work. */
typedef struct gl_request gl_request;
int gl_request_create(gl_lens* lens, int ray_grid, const gl_spectral_sample* spec, int n_spec,
                      const gl_flare_source* sources, int n_sources,
                      const gl_ghost_render_params* params, void* stream, gl_request** out);
/* Null outputs render into the request's own planes (r | g | b, contiguous,
 * W x H float32 each): gl_request_planes gives their device address and
 * gl_request_copy_out enqueues one copy of all three to host memory (pinned
 * for an asynchronous copy) or to device memory. */
/* Wavelength split of the request's probe and render work (as
 * gl_ghost_plan_set_lambda_split): each item becomes `chunks` tasks over
 * consecutive wavelength ranges, and one-shot CTAs are sized by tasks, so a
 * long request runs as more, shorter CTAs.  Before gl_request_enqueue. */
int gl_request_set_lambda_split(gl_request* req, int chunks);
int gl_request_enqueue(gl_request* req, float* d_out_r, float* d_out_g, float* d_out_b,
                       int items_per_warp, void* stream);
int gl_request_planes(const gl_request* req, float** d_rgb);
int gl_request_copy_out(const gl_request* req, void* host_rgb, void* stream);
int gl_request_info(const gl_request* req, long long* rays, long long* device_bytes,
                    int* grid_samples);
/* Ray-wavelength traces of the last enqueue.  stream == NULL: the caller has
 * seen that work complete, and the count is read from a pinned host word the
 * enqueue filled (no CUDA call); otherwise a synchronous read on `stream`. */
int gl_request_traced(const gl_request* req, long long* out, void* stream);
int gl_request_destroy(gl_request* req, void* stream);
/* The request pool of the current device: bytes reserved / in use; trim
 * releases reserved bytes above keep_bytes back to the driver. */
int gl_pool_info(long long* reserved, long long* used);
int gl_pool_trim(long long keep_bytes);

/* ---- First-order calibration and the source-position solve (host) ---------
 * calibrate_lens (lens_calibration.cpp:344) — covered field, image circle,
 * per-axis EFL, entrance pupil and f-number by tracing the spawn disc — and
 * solve_source_angle / source_map_screen (source_map.cpp:182, :456).
 * GL_SETUP_FP32 runs the reference's float32 arithmetic (the values equal the
 * reference's bit for bit); GL_SETUP_FP64 runs the same measurement with
 * double-precision traces and solves (results rounded to float at the end). */
#define GL_SETUP_FP32 0
#define GL_SETUP_FP64 1
typedef struct gl_lens_calibration {
    float sensor_half_w, sensor_half_h;        /* covered field landing (mm)    */
    float max_half_angle_h, max_half_angle_v;  /* covered field (rad)           */
    float image_circle_semi_w, image_circle_semi_h;
    float focal_length_x, focal_length_y;
    float entrance_pupil_semi_x, entrance_pupil_semi_y;
    float f_number_x, f_number_y;
    float pupil_area_frac;
    int32_t field_crossed;                     /* 0: field probe hit the 60 deg ceiling */
} gl_lens_calibration;

#define GL_SOURCE_SOLVED    0
#define GL_SOURCE_CONTINUED 1
#define GL_SOURCE_FALLBACK  2

typedef struct gl_source_solve {
    float angle_x, angle_y;                    /* radians: the answer           */
    int32_t status;                            /* GL_SOURCE_*                   */
    float residual_mm;
    float anchor_ax, anchor_ay, anchor_x, anchor_y;
    float J[4];                                /* d(landing mm)/d(angle), row-major */
    float eff_half_w, eff_half_h;
    float inv_tan_w, inv_tan_h;
    int32_t probe_evals;
} gl_source_solve;

int gl_calibrate_lens(const gl_surface* surfaces, int n_surfaces, float lens_focal_length,
                      float d_line_nm, gl_lens_calibration* out);
/* gl_calibrate_lens with a precision: GL_SETUP_FP32 (= gl_calibrate_lens) or
 * GL_SETUP_FP64. */
int gl_calibrate_lens2(const gl_surface* surfaces, int n_surfaces, float lens_focal_length,
                       float d_line_nm, int precision, gl_lens_calibration* out);
/* ndc in [-1, 1] (0 on the axis); eff_half_w/h: the rendered frame's half
 * extents in mm.  A lens with no surfaces gives the FALLBACK solve. */
int gl_solve_source_angle(const gl_surface* surfaces, int n_surfaces,
                          const gl_lens_calibration* calib, float ndc_x, float ndc_y,
                          float eff_half_w, float eff_half_h, gl_source_solve* out);
/* gl_solve_source_angle with a precision (GL_SETUP_FP32 or GL_SETUP_FP64). */
int gl_solve_source_angle2(const gl_surface* surfaces, int n_surfaces,
                           const gl_lens_calibration* calib, float ndc_x, float ndc_y,
                           float eff_half_w, float eff_half_h, int precision, gl_source_solve* out);
int gl_source_map_screen(const gl_source_solve* base, float angle_x, float angle_y,
                         float* out_sx, float* out_sy);

/* ---- Veiling glare (render_veil, veil_render.cu:243-414) -------------------
 * The analytic glare-spread function g(r) = (a^2 / (r^2 + a^2))^p, a =
 * spread * sensor half-height, baked once per falloff p (clamped to [1, 3])
 * into a resident 1024^2 sprite normalised to unit sum; each execute box-
 * downsamples it toward the output pitch and area-resamples it onto the frame
 * around every source, tinted by the source colour times gain.  Sources are
 * a device array (buffer-pixel position, output-space colour). */
typedef struct gl_veil_source { float px, py, r, g, b; } gl_veil_source;
typedef struct gl_veil_params {
    int32_t width, height, fmt_w, fmt_h;
    float sensor_half_w, sensor_half_h;
    float spread;                              /* core radius / sensor half-height */
    float gain;                                /* fraction of the source flux      */
    int32_t accumulate;                        /* add into the planes              */
} gl_veil_params;
typedef struct gl_veil_plan gl_veil_plan;
int gl_veil_plan_create(float falloff, void* stream, gl_veil_plan** out);
int gl_veil_plan_execute(gl_veil_plan* plan, const gl_veil_source* d_sources, int n_sources,
                         const gl_veil_params* params, float* d_out_r, float* d_out_g,
                         float* d_out_b, void* stream);
int gl_veil_plan_destroy(gl_veil_plan* plan);
/* The scale an execute with these params uses and the resident sprite — what
 * the reference's VeilDebug capture reports (veil_render.h:31-40, filled at
 * veil_render.cu:400-412; Python _render_veil_debug, bind_renderers.cpp:244).
 * gl_veil_plan_read copies the grid x grid unit-sum GSF (the reference
 * replicates it into its neutral RGB sprite) on the stream. */
typedef struct gl_veil_geometry {
    int32_t grid;            /* sprite side N (1024)                        */
    int32_t ds;              /* box-sum factor toward the output pitch      */
    float dx_mm;             /* sensor mm per sprite texel (isotropic)      */
    float core_mm;           /* GSF core radius a on the sensor             */
    float falloff;           /* radial power p actually used                */
    float core_texels;       /* core radius in sprite texels (N / 32)       */
} gl_veil_geometry;
int gl_veil_plan_geometry(const gl_veil_plan* plan, const gl_veil_params* params, gl_veil_geometry* out);
int gl_veil_plan_read(const gl_veil_plan* plan, float* d_reference, void* stream);

/* ---- PSF grid (render_psf: PSFRenderer.cpp:243-465, psf_render.cu) --------
 * Per source, the lens's primary-ray spot in its own tile of a composite
 * atlas.  gl_psf_prepass centres each tile (host, float32, the reference's
 * arithmetic): CHIEF_CENTROID = the unweighted 7 x 7 pupil-mean landing;
 * FIXED_TARGET = the chief ray aimed at (target_x, target_y) mm by 2x2
 * Newton, with the survivor-mean and tracked-window fallbacks.
 * sources7: per source [angle_x, angle_y, r, g, b, target_x_mm, target_y_mm]. */
#define GL_PSF_CENTER_CHIEF_CENTROID 0
#define GL_PSF_CENTER_FIXED_TARGET   1
#define GL_PSF_CELL_OK               0
#define GL_PSF_CELL_CHIEF_VIGNETTED  1
#define GL_PSF_CELL_DARK             2
typedef struct gl_psf_cell {
    float beam_ax, beam_ay;          /* field direction the tile's rays are traced at */
    float chief_x_mm, chief_y_mm;    /* tile centre on the sensor                     */
    int32_t status;                  /* GL_PSF_CELL_*                                 */
    float pupil_fraction;
    float aim_residual_mm;
} gl_psf_cell;
int gl_psf_prepass(const gl_surface* surfaces, int n_surfaces, const float* sources7, int n_sources,
                   int center_mode, gl_psf_cell* out);
typedef struct gl_psf_source {
    float angle_x, angle_y, r, g, b, chief_x_mm, chief_y_mm;
    int32_t tile_x0, tile_y0;
} gl_psf_source;
/* Accumulates into caller-zeroed planes (d_out_g/b unused when monochromatic);
 * splat_sigma_px <= 0: bilinear; else a normalised Gaussian of radius
 * splat_radius_px (<= 16).  Synchronous. */
int gl_psf_render(const gl_surface* surfaces, int n_surfaces, const gl_psf_source* sources,
                  int n_sources, const gl_pupil_sample* grid, int n_grid,
                  const gl_spectral_sample* spec, int n_spec, int tile_w, int tile_h,
                  int composite_w, int composite_h, float mm_per_pixel, int monochromatic,
                  float splat_sigma_px, int splat_radius_px, float* d_out_r, float* d_out_g,
                  float* d_out_b, void* stream);
/* The same render, stream-ordered for a serving loop (a PSF request among
 * flare requests): its device scratch comes from the device's memory pool and
 * is freed in stream order, and the call returns without waiting; the planes
 * are complete when the stream reaches this point.  (gl_psf_render frees
 * with cudaFree, which waits for the whole device.) */
int gl_psf_render_async(const gl_surface* surfaces, int n_surfaces, const gl_psf_source* sources,
                        int n_sources, const gl_pupil_sample* grid, int n_grid,
                        const gl_spectral_sample* spec, int n_spec, int tile_w, int tile_h,
                        int composite_w, int composite_h, float mm_per_pixel, int monochromatic,
                        float splat_sigma_px, int splat_radius_px, float* d_out_r, float* d_out_g,
                        float* d_out_b, void* stream);

/* Number of kernel launches issued by the last device call on this thread. */
int gl_last_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif /* GHOSTLIGHT_GB300_H */
