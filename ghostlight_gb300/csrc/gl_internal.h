// gl_internal.h — declarations shared by the translation units of
// libghostlight_gb300 (host builders, culler, render, starburst, conv).
#pragma once

#include "ghostlight_gb300.h"
#include "gl_trace.cuh"

#include <string>
#include <vector>

namespace gl {

extern thread_local std::string g_last_error;
extern thread_local int g_last_launches;
int fail(int code, const std::string& msg);

// Raise (never lower) a kernel's dynamic shared-memory limit on the current
// device; returns a cudaError_t.  The limit belongs to the function, shared
// by every plan on the device, so a plan prepared for a smaller size must not
// shrink it under the launches of a plan prepared earlier for a larger one.
int raise_smem_limit(const void* kernel, size_t bytes);

// Entrance-pupil silhouette (aperture_sampler.h:49-83), plain polygon form.
struct PupilMask {
    float aspect = 1.0f;
    int n_blades = 0;
    float rot_rad = 0.0f;
    float apothem = 1.0f;
    float sector = 1.0f;
    BladeProfile blade{};       // the stop's authored blade shape (blade.deformed), dropped under an override
};

// Pack the trace records of a lens.  Table coatings resolve to their table
// in the memory space of the trace that reads the records: the host
// (kTablesHost) or device `tables` (copied there on first use unless
// `may_upload` is false).
constexpr int kTablesHost = -1;
constexpr int kStoreImage = 100;     // store entries that hold an aperture bitmap
int pack_lens(const gl_surface* in, int n, SurfRec* out, int tables, bool may_upload = true);
int coating_table_address(int id, int model, int device, bool may_upload, const float** out, int* n0, int* n1,
                          int* discard, float* ref_ior);
float ior_at(const gl_surface& s, float lam);
float ior_before_nd(const gl_surface* s, int idx);
void build_ior_tables(const gl_surface* s, int n, const float* lambdas, int n_lam, float* at, float* bf);
PupilMask resolve_pupil_mask(const gl_surface* surfs, int n, int blades_override, float rotation_deg);
bool pupil_contains(const PupilMask& m, float u, float v);
int build_aperture_samples(const gl_surface* surfs, int n, const gl_sampler_params& p,
                           std::vector<gl_pupil_sample>& out);
int output_matrix(int cs, const float* custom, float M[9]);
int input_matrix(int cs, const float* custom, float M[9]);
std::vector<gl_spectral_sample> spectral_table(int n, float lmin, float lmax, const float M[9]);
void spectral_correction(const std::vector<gl_spectral_sample>& tn, float lmin, float lmax,
                         const float M[9], float C[9]);
// The culler's per-pair probes (ghost.cpp:34-102): the three axial rays of
// the intensity estimate and the 8 x 8 spread probe's landing box.
struct FilterProbe {
    float w[3];        // per-wavelength weight of the axial ray
    int wok[3];        // 1 when that ray reached the sensor
    float mnx, mxx, mny, mxy;
    int valid;         // spread-probe rays that reached the sensor
};
void host_filter_probe(const gl_surface* s, const SurfRec* recs, int n, int a, int b, FilterProbe* out);
float host_intensity_estimate(const gl_surface* s, const SurfRec* recs, int n, int a, int b);
float host_spread_boost(const gl_surface* s, const SurfRec* recs, int n, int a, int b,
                        float hw, float hh, float max_boost);

}  // namespace gl

#define GL_CUDA_TRY(expr)                                                          \
    do {                                                                           \
        cudaError_t _e = (expr);                                                   \
        if (_e != cudaSuccess)                                                     \
            return ::gl::fail(_e == cudaErrorMemoryAllocation ? GL_ERR_OOM         \
                                                              : GL_ERR_CUDA,       \
                              std::string(#expr) + ": " + cudaGetErrorString(_e)); \
    } while (0)
