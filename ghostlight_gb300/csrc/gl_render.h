// gl_render.h — the render kernel's device-side argument block and the
// launch helpers shared by the plan path (gl_ghost.cu) and the serving path
// (gl_serve.cu).
#pragma once

#include "gl_internal.h"

#include <cuda_runtime.h>

#include <vector>

namespace gl {

constexpr int kRenderThreads = 128;
constexpr int kTile = 32;          // pupil samples per work item = one warp
constexpr int kMaxSpec = 256;

struct PairDev {
    int a, b;
    float boost, w_ray;
};

struct SourceDev {
    float dx, dy, dz, sdx;
    float sdy, r, g, b;
};

struct RenderArgs {
    const SurfRec* recs;
    const float* ior_at;
    const float* ior_bf;
    const float4* spec;
    const int4* items;        // (pair, source, sample_start, sample_count)
    const PairDev* pairs;
    const SourceDev* sources;
    const float2* samples;
    int* counter;             // persistent queue head; null = static item assignment
    float4* accum;            // RGBA, width x height
    int* pair_hits;           // off-sensor cull: per-pair probe hits (null = no cull)
    unsigned long long* traced;   // ray-wavelength traces executed (null = not counted)
    unsigned long long* stats;    // diagnostic pass: per pair {traces, survived, on sensor} (null = off)
    int n_surf, n_spec, n_items, item_base;
    int l_chunks;             // wavelength ranges per item (tasks = items x l_chunks); <= 1: one
    // Uniform-grid items (items == null): every pair x source traces the same
    // grid, item i = (pair, source, 32-sample tile) in pair-major order,
    // computed from the index; w_uniform replaces the pairs' per-ray weight.
    int u_tiles, u_n_src, u_grid_base, u_grid_n;
    float w_uniform;
    // Up to three uniform item ranges in one queue (the off-sensor probe
    // passes): items [u_start[q], u_start[q + 1]) trace grid u_base[q] ..
    // + u_n[q] in u_tl[q] tiles.  u_npass = 0: the single range above.
    int u_npass;
    int u_start[4], u_base[3], u_n[3], u_tl[3];
    int width, height;
    float fmt_w, fmt_h, fmt_x0, fmt_y0;
    float hw2, hh2, gain, front_R, start_z;
    // Probe in two stages (plan path, one source): stage 1 traces wavelength
    // lam_lo..lam_hi (the first) and writes each ray's death step to
    // death[pair * perm_stride + sample]; stage 2 traces the rest with each
    // pair's samples read through perm[pair * perm_stride + i] (sorted by
    // that death step).  lam_hi = 0: the task's own wavelength range.
    int lam_lo, lam_hi;
    unsigned char* death;
    const unsigned short* perm;
    int perm_stride;
};

// The device's stream-ordered memory pool (freed blocks stay reserved).
cudaError_t shared_device_pool(int dev, cudaMemPool_t* out);
// Default wavelength split of a render's items (tasks per item) for n_spec wavelengths.
int default_lambda_split(int n_spec);
// Shared memory of one render CTA for a lens of n_surf surfaces and n_spec wavelengths.
size_t render_smem(int n_surf, int n_spec);
// Opt the render kernels in to `smem` bytes of dynamic shared memory and
// report resident CTAs per SM and the SM count.
cudaError_t render_prepare(size_t smem, int* per_sm, int* n_sm);
cudaError_t render_launch(const RenderArgs& A, bool probe, int grid, size_t smem, cudaStream_t st);
cudaError_t flush_launch(const float4* accum, size_t n_px, float* r, float* g, float* b, int apply, const float* C,
                         cudaStream_t st);
// Beam of one source (direction, spawn-plane shift, colour), ghost_render.cu:349-358.
SourceDev make_source(const gl_flare_source& s);
// Samples of [begin, end) reordered along a Morton curve over the pupil square.
void morton_order(const gl_pupil_sample* in, int n, gl_pupil_sample* out);
// Pupil samples of the three off-sensor probe passes (40x40, wang jitter,
// fixed seeds; ghost_render.cu:1022-1027), concatenated; pass p starts at begin[p].
int probe_grids(const gl_surface* surfaces, int n_surf, int blades_override, float rotation_deg,
                std::vector<gl_pupil_sample>& out, int begin[4]);

}  // namespace gl
