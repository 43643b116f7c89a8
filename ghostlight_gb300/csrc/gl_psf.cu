// gl_psf.cu — PSF grid renderer: per source, the lens's primary-ray spot
// (every pupil sample at every wavelength) splatted into its own tile of a
// composite atlas (psf_kernel, psf_render.cu:30-232).
//
// GB300 layout: the packed lens records and the per-wavelength IOR slices are
// staged in shared memory once per CTA; one thread per (source, pupil sample)
// walks the wavelengths with the reference-formulation primary trace; the
// splat is bilinear, or a normalised Gaussian of the configured physical
// width, clipped to the source's tile.
#include "gl_internal.h"
#include "gl_render.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

namespace gl {
namespace {

constexpr int kPsfThreads = 256;

struct PsfArgs {
    const SurfRec* recs;
    const float* ior_at;         // [spec][surf]
    const float4* spec;          // lambda, cmf r g b
    const gl_psf_source* src;
    const float2* grid;
    int n_surf, n_spec, n_src, n_grid;
    float front_R, start_z, mm_per_pixel, ray_weight;
    int tile_w, tile_h, comp_w, comp_h, mono;
    float sigma_px;
    int radius_px;
    float* out_r;
    float* out_g;
    float* out_b;
    int tile_smem;       // 1: the CTA's source tile is accumulated in shared memory
};

// Adds a ray-wavelength's weighted colour to one composite pixel: into the
// CTA's shared-memory copy of its source's tile (planes of tile_w x tile_h),
// or straight into the composite with global atomics.
__device__ __forceinline__ void deposit(const PsfArgs& A, float* tile, int tx, int ty, int pix, float lum,
                                       float cr, float cg, float cb, float wt)
{
    if (tile != nullptr)
    {
        const int t = ty * A.tile_w + tx, plane = A.tile_w * A.tile_h;
        if (A.mono)
        {
            if (fabsf(lum) > 1e-14f) atomicAdd(tile + t, lum * wt);
        }
        else
        {
            if (fabsf(cr) > 1e-14f) atomicAdd(tile + t, cr * wt);
            if (fabsf(cg) > 1e-14f) atomicAdd(tile + plane + t, cg * wt);
            if (fabsf(cb) > 1e-14f) atomicAdd(tile + 2 * plane + t, cb * wt);
        }
        return;
    }
    if (A.mono)
    {
        if (fabsf(lum) > 1e-14f) atomicAdd(A.out_r + pix, lum * wt);
    }
    else
    {
        if (fabsf(cr) > 1e-14f) atomicAdd(A.out_r + pix, cr * wt);
        if (fabsf(cg) > 1e-14f) atomicAdd(A.out_g + pix, cg * wt);
        if (fabsf(cb) > 1e-14f) atomicAdd(A.out_b + pix, cb * wt);
    }
}

__device__ __forceinline__ void psf_trace_one(const PsfArgs& A, const SurfRec* lens, const float* at, float* tile,
                                              int si, int gi);

__global__ void __launch_bounds__(kPsfThreads) psf_kernel(PsfArgs A)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    SurfRec* lens = reinterpret_cast<SurfRec*>(smem_raw);
    float* at = reinterpret_cast<float*>(lens + A.n_surf);
    {
        const int words = A.n_surf * (int)(sizeof(SurfRec) / 4);
        const int* s = reinterpret_cast<const int*>(A.recs);
        int* d = reinterpret_cast<int*>(lens);
        for (int i = threadIdx.x; i < words; i += blockDim.x) d[i] = s[i];
        for (int i = threadIdx.x; i < A.n_spec * A.n_surf; i += blockDim.x) at[i] = A.ior_at[i];
    }
    // every ray of this CTA belongs to source blockIdx.x and deposits only in
    // its tile: accumulate the tile in shared memory, add it to the composite once
    float* tile = nullptr;
    const int planes = A.mono ? 1 : 3, tile_px = A.tile_w * A.tile_h;
    if (A.tile_smem)
    {
        tile = reinterpret_cast<float*>(reinterpret_cast<unsigned char*>(at + A.n_spec * A.n_surf) +
                                        ((16 - (((uintptr_t)(at + A.n_spec * A.n_surf)) & 15)) & 15));
        for (int i = threadIdx.x; i < planes * tile_px; i += blockDim.x) tile[i] = 0.0f;
    }
    __syncthreads();
    const int si = blockIdx.x;
    const int gi = blockIdx.y * kPsfThreads + threadIdx.x;
    if (si < A.n_src && gi < A.n_grid) psf_trace_one(A, lens, at, tile, si, gi);
    if (!A.tile_smem || si >= A.n_src) return;
    __syncthreads();
    const gl_psf_source S = A.src[si];
    float* outs[3] = {A.out_r, A.out_g, A.out_b};
    for (int i = threadIdx.x; i < planes * tile_px; i += blockDim.x)
    {
        const float v = tile[i];
        if (v == 0.0f) continue;
        const int pl = i / tile_px, t = i - pl * tile_px;
        const int xi = S.tile_x0 + t % A.tile_w, yi = S.tile_y0 + t / A.tile_w;
        if (xi < 0 || xi >= A.comp_w || yi < 0 || yi >= A.comp_h) continue;
        atomicAdd(outs[pl] + (size_t)yi * A.comp_w + xi, v);
    }
}

// One pupil sample of one source through every wavelength, splatted into the
// source's tile (tile != nullptr: the CTA's shared-memory copy of it).
__device__ __forceinline__ void psf_trace_one(const PsfArgs& A, const SurfRec* lens, const float* at, float* tile,
                                              int si, int gi)
{
    const gl_psf_source S = A.src[si];
    const float2 uv = A.grid[gi];
    const float bx = tanf(S.angle_x), by = tanf(S.angle_y);
    const V3 dir = normalized(v3(bx, by, 1.0f));
    const V3 org = v3(uv.x * A.front_R - kSpawnOffset * bx, uv.y * A.front_R - kSpawnOffset * by, A.start_z);
    const int tx_min = S.tile_x0, ty_min = S.tile_y0, tx_max = S.tile_x0 + A.tile_w, ty_max = S.tile_y0 + A.tile_h;
    for (int l = 0; l < A.n_spec; ++l)
    {
        const float4 sp = A.spec[l];
        const TraceOut r = trace_primary(lens, A.n_surf, at + l * A.n_surf, org, dir, sp.x);
        if (r.status != GL_TRACE_OK || !isfinite(r.x) || !isfinite(r.y)) continue;
        const float tx = (r.x - S.chief_x_mm) / A.mm_per_pixel + (float)A.tile_w * 0.5f;
        const float ty = (r.y - S.chief_y_mm) / A.mm_per_pixel + (float)A.tile_h * 0.5f;
        const float margin = (float)(A.radius_px > 0 ? A.radius_px + 1 : 1);
        if (tx < -margin || tx > (float)A.tile_w + margin || ty < -margin || ty > (float)A.tile_h + margin) continue;
        const float px = tx + (float)S.tile_x0, py = ty + (float)S.tile_y0;
        const float w = r.w * A.ray_weight;
        const float lum = (S.r + S.g + S.b) * (1.0f / 3.0f) * sp.z * w;
        const float cr = S.r * sp.y * w, cg = S.g * sp.z * w, cb = S.b * sp.w * w;
        if (A.sigma_px <= 0.0f)
        {
            const int x0 = (int)floorf(px - 0.5f), y0 = (int)floorf(py - 0.5f);
            const float fx = (px - 0.5f) - (float)x0, fy = (py - 0.5f) - (float)y0;
            const float bw[4] = {(1.0f - fx) * (1.0f - fy), fx * (1.0f - fy), (1.0f - fx) * fy, fx * fy};
            #pragma unroll
            for (int k = 0; k < 4; ++k)
            {
                const int xi = x0 + (k & 1), yi = y0 + (k >> 1);
                if (xi < tx_min || xi >= tx_max || yi < ty_min || yi >= ty_max || xi < 0 || xi >= A.comp_w ||
                    yi < 0 || yi >= A.comp_h)
                    continue;
                deposit(A, tile, xi - S.tile_x0, yi - S.tile_y0, yi * A.comp_w + xi, lum, cr, cg, cb, bw[k]);
            }
        }
        else
        {
            const float inv2 = 1.0f / (2.0f * A.sigma_px * A.sigma_px);
            const int cx = (int)floorf(px), cy = (int)floorf(py);
            const float ox = px - ((float)cx + 0.5f), oy = py - ((float)cy + 0.5f);
            const int R = A.radius_px;
            float wsum = 0.0f;
            for (int dy = -R; dy <= R; ++dy)
            {
                const float dyr = (float)dy - oy;
                for (int dx = -R; dx <= R; ++dx)
                {
                    const float dxr = (float)dx - ox;
                    wsum += expf(-(dxr * dxr + dyr * dyr) * inv2);
                }
            }
            const float inv_wsum = wsum > 1e-20f ? 1.0f / wsum : 0.0f;
            for (int dy = -R; dy <= R; ++dy)
            {
                const int yi = cy + dy;
                if (yi < ty_min || yi >= ty_max || yi < 0 || yi >= A.comp_h) continue;
                const float dyr = (float)dy - oy;
                for (int dx = -R; dx <= R; ++dx)
                {
                    const int xi = cx + dx;
                    if (xi < tx_min || xi >= tx_max || xi < 0 || xi >= A.comp_w) continue;
                    const float dxr = (float)dx - ox;
                    const float wt = expf(-(dxr * dxr + dyr * dyr) * inv2) * inv_wsum;
                    if (wt < 1e-6f) continue;
                    deposit(A, tile, xi - S.tile_x0, yi - S.tile_y0, yi * A.comp_w + xi, lum, cr, cg, cb, wt);
                }
            }
        }
    }
}

}  // namespace
}  // namespace gl

using namespace gl;

// The render of both entries: `ordered` takes the scratch (lens records,
// index table, spectrum, sources, pupil grid: one block) from the device's
// stream-ordered pool and frees it in stream order without waiting; otherwise
// plain allocations and a wait on the stream before they are freed.
static int psf_render_impl(const gl_surface* surfaces, int n_surfaces, const gl_psf_source* sources, int n_sources,
                           const gl_pupil_sample* grid, int n_grid, const gl_spectral_sample* spec, int n_spec,
                           int tile_w, int tile_h, int composite_w, int composite_h, float mm_per_pixel,
                           int monochromatic, float splat_sigma_px, int splat_radius_px, float* d_out_r,
                           float* d_out_g, float* d_out_b, void* stream, bool ordered)
{
    if (!surfaces || n_surfaces <= 0) return fail(GL_ERR_INVALID, "psf_render: lens has no surfaces");
    if (n_sources < 0 || n_grid < 0 || n_spec < 1 || (n_sources > 0 && !sources) || (n_grid > 0 && !grid) || !spec)
        return fail(GL_ERR_INVALID, "psf_render: bad arguments");
    if (tile_w <= 0 || tile_h <= 0 || composite_w <= 0 || composite_h <= 0 || !(mm_per_pixel > 0.0f))
        return fail(GL_ERR_INVALID, "psf_render: grid and tile dimensions must be positive");
    if ((long long)composite_w * composite_h > (1LL << 31)) return fail(GL_ERR_INVALID, "psf_render: too many pixels");
    if (!d_out_r || (!monochromatic && (!d_out_g || !d_out_b))) return fail(GL_ERR_INVALID, "psf_render: null output");
    if (splat_radius_px < 0 || splat_radius_px > 16) return fail(GL_ERR_INVALID, "psf_render: splat radius must be 0..16");
    if (n_sources == 0 || n_grid == 0) return GL_OK;
    int dev = 0;
    GL_CUDA_TRY(cudaGetDevice(&dev));
    std::vector<SurfRec> recs((size_t)n_surfaces);
    int rc = pack_lens(surfaces, n_surfaces, recs.data(), dev);
    if (rc) return rc;
    std::vector<float> lams((size_t)n_spec), at((size_t)n_spec * n_surfaces), bf((size_t)n_spec * n_surfaces);
    std::vector<float4> sp((size_t)n_spec);
    for (int i = 0; i < n_spec; ++i)
    {
        lams[i] = spec[i].lambda;
        sp[i] = make_float4(spec[i].lambda, spec[i].cmf_r, spec[i].cmf_g, spec[i].cmf_b);
    }
    build_ior_tables(surfaces, n_surfaces, lams.data(), n_spec, at.data(), bf.data());
    cudaStream_t st = (cudaStream_t)stream;
    // one scratch block, each part 256-byte aligned
    auto up = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t o_recs = 0, o_at = o_recs + up(recs.size() * sizeof(SurfRec)), o_spec = o_at + up(at.size() * sizeof(float)),
                 o_src = o_spec + up(sp.size() * sizeof(float4)), o_grid = o_src + up((size_t)n_sources * sizeof(gl_psf_source)),
                 total = o_grid + up((size_t)n_grid * sizeof(float2));
    char* block = nullptr;
    cudaError_t e;
    if (ordered)
    {
        cudaMemPool_t pool;
        e = shared_device_pool(dev, &pool);
        if (e == cudaSuccess) e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&block), total, pool, st);
    }
    else
        e = cudaMalloc(&block, total);
    if (e != cudaSuccess)
        return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA, std::string("psf_render: ") + cudaGetErrorString(e));
    SurfRec* d_recs = reinterpret_cast<SurfRec*>(block + o_recs);
    float* d_at = reinterpret_cast<float*>(block + o_at);
    float4* d_spec = reinterpret_cast<float4*>(block + o_spec);
    gl_psf_source* d_src = reinterpret_cast<gl_psf_source*>(block + o_src);
    float2* d_grid = reinterpret_cast<float2*>(block + o_grid);
    e = cudaMemcpyAsync(d_recs, recs.data(), recs.size() * sizeof(SurfRec), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_at, at.data(), at.size() * sizeof(float), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_spec, sp.data(), sp.size() * sizeof(float4), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_src, sources, (size_t)n_sources * sizeof(gl_psf_source), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_grid, grid, (size_t)n_grid * sizeof(float2), cudaMemcpyHostToDevice, st);
    // the CTA's source tile in shared memory when it fits (96 KB of tile)
    const size_t tile_bytes = (size_t)(monochromatic ? 1 : 3) * tile_w * tile_h * sizeof(float);
    const bool tile_smem = tile_bytes <= 96 * 1024;
    const size_t smem = recs.size() * sizeof(SurfRec) + at.size() * sizeof(float) + (tile_smem ? tile_bytes + 16 : 0);
    if (e == cudaSuccess && smem > 48 * 1024)
        e = (cudaError_t)raise_smem_limit((const void*)psf_kernel, smem);
    if (e == cudaSuccess)
    {
        PsfArgs A;
        A.recs = d_recs; A.ior_at = d_at; A.spec = d_spec; A.src = d_src; A.grid = d_grid;
        A.n_surf = n_surfaces; A.n_spec = n_spec; A.n_src = n_sources; A.n_grid = n_grid;
        A.front_R = surfaces[0].semi_aperture; A.start_z = surfaces[0].z - kSpawnOffset;
        A.mm_per_pixel = mm_per_pixel; A.ray_weight = 1.0f / (float)n_grid;
        A.tile_w = tile_w; A.tile_h = tile_h; A.comp_w = composite_w; A.comp_h = composite_h;
        A.mono = monochromatic ? 1 : 0;
        A.sigma_px = splat_sigma_px; A.radius_px = splat_radius_px;
        A.out_r = d_out_r; A.out_g = d_out_g; A.out_b = d_out_b;
        A.tile_smem = tile_smem ? 1 : 0;
        const dim3 g((unsigned)n_sources, (unsigned)((n_grid + kPsfThreads - 1) / kPsfThreads));
        psf_kernel<<<g, kPsfThreads, smem, st>>>(A);
        e = cudaGetLastError();
    }
    if (ordered)
    {
        const cudaError_t f = cudaFreeAsync(block, st);
        if (e == cudaSuccess) e = f;
    }
    else
    {
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        cudaFree(block);
    }
    if (e != cudaSuccess)
        return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA, std::string("psf_render: ") + cudaGetErrorString(e));
    g_last_launches = 1;
    return GL_OK;
}

extern "C" int gl_psf_render(const gl_surface* surfaces, int n_surfaces, const gl_psf_source* sources, int n_sources,
                             const gl_pupil_sample* grid, int n_grid, const gl_spectral_sample* spec, int n_spec,
                             int tile_w, int tile_h, int composite_w, int composite_h, float mm_per_pixel,
                             int monochromatic, float splat_sigma_px, int splat_radius_px, float* d_out_r,
                             float* d_out_g, float* d_out_b, void* stream)
{
    return psf_render_impl(surfaces, n_surfaces, sources, n_sources, grid, n_grid, spec, n_spec, tile_w, tile_h,
                           composite_w, composite_h, mm_per_pixel, monochromatic, splat_sigma_px, splat_radius_px,
                           d_out_r, d_out_g, d_out_b, stream, false);
}

extern "C" int gl_psf_render_async(const gl_surface* surfaces, int n_surfaces, const gl_psf_source* sources,
                                   int n_sources, const gl_pupil_sample* grid, int n_grid,
                                   const gl_spectral_sample* spec, int n_spec, int tile_w, int tile_h,
                                   int composite_w, int composite_h, float mm_per_pixel, int monochromatic,
                                   float splat_sigma_px, int splat_radius_px, float* d_out_r, float* d_out_g,
                                   float* d_out_b, void* stream)
{
    return psf_render_impl(surfaces, n_surfaces, sources, n_sources, grid, n_grid, spec, n_spec, tile_w, tile_h,
                           composite_w, composite_h, mm_per_pixel, monochromatic, splat_sigma_px, splat_radius_px,
                           d_out_r, d_out_g, d_out_b, stream, true);
}
