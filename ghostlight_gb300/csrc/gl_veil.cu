// gl_veil.cu — veiling-glare layer: the analytic glare-spread function
// g(r) = (a^2 / (r^2 + a^2))^p around each source, energy-normalised and
// area-resampled onto the output grid (render_veil, veil_render.cu:243-414).
//
// GB300 layout: the sprite is monochrome (the halo is achromatic; the source
// colour tints it at the splat), baked once per falloff into a resident
// 1024^2 grid whose sum is reduced in FP64 on the device; the per-execute
// work is a power-of-two box downsample toward the output pitch and one
// thread per output pixel that integrates the sprite over its own footprint
// for every source and writes (or adds) its three channels — no atomics.
#include "gl_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>

namespace gl {
namespace {

constexpr int kVeilGrid = 1024;       // sprite side (texels)
constexpr int kVeilCoreDiv = 32;      // core radius = grid / 32 texels: the sprite spans 16 core radii
constexpr int kSpriteOversample = 3;  // sprite texels kept per output pixel after the downsample

__global__ void veil_bake_kernel(float* __restrict__ ref, int N, float a_texels, float p)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= N * N) return;
    const int i = idx % N, j = idx / N;
    const float dx = (float)(i - N / 2), dy = (float)(j - N / 2);
    const float a2 = a_texels * a_texels;
    ref[idx] = powf(a2 / (dx * dx + dy * dy + a2), p);
}

// One block: FP64 sum of the grid (deterministic order), then scale to unit sum.
__global__ void __launch_bounds__(1024) veil_normalise_kernel(float* __restrict__ ref, int n)
{
    __shared__ double part[1024];
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) s += (double)ref[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1)
    {
        if ((int)threadIdx.x < h) part[threadIdx.x] += part[threadIdx.x + h];
        __syncthreads();
    }
    const double total = part[0];
    if (!(total > 0.0)) return;
    const float k = (float)(1.0 / total);
    for (int i = threadIdx.x; i < n; i += blockDim.x) ref[i] *= k;
}

// Box-sum the N x N sprite into M x M (M = N / ds): summing keeps the deposit
// an exact integral of the fine pattern over each coarse texel.
__global__ void veil_downsample_kernel(const float* __restrict__ fine, int N, int ds, float* __restrict__ coarse,
                                       int M)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= M * M) return;
    const int a = idx % M, b = idx / M;
    float s = 0.0f;
    for (int jj = 0; jj < ds; ++jj)
        for (int ii = 0; ii < ds; ++ii) s += fine[(size_t)(b * ds + jj) * N + a * ds + ii];
    coarse[idx] = s;
}

struct VeilArgs {
    const float* sprite;
    int M;
    float sx_ds, sy_ds;        // sensor mm per coarse texel
    float px_mm_x, px_mm_y;    // sensor mm per output pixel
    int rx, ry;                // footprint half-extent in pixels
    const gl_veil_source* src;
    int n_src;
    float gain;
    float* out_r;
    float* out_g;
    float* out_b;
    int width, height, x0, y0, bw, bh;   // pixel box covering every source's footprint
    int accumulate;
};

// One thread per output pixel of the box: for every source whose footprint
// holds the pixel, integrate the sprite over the pixel's sensor footprint
// (texel overlap areas; at most 65 x 65 texels), tint, sum, store.
__global__ void veil_splat_kernel(VeilArgs A)
{
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)A.bw * A.bh) return;
    const int ix = A.x0 + (int)(t % A.bw), iy = A.y0 + (int)(t / A.bw);
    if (ix < 0 || ix >= A.width || iy < 0 || iy >= A.height) return;
    const int M = A.M;
    float ar = 0.0f, ag = 0.0f, ab = 0.0f;
    for (int si = 0; si < A.n_src; ++si)
    {
        const gl_veil_source s = A.src[si];
        const int cx = (int)floorf(s.px), cy = (int)floorf(s.py);
        if (ix < cx - A.rx || ix > cx + A.rx || iy < cy - A.ry || iy > cy + A.ry) continue;
        // texel coordinates of the pixel's edges (splat_resample_kernel, veil_render.cu:196-201)
        const float ax0 = (((float)ix - s.px) * A.px_mm_x) / A.sx_ds + 0.5f * (float)M - 0.5f;
        const float ax1 = (((float)ix + 1.0f - s.px) * A.px_mm_x) / A.sx_ds + 0.5f * (float)M - 0.5f;
        const float by0 = (((float)iy - s.py) * A.px_mm_y) / A.sy_ds + 0.5f * (float)M - 0.5f;
        const float by1 = (((float)iy + 1.0f - s.py) * A.px_mm_y) / A.sy_ds + 0.5f * (float)M - 0.5f;
        const float xlo = ax0 + 0.5f, xhi = ax1 + 0.5f, ylo = by0 + 0.5f, yhi = by1 + 0.5f;
        int i0 = (int)floorf(xlo), i1 = (int)floorf(xhi - 1e-6f);
        int j0 = (int)floorf(ylo), j1 = (int)floorf(yhi - 1e-6f);
        i0 = max(i0, 0); i1 = min(i1, M - 1);
        j0 = max(j0, 0); j1 = min(j1, M - 1);
        if (i1 < i0 || j1 < j0) continue;
        i1 = min(i1, i0 + 64);
        j1 = min(j1, j0 + 64);
        float acc = 0.0f;
        for (int j = j0; j <= j1; ++j)
        {
            const float yov = fminf(yhi, (float)(j + 1)) - fmaxf(ylo, (float)j);
            if (yov <= 0.0f) continue;
            const float* row = A.sprite + (size_t)j * M;
            for (int i = i0; i <= i1; ++i)
            {
                const float xov = fminf(xhi, (float)(i + 1)) - fmaxf(xlo, (float)i);
                if (xov <= 0.0f) continue;
                acc += __ldg(row + i) * (xov * yov);
            }
        }
        ar += acc * s.r * A.gain;
        ag += acc * s.g * A.gain;
        ab += acc * s.b * A.gain;
    }
    const size_t o = (size_t)iy * A.width + ix;
    if (A.accumulate) { A.out_r[o] += ar; A.out_g[o] += ag; A.out_b[o] += ab; }
    else { A.out_r[o] = ar; A.out_g[o] = ag; A.out_b[o] = ab; }
}

}  // namespace

struct VeilPlan {
    float falloff = 1.0f;
    float* ref = nullptr;       // N x N, unit sum
    float* coarse = nullptr;    // up to (N/2)^2 downsampled
};

}  // namespace gl

struct gl_veil_plan { gl::VeilPlan* p; };

using namespace gl;

extern "C" int gl_veil_plan_create(float falloff, void* stream, gl_veil_plan** out)
{
    if (!out) return fail(GL_ERR_INVALID, "veil_plan_create: null out");
    float p = falloff;
    if (!(p >= 1.0f)) p = 1.0f;      // the reference's clamp (veil_render.cu:286-288)
    if (p > 3.0f) p = 3.0f;
    VeilPlan* v = new VeilPlan();
    v->falloff = p;
    const int N = kVeilGrid;
    const size_t NN = (size_t)N * N;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMalloc(&v->ref, NN * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&v->coarse, (NN / 4) * sizeof(float));
    if (e == cudaSuccess)
    {
        veil_bake_kernel<<<(int)((NN + 255) / 256), 256, 0, st>>>(v->ref, N, (float)N / (float)kVeilCoreDiv, p);
        veil_normalise_kernel<<<1, 1024, 0, st>>>(v->ref, (int)NN);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
    {
        cudaFree(v->ref); cudaFree(v->coarse);
        delete v;
        return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA, std::string("veil_plan_create: ") + cudaGetErrorString(e));
    }
    *out = new gl_veil_plan{v};
    return GL_OK;
}

namespace gl {
namespace {

// The scale of one execute (veil_render.cu:276-296): core radius a = spread x
// the sensor half-height (half-width when that is unset), the fine texel
// pitch a / (N / 32), and the power-of-two box sum ds toward three texels per
// output pixel.
struct VeilGeom {
    float spread, half_ref, a_texels, dx_fine, px_mm_x, px_mm_y;
    int ds, M;
};

int veil_geometry(const gl_veil_params* prm, VeilGeom& g)
{
    if (prm->width <= 0 || prm->height <= 0 || prm->fmt_w <= 0 || prm->fmt_h <= 0)
        return fail(GL_ERR_INVALID, "veil_plan_execute: degenerate output dimensions");
    if ((long long)prm->width * prm->height > (1LL << 31)) return fail(GL_ERR_INVALID, "veil_plan_execute: too many pixels");
    g.half_ref = prm->sensor_half_h > 0.0f ? prm->sensor_half_h : prm->sensor_half_w;
    if (!(g.half_ref > 0.0f) || !(prm->sensor_half_w > 0.0f) || !(prm->sensor_half_h > 0.0f))
        return fail(GL_ERR_INVALID, "veil_plan_execute: degenerate sensor half-size");
    float spread = prm->spread;
    if (!(spread > 0.0f)) spread = 0.12f;
    g.spread = spread < 1e-3f ? 1e-3f : (spread > 4.0f ? 4.0f : spread);
    const int N = kVeilGrid;
    g.a_texels = (float)N / (float)kVeilCoreDiv;
    g.dx_fine = g.spread * g.half_ref / g.a_texels;                 // sensor mm per fine texel
    g.px_mm_x = 2.0f * prm->sensor_half_w / (float)prm->fmt_w;
    g.px_mm_y = 2.0f * prm->sensor_half_h / (float)prm->fmt_h;
    const double target = std::min((double)g.px_mm_x / (g.dx_fine * kSpriteOversample),
                                    (double)g.px_mm_y / (g.dx_fine * kSpriteOversample));
    g.ds = 1;
    while (g.ds * 2 <= target && g.ds * 2 <= N / 8) g.ds *= 2;
    g.M = N / g.ds;
    return GL_OK;
}

}  // namespace
}  // namespace gl

extern "C" int gl_veil_plan_execute(gl_veil_plan* plan, const gl_veil_source* d_sources, int n_sources,
                                    const gl_veil_params* prm, float* d_out_r, float* d_out_g, float* d_out_b,
                                    void* stream)
{
    if (!plan || !prm || !d_out_r || !d_out_g || !d_out_b) return fail(GL_ERR_INVALID, "veil_plan_execute: null argument");
    if (n_sources < 0 || n_sources > 65536 || (n_sources > 0 && !d_sources))
        return fail(GL_ERR_INVALID, "veil_plan_execute: bad source list");
    VeilGeom G;
    if (int rc = veil_geometry(prm, G)) return rc;
    VeilPlan* v = plan->p;
    cudaStream_t st = (cudaStream_t)stream;
    const int N = kVeilGrid;
    const int ds = G.ds, M = G.M;
    const float dx_fine = G.dx_fine, px_mm_x = G.px_mm_x, px_mm_y = G.px_mm_y;
    int launches = 0;
    const float* sprite = v->ref;
    if (ds > 1)
    {
        veil_downsample_kernel<<<(M * M + 255) / 256, 256, 0, st>>>(v->ref, N, ds, v->coarse, M);
        sprite = v->coarse;
        ++launches;
    }
    VeilArgs A;
    A.sprite = sprite; A.M = M;
    A.sx_ds = dx_fine * ds; A.sy_ds = dx_fine * ds;
    A.px_mm_x = px_mm_x; A.px_mm_y = px_mm_y;
    A.rx = std::min((int)std::ceil(0.5 * M * A.sx_ds / px_mm_x) + 1, prm->width);
    A.ry = std::min((int)std::ceil(0.5 * M * A.sy_ds / px_mm_y) + 1, prm->height);
    A.src = d_sources; A.n_src = n_sources; A.gain = prm->gain;
    A.out_r = d_out_r; A.out_g = d_out_g; A.out_b = d_out_b;
    A.width = prm->width; A.height = prm->height;
    A.accumulate = prm->accumulate;
    // the whole frame: sources may move between executes of a captured graph
    A.x0 = 0; A.y0 = 0; A.bw = prm->width; A.bh = prm->height;
    if (!prm->accumulate || n_sources > 0)
    {
        const long long total = (long long)A.bw * A.bh;
        veil_splat_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(A);
        ++launches;
    }
    GL_CUDA_TRY(cudaGetLastError());
    g_last_launches = launches;
    return GL_OK;
}

extern "C" int gl_veil_plan_destroy(gl_veil_plan* plan)
{
    if (!plan) return GL_OK;
    cudaFree(plan->p->ref);
    cudaFree(plan->p->coarse);
    delete plan->p;
    delete plan;
    return GL_OK;
}

extern "C" int gl_veil_plan_geometry(const gl_veil_plan* plan, const gl_veil_params* prm, gl_veil_geometry* out)
{
    if (!plan || !prm || !out) return fail(GL_ERR_INVALID, "veil_plan_geometry: null argument");
    VeilGeom G;
    if (int rc = veil_geometry(prm, G)) return rc;
    out->grid = kVeilGrid;
    out->ds = G.ds;
    out->dx_mm = G.dx_fine;
    out->core_mm = G.spread * G.half_ref;
    out->falloff = plan->p->falloff;
    out->core_texels = G.a_texels;
    return GL_OK;
}

extern "C" int gl_veil_plan_read(const gl_veil_plan* plan, float* d_reference, void* stream)
{
    if (!plan || !d_reference) return fail(GL_ERR_INVALID, "veil_plan_read: null argument");
    const size_t NN = (size_t)kVeilGrid * kVeilGrid;
    GL_CUDA_TRY(cudaMemcpyAsync(d_reference, plan->p->ref, NN * sizeof(float), cudaMemcpyDeviceToDevice,
                                (cudaStream_t)stream));
    return GL_OK;
}
