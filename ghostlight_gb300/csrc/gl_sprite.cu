// gl_sprite.cu — the SPRITE starburst engine: one FFT of the stop pupil,
// baked over wavelength into an RGB sprite, splatted at every source.
//
// Restates the reference's default engine (render_starburst's sprite path,
// ghostlight/src/starburst_render.cu:969-1073, kernels :194-389):
//   |FFT(A)|^2 with DC at the grid centre -> normalised to unit sum -> the
//   sprite texel (i, j) = sum_l cmf_l * PSF(c + (i, j - c) lambda_ref /
//   lambda_l) (lambda_ref / lambda_l)^2 (Fourier scaling theorem, bilinear,
//   zero outside) -> box-summed by ds toward the output pitch -> each output
//   pixel integrates the sprite over its own footprint (area-weighted box
//   resample), times the source colour and the gain.
//
// GB300 layout (one GPU, everything resident in the plan):
//   * 2-D FFT as two shared-memory Stockham passes (gl_fft.cuh): row FFTs,
//     one CTA per row, skipping rows the pupil leaves dark (the pupil fills a
//     centred disc of `fill` of the grid, so most rows are zero); column FFTs
//     over groups of NB adjacent columns whose epilogue writes |X|^2 straight
//     to its fftshifted place and adds the block's energy to one FP64 sum;
//   * the wavelength bake and the ds x ds box sum fused in one kernel: each
//     coarse texel accumulates its fine texels in the reference's order, so
//     the N x N x 3 fine sprite (805 MB at N = 8192) never exists in HBM; the
//     1 / energy normalisation is read on the device (no host round trip);
//   * the splat: one thread per (source, output pixel in the footprint),
//     float atomics into the caller's planes (sources overlap), as the
//     reference does.
#include "gl_internal.h"
#include "gl_fft.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

namespace gl {
namespace {

constexpr int kSpriteThreads = 256;
constexpr int kMaxSpriteGrid = 8192;   // a complex row pair fits the 227 KB of shared memory

struct StarSource { float px, py, r, g, b; };

// columns per CTA in the column pass, so the interleaved pair of shared
// buffers stays within 8192 complex each
__host__ __device__ inline int col_group(int N) { return N >= 8192 ? 1 : (N >= 4096 ? 2 : 4); }

__global__ void __launch_bounds__(kSpriteThreads) sprite_rows(const float* __restrict__ pupil, int N, FftDims d,
                                                              const float2* __restrict__ tw, float2* __restrict__ work)
{
    extern __shared__ float2 sm[];
    float2* x = sm;
    float2* y = sm + padded((size_t)N);
    const int j = blockIdx.x;
    const float* row = pupil + (size_t)j * N;
    float2* out = work + (size_t)j * N;
    int lit = 0;
    for (int i = threadIdx.x; i < N; i += blockDim.x)
    {
        const float a = row[i];
        lit |= (a != 0.0f);
        x[pad(i)] = make_float2(a, 0.0f);
    }
    if (!__syncthreads_or(lit))
    {
        for (int i = threadIdx.x; i < N; i += blockDim.x) out[i] = make_float2(0.0f, 0.0f);
        return;
    }
    const float2* r = stockham<1>(x, y, d, tw, false);
    for (int i = threadIdx.x; i < N; i += blockDim.x) out[i] = r[pad(i)];
}

template <int NB>
__global__ void __launch_bounds__(kSpriteThreads) sprite_cols(const float2* __restrict__ work, int N, FftDims d,
                                                              const float2* __restrict__ tw, float* __restrict__ psf,
                                                              double* __restrict__ energy)
{
    extern __shared__ float2 sm[];
    float2* x = sm;
    float2* y = sm + padded((size_t)N * NB);
    __shared__ float red[kSpriteThreads / 32];
    const int c0 = blockIdx.x * NB;
    for (int it = threadIdx.x; it < N * NB; it += blockDim.x)
    {
        const int r = it / NB, s = it % NB;
        x[pad(r * NB + s)] = work[(size_t)r * N + c0 + s];
    }
    __syncthreads();
    const float2* X = stockham<NB>(x, y, d, tw, false);
    // fftshift: transform row k, column c lands at ((k + N/2) % N, (c + N/2) % N)
    const int h = N / 2;
    float part = 0.0f;
    for (int it = threadIdx.x; it < N * NB; it += blockDim.x)
    {
        const int k = it / NB, s = it % NB;
        const float2 z = X[pad(k * NB + s)];
        const float p = z.x * z.x + z.y * z.y;
        part += p;
        const int jj = (k + h) & (N - 1), ii = (c0 + s + h) & (N - 1);
        psf[(size_t)jj * N + ii] = p;
    }
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += (double)red[w];
        atomicAdd(energy, t);
    }
}

__device__ __forceinline__ float psf_bilinear(const float* __restrict__ psf, float fx, float fy, int N, float scale)
{
    if (fx < 0.0f || fy < 0.0f || fx >= (float)(N - 1) || fy >= (float)(N - 1)) return 0.0f;
    const int x0 = (int)floorf(fx), y0 = (int)floorf(fy);
    const float tx = fx - x0, ty = fy - y0;
    const float* r0 = psf + (size_t)y0 * N;
    const float* r1 = r0 + N;
    const float a = (r0[x0] * scale) * (1.0f - tx) + (r0[x0 + 1] * scale) * tx;
    const float b = (r1[x0] * scale) * (1.0f - tx) + (r1[x0 + 1] * scale) * tx;
    return a * (1.0f - ty) + b * ty;
}

// Column pass of the second transform of the matrix-DFT engine's compact
// autocorrelation (mdft_render.cu:88-99, 247-262): after the row pass of the
// fftshifted PSF, transform the columns whose x lag lies within +-mc of zero
// and write C[a][b] (a = y lag + mc, b = x lag + mc) = (-1)^(lx + ly)
// Re X[ly][lx] / (energy N^2).  The sign undoes the fftshift of the PSF
// (a shift by N/2 multiplies the transform by (-1)^l); energy = sum |FFT A|^2
// = G[0][0], summed on the device by the first column pass.  A real pupil has
// a real, point-symmetric autocorrelation: the imaginary part is rounding.
template <int NB>
__global__ void __launch_bounds__(kSpriteThreads) autocorr_cols(const float2* __restrict__ work, int N, FftDims d,
                                                                const float2* __restrict__ tw, int mc,
                                                                const double* __restrict__ energy,
                                                                float* __restrict__ C, int ldc)
{
    extern __shared__ float2 sm[];
    const int c0 = blockIdx.x * NB;
    const int h = N / 2;
    bool any = false;
    #pragma unroll
    for (int s = 0; s < NB; ++s)
    {
        const int c = c0 + s, lag = c <= h ? c : c - N;
        any |= (lag >= -mc && lag <= mc);
    }
    if (!any) return;                          // uniform over the block
    float2* x = sm;
    float2* y = sm + padded((size_t)N * NB);
    for (int it = threadIdx.x; it < N * NB; it += blockDim.x)
    {
        const int r = it / NB, s = it % NB;
        x[pad(r * NB + s)] = work[(size_t)r * N + c0 + s];
    }
    __syncthreads();
    const float2* X = stockham<NB>(x, y, d, tw, false);
    const double e = *energy;
    const float scale = e > 0.0 ? (float)(1.0 / (e * (double)N * (double)N)) : 0.0f;
    const int Mc = 2 * mc + 1;
    for (int it = threadIdx.x; it < Mc * NB; it += blockDim.x)
    {
        const int a = it / NB, s = it % NB;
        const int c = c0 + s, lx = c <= h ? c : c - N;
        if (lx < -mc || lx > mc) continue;
        const int ly = a - mc, r = (ly + N) & (N - 1);
        const float v = X[pad(r * NB + s)].x * scale;
        C[(size_t)a * ldc + (lx + mc)] = ((lx + ly) & 1) ? -v : v;
    }
}

// bake over wavelength + ds x ds box sum: coarse texel (a, b) of M x M
__global__ void __launch_bounds__(kSpriteThreads) sprite_bake(const float* __restrict__ psf, int N,
                                                              const float4* __restrict__ spec, int n_spec,
                                                              float lambda_ref, int ds, int M,
                                                              const double* __restrict__ energy,
                                                              float* __restrict__ sprite)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= M * M) return;
    const double e = *energy;
    const float scale = (e > 0.0) ? (float)(1.0 / e) : 0.0f;
    const int a = idx % M, b = idx / M;
    const float half = (float)(N / 2);
    float sr = 0.0f, sg = 0.0f, sb = 0.0f;
    for (int jj = 0; jj < ds; ++jj)
        for (int ii = 0; ii < ds; ++ii)
        {
            const int i = a * ds + ii, j = b * ds + jj;
            const float dx = (float)(i - N / 2), dy = (float)(j - N / 2);
            float cr = 0.0f, cg = 0.0f, cb = 0.0f;
            for (int l = 0; l < n_spec; ++l)
            {
                const float4 s = spec[l];
                const float k = lambda_ref / s.x;
                const float v = psf_bilinear(psf, half + dx * k, half + dy * k, N, scale) * k * k;
                cr += s.y * v;
                cg += s.z * v;
                cb += s.w * v;
            }
            sr += cr;
            sg += cg;
            sb += cb;
        }
    sprite[3 * (size_t)idx + 0] = sr;
    sprite[3 * (size_t)idx + 1] = sg;
    sprite[3 * (size_t)idx + 2] = sb;
}

// One output pixel of one source's footprint (offset t in its
// (2 rx + 1) x (2 ry + 1) box): the sprite integrated over the pixel's sensor
// footprint (texel overlap areas), tinted, added.
__device__ __forceinline__ void splat_pixel(const float* __restrict__ sprite, int M, float sx_ds, float sy_ds,
                                            float px_mm_x, float px_mm_y, int rx, int ry, const StarSource& s,
                                            long long t, float gain, float* __restrict__ out_r,
                                            float* __restrict__ out_g, float* __restrict__ out_b, int width,
                                            int height)
{
    const long long span_x = 2LL * rx + 1;
    const int oy = (int)(t / span_x) - ry, ox = (int)(t % span_x) - rx;
    const int ix = (int)floorf(s.px) + ox, iy = (int)floorf(s.py) + oy;
    if (ix < 0 || ix >= width || iy < 0 || iy >= height) return;
    // the pixel [ix, ix+1) x [iy, iy+1) in texel-cell coordinates (texel a
    // covers [a, a+1), its centre at sensor offset (a - M/2 + 0.5) pitch)
    const float xlo = ((ix - s.px) * px_mm_x) / sx_ds + 0.5f * M - 0.5f + 0.5f;
    const float xhi = ((ix + 1.0f - s.px) * px_mm_x) / sx_ds + 0.5f * M - 0.5f + 0.5f;
    const float ylo = ((iy - s.py) * px_mm_y) / sy_ds + 0.5f * M - 0.5f + 0.5f;
    const float yhi = ((iy + 1.0f - s.py) * px_mm_y) / sy_ds + 0.5f * M - 0.5f + 0.5f;
    int i0 = (int)floorf(xlo), i1 = (int)floorf(xhi - 1e-6f);
    int j0 = (int)floorf(ylo), j1 = (int)floorf(yhi - 1e-6f);
    i0 = max(i0, 0);
    i1 = min(i1, M - 1);
    j0 = max(j0, 0);
    j1 = min(j1, M - 1);
    if (i1 < i0 || j1 < j0) return;
    i1 = min(i1, i0 + 64);   // bounded box for a pathologically minified sprite
    j1 = min(j1, j0 + 64);
    float ar = 0.0f, ag = 0.0f, ab = 0.0f;
    for (int j = j0; j <= j1; ++j)
    {
        const float yov = fminf(yhi, (float)(j + 1)) - fmaxf(ylo, (float)j);
        if (yov <= 0.0f) continue;
        const float* row = sprite + 3 * ((size_t)j * M);
        for (int i = i0; i <= i1; ++i)
        {
            const float xov = fminf(xhi, (float)(i + 1)) - fmaxf(xlo, (float)i);
            if (xov <= 0.0f) continue;
            const float w = xov * yov;
            const float* p = row + 3 * i;
            ar += p[0] * w;
            ag += p[1] * w;
            ab += p[2] * w;
        }
    }
    const float vr = ar * s.r * gain, vg = ag * s.g * gain, vb = ab * s.b * gain;
    const size_t pix = (size_t)iy * width + ix;
    if (fabsf(vr) > 1e-20f) atomicAdd(&out_r[pix], vr);
    if (fabsf(vg) > 1e-20f) atomicAdd(&out_g[pix], vg);
    if (fabsf(vb) > 1e-20f) atomicAdd(&out_b[pix], vb);
}

__global__ void __launch_bounds__(kSpriteThreads) sprite_splat(const float* __restrict__ sprite, int M, float sx_ds,
                                                               float sy_ds, float px_mm_x, float px_mm_y, int rx,
                                                               int ry, const StarSource* __restrict__ src,
                                                               int n_src, float gain, float* __restrict__ out_r,
                                                               float* __restrict__ out_g, float* __restrict__ out_b,
                                                               int width, int height)
{
    const long long per_src = (2LL * rx + 1) * (2LL * ry + 1);
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= (long long)n_src * per_src) return;
    const int si = (int)(tid / per_src);
    splat_pixel(sprite, M, sx_ds, sy_ds, px_mm_x, px_mm_y, rx, ry, src[si], tid % per_src, gain, out_r, out_g,
                out_b, width, height);
}

// One source passed by value: no staging buffer, so splats of one resident
// sprite on many streams run side by side.
__global__ void __launch_bounds__(kSpriteThreads) sprite_splat_one(const float* __restrict__ sprite, int M,
                                                                   float sx_ds, float sy_ds, float px_mm_x,
                                                                   float px_mm_y, int rx, int ry, StarSource s,
                                                                   float gain, float* __restrict__ out_r,
                                                                   float* __restrict__ out_g,
                                                                   float* __restrict__ out_b, int width, int height)
{
    const long long per_src = (2LL * rx + 1) * (2LL * ry + 1);
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= per_src) return;
    splat_pixel(sprite, M, sx_ds, sy_ds, px_mm_x, px_mm_y, rx, ry, s, tid, gain, out_r, out_g, out_b, width, height);
}

}  // namespace

struct SpritePlan {
    int N = 0, n_spec = 0, M = 0, device = 0;
    float lambda_ref = 550.0f;
    FftDims dims{};
    float2* tw = nullptr;
    float2* work = nullptr;
    float* psf = nullptr;
    float* sprite = nullptr;
    size_t sprite_cap = 0;       // floats; grown by the bake to 3 M^2
    float4* spec = nullptr;
    double* energy = nullptr;
    StarSource* src = nullptr;
    int src_cap = 0;
    size_t smem_rows = 0, smem_cols = 0;
};

}  // namespace gl

struct gl_sprite_plan { gl::SpritePlan* p; };

using namespace gl;

static void sprite_free(SpritePlan* p)
{
    cudaFree(p->tw);
    cudaFree(p->work);
    cudaFree(p->psf);
    cudaFree(p->sprite);
    cudaFree(p->spec);
    cudaFree(p->energy);
    cudaFree(p->src);
    delete p;
}

extern "C" int gl_sprite_plan_create(int N, const gl_spectral_sample* spec, int n_spec, float lambda_ref,
                                     gl_sprite_plan** out)
{
    if (!out || !spec || n_spec < 1) return fail(GL_ERR_INVALID, "sprite_plan_create: bad arguments");
    if (N < 256 || N > kMaxSpriteGrid || (N & (N - 1)) != 0)
        return fail(GL_ERR_INVALID, "sprite_plan_create: grid must be a power of two in [256, 8192]");
    if (!(lambda_ref > 0.0f)) return fail(GL_ERR_INVALID, "sprite_plan_create: lambda_ref must be positive");
    for (int l = 0; l < n_spec; ++l)
        if (!(spec[l].lambda > 0.0f)) return fail(GL_ERR_INVALID, "sprite_plan_create: wavelengths must be positive");
    SpritePlan* p = new SpritePlan();
    p->N = N;
    p->n_spec = n_spec;
    p->lambda_ref = lambda_ref;
    p->dims = make_dims(N);
    cudaGetDevice(&p->device);
    const size_t NN = (size_t)N * N;
    const int nb = col_group(N);
    p->smem_rows = 2 * padded((size_t)N) * sizeof(float2);
    p->smem_cols = 2 * padded((size_t)N * nb) * sizeof(float2);
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    chk(cudaMalloc(&p->tw, sizeof(float2) * N));
    chk(cudaMalloc(&p->work, sizeof(float2) * NN));
    chk(cudaMalloc(&p->psf, sizeof(float) * NN));
    chk(cudaMalloc(&p->spec, sizeof(float4) * n_spec));
    chk(cudaMalloc(&p->energy, sizeof(double)));
    if (e == cudaSuccess)
    {
        const std::vector<float2> tw = twiddles(N);
        std::vector<float4> sp((size_t)n_spec);
        for (int l = 0; l < n_spec; ++l) sp[l] = make_float4(spec[l].lambda, spec[l].cmf_r, spec[l].cmf_g, spec[l].cmf_b);
        chk(cudaMemcpy(p->tw, tw.data(), sizeof(float2) * N, cudaMemcpyHostToDevice));
        chk(cudaMemcpy(p->spec, sp.data(), sizeof(float4) * n_spec, cudaMemcpyHostToDevice));
        chk((cudaError_t)raise_smem_limit((const void*)sprite_rows, p->smem_rows));
        if (nb == 4) chk((cudaError_t)raise_smem_limit((const void*)sprite_cols<4>, p->smem_cols));
        if (nb == 2) chk((cudaError_t)raise_smem_limit((const void*)sprite_cols<2>, p->smem_cols));
        if (nb == 1) chk((cudaError_t)raise_smem_limit((const void*)sprite_cols<1>, p->smem_cols));
        if (nb == 4) chk((cudaError_t)raise_smem_limit((const void*)autocorr_cols<4>, p->smem_cols));
        if (nb == 2) chk((cudaError_t)raise_smem_limit((const void*)autocorr_cols<2>, p->smem_cols));
        if (nb == 1) chk((cudaError_t)raise_smem_limit((const void*)autocorr_cols<1>, p->smem_cols));
    }
    if (e != cudaSuccess)
    {
        sprite_free(p);
        return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA,
                    std::string("sprite_plan_create: ") + cudaGetErrorString(e));
    }
    *out = new gl_sprite_plan{p};
    return GL_OK;
}

extern "C" int gl_sprite_plan_bake(gl_sprite_plan* plan, const float* d_pupil, int ds, void* stream)
{
    if (!plan || !d_pupil) return fail(GL_ERR_INVALID, "sprite_bake: bad arguments");
    SpritePlan* p = plan->p;
    const int N = p->N;
    if (ds < 1 || (ds & (ds - 1)) != 0 || ds > N / 8)
        return fail(GL_ERR_INVALID, "sprite_bake: ds must be a power of two in [1, N/8]");
    cudaStream_t st = (cudaStream_t)stream;
    const size_t need = 3 * (size_t)(N / ds) * (N / ds);
    if (need > p->sprite_cap)
    {
        // an earlier splat on this stream may still read the old sprite
        GL_CUDA_TRY(cudaStreamSynchronize(st));
        cudaFree(p->sprite);
        p->sprite = nullptr;
        p->sprite_cap = 0;
        GL_CUDA_TRY(cudaMalloc(&p->sprite, sizeof(float) * need));
        p->sprite_cap = need;
    }
    p->M = N / ds;
    GL_CUDA_TRY(cudaMemsetAsync(p->energy, 0, sizeof(double), st));
    sprite_rows<<<N, kSpriteThreads, p->smem_rows, st>>>(d_pupil, N, p->dims, p->tw, p->work);
    const int nb = col_group(N);
    if (nb == 4)
        sprite_cols<4><<<N / 4, kSpriteThreads, p->smem_cols, st>>>(p->work, N, p->dims, p->tw, p->psf, p->energy);
    else if (nb == 2)
        sprite_cols<2><<<N / 2, kSpriteThreads, p->smem_cols, st>>>(p->work, N, p->dims, p->tw, p->psf, p->energy);
    else
        sprite_cols<1><<<N, kSpriteThreads, p->smem_cols, st>>>(p->work, N, p->dims, p->tw, p->psf, p->energy);
    const int MM = p->M * p->M;
    sprite_bake<<<(MM + kSpriteThreads - 1) / kSpriteThreads, kSpriteThreads, 0, st>>>(
        p->psf, N, p->spec, p->n_spec, p->lambda_ref, ds, p->M, p->energy, p->sprite);
    GL_CUDA_TRY(cudaGetLastError());
    g_last_launches = 3;
    return GL_OK;
}

extern "C" int gl_sprite_plan_splat(gl_sprite_plan* plan, const float* sources, int n_src, float sx_ds, float sy_ds,
                                    float px_mm_x, float px_mm_y, int rx, int ry, float gain, float* d_out_r,
                                    float* d_out_g, float* d_out_b, int width, int height, void* stream)
{
    if (!plan || n_src < 0 || (n_src > 0 && !sources) || !d_out_r || !d_out_g || !d_out_b || width < 1 || height < 1)
        return fail(GL_ERR_INVALID, "sprite_splat: bad arguments");
    SpritePlan* p = plan->p;
    if (p->M == 0) return fail(GL_ERR_INVALID, "sprite_splat: bake the sprite first");
    if (!(sx_ds > 0.0f) || !(sy_ds > 0.0f) || !(px_mm_x > 0.0f) || !(px_mm_y > 0.0f) || rx < 0 || ry < 0)
        return fail(GL_ERR_INVALID, "sprite_splat: pitches must be positive");
    if (n_src == 0) return GL_OK;
    cudaStream_t st = (cudaStream_t)stream;
    if (n_src > p->src_cap)
    {
        // the previous buffer may still be read by an earlier splat on this stream
        GL_CUDA_TRY(cudaStreamSynchronize(st));
        cudaFree(p->src);
        p->src = nullptr;
        p->src_cap = 0;
        GL_CUDA_TRY(cudaMalloc(&p->src, sizeof(StarSource) * n_src));
        p->src_cap = n_src;
    }
    GL_CUDA_TRY(cudaMemcpyAsync(p->src, sources, sizeof(StarSource) * n_src, cudaMemcpyHostToDevice, st));
    const long long total = (long long)n_src * (2LL * rx + 1) * (2LL * ry + 1);
    if (total > (1LL << 40)) return fail(GL_ERR_INVALID, "sprite_splat: footprint too large");
    const long long blocks = (total + kSpriteThreads - 1) / kSpriteThreads;
    if (blocks > 0x7fffffffLL) return fail(GL_ERR_INVALID, "sprite_splat: footprint too large");
    sprite_splat<<<(unsigned)blocks, kSpriteThreads, 0, st>>>(p->sprite, p->M, sx_ds, sy_ds, px_mm_x, px_mm_y, rx, ry,
                                                              p->src, n_src, gain, d_out_r, d_out_g, d_out_b, width,
                                                              height);
    GL_CUDA_TRY(cudaGetLastError());
    // the host sources are staged through pageable memory: the copy is done
    // when the call returns, so the caller may reuse them
    g_last_launches = 1;
    return GL_OK;
}

extern "C" int gl_sprite_splat_source(const float* d_sprite, int M, float px, float py, float r, float g, float b,
                                      float sx_ds, float sy_ds, float px_mm_x, float px_mm_y, int rx, int ry,
                                      float gain, float* d_out_r, float* d_out_g, float* d_out_b, int width,
                                      int height, void* stream)
{
    if (!d_sprite || M < 1 || !d_out_r || !d_out_g || !d_out_b || width < 1 || height < 1)
        return fail(GL_ERR_INVALID, "sprite_splat_source: bad arguments");
    if (!(sx_ds > 0.0f) || !(sy_ds > 0.0f) || !(px_mm_x > 0.0f) || !(px_mm_y > 0.0f) || rx < 0 || ry < 0)
        return fail(GL_ERR_INVALID, "sprite_splat_source: pitches must be positive");
    const long long total = (2LL * rx + 1) * (2LL * ry + 1);
    const long long blocks = (total + kSpriteThreads - 1) / kSpriteThreads;
    if (blocks > 0x7fffffffLL) return fail(GL_ERR_INVALID, "sprite_splat_source: footprint too large");
    const StarSource s{px, py, r, g, b};
    sprite_splat_one<<<(unsigned)blocks, kSpriteThreads, 0, (cudaStream_t)stream>>>(
        d_sprite, M, sx_ds, sy_ds, px_mm_x, px_mm_y, rx, ry, s, gain, d_out_r, d_out_g, d_out_b, width, height);
    GL_CUDA_TRY(cudaGetLastError());
    g_last_launches = 1;
    return GL_OK;
}

extern "C" int gl_sprite_plan_autocorr(gl_sprite_plan* plan, const float* d_pupil, int mc, float* d_C, int ldc,
                                       int rows, void* stream)
{
    if (!plan || !d_pupil || !d_C) return fail(GL_ERR_INVALID, "autocorr: bad arguments");
    SpritePlan* p = plan->p;
    const int N = p->N;
    if (mc < 0 || mc > N / 2 - 1) return fail(GL_ERR_INVALID, "autocorr: lag radius must lie in [0, N/2 - 1]");
    if (ldc < 2 * mc + 1 || rows < 2 * mc + 1)
        return fail(GL_ERR_INVALID, "autocorr: the output must hold (2 mc + 1)^2 lags");
    cudaStream_t st = (cudaStream_t)stream;
    GL_CUDA_TRY(cudaMemsetAsync(d_C, 0, sizeof(float) * (size_t)ldc * rows, st));
    GL_CUDA_TRY(cudaMemsetAsync(p->energy, 0, sizeof(double), st));
    const int nb = col_group(N);
    // |FFT A|^2 (fftshifted) and its sum, as the sprite bake computes them
    sprite_rows<<<N, kSpriteThreads, p->smem_rows, st>>>(d_pupil, N, p->dims, p->tw, p->work);
    if (nb == 4)
        sprite_cols<4><<<N / 4, kSpriteThreads, p->smem_cols, st>>>(p->work, N, p->dims, p->tw, p->psf, p->energy);
    else if (nb == 2)
        sprite_cols<2><<<N / 2, kSpriteThreads, p->smem_cols, st>>>(p->work, N, p->dims, p->tw, p->psf, p->energy);
    else
        sprite_cols<1><<<N, kSpriteThreads, p->smem_cols, st>>>(p->work, N, p->dims, p->tw, p->psf, p->energy);
    // the second transform, kept only at lags within +-mc
    sprite_rows<<<N, kSpriteThreads, p->smem_rows, st>>>(p->psf, N, p->dims, p->tw, p->work);
    if (nb == 4)
        autocorr_cols<4><<<N / 4, kSpriteThreads, p->smem_cols, st>>>(p->work, N, p->dims, p->tw, mc, p->energy, d_C, ldc);
    else if (nb == 2)
        autocorr_cols<2><<<N / 2, kSpriteThreads, p->smem_cols, st>>>(p->work, N, p->dims, p->tw, mc, p->energy, d_C, ldc);
    else
        autocorr_cols<1><<<N, kSpriteThreads, p->smem_cols, st>>>(p->work, N, p->dims, p->tw, mc, p->energy, d_C, ldc);
    GL_CUDA_TRY(cudaGetLastError());
    // the bake's sprite no longer matches the PSF buffer's contents
    p->M = 0;
    g_last_launches = 4;
    return GL_OK;
}

extern "C" int gl_sprite_plan_read(gl_sprite_plan* plan, float* d_psf, float* d_sprite, double* energy, int* M,
                                   void* stream)
{
    if (!plan) return fail(GL_ERR_INVALID, "sprite_read: bad arguments");
    SpritePlan* p = plan->p;
    cudaStream_t st = (cudaStream_t)stream;
    const size_t NN = (size_t)p->N * p->N;
    if (d_psf) GL_CUDA_TRY(cudaMemcpyAsync(d_psf, p->psf, sizeof(float) * NN, cudaMemcpyDeviceToDevice, st));
    if (d_sprite && p->M)
        GL_CUDA_TRY(cudaMemcpyAsync(d_sprite, p->sprite, sizeof(float) * 3 * (size_t)p->M * p->M,
                                    cudaMemcpyDeviceToDevice, st));
    if (energy)
    {
        GL_CUDA_TRY(cudaMemcpyAsync(energy, p->energy, sizeof(double), cudaMemcpyDeviceToHost, st));
        GL_CUDA_TRY(cudaStreamSynchronize(st));
    }
    if (M) *M = p->M;
    return GL_OK;
}

extern "C" int gl_sprite_plan_destroy(gl_sprite_plan* plan)
{
    if (!plan) return GL_OK;
    cudaDeviceSynchronize();
    sprite_free(plan->p);
    delete plan;
    return GL_OK;
}
