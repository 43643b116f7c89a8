// gl_conv.cu — PSF / veil convolution of the flare image with a large FP32
// kernel, by FFT.
//
// The reference has no image convolution on this path (its veil is an
// analytic glare-spread sprite splatted per source, veil_render.cu:94-243);
// the flare path adds one: out_c = in_c (*) k, 'same' size, k centred.
//
// GB300 route: the transform is memory-bound, so it is laid out for HBM.
//   * linear convolution by zero-padded circular convolution of size P x Q,
//     P, Q = the smallest 2^a 3^b >= image + kernel - 1 (2048 + 257 - 1 = 2304
//     = 16 * 16 * 9: no power-of-two padding waste);
//   * two real channels per complex transform (the kernel is real, so the
//     real and imaginary parts of the result are the two channels);
//   * Stockham FFTs in shared memory with large radices held in registers
//     (16, 8, 4, 2 and 9, 3: three passes over shared memory for 2304
//     points), twiddles from a per-plan table computed in FP64; the shared
//     arrays carry one pad word per 16 so the strided radix writes do not
//     collide in banks;
//   * three HBM passes: (1) forward row FFTs, two rows per CTA; (2) per group
//     of four columns: forward column FFT, multiply by the kernel spectrum,
//     inverse column FFT, all in one shared-memory residency; (3) inverse row
//     FFTs writing the cropped W x H planes.
// The kernel spectrum (normalisation 1/(PQ) folded in) is built once per plan
// and stays resident.
#include "gl_internal.h"
#include "gl_fft.cuh"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

namespace gl {
namespace {

// HBM layout of the intermediate ("column-group tiles"): complex element
// (row r, column q) of channel pair p at ((p * G + q / 4) * rows + r) * 4 + q % 4,
// G = ceil(Q / 4).  A column group (4 columns x all rows) is one contiguous
// block, so the column pass streams it with coalesced 16-byte accesses; the
// row passes touch 32-byte pieces (4 complex) per group, whole DRAM sectors.
__device__ __forceinline__ size_t tile_index(int pair, int G, int rows, int r, int q)
{
    return (((size_t)pair * G + (q >> 2)) * rows + r) * 4 + (q & 3);
}

constexpr int kRowsPerCta = 2;
constexpr int kRowLoads = 8;   // per-thread loads in flight per row pass

// Pass 1: forward row FFTs, two rows per CTA (rows 2b, 2b+1; blockIdx.y =
// packed pair: 0 = in0 + i in1, 1 = in2).  An optional second layer is summed
// in on load (flare composite = ghosts + starburst).  Rows of width W,
// zero-padded to Q, written as column-group tiles of `rows` rows.
__global__ void __launch_bounds__(1024) conv_rows_fwd(const float* __restrict__ in0, const float* __restrict__ in1,
                              const float* __restrict__ in2, const float* __restrict__ add0,
                              const float* __restrict__ add1, const float* __restrict__ add2, int W, int rows,
                              float2* __restrict__ buf, FftDims dq, const float2* __restrict__ tw)
{
    extern __shared__ float2 sm[];
    const int Q = dq.n, G = (Q + 3) >> 2;
    float2* x = sm;
    float2* y = sm + padded((size_t)Q * kRowsPerCta);
    const int pair = blockIdx.y;
    const int row0 = blockIdx.x * kRowsPerCta;
    const float* re = pair == 0 ? in0 : in2;
    const float* im = pair == 0 ? in1 : nullptr;
    const float* are = pair == 0 ? add0 : add2;
    const float* aim = pair == 0 ? add1 : nullptr;
    const int total = Q * kRowsPerCta;
    for (int e0 = 0; e0 < total; e0 += blockDim.x * kRowLoads)
    {
        float a[kRowLoads], b[kRowLoads];
        #pragma unroll
        for (int u = 0; u < kRowLoads; ++u)
        {
            const int e = e0 + u * blockDim.x + threadIdx.x;
            const int rr = e / Q, i = e - rr * Q;
            const int row = row0 + rr;
            a[u] = 0.0f; b[u] = 0.0f;
            if (e < total && i < W && row < rows)
            {
                const size_t o = (size_t)row * W + i;
                a[u] = re[o];
                if (are) a[u] += are[o];
                if (im) b[u] = im[o];
                if (aim) b[u] += aim[o];
            }
        }
        #pragma unroll
        for (int u = 0; u < kRowLoads; ++u)
        {
            const int e = e0 + u * blockDim.x + threadIdx.x;
            if (e < total)
            {
                const int rr = e / Q, i = e - rr * Q;
                x[pad(i * kRowsPerCta + rr)] = make_float2(a[u], b[u]);
            }
        }
    }
    __syncthreads();
    const float2* r = stockham<kRowsPerCta>(x, y, dq, tw, false);
    // two complex of one row per thread -> one 16-byte store into the tile
    const int half = (Q + 1) / 2;
    for (int h = threadIdx.x; h < half * kRowsPerCta; h += blockDim.x)
    {
        const int rr = h / half, q = 2 * (h - rr * half);
        const int row = row0 + rr;
        if (row >= rows) continue;
        const float2 v0 = r[pad(q * kRowsPerCta + rr)];
        const float2 v1 = (q + 1 < Q) ? r[pad((q + 1) * kRowsPerCta + rr)] : make_float2(0.0f, 0.0f);
        *reinterpret_cast<float4*>(buf + tile_index(pair, G, rows, row, q)) = make_float4(v0.x, v0.y, v1.x, v1.y);
    }
}

constexpr int kColGroup = 4;      // columns per tile group in the HBM layout
constexpr int kColsPerCta = 2;    // columns per CTA: half a group, so two CTAs fit an SM

// Pass 2: two columns (half a tile group) per CTA: forward column FFT over P
// rows (rows >= rows_in are zero), times the kernel spectrum, inverse column
// FFT; rows [0, rows_out) back in place.  mode 1 (kernel-spectrum setup):
// forward only, result for all P rows.  The two halves of a group are
// neighbouring CTAs, so each 32-byte sector they share is read from DRAM once.
__global__ void __launch_bounds__(1024) conv_cols(float2* __restrict__ buf, const float2* __restrict__ khat,
                                                  int rows_in, int rows_out, FftDims dp, int Q, int mode,
                                                  const float2* __restrict__ tw)
{
    extern __shared__ float2 sm[];
    const int P = dp.n, G = (Q + 3) >> 2;
    float2* x = sm;
    float2* y = sm + padded((size_t)P * kColsPerCta);
    const int g = blockIdx.x >> 1, hcol = (blockIdx.x & 1) * kColsPerCta;
    float2* base = buf + ((size_t)blockIdx.y * G + g) * rows_in * kColGroup;
    const int valid = max(0, min(kColsPerCta, Q - g * kColGroup - hcol));
    if (valid == 0) return;
    {
        constexpr int U = 8;
        for (int r0 = 0; r0 < P; r0 += blockDim.x * U)
        {
            float4 v[U];
            #pragma unroll
            for (int u = 0; u < U; ++u)
            {
                const int r = r0 + u * blockDim.x + threadIdx.x;
                v[u] = r < rows_in ? *reinterpret_cast<const float4*>(base + (size_t)r * kColGroup + hcol)
                                   : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
            #pragma unroll
            for (int u = 0; u < U; ++u)
            {
                const int r = r0 + u * blockDim.x + threadIdx.x;
                if (r < P)
                {
                    x[pad(2 * r)] = make_float2(v[u].x, v[u].y);
                    x[pad(2 * r + 1)] = valid > 1 ? make_float2(v[u].z, v[u].w) : make_float2(0.0f, 0.0f);
                }
            }
        }
    }
    __syncthreads();
    float2* f = stockham<kColsPerCta>(x, y, dp, tw, false);
    float2* other = (f == x) ? y : x;
    if (mode == 1)
    {
        for (int r = threadIdx.x; r < P; r += blockDim.x)
        {
            const float2 a = f[pad(2 * r)], b = f[pad(2 * r + 1)];
            *reinterpret_cast<float4*>(base + (size_t)r * kColGroup + hcol) = make_float4(a.x, a.y, b.x, b.y);
        }
        return;
    }
    const float2* kb = khat + (size_t)g * P * kColGroup + hcol;
    for (int r = threadIdx.x; r < P; r += blockDim.x)
    {
        const float4 k = __ldg(reinterpret_cast<const float4*>(kb + (size_t)r * kColGroup));
        f[pad(2 * r)] = cmul(f[pad(2 * r)], make_float2(k.x, k.y));
        f[pad(2 * r + 1)] = cmul(f[pad(2 * r + 1)], make_float2(k.z, k.w));
    }
    __syncthreads();
    const float2* res = stockham<kColsPerCta>(f, other, dp, tw, true);
    for (int r = threadIdx.x; r < rows_out; r += blockDim.x)
    {
        const float2 a = res[pad(2 * r)], b = res[pad(2 * r + 1)];
        *reinterpret_cast<float4*>(base + (size_t)r * kColGroup + hcol) = make_float4(a.x, a.y, b.x, b.y);
    }
}

// Pass 3: inverse row FFTs from the tiles, two rows per CTA; real part ->
// out0 (pair 0) / out2 (pair 1), imaginary part -> out1 (pair 0).  Crop to W.
__global__ void __launch_bounds__(1024) conv_rows_inv(const float2* __restrict__ buf, int W, int H, float* __restrict__ out0,
                              float* __restrict__ out1, float* __restrict__ out2, FftDims dq,
                              const float2* __restrict__ tw)
{
    extern __shared__ float2 sm[];
    const int Q = dq.n, G = (Q + 3) >> 2;
    float2* x = sm;
    float2* y = sm + padded((size_t)Q * kRowsPerCta);
    const int pair = blockIdx.y;
    const int row0 = blockIdx.x * kRowsPerCta;
    const int half = (Q + 1) / 2;
    const int total = half * kRowsPerCta;
    constexpr int U = 6;
    for (int h0 = 0; h0 < total; h0 += blockDim.x * U)
    {
        float4 v[U];
        #pragma unroll
        for (int u = 0; u < U; ++u)
        {
            const int h = h0 + u * blockDim.x + threadIdx.x;
            const int rr = h / half, q = 2 * (h - rr * half);
            const int row = row0 + rr;
            v[u] = (h < total && row < H) ? __ldg(reinterpret_cast<const float4*>(buf + tile_index(pair, G, H, row, q)))
                                          : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        #pragma unroll
        for (int u = 0; u < U; ++u)
        {
            const int h = h0 + u * blockDim.x + threadIdx.x;
            if (h < total)
            {
                const int rr = h / half, q = 2 * (h - rr * half);
                x[pad(q * kRowsPerCta + rr)] = make_float2(v[u].x, v[u].y);
                if (q + 1 < Q) x[pad((q + 1) * kRowsPerCta + rr)] = make_float2(v[u].z, v[u].w);
            }
        }
    }
    __syncthreads();
    const float2* r = stockham<kRowsPerCta>(x, y, dq, tw, true);
    for (int e = threadIdx.x; e < W * kRowsPerCta; e += blockDim.x)
    {
        const int rr = e / W, i = e - rr * W;
        const int row = row0 + rr;
        if (row >= H) continue;
        const float2 v = r[pad(i * kRowsPerCta + rr)];
        const size_t o = (size_t)row * W + i;
        if (pair == 0) { out0[o] = v.x; out1[o] = v.y; }
        else out2[o] = v.x;
    }
}

int good_size(int need)
{
    int best = 1 << 30;
    for (long long p2 = 1; p2 < (1LL << 31); p2 *= 2)
        for (long long v = p2; v < (1LL << 31); v *= 3)
        {
            if (v >= need && v < best) best = (int)v;
            if (v >= need) break;
        }
    return best;
}

}  // namespace

struct ConvPlan {
    int W = 0, H = 0, KW = 0, KH = 0, P = 0, Q = 0, G = 0;
    float2* khat = nullptr;   // column-group tiles, P rows
    float2* buf = nullptr;    // column-group tiles, 2 pairs x H rows
    float2* tw_p = nullptr;   // twiddles for P (== tw_q when P == Q)
    float2* tw_q = nullptr;
    size_t smem_row = 0, smem_col = 0;
    int thr_row = 0, thr_col = 0;
};

}  // namespace gl

struct gl_conv_plan { gl::ConvPlan* p; };

using namespace gl;

static void conv_free(ConvPlan* p)
{
    cudaFree(p->khat);
    cudaFree(p->buf);
    if (p->tw_p != p->tw_q) cudaFree(p->tw_p);
    cudaFree(p->tw_q);
    delete p;
}

extern "C" int gl_conv2d_plan_create(int width, int height, const float* h_kernel, int kw, int kh, void* stream,
                                     gl_conv_plan** out)
{
    if (!out || !h_kernel) return fail(GL_ERR_INVALID, "conv2d_plan_create: null argument");
    if (width <= 0 || height <= 0 || kw <= 0 || kh <= 0 || (kw % 2) == 0 || (kh % 2) == 0)
        return fail(GL_ERR_INVALID, "conv2d_plan_create: positive sizes and an odd (centred) kernel required");
    ConvPlan* p = new ConvPlan();
    p->W = width; p->H = height; p->KW = kw; p->KH = kh;
    p->Q = good_size(width + kw - 1);
    p->P = good_size(height + kh - 1);
    p->G = (p->Q + 3) / 4;
    if (p->P > 3072 || p->Q > 3072)
    {
        delete p;
        return fail(GL_ERR_INVALID, "conv2d_plan_create: padded transform above 3072 points per axis");
    }
    p->smem_row = 2 * padded((size_t)p->Q * kRowsPerCta) * sizeof(float2);
    p->smem_col = 2 * padded((size_t)p->P * kColsPerCta) * sizeof(float2);
    {
        // one thread per butterfly of the largest-radix stage
        const FftDims dq = make_dims(p->Q), dp = make_dims(p->P);
        auto threads = [](const FftDims& d, int nb) {
            int rmax = 2;
            for (int i = 0; i < d.nrad; ++i) rmax = std::max(rmax, d.rad[i]);
            const int t = (d.n * nb / rmax + 31) / 32 * 32;
            return std::min(1024, std::max(64, t));
        };
        p->thr_row = threads(dq, kRowsPerCta);
        p->thr_col = threads(dp, kColsPerCta);
    }
    if (p->smem_col > 227 * 1024 || p->smem_row > 227 * 1024)
    {
        delete p;
        return fail(GL_ERR_INVALID, "conv2d_plan_create: transform too large for one shared-memory residency");
    }
    cudaStream_t st = (cudaStream_t)stream;
    // Kernel placed with its centre at the origin, wrapped (so the circular
    // convolution lands 'same'-aligned), as a P x Q real plane, 1/(PQ) folded in.
    std::vector<float> kplane((size_t)p->P * p->Q, 0.0f);
    const int cy = kh / 2, cx = kw / 2;
    const float norm = 1.0f / ((float)p->P * (float)p->Q);
    for (int u = 0; u < kh; ++u)
        for (int v = 0; v < kw; ++v)
        {
            const int yy = ((u - cy) % p->P + p->P) % p->P, xx = ((v - cx) % p->Q + p->Q) % p->Q;
            kplane[(size_t)yy * p->Q + xx] = h_kernel[(size_t)u * kw + v] * norm;
        }
    const std::vector<float2> twq = twiddles(p->Q);
    const std::vector<float2> twp = p->P == p->Q ? std::vector<float2>() : twiddles(p->P);
    float* kdev = nullptr;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    chk(cudaMalloc(&p->khat, sizeof(float2) * (size_t)p->G * 4 * p->P));
    chk(cudaMalloc(&p->buf, sizeof(float2) * 2 * (size_t)p->G * 4 * p->H));
    chk(cudaMalloc(&p->tw_q, sizeof(float2) * (size_t)p->Q));
    if (p->P != p->Q) chk(cudaMalloc(&p->tw_p, sizeof(float2) * (size_t)p->P));
    else p->tw_p = p->tw_q;
    chk(cudaMalloc(&kdev, sizeof(float) * kplane.size()));
    chk((cudaError_t)raise_smem_limit((const void*)conv_cols, p->smem_col));
    chk((cudaError_t)raise_smem_limit((const void*)conv_rows_fwd, p->smem_row));
    chk((cudaError_t)raise_smem_limit((const void*)conv_rows_inv, p->smem_row));
    if (e == cudaSuccess)
    {
        chk(cudaMemcpyAsync(p->tw_q, twq.data(), sizeof(float2) * twq.size(), cudaMemcpyHostToDevice, st));
        if (p->P != p->Q)
            chk(cudaMemcpyAsync(p->tw_p, twp.data(), sizeof(float2) * twp.size(), cudaMemcpyHostToDevice, st));
        chk(cudaMemcpyAsync(kdev, kplane.data(), sizeof(float) * kplane.size(), cudaMemcpyHostToDevice, st));
        const FftDims dq = make_dims(p->Q), dp = make_dims(p->P);
        if (e == cudaSuccess)
        {
            // kernel spectrum: row FFTs of the real plane into tiles, then forward column FFTs in place
            conv_rows_fwd<<<dim3((p->P + kRowsPerCta - 1) / kRowsPerCta, 1), p->thr_row, p->smem_row, st>>>(kdev, nullptr, nullptr, nullptr, nullptr,
                                                                            nullptr, p->Q, p->P, p->khat, dq,
                                                                            p->tw_q);
            conv_cols<<<dim3(2 * p->G, 1), p->thr_col, p->smem_col, st>>>(p->khat, nullptr, p->P, p->P, dp, p->Q, 1,
                                                                       p->tw_p);
            chk(cudaGetLastError());
        }
        chk(cudaStreamSynchronize(st));
    }
    cudaFree(kdev);
    if (e != cudaSuccess)
    {
        conv_free(p);
        return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA, std::string("conv2d_plan_create: ") + cudaGetErrorString(e));
    }
    *out = new gl_conv_plan{p};
    return GL_OK;
}

extern "C" int gl_conv2d_plan_execute2(gl_conv_plan* plan, const float* d_in_r, const float* d_in_g,
                                       const float* d_in_b, const float* d_add_r, const float* d_add_g,
                                       const float* d_add_b, float* d_out_r, float* d_out_g, float* d_out_b,
                                       void* stream)
{
    if (!plan || !d_in_r || !d_in_g || !d_in_b || !d_out_r || !d_out_g || !d_out_b)
        return fail(GL_ERR_INVALID, "conv2d_plan_execute: null argument");
    if ((d_add_r == nullptr) != (d_add_g == nullptr) || (d_add_r == nullptr) != (d_add_b == nullptr))
        return fail(GL_ERR_INVALID, "conv2d_plan_execute: the added layer needs all three planes or none");
    ConvPlan* p = plan->p;
    cudaStream_t st = (cudaStream_t)stream;
    const FftDims dq = make_dims(p->Q), dp = make_dims(p->P);
    const unsigned rb = (unsigned)((p->H + kRowsPerCta - 1) / kRowsPerCta);
    conv_rows_fwd<<<dim3(rb, 2), p->thr_row, p->smem_row, st>>>(d_in_r, d_in_g, d_in_b, d_add_r, d_add_g, d_add_b,
                                                                    p->W, p->H, p->buf, dq, p->tw_q);
    conv_cols<<<dim3(2 * p->G, 2), p->thr_col, p->smem_col, st>>>(p->buf, p->khat, p->H, p->H, dp, p->Q, 0, p->tw_p);
    conv_rows_inv<<<dim3(rb, 2), p->thr_row, p->smem_row, st>>>(p->buf, p->W, p->H, d_out_r, d_out_g, d_out_b, dq,
                                                                    p->tw_q);
    GL_CUDA_TRY(cudaGetLastError());
    g_last_launches = 3;
    return GL_OK;
}

extern "C" int gl_conv2d_plan_execute(gl_conv_plan* plan, const float* d_in_r, const float* d_in_g, const float* d_in_b,
                                      float* d_out_r, float* d_out_g, float* d_out_b, void* stream)
{
    return gl_conv2d_plan_execute2(plan, d_in_r, d_in_g, d_in_b, nullptr, nullptr, nullptr, d_out_r, d_out_g, d_out_b,
                                   stream);
}

extern "C" int gl_conv2d_plan_info(const gl_conv_plan* plan, int* P, int* Q)
{
    if (!plan) return fail(GL_ERR_INVALID, "conv2d_plan_info: null plan");
    if (P) *P = plan->p->P;
    if (Q) *Q = plan->p->Q;
    return GL_OK;
}

extern "C" int gl_conv2d_plan_destroy(gl_conv_plan* plan)
{
    if (!plan) return GL_OK;
    conv_free(plan->p);
    delete plan;
    return GL_OK;
}
