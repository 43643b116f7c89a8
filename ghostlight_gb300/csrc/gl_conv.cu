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
//     = 4^4 * 3^2: no power-of-two padding waste);
//   * two real channels per complex transform (the kernel is real, so the
//     real and imaginary parts of the result are the two channels);
//   * mixed-radix (4, 3, 2) Stockham FFTs in shared memory, twiddles from
//     sincospif;
//   * three HBM passes: (1) forward row FFTs of the H image rows; (2) per
//     group of four columns: forward column FFT, multiply by the kernel
//     spectrum, inverse column FFT, all in one shared-memory residency;
//     (3) inverse row FFTs writing the cropped W x H planes.
// The kernel spectrum (normalisation 1/(PQ) folded in) is built once per plan
// and stays resident.
#include "gl_internal.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

namespace gl {
namespace {

struct FftDims {
    int n, nrad;
    int rad[16];
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// One Stockham stage over `nb` interleaved sequences (element i of sequence s
// at x[i * nb + s]); radix r, span Ls of the sub-transforms done so far.
__device__ __forceinline__ void stockham_stage(const float2* __restrict__ x, float2* __restrict__ y, int n, int nb,
                                               int r, int Ls, float sign)
{
    const int m = n / r;
    const int items = m * nb;
    for (int it = threadIdx.x; it < items; it += blockDim.x)
    {
        const int s = it % nb, j = it / nb;
        const int k = j % Ls, g = j / Ls;
        float2 v[4];
        #pragma unroll
        for (int q = 0; q < 4; ++q)
        {
            if (q >= r) break;
            float2 a = x[(size_t)(j + q * m) * nb + s];
            if (q > 0 && k > 0)
            {
                float sn, cs;
                sincospif(sign * 2.0f * (float)(q * k) / (float)(Ls * r), &sn, &cs);
                a = cmul(a, make_float2(cs, sn));
            }
            v[q] = a;
        }
        float2 z[4];
        if (r == 4)
        {
            const float2 t0 = make_float2(v[0].x + v[2].x, v[0].y + v[2].y);
            const float2 t1 = make_float2(v[0].x - v[2].x, v[0].y - v[2].y);
            const float2 t2 = make_float2(v[1].x + v[3].x, v[1].y + v[3].y);
            const float2 t3 = make_float2(v[1].x - v[3].x, v[1].y - v[3].y);
            // (s i) * t3
            const float2 it3 = make_float2(-sign * t3.y, sign * t3.x);
            z[0] = make_float2(t0.x + t2.x, t0.y + t2.y);
            z[1] = make_float2(t1.x + it3.x, t1.y + it3.y);
            z[2] = make_float2(t0.x - t2.x, t0.y - t2.y);
            z[3] = make_float2(t1.x - it3.x, t1.y - it3.y);
        }
        else if (r == 3)
        {
            const float c = 0.86602540378443864676f;   // sqrt(3)/2
            const float2 t1 = make_float2(v[1].x + v[2].x, v[1].y + v[2].y);
            const float2 t2 = make_float2(v[1].x - v[2].x, v[1].y - v[2].y);
            const float2 base = make_float2(v[0].x - 0.5f * t1.x, v[0].y - 0.5f * t1.y);
            const float2 rot = make_float2(-sign * c * t2.y, sign * c * t2.x);   // s i (sqrt3/2) t2
            z[0] = make_float2(v[0].x + t1.x, v[0].y + t1.y);
            z[1] = make_float2(base.x + rot.x, base.y + rot.y);
            z[2] = make_float2(base.x - rot.x, base.y - rot.y);
        }
        else
        {
            z[0] = make_float2(v[0].x + v[1].x, v[0].y + v[1].y);
            z[1] = make_float2(v[0].x - v[1].x, v[0].y - v[1].y);
        }
        const int ob = g * Ls * r + k;
        #pragma unroll
        for (int p = 0; p < 4; ++p)
        {
            if (p >= r) break;
            y[(size_t)(ob + p * Ls) * nb + s] = z[p];
        }
    }
}

// Full transform; returns the buffer holding the result (x or y).
__device__ float2* stockham(float2* x, float2* y, const FftDims& d, int nb, float sign)
{
    int Ls = 1;
    for (int st = 0; st < d.nrad; ++st)
    {
        stockham_stage(x, y, d.n, nb, d.rad[st], Ls, sign);
        __syncthreads();
        Ls *= d.rad[st];
        float2* t = x; x = y; y = t;
    }
    return x;
}

// Pass 1: forward row FFTs.  blockIdx.y selects the packed pair:
// pair 0 = in0 + i in1, pair 1 = in2 (+ i 0).  Rows [0, H) of width Q.
__global__ void __launch_bounds__(256) conv_rows_fwd(const float* __restrict__ in0, const float* __restrict__ in1,
                                                     const float* __restrict__ in2, const float* __restrict__ add0,
                                                     const float* __restrict__ add1, const float* __restrict__ add2,
                                                     int W, int H, float2* __restrict__ buf, FftDims dq)
{
    extern __shared__ float2 sm[];
    float2* x = sm;
    float2* y = sm + dq.n;
    const int row = blockIdx.x, pair = blockIdx.y;
    const float* re = pair == 0 ? in0 : in2;
    const float* im = pair == 0 ? in1 : nullptr;
    // optional second layer summed on load (flare composite = ghosts + starburst)
    const float* are = pair == 0 ? add0 : add2;
    const float* aim = pair == 0 ? add1 : nullptr;
    for (int i = threadIdx.x; i < dq.n; i += blockDim.x)
    {
        float a = 0.0f, b = 0.0f;
        if (i < W)
        {
            const size_t o = (size_t)row * W + i;
            a = re[o];
            if (are) a += are[o];
            if (im) b = im[o];
            if (aim) b += aim[o];
        }
        x[i] = make_float2(a, b);
    }
    __syncthreads();
    float2* r = stockham(x, y, dq, 1, -1.0f);
    float2* out = buf + ((size_t)pair * H + row) * dq.n;
    for (int i = threadIdx.x; i < dq.n; i += blockDim.x) out[i] = r[i];
}

// Forward row FFT of a complex P x Q buffer in place (kernel spectrum setup).
__global__ void __launch_bounds__(256) conv_rows_fwd_complex(float2* __restrict__ buf, int Q, FftDims dq)
{
    extern __shared__ float2 sm[];
    float2* x = sm;
    float2* y = sm + dq.n;
    float2* row = buf + (size_t)blockIdx.x * Q;
    for (int i = threadIdx.x; i < dq.n; i += blockDim.x) x[i] = row[i];
    __syncthreads();
    float2* r = stockham(x, y, dq, 1, -1.0f);
    for (int i = threadIdx.x; i < dq.n; i += blockDim.x) row[i] = r[i];
}

constexpr int kColGroup = 4;

// Pass 2: per group of 4 columns: forward column FFT over P rows (rows >= H
// are zero), times the kernel spectrum, inverse column FFT; rows [0, H) back.
// mode 1 (kernel precompute): forward only, all P rows present, no multiply.
__global__ void __launch_bounds__(512) conv_cols(float2* __restrict__ buf, const float2* __restrict__ khat, int H,
                                                 int rows_in, FftDims dp, int Q, int mode)
{
    extern __shared__ float2 sm[];
    float2* x = sm;
    float2* y = sm + (size_t)dp.n * kColGroup;
    const int c0 = blockIdx.x * kColGroup;
    float2* base = buf + (size_t)blockIdx.y * rows_in * Q;
    for (int e = threadIdx.x; e < dp.n * kColGroup; e += blockDim.x)
    {
        const int rr = e / kColGroup, cc = e % kColGroup;
        x[e] = (rr < rows_in && c0 + cc < Q) ? base[(size_t)rr * Q + c0 + cc] : make_float2(0.0f, 0.0f);
    }
    __syncthreads();
    float2* f = stockham(x, y, dp, kColGroup, -1.0f);
    float2* other = (f == x) ? y : x;
    if (mode == 1)
    {
        for (int e = threadIdx.x; e < dp.n * kColGroup; e += blockDim.x)
        {
            const int rr = e / kColGroup, cc = e % kColGroup;
            if (c0 + cc < Q) base[(size_t)rr * Q + c0 + cc] = f[e];
        }
        return;
    }
    for (int e = threadIdx.x; e < dp.n * kColGroup; e += blockDim.x)
    {
        const int rr = e / kColGroup, cc = e % kColGroup;
        const float2 k = (c0 + cc < Q) ? khat[(size_t)rr * Q + c0 + cc] : make_float2(0.0f, 0.0f);
        f[e] = cmul(f[e], k);
    }
    __syncthreads();
    float2* g = stockham(f, other, dp, kColGroup, 1.0f);
    for (int e = threadIdx.x; e < H * kColGroup; e += blockDim.x)
    {
        const int rr = e / kColGroup, cc = e % kColGroup;
        if (c0 + cc < Q) base[(size_t)rr * Q + c0 + cc] = g[e];
    }
}

// Pass 3: inverse row FFTs; real part -> out0 (pair 0) / out2 (pair 1),
// imaginary part -> out1 (pair 0).  Crop to W.
__global__ void __launch_bounds__(256) conv_rows_inv(const float2* __restrict__ buf, int W, int H, float* __restrict__ out0,
                                                     float* __restrict__ out1, float* __restrict__ out2, FftDims dq)
{
    extern __shared__ float2 sm[];
    float2* x = sm;
    float2* y = sm + dq.n;
    const int row = blockIdx.x, pair = blockIdx.y;
    const float2* in = buf + ((size_t)pair * H + row) * dq.n;
    for (int i = threadIdx.x; i < dq.n; i += blockDim.x) x[i] = in[i];
    __syncthreads();
    float2* r = stockham(x, y, dq, 1, 1.0f);
    float* o_re = pair == 0 ? out0 : out2;
    float* o_im = pair == 0 ? out1 : nullptr;
    for (int i = threadIdx.x; i < W; i += blockDim.x)
    {
        o_re[(size_t)row * W + i] = r[i].x;
        if (o_im) o_im[(size_t)row * W + i] = r[i].y;
    }
}

FftDims make_dims(int n)
{
    FftDims d{};
    d.n = n;
    int m = n;
    while (m % 4 == 0) { d.rad[d.nrad++] = 4; m /= 4; }
    while (m % 2 == 0) { d.rad[d.nrad++] = 2; m /= 2; }
    while (m % 3 == 0) { d.rad[d.nrad++] = 3; m /= 3; }
    return d;
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
    int W = 0, H = 0, KW = 0, KH = 0, P = 0, Q = 0;
    float2* khat = nullptr;   // P x Q
    float2* buf = nullptr;    // 2 x H x Q
    size_t smem_row = 0, smem_col = 0;
};

}  // namespace gl

struct gl_conv_plan { gl::ConvPlan* p; };

using namespace gl;

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
    if (p->P > 8192 || p->Q > 8192)
    {
        delete p;
        return fail(GL_ERR_INVALID, "conv2d_plan_create: padded transform above 8192 points per axis");
    }
    p->smem_row = 2 * (size_t)p->Q * sizeof(float2);
    p->smem_col = 2 * (size_t)p->P * kColGroup * sizeof(float2);
    if (p->smem_col > 227 * 1024 || p->smem_row > 227 * 1024)
    {
        delete p;
        return fail(GL_ERR_INVALID, "conv2d_plan_create: transform too large for one shared-memory residency");
    }
    cudaStream_t st = (cudaStream_t)stream;
    // Kernel placed with its centre at the origin, wrapped (so the circular
    // convolution lands 'same'-aligned), as P x Q real, then 2-D FFT in place.
    std::vector<float2> kw_host((size_t)p->P * p->Q, make_float2(0.0f, 0.0f));
    const int cy = kh / 2, cx = kw / 2;
    const float norm = 1.0f / ((float)p->P * (float)p->Q);
    for (int u = 0; u < kh; ++u)
        for (int v = 0; v < kw; ++v)
        {
            const int yy = ((u - cy) % p->P + p->P) % p->P, xx = ((v - cx) % p->Q + p->Q) % p->Q;
            kw_host[(size_t)yy * p->Q + xx].x = h_kernel[(size_t)u * kw + v] * norm;
        }
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    chk(cudaMalloc(&p->khat, sizeof(float2) * (size_t)p->P * p->Q));
    chk(cudaMalloc(&p->buf, sizeof(float2) * 2 * (size_t)p->H * p->Q));
    chk(cudaFuncSetAttribute(conv_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem_col));
    chk(cudaFuncSetAttribute(conv_rows_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem_row));
    chk(cudaFuncSetAttribute(conv_rows_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem_row));
    if (e == cudaSuccess)
    {
        chk(cudaMemcpyAsync(p->khat, kw_host.data(), sizeof(float2) * kw_host.size(), cudaMemcpyHostToDevice, st));
        const FftDims dq = make_dims(p->Q), dp = make_dims(p->P);
        chk(cudaFuncSetAttribute(conv_rows_fwd_complex, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem_row));
        if (e == cudaSuccess)
        {
            conv_rows_fwd_complex<<<p->P, 256, p->smem_row, st>>>(p->khat, p->Q, dq);
            conv_cols<<<dim3((p->Q + kColGroup - 1) / kColGroup, 1), 512, p->smem_col, st>>>(p->khat, nullptr, p->P,
                                                                                         p->P, dp, p->Q, 1);
            chk(cudaGetLastError());
        }
        chk(cudaStreamSynchronize(st));
    }
    if (e != cudaSuccess)
    {
        cudaFree(p->khat); cudaFree(p->buf);
        delete p;
        return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA, std::string("conv2d_plan_create: ") + cudaGetErrorString(e));
    }
    *out = new gl_conv_plan{p};
    return GL_OK;
}

// in_r/g/b, out_r/g/b: W x H planar float32 on the device; the outputs must
// not overlap the inputs.
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
    conv_rows_fwd<<<dim3(p->H, 2), 256, p->smem_row, st>>>(d_in_r, d_in_g, d_in_b, d_add_r, d_add_g, d_add_b, p->W,
                                                           p->H, p->buf, dq);
    conv_cols<<<dim3((p->Q + kColGroup - 1) / kColGroup, 2), 512, p->smem_col, st>>>(p->buf, p->khat, p->H, p->H, dp,
                                                                                  p->Q, 0);
    conv_rows_inv<<<dim3(p->H, 2), 256, p->smem_row, st>>>(p->buf, p->W, p->H, d_out_r, d_out_g, d_out_b, dq);
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
    cudaFree(plan->p->khat);
    cudaFree(plan->p->buf);
    delete plan->p;
    delete plan;
    return GL_OK;
}
