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

// Radix plan of one transform length n = 2^a 3^b: per stage its radix r, the
// span Ls of the sub-transforms done before it, ceil(2^32 / Ls) for an exact
// division by multiply-high (indices < 2^14), and the twiddle-table stride
// n / (Ls r).
struct FftDims {
    int n, nrad;
    int rad[16];
    int ls[16];
    uint32_t lmag[16];
    int twstep[16];
};

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// One Stockham stage over NB interleaved sequences (element i of sequence s
// at x[i * NB + s]).  tw[t] = exp(-2 pi i t / n); the inverse uses conj.
template <int NB>
__device__ __forceinline__ void stockham_stage(const float2* __restrict__ x, float2* __restrict__ y, int n, int r,
                                               int Ls, uint32_t lmag, int twstep, const float2* __restrict__ tw,
                                               bool inv)
{
    const int m = n / r;
    const int items = m * NB;
    const float sign = inv ? 1.0f : -1.0f;
    for (int it = threadIdx.x; it < items; it += blockDim.x)
    {
        const int s = it % NB, j = it / NB;
        int g, k;
        if (Ls == 1) { g = j; k = 0; }
        else
        {
            g = (int)__umulhi((uint32_t)j, lmag);
            k = j - g * Ls;
        }
        float2 v[4];
        #pragma unroll
        for (int q = 0; q < 4; ++q)
        {
            if (q >= r) break;
            float2 a = x[(j + q * m) * NB + s];
            if (q > 0 && k > 0)
            {
                float2 w = __ldg(&tw[q * k * twstep]);   // q k < r Ls, so the index is < n
                if (inv) w.y = -w.y;
                a = cmul(a, w);
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
            const float2 it3 = make_float2(-sign * t3.y, sign * t3.x);   // (sign i) t3
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
            const float2 rot = make_float2(-sign * c * t2.y, sign * c * t2.x);   // (sign i) (sqrt3/2) t2
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
            y[(ob + p * Ls) * NB + s] = z[p];
        }
    }
}

// Full transform; returns the buffer holding the result (x or y).
template <int NB>
__device__ float2* stockham(float2* x, float2* y, const FftDims& d, const float2* __restrict__ tw, bool inv)
{
    for (int st = 0; st < d.nrad; ++st)
    {
        stockham_stage<NB>(x, y, d.n, d.rad[st], d.ls[st], d.lmag[st], d.twstep[st], tw, inv);
        __syncthreads();
        float2* t = x; x = y; y = t;
    }
    return x;
}

// HBM layout of the intermediate ("column-group tiles"): complex element
// (row r, column q) of channel pair p at ((p * G + q / 4) * rows + r) * 4 + q % 4,
// G = ceil(Q / 4).  A column group (4 columns x all rows) is one contiguous
// block, so the column pass streams it with coalesced 16-byte accesses; the
// row passes touch 32-byte pieces (4 complex) per group, whole DRAM sectors.
__device__ __forceinline__ size_t tile_index(int pair, int G, int rows, int r, int q)
{
    return (((size_t)pair * G + (q >> 2)) * rows + r) * 4 + (q & 3);
}

constexpr int kRowThreads = 256;
constexpr int kRowLoads = 12;   // per-thread loads issued before use (covers rows of up to 3072)

// Pass 1: forward row FFTs.  blockIdx.y selects the packed pair:
// pair 0 = in0 + i in1, pair 1 = in2 (+ i 0); an optional second layer is
// summed in on load (flare composite = ghosts + starburst).  Rows [0, H) of
// width W, zero-padded to Q, written as column-group tiles of `rows` rows.
__global__ void __launch_bounds__(kRowThreads) conv_rows_fwd(const float* __restrict__ in0,
                                                             const float* __restrict__ in1,
                                                             const float* __restrict__ in2,
                                                             const float* __restrict__ add0,
                                                             const float* __restrict__ add1,
                                                             const float* __restrict__ add2, int W, int rows,
                                                             float2* __restrict__ buf, FftDims dq,
                                                             const float2* __restrict__ tw)
{
    extern __shared__ float2 sm[];
    float2* x = sm;
    float2* y = sm + dq.n;
    const int row = blockIdx.x, pair = blockIdx.y;
    const int Q = dq.n, G = (Q + 3) >> 2;
    const float* re = pair == 0 ? in0 : in2;
    const float* im = pair == 0 ? in1 : nullptr;
    const float* are = pair == 0 ? add0 : add2;
    const float* aim = pair == 0 ? add1 : nullptr;
    const size_t ro = (size_t)row * W;
    // issue every load of this thread first (bytes in flight), then stage
    for (int i0 = 0; i0 < Q; i0 += kRowThreads * kRowLoads)
    {
        float a[kRowLoads], b[kRowLoads];
        #pragma unroll
        for (int u = 0; u < kRowLoads; ++u)
        {
            const int i = i0 + u * kRowThreads + threadIdx.x;
            a[u] = 0.0f; b[u] = 0.0f;
            if (i < W)
            {
                a[u] = re[ro + i];
                if (are) a[u] += are[ro + i];
                if (im) b[u] = im[ro + i];
                if (aim) b[u] += aim[ro + i];
            }
        }
        #pragma unroll
        for (int u = 0; u < kRowLoads; ++u)
        {
            const int i = i0 + u * kRowThreads + threadIdx.x;
            if (i < Q) x[i] = make_float2(a[u], b[u]);
        }
    }
    __syncthreads();
    const float2* r = stockham<1>(x, y, dq, tw, false);
    // two complex per thread -> one 16-byte store into the tile
    for (int h = threadIdx.x; 2 * h < Q; h += kRowThreads)
    {
        const int q = 2 * h;
        const float2 v0 = r[q];
        const float2 v1 = (q + 1 < Q) ? r[q + 1] : make_float2(0.0f, 0.0f);
        *reinterpret_cast<float4*>(buf + tile_index(pair, G, rows, row, q)) = make_float4(v0.x, v0.y, v1.x, v1.y);
    }
}

constexpr int kColGroup = 4;
constexpr int kColThreads = 512;

// Pass 2: one column group (4 columns) per CTA: forward column FFT over P rows
// (rows >= rows_in are zero), times the kernel spectrum, inverse column FFT;
// rows [0, rows_out) back in place.  mode 1 (kernel-spectrum setup): forward
// only, result for all P rows.
__global__ void __launch_bounds__(kColThreads) conv_cols(float2* __restrict__ buf, const float2* __restrict__ khat,
                                                         int rows_in, int rows_out, FftDims dp, int Q, int mode,
                                                         const float2* __restrict__ tw)
{
    extern __shared__ float2 sm[];
    float2* x = sm;
    float2* y = sm + (size_t)dp.n * kColGroup;
    const int P = dp.n, G = (Q + 3) >> 2;
    const int g = blockIdx.x;
    float2* base = buf + ((size_t)blockIdx.y * G + g) * rows_in * kColGroup;
    const int valid = min(kColGroup, Q - g * kColGroup);
    {
        const float4* src = reinterpret_cast<const float4*>(base);
        float4* xs = reinterpret_cast<float4*>(x);
        const int n4 = rows_in * 2, p4 = P * 2;
        constexpr int U = 8;
        for (int e0 = 0; e0 < p4; e0 += kColThreads * U)
        {
            float4 v[U];
            #pragma unroll
            for (int u = 0; u < U; ++u)
            {
                const int e = e0 + u * kColThreads + threadIdx.x;
                v[u] = e < n4 ? src[e] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            }
            #pragma unroll
            for (int u = 0; u < U; ++u)
            {
                const int e = e0 + u * kColThreads + threadIdx.x;
                if (e < p4) xs[e] = v[u];
            }
        }
    }
    if (valid < kColGroup)
    {
        __syncthreads();
        for (int e = threadIdx.x; e < P * kColGroup; e += kColThreads)
            if ((e & 3) >= valid) x[e] = make_float2(0.0f, 0.0f);
    }
    __syncthreads();
    float2* f = stockham<kColGroup>(x, y, dp, tw, false);
    float2* other = (f == x) ? y : x;
    float4* f4 = reinterpret_cast<float4*>(f);
    float4* dst = reinterpret_cast<float4*>(base);
    if (mode == 1)
    {
        for (int e = threadIdx.x; e < P * 2; e += kColThreads) dst[e] = f4[e];
        return;
    }
    const float4* k4 = reinterpret_cast<const float4*>(khat + (size_t)g * P * kColGroup);
    for (int e = threadIdx.x; e < P * 2; e += kColThreads)
    {
        const float4 a = f4[e], k = __ldg(&k4[e]);
        const float2 lo = cmul(make_float2(a.x, a.y), make_float2(k.x, k.y));
        const float2 hi = cmul(make_float2(a.z, a.w), make_float2(k.z, k.w));
        f4[e] = make_float4(lo.x, lo.y, hi.x, hi.y);
    }
    __syncthreads();
    const float4* r4 = reinterpret_cast<const float4*>(stockham<kColGroup>(f, other, dp, tw, true));
    for (int e = threadIdx.x; e < rows_out * 2; e += kColThreads) dst[e] = r4[e];
}

// Pass 3: inverse row FFTs from the tiles; real part -> out0 (pair 0) / out2
// (pair 1), imaginary part -> out1 (pair 0).  Crop to W.
__global__ void __launch_bounds__(kRowThreads) conv_rows_inv(const float2* __restrict__ buf, int W, int H,
                                                             float* __restrict__ out0, float* __restrict__ out1,
                                                             float* __restrict__ out2, FftDims dq,
                                                             const float2* __restrict__ tw)
{
    extern __shared__ float2 sm[];
    float2* x = sm;
    float2* y = sm + dq.n;
    const int row = blockIdx.x, pair = blockIdx.y;
    const int Q = dq.n, G = (Q + 3) >> 2;
    const int nh = (Q + 1) / 2;
    for (int h0 = 0; h0 < nh; h0 += kRowThreads * 6)
    {
        float4 v[6];
        #pragma unroll
        for (int u = 0; u < 6; ++u)
        {
            const int h = h0 + u * kRowThreads + threadIdx.x;
            v[u] = h < nh ? __ldg(reinterpret_cast<const float4*>(buf + tile_index(pair, G, H, row, 2 * h)))
                          : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
        #pragma unroll
        for (int u = 0; u < 6; ++u)
        {
            const int h = h0 + u * kRowThreads + threadIdx.x;
            if (h < nh)
            {
                x[2 * h] = make_float2(v[u].x, v[u].y);
                if (2 * h + 1 < Q) x[2 * h + 1] = make_float2(v[u].z, v[u].w);
            }
        }
    }
    __syncthreads();
    const float2* r = stockham<1>(x, y, dq, tw, true);
    float* o_re = pair == 0 ? out0 : out2;
    float* o_im = pair == 0 ? out1 : nullptr;
    for (int i = threadIdx.x; i < W; i += kRowThreads)
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
    int Ls = 1;
    for (int s = 0; s < d.nrad; ++s)
    {
        d.ls[s] = Ls;
        d.lmag[s] = Ls > 1 ? (uint32_t)((((uint64_t)1 << 32) + Ls - 1) / Ls) : 0u;
        d.twstep[s] = n / (Ls * d.rad[s]);
        Ls *= d.rad[s];
    }
    return d;
}

// exp(-2 pi i t / n), t < n, in double then rounded
std::vector<float2> twiddles(int n)
{
    std::vector<float2> t((size_t)n);
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < n; ++i)
    {
        const double a = 2.0 * pi * (double)i / (double)n;
        t[i] = make_float2((float)std::cos(a), (float)-std::sin(a));
    }
    return t;
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
    if (p->P > 8192 || p->Q > 3072)
    {
        delete p;
        return fail(GL_ERR_INVALID, "conv2d_plan_create: padded transform above 8192 rows or 3072 columns");
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
    chk(cudaFuncSetAttribute(conv_cols, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem_col));
    chk(cudaFuncSetAttribute(conv_rows_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem_row));
    chk(cudaFuncSetAttribute(conv_rows_inv, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smem_row));
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
            conv_rows_fwd<<<dim3(p->P, 1), kRowThreads, p->smem_row, st>>>(kdev, nullptr, nullptr, nullptr, nullptr,
                                                                            nullptr, p->Q, p->P, p->khat, dq,
                                                                            p->tw_q);
            conv_cols<<<dim3(p->G, 1), kColThreads, p->smem_col, st>>>(p->khat, nullptr, p->P, p->P, dp, p->Q, 1,
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
    conv_rows_fwd<<<dim3(p->H, 2), kRowThreads, p->smem_row, st>>>(d_in_r, d_in_g, d_in_b, d_add_r, d_add_g, d_add_b,
                                                                    p->W, p->H, p->buf, dq, p->tw_q);
    conv_cols<<<dim3(p->G, 2), kColThreads, p->smem_col, st>>>(p->buf, p->khat, p->H, p->H, dp, p->Q, 0, p->tw_p);
    conv_rows_inv<<<dim3(p->H, 2), kRowThreads, p->smem_row, st>>>(p->buf, p->W, p->H, d_out_r, d_out_g, d_out_b, dq,
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
