// gl_fft.cuh — shared-memory Stockham FFT building blocks (complex float):
// radix 16 / 9 / 8 / 4 / 3 / 2 butterflies held in registers, one stage per
// pass over shared memory, twiddles from a table computed in FP64.  Used by
// the image convolution (gl_conv.cu) and the starburst sprite (gl_sprite.cu).
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <vector>

namespace gl {

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
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// (sign i) * a
__device__ __forceinline__ float2 cis(float2 a, float sign) { return make_float2(-sign * a.y, sign * a.x); }

// Padded shared-memory index: one spare word per 16 elements, so a warp
// writing 16-element runs at a stride of 16 hits 16 different banks.
__device__ __forceinline__ int pad(int i) { return i + (i >> 4); }
__host__ __device__ inline size_t padded(size_t n) { return n + (n >> 4) + 1; }

// ---- small DFTs in registers: X[p] = sum_q v[q] w^(pq), w = exp(sign 2 pi i / R) ----
__device__ __forceinline__ void dft2(float2& a, float2& b)
{
    const float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

__device__ __forceinline__ void dft4(float2& v0, float2& v1, float2& v2, float2& v3, float sign)
{
    const float2 t0 = cadd(v0, v2), t1 = csub(v0, v2), t2 = cadd(v1, v3), t3 = cis(csub(v1, v3), sign);
    v0 = cadd(t0, t2);
    v2 = csub(t0, t2);
    v1 = cadd(t1, t3);
    v3 = csub(t1, t3);
}

__device__ __forceinline__ void dft3(float2& v0, float2& v1, float2& v2, float sign)
{
    const float c = 0.86602540378443864676f;   // sqrt(3)/2
    const float2 t1 = cadd(v1, v2);
    const float2 t2 = csub(v1, v2);
    const float2 base = make_float2(v0.x - 0.5f * t1.x, v0.y - 0.5f * t1.y);
    const float2 rot = cis(make_float2(c * t2.x, c * t2.y), sign);
    v0 = cadd(v0, t1);
    v1 = cadd(base, rot);
    v2 = csub(base, rot);
}

// w_N^k = (cos 2 pi k / N, sign sin 2 pi k / N) for the in-register twiddles
__device__ __forceinline__ float2 wk(float c, float s, float sign) { return make_float2(c, sign * s); }

template <int R>
__device__ __forceinline__ void dft(float2 (&v)[R], float sign);

template <>
__device__ __forceinline__ void dft<2>(float2 (&v)[2], float) { dft2(v[0], v[1]); }

template <>
__device__ __forceinline__ void dft<3>(float2 (&v)[3], float sign) { dft3(v[0], v[1], v[2], sign); }

template <>
__device__ __forceinline__ void dft<4>(float2 (&v)[4], float sign) { dft4(v[0], v[1], v[2], v[3], sign); }

// 8 = 2 x 4: q = q1 + 2 q2; inner DFT4 over q2, twiddle w8^(q1 p1), outer DFT2.
template <>
__device__ __forceinline__ void dft<8>(float2 (&v)[8], float sign)
{
    const float h = 0.70710678118654752440f;
    dft4(v[0], v[2], v[4], v[6], sign);   // q1 = 0 -> A0[p1] at v[0], v[2], v[4], v[6]
    dft4(v[1], v[3], v[5], v[7], sign);   // q1 = 1 -> A1[p1]
    v[3] = cmul(v[3], wk(h, h, sign));
    v[5] = cis(v[5], sign);
    v[7] = cmul(v[7], wk(-h, h, sign));
    float2 x[8];
    #pragma unroll
    for (int p1 = 0; p1 < 4; ++p1)
    {
        x[p1] = cadd(v[2 * p1], v[2 * p1 + 1]);
        x[p1 + 4] = csub(v[2 * p1], v[2 * p1 + 1]);
    }
    #pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = x[i];
}

// 16 = 4 x 4: q = q1 + 4 q2; inner DFT4 over q2, twiddle w16^(q1 p1), outer DFT4 over q1.
template <>
__device__ __forceinline__ void dft<16>(float2 (&v)[16], float sign)
{
    const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f, h = 0.70710678118654752440f;
    #pragma unroll
    for (int q1 = 0; q1 < 4; ++q1) dft4(v[q1], v[q1 + 4], v[q1 + 8], v[q1 + 12], sign);
    // v[q1 + 4 p1] = A[q1][p1]; multiply by w16^(q1 p1)
    v[5] = cmul(v[5], wk(c1, s1, sign));     // q1 1, p1 1: k 1
    v[9] = cmul(v[9], wk(h, h, sign));       // 1,2: k 2
    v[13] = cmul(v[13], wk(s1, c1, sign));   // 1,3: k 3
    v[6] = cmul(v[6], wk(h, h, sign));       // 2,1: k 2
    v[10] = cis(v[10], sign);                // 2,2: k 4
    v[14] = cmul(v[14], wk(-h, h, sign));    // 2,3: k 6
    v[7] = cmul(v[7], wk(s1, c1, sign));     // 3,1: k 3
    v[11] = cmul(v[11], wk(-h, h, sign));    // 3,2: k 6
    v[15] = cmul(v[15], wk(-c1, -s1, sign)); // 3,3: k 9
    #pragma unroll
    for (int p1 = 0; p1 < 4; ++p1) dft4(v[4 * p1], v[4 * p1 + 1], v[4 * p1 + 2], v[4 * p1 + 3], sign);
    // now v[4 p1 + p2] = X[p1 + 4 p2]: transpose the 4 x 4 index
    float2 x[16];
    #pragma unroll
    for (int p1 = 0; p1 < 4; ++p1)
        #pragma unroll
        for (int p2 = 0; p2 < 4; ++p2) x[p1 + 4 * p2] = v[4 * p1 + p2];
    #pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = x[i];
}

// 9 = 3 x 3: q = q1 + 3 q2; inner DFT3 over q2, twiddle w9^(q1 p1), outer DFT3 over q1.
template <>
__device__ __forceinline__ void dft<9>(float2 (&v)[9], float sign)
{
    const float c1 = 0.76604444311897803520f, s1 = 0.64278760968653932632f;   // 2 pi / 9
    const float c2 = 0.17364817766693034885f, s2 = 0.98480775301220805936f;   // 4 pi / 9
    const float c4 = -0.93969262078590838405f, s4 = 0.34202014332566873304f; // 8 pi / 9
    #pragma unroll
    for (int q1 = 0; q1 < 3; ++q1) dft3(v[q1], v[q1 + 3], v[q1 + 6], sign);
    v[4] = cmul(v[4], wk(c1, s1, sign));   // q1 1, p1 1: k 1
    v[7] = cmul(v[7], wk(c2, s2, sign));   // 1,2: k 2
    v[5] = cmul(v[5], wk(c2, s2, sign));   // 2,1: k 2
    v[8] = cmul(v[8], wk(c4, s4, sign));   // 2,2: k 4
    #pragma unroll
    for (int p1 = 0; p1 < 3; ++p1) dft3(v[3 * p1], v[3 * p1 + 1], v[3 * p1 + 2], sign);
    float2 x[9];
    #pragma unroll
    for (int p1 = 0; p1 < 3; ++p1)
        #pragma unroll
        for (int p2 = 0; p2 < 3; ++p2) x[p1 + 3 * p2] = v[3 * p1 + p2];
    #pragma unroll
    for (int i = 0; i < 9; ++i) v[i] = x[i];
}

// One Stockham stage of radix R over NB interleaved sequences (element i of
// sequence s at logical index i * NB + s, stored at pad()), x -> y.
template <int R, int NB>
__device__ __forceinline__ void radix_stage(const float2* __restrict__ x, float2* __restrict__ y, int n, int Ls,
                                            uint32_t lmag, int twstep, const float2* __restrict__ tw, bool inv)
{
    const int m = n / R;
    const int items = m * NB;
    const float sign = inv ? 1.0f : -1.0f;
    for (int it = threadIdx.x; it < items; it += blockDim.x)
    {
        const int s = it % NB, j = it / NB;
        int g = j, k = 0;
        if (Ls > 1)
        {
            g = (int)__umulhi((uint32_t)j, lmag);
            k = j - g * Ls;
        }
        float2 v[R];
        #pragma unroll
        for (int q = 0; q < R; ++q) v[q] = x[pad((j + q * m) * NB + s)];
        if (k > 0)
        {
            #pragma unroll
            for (int q = 1; q < R; ++q)
            {
                float2 w = __ldg(&tw[q * k * twstep]);   // q k < R Ls: index < n
                if (inv) w.y = -w.y;
                v[q] = cmul(v[q], w);
            }
        }
        dft<R>(v, sign);
        const int ob = g * Ls * R + k;
        #pragma unroll
        for (int p = 0; p < R; ++p) y[pad((ob + p * Ls) * NB + s)] = v[p];
    }
}

// Full transform; returns the buffer holding the result (x or y).
template <int NB>
__device__ float2* stockham(float2* x, float2* y, const FftDims& d, const float2* __restrict__ tw, bool inv)
{
    for (int st = 0; st < d.nrad; ++st)
    {
        const int n = d.n, L = d.ls[st], ts = d.twstep[st];
        const uint32_t lm = d.lmag[st];
        switch (d.rad[st])
        {
        case 16: radix_stage<16, NB>(x, y, n, L, lm, ts, tw, inv); break;
        case 9: radix_stage<9, NB>(x, y, n, L, lm, ts, tw, inv); break;
        case 8: radix_stage<8, NB>(x, y, n, L, lm, ts, tw, inv); break;
        case 4: radix_stage<4, NB>(x, y, n, L, lm, ts, tw, inv); break;
        case 3: radix_stage<3, NB>(x, y, n, L, lm, ts, tw, inv); break;
        default: radix_stage<2, NB>(x, y, n, L, lm, ts, tw, inv); break;
        }
        __syncthreads();
        float2* t = x; x = y; y = t;
    }
    return x;
}

inline FftDims make_dims(int n)
{
    FftDims d{};
    d.n = n;
    int m = n;
    while (m % 16 == 0) { d.rad[d.nrad++] = 16; m /= 16; }
    if (m % 8 == 0) { d.rad[d.nrad++] = 8; m /= 8; }
    if (m % 4 == 0) { d.rad[d.nrad++] = 4; m /= 4; }
    if (m % 2 == 0) { d.rad[d.nrad++] = 2; m /= 2; }
    while (m % 9 == 0) { d.rad[d.nrad++] = 9; m /= 9; }
    if (m % 3 == 0) { d.rad[d.nrad++] = 3; m /= 3; }
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
inline std::vector<float2> twiddles(int n)
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

}  // namespace gl
