// gl_mdft.cu — tensor-core matrix products for the matrix-DFT starburst.
//
// This unit holds the tcgen05 machinery shared by the MDFT forms: TMA tensor
// maps built on the host, a warp-specialised CTA (one TMA producer thread,
// one MMA-issuing thread, four epilogue warps reading TMEM) and the plain
// BF16 GEMM C = A * B^T that pins the descriptors against torch.
#include "gl_internal.h"
#include "gl_tc.cuh"

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>
#include <cstring>
#include <mutex>
#include <string>

namespace gl {

// ---- host: tensor maps --------------------------------------------------------
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn()
{
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// 2-D row-major matrix of `rows` x `cols` elements (cols contiguous) with a
// box of box_rows x box_cols, 128-byte swizzle (box_cols * elem = 128 B).
int make_tmap_2d(CUtensorMap* map, const void* base, CUtensorMapDataType dtype, int elem_bytes, uint64_t rows,
                 uint64_t cols, uint32_t box_rows, uint32_t box_cols)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn) return fail(GL_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    if (((uintptr_t)base & 15) != 0) return fail(GL_ERR_INVALID, "tensor base must be 16-byte aligned");
    if ((cols * elem_bytes) % 16 != 0) return fail(GL_ERR_INVALID, "tensor row pitch must be a multiple of 16 bytes");
    cuuint64_t gdim[2] = {cols, rows};
    cuuint64_t gstride[1] = {cols * (uint64_t)elem_bytes};
    cuuint32_t box[2] = {box_cols, box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, dtype, 2, const_cast<void*>(base), gdim, gstride, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(GL_ERR_INVALID, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return GL_OK;
}

namespace {

constexpr int kBM = 128, kBN = 128, kBK = 64, kStages = 4;
constexpr int kTileBytes = kBM * kBK * 2;   // 16 KB per operand tile

__device__ __forceinline__ uint8_t* align1024(uint8_t* p)
{
    return reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(p) + 1023) & ~uintptr_t(1023));
}

// C[M x N] (fp32, row-major) = A[M x K] * B[N x K]^T, BF16 operands, FP32
// accumulation in TMEM.  One 128x128 tile per CTA; 128 threads.
__global__ void __launch_bounds__(128, 1) tc_gemm_bf16_kernel(const __grid_constant__ CUtensorMap ta,
                                                              const __grid_constant__ CUtensorMap tb, float* C,
                                                              int M, int N, int K, int* err)
{
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = align1024(smem_raw);
    uint8_t* sa = smem;
    uint8_t* sb = smem + kStages * kTileBytes;
    __shared__ uint64_t full[kStages], empty[kStages], accbar;
    __shared__ uint32_t tmem_base;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
    const int nk = K / kBK;

    if (warp == 0) tc::tmem_alloc(&tmem_base, 128);
    if (threadIdx.x == 32)
    {
        for (int s = 0; s < kStages; ++s) { tc::mbar_init(&full[s], 1); tc::mbar_init(&empty[s], 1); }
        tc::mbar_init(&accbar, 1);
        tc::fence_mbar_init();
        tc::tma_prefetch(&ta);
        tc::tma_prefetch(&tb);
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;

    if (warp == 0 && lane == 0)
    {
        // TMA producer
        int issued = 0;
        for (int kb = 0; kb < nk; ++kb)
        {
            const int s = kb % kStages;
            if (kb >= kStages && !tc::mbar_wait(&empty[s], ((kb / kStages) - 1) & 1, err, tc::TC_TIMEOUT_EMPTY)) break;
            tc::mbar_expect_tx(&full[s], 2 * kTileBytes);
            tc::tma_load_2d(sa + s * kTileBytes, &ta, kb * kBK, m0, &full[s]);
            tc::tma_load_2d(sb + s * kTileBytes, &tb, kb * kBK, n0, &full[s]);
            ++issued;
        }
        // our own copies must have landed before the CTA can retire
        for (int kb = (issued > kStages ? issued - kStages : 0); kb < issued; ++kb)
            tc::mbar_wait(&full[kb % kStages], (kb / kStages) & 1, err, tc::TC_TIMEOUT_FULL);
    }
    else if (warp == 1 && lane == 0)
    {
        // MMA issuer
        const uint32_t idesc = tc::idesc_bf16(kBM, kBN, false);
        for (int kb = 0; kb < nk; ++kb)
        {
            const int s = kb % kStages;
            if (!tc::mbar_wait(&full[s], (kb / kStages) & 1, err, tc::TC_TIMEOUT_FULL)) break;
            tc::tc_fence_after();
            const uint64_t da = tc::sw128_desc(tc::smem_u32(sa + s * kTileBytes));
            const uint64_t db = tc::sw128_desc(tc::smem_u32(sb + s * kTileBytes));
            #pragma unroll
            for (int kk = 0; kk < kBK / 16; ++kk)
                tc::mma_f16(tmem, da + 2 * kk, db + 2 * kk, idesc, (kb | kk) != 0);
            tc::mma_commit(&empty[s]);
        }
        tc::mma_commit(&accbar);   // also on the error path: no MMA may outlive TMEM
    }
    __syncwarp();

    // Epilogue: TMEM lane = tile row; 8 chunks of 16 columns.
    const bool ok = tc::mbar_wait(&accbar, 0, err, tc::TC_TIMEOUT_ACC);
    tc::tc_fence_after();
    const int row = warp * 32 + lane;
    #pragma unroll 1
    for (int c = 0; c < kBN / 16; ++c)
    {
        float v[16];
        tc::tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 16), v);
        if (ok && m0 + row < M)
        {
            float* dst = C + (size_t)(m0 + row) * N + n0 + c * 16;
            #pragma unroll
            for (int i = 0; i < 16; i += 4) *reinterpret_cast<float4*>(dst + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 128);
}

}  // namespace
}  // namespace gl

using namespace gl;

extern "C" int gl_gemm_bf16_tc(const void* d_a, const void* d_b, float* d_c, int M, int N, int K, void* stream)
{
    if (!d_a || !d_b || !d_c) return fail(GL_ERR_INVALID, "gemm_bf16_tc: null pointer");
    if (M <= 0 || N <= 0 || K <= 0 || M % 128 || N % 128 || K % 64)
        return fail(GL_ERR_INVALID, "gemm_bf16_tc: M and N must be multiples of 128, K of 64");
    CUtensorMap ta, tb;
    int rc = make_tmap_2d(&ta, d_a, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (uint64_t)M, (uint64_t)K, 128, 64);
    if (rc) return rc;
    rc = make_tmap_2d(&tb, d_b, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (uint64_t)N, (uint64_t)K, 128, 64);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    int* d_err = nullptr;
    GL_CUDA_TRY(cudaMallocAsync(&d_err, sizeof(int), st));
    GL_CUDA_TRY(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    const size_t smem = 2 * kStages * kTileBytes + 1024;
    GL_CUDA_TRY(cudaFuncSetAttribute(tc_gemm_bf16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid(N / 128, M / 128);
    tc_gemm_bf16_kernel<<<grid, 128, smem, st>>>(ta, tb, d_c, M, N, K, d_err);
    GL_CUDA_TRY(cudaGetLastError());
    int h_err = 0;
    GL_CUDA_TRY(cudaMemcpyAsync(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    GL_CUDA_TRY(cudaStreamSynchronize(st));
    cudaFreeAsync(d_err, st);
    g_last_launches = 1;
    if (h_err) return fail(GL_ERR_TIMEOUT, "gemm_bf16_tc: a pipeline wait timed out (code " + std::to_string(h_err) + ")");
    return GL_OK;
}

// ===========================================================================
// Matrix-DFT starburst, field form:  E_l = W_y(l) A W_x(l)^T,  I_l = |E_l|^2,
// out_c = sum_l w_c(l) I_l   (the field form of mdft_render.cu's
// per-wavelength triple product, evaluated on the tensor cores).
//
//   W_x[k][j] = exp(-2 pi i s_x(l) (j - c_j)(k - c_x)),  same for y.
//
// Step 1: T'[k][i] = sum_j W_x[k][j] A[i][j]          (K_out x n, complex)
// Step 2: E[l][k]  = sum_i W_y[l][i] T'[k][i]         (K_out x K_out, complex)
//
// FORM 0 (split BF16): every operand X is stored as X_hi = bf16(X) and
// X_lo = bf16(X - X_hi); the three-term product A_hi B_hi + A_hi B_lo +
// A_lo B_hi is one GEMM over a tripled reduction axis, A' = [hi | hi | lo],
// B' = [hi | lo | hi].  FORM 1 (TF32): FP32 operands, kind::tf32 MMAs.
// Accumulation is FP32 in TMEM throughout.
//
// Complex products: T' holds, per 128 output columns, the two row blocks
// [Tr | Ti]; step 2 stages them next to each other in shared memory and
// accumulates two products with the same B operand, D1 = Wr [Tr | Ti] and
// D2 = Wi [Tr | Ti] (N = 2 x tile width each), which its epilogue combines:
// Re E = Wr Tr - Wi Ti = D1[Tr] - D2[Ti], Im E = Wr Ti + Wi Tr = D1[Ti] +
// D2[Tr].
// ===========================================================================
namespace gl {
namespace {

constexpr int kMdftThreads = 192;     // warps 0-3 epilogue, warp 4 TMA, warp 5 MMA
constexpr int kOpTile = 128 * 128;    // bytes of one 128-row x 128-byte operand tile

struct MdftArgs {
    int KA;       // rows of the A operand per (wavelength, re/im part): Kx in step 1, Ky in step 2
    int Kx;       // output width = T' k range; row stride of the output planes
    int NBm;      // 128-row blocks of the A operand (step 1: Kx / 128, step 2: Ky / 128)
    int n, n_lambda, Kp, nkb, NB, NI, n_units;   // NB = Kx / 128 (T' blocks per wavelength)
    void* tprime;                     // step 1 output / step 2 B operand
    float* out_r;
    float* out_g;
    float* out_b;
    const float4* weights;            // per wavelength (w_r, w_g, w_b, 0)
    int* err;
    // step-2 output placement: plan pixel (l, k) -> frame (y0 + l, x0 + k) of
    // planes out_w wide, kept when l < win_h and k < win_w
    int out_w, x0, y0, win_w, win_h;
    int box;                          // 1: accumulate Re E (pixel-integrated form); 0: |E|^2
    float4 tint;                      // per-launch colour factor on the weights
    int lam_base;                     // first wavelength of this launch's range
    int NBt;                          // step 2: output tiles per row of the frame (Kx / tile width)
};

template <int FORM>
__device__ __forceinline__ void mma_any(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    if (FORM == 0) tc::mma_f16(d, a, b, idesc, acc);
    else tc::mma_tf32(d, a, b, idesc, acc);
}

template <int FORM>
__host__ __device__ constexpr uint32_t idesc_any(int M, int N)
{
    return FORM == 0 ? tc::idesc_bf16(M, N, false) : tc::idesc_tf32(M, N, false);
}

__device__ __forceinline__ void store_split16(__nv_bfloat16* row, int n, int i0, const float (&v)[16], float sign)
{
    // [hi | lo | hi] at columns i0, n + i0, 2n + i0
    __align__(16) __nv_bfloat16 hi[16], lo[16];
    #pragma unroll
    for (int j = 0; j < 16; ++j)
    {
        const float x = sign * v[j];
        hi[j] = __float2bfloat16_rn(x);
        lo[j] = __float2bfloat16_rn(x - __bfloat162float(hi[j]));
    }
    const uint4* h4 = reinterpret_cast<const uint4*>(hi);
    const uint4* l4 = reinterpret_cast<const uint4*>(lo);
    uint4* d0 = reinterpret_cast<uint4*>(row + i0);
    uint4* d1 = reinterpret_cast<uint4*>(row + n + i0);
    uint4* d2 = reinterpret_cast<uint4*>(row + 2 * n + i0);
    d0[0] = h4[0]; d0[1] = h4[1];
    d1[0] = l4[0]; d1[1] = l4[1];
    d2[0] = h4[0]; d2[1] = h4[1];
}

// TN (step 2): complex output columns per unit, 128 or 64 (the autotuner's
// tile-shape knob).  A 64-column unit stages three 64-row blocks of T' (8 KB
// each, box rows 64 in tB) and issues N = 128 MMAs; its smaller stages allow
// a three-deep pipeline, and twice the units spread a small frame over more
// SMs.
template <int FORM, int STEP, int TN = 128>
__global__ void __launch_bounds__(kMdftThreads, 1) mdft_kernel(const __grid_constant__ CUtensorMap tA,
                                                              const __grid_constant__ CUtensorMap tB, MdftArgs args)
{
    static_assert(TN == 128 || TN == 64, "tile width");
    constexpr int kBBytes = (STEP == 2) ? 2 * TN * 128 : kOpTile;   // B operand bytes per stage
    constexpr int kStagesM = (STEP == 2) ? (TN == 128 ? 3 : 4) : 4;
    constexpr int kStageBytes = 2 * kOpTile + kBBytes;
    // accumulator buffers in TMEM's 512 columns: a unit of step 2 takes
    // 4 TN columns (D1 and D2), so the 128-column tile is single-buffered
    constexpr int kAccBufs = (STEP == 2 && TN == 128) ? 1 : 2;
    constexpr int kbe = (FORM == 0) ? 64 : 32;                   // reduction elements per 128-byte row
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = align1024(smem_raw);
    __shared__ uint64_t full[kStagesM], empty[kStagesM], acc_full[2], acc_empty[2], mma_done;
    __shared__ uint32_t tmem_base;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int* err = args.err;

    if (warp == 5) tc::tmem_alloc(&tmem_base, 512);
    if (threadIdx.x == 128)
    {
        for (int s = 0; s < kStagesM; ++s) { tc::mbar_init(&full[s], 1); tc::mbar_init(&empty[s], 1); }
        for (int b = 0; b < 2; ++b) { tc::mbar_init(&acc_full[b], 1); tc::mbar_init(&acc_empty[b], 128); }
        tc::mbar_init(&mma_done, 1);
        tc::fence_mbar_init();
        tc::tma_prefetch(&tA);
        tc::tma_prefetch(&tB);
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = tmem_base;

    // Units are dealt round-robin (unit u to CTA u mod G), so the units in
    // flight at any moment are consecutive: with wavelength-major unit order
    // they share one wavelength's operands, which then stay in L2.
    const int G = gridDim.x;
    const int u0 = blockIdx.x, u1 = args.n_units;

    auto decode = [&](int u, int& lam, int& mb, int& xb) {
        if (STEP == 2)
        {
            // wavelength-major: all output tiles of one wavelength, then the next
            const int tiles = args.NBm * args.NBt;
            const int lr = u / tiles;               // wavelength within this launch's range
            lam = args.lam_base + lr;
            const int tile = u - lr * tiles;
            mb = tile / args.NBt;
            xb = tile % args.NBt;
        }
        else
        {
            lam = args.lam_base + u / (args.NBm * args.NI);
            const int r = u % (args.NBm * args.NI);
            mb = r / args.NI;
            xb = r % args.NI;
        }
    };

    if (warp == 4)
    {
        if (lane == 0)
        {
            int it = 0, issued = 0;
            bool stop = false;
            for (int u = u0; u < u1 && !stop; u += G)
            {
                int lam, mb, xb;
                decode(u, lam, mb, xb);
                const int rowA = (lam * 2) * args.KA + mb * 128;
                for (int kb = 0; kb < args.nkb; ++kb, ++it)
                {
                    const int s = it % kStagesM, r = it / kStagesM;
                    if (it >= kStagesM && !tc::mbar_wait(&empty[s], (r - 1) & 1, err, tc::TC_TIMEOUT_EMPTY)) { stop = true; break; }
                    uint8_t* st = smem + s * kStageBytes;
                    tc::mbar_expect_tx(&full[s], kStageBytes);
                    const int x = kb * kbe;
                    tc::tma_load_2d(st, &tA, x, rowA, &full[s]);
                    tc::tma_load_2d(st + kOpTile, &tA, x, rowA + args.KA, &full[s]);
                    if (STEP == 2)
                    {
                        // rows [Tr | Ti] of this tile's columns: T' holds them in
                        // 128-row blocks, a 64-column tile takes one half of each
                        const int xb128 = (TN == 128) ? xb : (xb >> 1);
                        const int half = (TN == 128) ? 0 : (xb & 1) * 64;
                        const int rowB = ((lam * args.NB + xb128) * 2) * 128 + half;
                        #pragma unroll
                        for (int j = 0; j < 2; ++j)
                            tc::tma_load_2d(st + 2 * kOpTile + j * TN * 128, &tB, x, rowB + j * 128, &full[s]);
                    }
                    else
                    {
                        tc::tma_load_2d(st + 2 * kOpTile, &tB, x, xb * 128, &full[s]);
                    }
                    ++issued;
                }
            }
            for (int q = (issued > kStagesM ? issued - kStagesM : 0); q < issued; ++q)
                tc::mbar_wait(&full[q % kStagesM], (q / kStagesM) & 1, err, tc::TC_TIMEOUT_FULL);
        }
        __syncwarp();
    }
    else if (warp == 5)
    {
        if (lane == 0)
        {
            const uint32_t id2 = idesc_any<FORM>(128, 2 * TN);
            const uint32_t id128 = idesc_any<FORM>(128, 128);
            int it = 0, ui = 0;
            bool stop = false;
            for (int u = u0; u < u1 && !stop; u += G, ++ui)
            {
                const int b = ui % kAccBufs, ur = ui / kAccBufs;
                if (ui >= kAccBufs && !tc::mbar_wait(&acc_empty[b], (ur - 1) & 1, err, tc::TC_TIMEOUT_ACC_FREE)) break;
                tc::tc_fence_after();
                const uint32_t d = tmem + (uint32_t)(b * 256);
                for (int kb = 0; kb < args.nkb; ++kb, ++it)
                {
                    const int s = it % kStagesM, r = it / kStagesM;
                    if (!tc::mbar_wait(&full[s], r & 1, err, tc::TC_TIMEOUT_FULL)) { stop = true; break; }
                    tc::tc_fence_after();
                    uint8_t* st = smem + s * kStageBytes;
                    const uint64_t aR = tc::sw128_desc(tc::smem_u32(st));
                    const uint64_t aI = tc::sw128_desc(tc::smem_u32(st + kOpTile));
                    if (STEP == 2)
                    {
                        // D1 = Wr [Tr | Ti] at d, D2 = Wi [Tr | Ti] at d + 2 TN
                        const uint64_t bRI = tc::sw128_desc(tc::smem_u32(st + 2 * kOpTile));   // [Tr | Ti]
                        #pragma unroll
                        for (int kk = 0; kk < 4; ++kk)
                        {
                            mma_any<FORM>(d, aR + 2 * kk, bRI + 2 * kk, id2, (kb | kk) != 0);
                            mma_any<FORM>(d + 2 * TN, aI + 2 * kk, bRI + 2 * kk, id2, (kb | kk) != 0);
                        }
                    }
                    else
                    {
                        const uint64_t bM = tc::sw128_desc(tc::smem_u32(st + 2 * kOpTile));
                        #pragma unroll
                        for (int kk = 0; kk < 4; ++kk)
                        {
                            mma_any<FORM>(d, aR + 2 * kk, bM + 2 * kk, id128, (kb | kk) != 0);
                            mma_any<FORM>(d + 128, aI + 2 * kk, bM + 2 * kk, id128, (kb | kk) != 0);
                        }
                    }
                    tc::mma_commit(&empty[s]);
                }
                tc::mma_commit(&acc_full[b]);
            }
            // every MMA this thread issued must be complete before TMEM is freed
            tc::mma_commit(&mma_done);
            tc::mbar_wait(&mma_done, 0, err, tc::TC_TIMEOUT_ACC);
        }
        __syncwarp();
    }
    else
    {
        // Epilogue warps 0-3: TMEM lane = tile row.
        int ui = 0;
        const int row = warp * 32 + lane;
        for (int u = u0; u < u1; u += G, ++ui)
        {
            int lam, mb, xb;
            decode(u, lam, mb, xb);
            const int b = ui % kAccBufs, ur = ui / kAccBufs;
            const bool ok = tc::mbar_wait(&acc_full[b], ur & 1, err, tc::TC_TIMEOUT_ACC);
            tc::tc_fence_after();
            const uint32_t ta = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(b * 256);
            if (STEP == 2)
            {
                const float4 w0 = args.weights[lam];
                const float4 w = make_float4(w0.x * args.tint.x, w0.y * args.tint.y, w0.z * args.tint.z, 0.0f);
                const int l = mb * 128 + row;
                const bool row_in = l < args.win_h;
                const size_t orow = (size_t)(args.y0 + l) * (size_t)args.out_w + (size_t)args.x0;
                #pragma unroll 1
                for (int c = 0; c < TN / 16; ++c)
                {
                    // Re E = D1[Tr] - D2[Ti], Im E = D1[Ti] + D2[Tr]
                    float re[16], im[16], u2[16], v2[16];
                    tc::tmem_ld16(ta + (uint32_t)(c * 16), re);
                    tc::tmem_ld16(ta + (uint32_t)TN + (uint32_t)(c * 16), im);
                    tc::tmem_ld16(ta + (uint32_t)(2 * TN) + (uint32_t)(c * 16), u2);
                    tc::tmem_ld16(ta + (uint32_t)(3 * TN) + (uint32_t)(c * 16), v2);
                    #pragma unroll
                    for (int j = 0; j < 16; ++j)
                    {
                        re[j] -= v2[j];
                        im[j] += u2[j];
                    }
                    if (!ok || !row_in) continue;
                    const int kc = xb * TN + c * 16;
                    #pragma unroll
                    for (int j = 0; j < 16; j += 4)
                    {
                        float I[4];
                        #pragma unroll
                        for (int q = 0; q < 4; ++q)
                            I[q] = args.box ? re[j + q] : re[j + q] * re[j + q] + im[j + q] * im[j + q];
                        const int k = kc + j;
                        const size_t o = orow + (size_t)k;
                        if (k + 3 < args.win_w && (o & 3) == 0)
                        {
                            atomicAdd(reinterpret_cast<float4*>(args.out_r + o), make_float4(w.x * I[0], w.x * I[1], w.x * I[2], w.x * I[3]));
                            atomicAdd(reinterpret_cast<float4*>(args.out_g + o), make_float4(w.y * I[0], w.y * I[1], w.y * I[2], w.y * I[3]));
                            atomicAdd(reinterpret_cast<float4*>(args.out_b + o), make_float4(w.z * I[0], w.z * I[1], w.z * I[2], w.z * I[3]));
                        }
                        else
                        {
                            #pragma unroll
                            for (int q = 0; q < 4; ++q)
                            {
                                if (k + q >= args.win_w) break;
                                atomicAdd(args.out_r + o + q, w.x * I[q]);
                                atomicAdd(args.out_g + o + q, w.y * I[q]);
                                atomicAdd(args.out_b + o + q, w.z * I[q]);
                            }
                        }
                    }
                }
            }
            else
            {
                // T' rows of this k: [Tr | Ti] blocks of 128 rows.
                const int k = row;
                const size_t blk = ((size_t)(lam * args.NB + mb) * 2) * 128;
                #pragma unroll 1
                for (int c = 0; c < 8; ++c)
                {
                    float re[16], im[16];
                    tc::tmem_ld16(ta + (uint32_t)(c * 16), re);
                    tc::tmem_ld16(ta + 128u + (uint32_t)(c * 16), im);
                    if (!ok) continue;
                    const int i0 = xb * 128 + c * 16;
                    if (FORM == 0)
                    {
                        __nv_bfloat16* T = static_cast<__nv_bfloat16*>(args.tprime);
                        store_split16(T + (blk + 0 * 128 + k) * (size_t)args.Kp, args.n, i0, re, 1.0f);
                        store_split16(T + (blk + 1 * 128 + k) * (size_t)args.Kp, args.n, i0, im, 1.0f);
                    }
                    else
                    {
                        float* T = static_cast<float*>(args.tprime);
                        float* r0 = T + (blk + 0 * 128 + k) * (size_t)args.Kp + i0;
                        float* r1 = T + (blk + 1 * 128 + k) * (size_t)args.Kp + i0;
                        #pragma unroll
                        for (int j = 0; j < 16; j += 4)
                        {
                            *reinterpret_cast<float4*>(r0 + j) = make_float4(re[j], re[j + 1], re[j + 2], re[j + 3]);
                            *reinterpret_cast<float4*>(r1 + j) = make_float4(im[j], im[j + 1], im[j + 2], im[j + 3]);
                        }
                    }
                }
            }
            tc::tc_fence_before();
            tc::mbar_arrive(&acc_empty[b]);
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 5) tc::tmem_dealloc(tmem, 512);
}

// DFT matrices W'[lam][part][k][Kp]: part 0 = Re, 1 = Im of
// exp(-2 pi i s(lam) (j - cj)(k - ck)).  The phase is formed in FP32
// double-float arithmetic (Dekker / Ogita-Rump-Oishi error-free products
// with FMA): s = s_hi + s_lo and ck = ck_hi + ck_lo are split on the host,
// a = j - cj is exact (cj a half-integer), b = k - ck is carried as a
// two-float sum, and the product's integer cycles are removed from
// the leading term exactly; the reduced phase is accurate to ~1e-9 cycles,
// then evaluated with sincospif.  (The FP64 units of this part are slow.)
// With box set each entry also carries the pixel-box factor sinc(s (j - cj))
// of the reference's pixel-integrated form (mdft_render.cu:109-135).
// FORM 0 stores [hi | hi | lo] along the reduction axis, FORM 1 the FP32 value.
template <int FORM>
__global__ void mdft_dft_kernel(void* out, int n_lambda, int K_rows, int n, int Kp, const float2* __restrict__ scale,
                                float ck_hi, float ck_lo, float cj, int box)
{
    const size_t total = (size_t)n_lambda * K_rows * n;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
    {
        const int j = (int)(e % n);
        const int k = (int)((e / n) % K_rows);
        const int lam = (int)(e / ((size_t)n * K_rows));
        const float2 sc = scale[lam];                  // (s_hi, s_lo)
        const float a = (float)j - cj;                 // exact
        // b = k - ck as bh + bl: Knuth's two-sum of k and -ck_hi, then -ck_lo
        const float kf = (float)k;
        const float bh = kf - ck_hi;
        const float bb = bh - kf;
        const float bl = ((kf - (bh - bb)) + (-ck_hi - bb)) - ck_lo;
        const float p1 = a * bh;
        const float e1 = fmaf(a, bh, -p1);             // a*bh = p1 + e1 exactly
        const float m_lo = e1 + a * bl;
        const float q = sc.x * p1;
        const float eq = fmaf(sc.x, p1, -q);           // s_hi*p1 = q + eq exactly
        const float rest = eq + sc.x * m_lo + sc.y * p1;
        float fr = (q - rintf(q)) + rest;              // q - rint(q) is exact
        fr -= rintf(fr);
        float sv, cv;
        sincospif(2.0f * fr, &sv, &cv);
        float amp = 1.0f;
        if (box)
        {
            // pixel-box factor of the pixel-integrated form: sinc(m s), m = j - cj
            // the lag, s = pixel pitch / pattern period at this wavelength
            const float x = a * (sc.x + sc.y);
            amp = fabsf(x) < 1e-7f ? 1.0f : sinpif(x) / (3.14159265358979323846f * x);
        }
        const float re = amp * cv, im = -amp * sv;
        const size_t rr = ((size_t)(lam * 2 + 0) * K_rows + k) * Kp;
        const size_t ri = ((size_t)(lam * 2 + 1) * K_rows + k) * Kp;
        if (FORM == 0)
        {
            __nv_bfloat16* W = static_cast<__nv_bfloat16*>(out);
            const __nv_bfloat16 rh = __float2bfloat16_rn(re), ih = __float2bfloat16_rn(im);
            const __nv_bfloat16 rl = __float2bfloat16_rn(re - __bfloat162float(rh));
            const __nv_bfloat16 il = __float2bfloat16_rn(im - __bfloat162float(ih));
            W[rr + j] = rh; W[rr + n + j] = rh; W[rr + 2 * n + j] = rl;
            W[ri + j] = ih; W[ri + n + j] = ih; W[ri + 2 * n + j] = il;
        }
        else
        {
            float* W = static_cast<float*>(out);
            W[rr + j] = re;
            W[ri + j] = im;
        }
    }
}

// Pupil amplitude of the lens's stop (build_pupil_kernel,
// starburst_render.cu:155-191, stop term): grid coordinate g in [-1, 1) maps
// to pupil coordinate g / pupil_fill; 4 x 4 supersamples per texel tested
// against the stop silhouette (PupilMask::contains, aperture_sampler.h:63-82:
// ellipse of the stop's aspect, then the regular n-gon or the authored blade
// profile).
struct PupilDev {
    float aspect, rot_rad, apothem, sector;
    int n_blades;
    BladeProfile blade;
};

__device__ __forceinline__ bool pupil_in(const PupilDev& m, float u, float v)
{
    const float ux = u / m.aspect;
    const float r2 = ux * ux + v * v;
    if (r2 > 1.0f) return false;
    if (m.n_blades >= 3)
    {
        if (m.blade.deformed) return sqrtf(r2) <= blade_radius_at(m.blade, atan2f(v, ux));
        const float angle = atan2f(v, ux) - m.rot_rad;
        float sector = fmodf(angle, m.sector);
        if (sector < 0.0f) sector += m.sector;
        if (sqrtf(r2) * cosf(sector - m.sector * 0.5f) > m.apothem) return false;
    }
    return true;
}

// bilinear sample of the cat's-eye envelope (ME x ME over pupil [-1, 1]^2,
// cell centres, clamped at the edges): sample_env, starburst_render.cu:136-149
__device__ __forceinline__ float pupil_env(const float* __restrict__ env, int ME, float u, float v)
{
    float fx = (u * 0.5f + 0.5f) * ME - 0.5f;
    float fy = (v * 0.5f + 0.5f) * ME - 0.5f;
    fx = fminf(fmaxf(fx, 0.0f), (float)(ME - 1));
    fy = fminf(fmaxf(fy, 0.0f), (float)(ME - 1));
    const int x0 = (int)floorf(fx), y0 = (int)floorf(fy);
    const int x1 = min(x0 + 1, ME - 1), y1 = min(y0 + 1, ME - 1);
    const float tx = fx - x0, ty = fy - y0;
    const float a = env[(size_t)y0 * ME + x0] * (1.0f - tx) + env[(size_t)y0 * ME + x1] * tx;
    const float b = env[(size_t)y1 * ME + x0] * (1.0f - tx) + env[(size_t)y1 * ME + x1] * tx;
    return a * (1.0f - ty) + b * ty;
}

// env == nullptr: the plain stop (coverage of the 16 supersamples); else
// each inside supersample weighs the envelope at its own position
__global__ void pupil_build_kernel(float* __restrict__ out, int N, float fill, PupilDev m,
                                   const float* __restrict__ env, int ME)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= N * N) return;
    const int i = idx % N, j = idx / N;
    int cnt = 0;
    float acc = 0.0f;
    #pragma unroll
    for (int sy = 0; sy < 4; ++sy)
        #pragma unroll
        for (int sx = 0; sx < 4; ++sx)
        {
            const float u = (((float)i + ((float)sx + 0.5f) * 0.25f) / (float)N * 2.0f - 1.0f) / fill;
            const float v = (((float)j + ((float)sy + 0.5f) * 0.25f) / (float)N * 2.0f - 1.0f) / fill;
            if (!pupil_in(m, u, v)) continue;
            ++cnt;
            if (env) acc += pupil_env(env, ME, u, v);
        }
    out[idx] = (env ? acc : (float)cnt) * (1.0f / 16.0f);
}

// Pupil amplitude A[i][j] (float, n x n) -> B operand [hi | lo | hi] or FP32.
template <int FORM>
__global__ void mdft_mask_kernel(const float* __restrict__ a, void* out, int n, int Kp)
{
    const size_t total = (size_t)n * n;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x)
    {
        const int j = (int)(e % n), i = (int)(e / n);
        const float v = a[e];
        if (FORM == 0)
        {
            __nv_bfloat16* M = static_cast<__nv_bfloat16*>(out);
            const __nv_bfloat16 h = __float2bfloat16_rn(v);
            const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
            M[(size_t)i * Kp + j] = h; M[(size_t)i * Kp + n + j] = l; M[(size_t)i * Kp + 2 * n + j] = h;
        }
        else
        {
            static_cast<float*>(out)[(size_t)i * Kp + j] = v;
        }
    }
}


// ---- FP32 CUDA-core form -------------------------------------------------------
// Register-tiled FP32 products on the SIMT pipes over the TF32 form's storage
// (W' [lam][2][K_out][n], T' [lam][NB][3][128][n]); 256 threads, 128x128
// tiles, 8x8 outputs per thread, K chunks of 16 staged in shared memory.
constexpr int kSB = 128, kSK = 16;

__global__ void __launch_bounds__(256) mdft_simt_step1(const float* __restrict__ W, const float* __restrict__ A,
                                                       float* __restrict__ T, int K_out, int n, int NB, int lam_base)
{
    // K_out = rows of W_x per (wavelength, part) = Kx
    __shared__ float sWr[kSK][kSB + 4], sWi[kSK][kSB + 4], sA[kSK][kSB + 4];
    const int lam = lam_base + (int)blockIdx.z, mb = blockIdx.y, ib = blockIdx.x;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    const float* Wr = W + ((size_t)(lam * 2 + 0) * K_out + mb * kSB) * n;
    const float* Wi = W + ((size_t)(lam * 2 + 1) * K_out + mb * kSB) * n;
    const float* Ab = A + (size_t)(ib * kSB) * n;
    float cr[8][8] = {}, ci[8][8] = {};
    for (int k0 = 0; k0 < n; k0 += kSK)
    {
        for (int e = threadIdx.x; e < kSB * kSK; e += 256)
        {
            const int r = e / kSK, c = e % kSK;
            sWr[c][r] = Wr[(size_t)r * n + k0 + c];
            sWi[c][r] = Wi[(size_t)r * n + k0 + c];
            sA[c][r] = Ab[(size_t)r * n + k0 + c];
        }
        __syncthreads();
        #pragma unroll
        for (int kk = 0; kk < kSK; ++kk)
        {
            float wr[8], wi[8], a[8];
            #pragma unroll
            for (int q = 0; q < 8; ++q) { wr[q] = sWr[kk][ty * 8 + q]; wi[q] = sWi[kk][ty * 8 + q]; a[q] = sA[kk][tx * 8 + q]; }
            #pragma unroll
            for (int p = 0; p < 8; ++p)
                #pragma unroll
                for (int q = 0; q < 8; ++q) { cr[p][q] += wr[p] * a[q]; ci[p][q] += wi[p] * a[q]; }
        }
        __syncthreads();
    }
    const size_t blk = ((size_t)(lam * NB + mb) * 3) * 128;
    #pragma unroll
    for (int p = 0; p < 8; ++p)
    {
        const int k = ty * 8 + p;
        #pragma unroll
        for (int q = 0; q < 8; ++q)
        {
            const int i = ib * kSB + tx * 8 + q;
            T[(blk + 0 * 128 + k) * n + i] = -ci[p][q];
            T[(blk + 1 * 128 + k) * n + i] = cr[p][q];
            T[(blk + 2 * 128 + k) * n + i] = ci[p][q];
        }
    }
}

__global__ void __launch_bounds__(256) mdft_simt_step2(const float* __restrict__ W, const float* __restrict__ T,
                                                       const float4* __restrict__ weights, float* out_r, float* out_g,
                                                       float* out_b, int K_rows, int K_out, int n, int NB, int lam0, int lam1,
                                                       int box, int out_w, int x0, int y0, int win_w, int win_h,
                                                       float4 tint)
{
    // K_rows = rows of W_y per (wavelength, part) = Ky; K_out = output width Kx
    __shared__ float sWr[kSK][kSB + 4], sWi[kSK][kSB + 4], sTr[kSK][kSB + 4], sTi[kSK][kSB + 4];
    const int mb = blockIdx.y, nb = blockIdx.x;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    for (int lam = lam0; lam < lam1; ++lam)
    {
        const float* Wr = W + ((size_t)(lam * 2 + 0) * K_rows + mb * kSB) * n;
        const float* Wi = W + ((size_t)(lam * 2 + 1) * K_rows + mb * kSB) * n;
        const size_t blk = ((size_t)(lam * NB + nb) * 3) * 128;
        const float* Tr = T + (blk + 128) * n;
        const float* Ti = T + (blk + 256) * n;
        float er[8][8] = {}, ei[8][8] = {};
        for (int k0 = 0; k0 < n; k0 += kSK)
        {
            for (int e = threadIdx.x; e < kSB * kSK; e += 256)
            {
                const int r = e / kSK, c = e % kSK;
                sWr[c][r] = Wr[(size_t)r * n + k0 + c];
                sWi[c][r] = Wi[(size_t)r * n + k0 + c];
                sTr[c][r] = Tr[(size_t)r * n + k0 + c];
                sTi[c][r] = Ti[(size_t)r * n + k0 + c];
            }
            __syncthreads();
            #pragma unroll 4
            for (int kk = 0; kk < kSK; ++kk)
            {
                float wr[8], wi[8], tr[8], ti[8];
                #pragma unroll
                for (int q = 0; q < 8; ++q)
                {
                    wr[q] = sWr[kk][ty * 8 + q]; wi[q] = sWi[kk][ty * 8 + q];
                    tr[q] = sTr[kk][tx * 8 + q]; ti[q] = sTi[kk][tx * 8 + q];
                }
                #pragma unroll
                for (int p = 0; p < 8; ++p)
                    #pragma unroll
                    for (int q = 0; q < 8; ++q)
                    {
                        er[p][q] += wr[p] * tr[q] - wi[p] * ti[q];
                        ei[p][q] += wr[p] * ti[q] + wi[p] * tr[q];
                    }
            }
            __syncthreads();
        }
        // this block owns the tile across wavelengths: plain read-modify-write
        const float4 w0 = weights[lam];
        const float4 w = make_float4(w0.x * tint.x, w0.y * tint.y, w0.z * tint.z, 0.0f);
        #pragma unroll
        for (int p = 0; p < 8; ++p)
        {
            const int l = mb * kSB + ty * 8 + p;
            if (l >= win_h) continue;
            const size_t row = (size_t)(y0 + l) * out_w + x0 + nb * kSB + tx * 8;
            #pragma unroll
            for (int q = 0; q < 8; ++q)
            {
                if (nb * kSB + tx * 8 + q >= win_w) continue;
                const float I = box ? er[p][q] : er[p][q] * er[p][q] + ei[p][q] * ei[p][q];
                out_r[row + q] += w.x * I; out_g[row + q] += w.y * I; out_b[row + q] += w.z * I;
            }
        }
    }
}

}  // namespace

// ---- MDFT plan ----------------------------------------------------------------
constexpr double kMaxCentre = 12288.0;   // pattern centre range (pixels)

struct MdftPlan {
    int n = 0, Kx = 0, Ky = 0, n_lambda = 0, form = 0, Kp = 0, elem = 2;
    void* wx = nullptr;     // W_x' [lam][2][Kx][Kp]
    void* wy = nullptr;     // W_y' [lam][2][Ky][Kp]
    void* mask = nullptr;   // A'   [n][Kp]
    void* tprime = nullptr; // T'   [lam][Kx/128][3][128][Kp]
    float4* weights = nullptr;
    float2* scales = nullptr;   // [2][n_lambda] (s_hi, s_lo) device copy
    double cx = 0.0, cy = 0.0;
    float cj = 0.0f;            // reduction-axis centre: (n - 1) / 2, or the zero lag mc of the box form
    int box = 0;                // pixel-integrated form (the reference's MDFT engine)
    int lam0 = 0, lam1 = -1;    // wavelength range of the next executes (lam1 < 0: all)
    int ctas = 0;               // GEMM grid (0 = one CTA per SM)
    int tile_n = 128;           // step-2 output tile width (complex columns): 128 or 64
    int* err = nullptr;
    CUtensorMap t_wx, t_wy, t_mask, t_tp, t_tp64;
    int sms = 0;
};

static void mdft_free(MdftPlan* p)
{
    if (!p) return;
    cudaFree(p->wx); cudaFree(p->wy); cudaFree(p->mask); cudaFree(p->tprime);
    cudaFree(p->weights); cudaFree(p->scales); cudaFree(p->err);
    delete p;
}

}  // namespace gl

struct gl_mdft_plan { gl::MdftPlan* p; };

namespace gl {

// Enqueue the DFT matrices of the plan's current centre.
static cudaError_t mdft_build_matrices(MdftPlan* p, cudaStream_t st)
{
    const int blocks = 4 * p->sms;
    const float cj = p->cj;
    const int box = p->box;
    const float cxh = (float)p->cx, cxl = (float)(p->cx - (double)cxh);
    const float cyh = (float)p->cy, cyl = (float)(p->cy - (double)cyh);
    if (p->form == 0)
    {
        mdft_dft_kernel<0><<<blocks, 256, 0, st>>>(p->wx, p->n_lambda, p->Kx, p->n, p->Kp, p->scales, cxh, cxl, cj, box);
        mdft_dft_kernel<0><<<blocks, 256, 0, st>>>(p->wy, p->n_lambda, p->Ky, p->n, p->Kp, p->scales + p->n_lambda, cyh,
                                                   cyl, cj, box);
    }
    else
    {
        mdft_dft_kernel<1><<<blocks, 256, 0, st>>>(p->wx, p->n_lambda, p->Kx, p->n, p->Kp, p->scales, cxh, cxl, cj, box);
        mdft_dft_kernel<1><<<blocks, 256, 0, st>>>(p->wy, p->n_lambda, p->Ky, p->n, p->Kp, p->scales + p->n_lambda, cyh,
                                                   cyl, cj, box);
    }
    return cudaGetLastError();
}

}  // namespace gl

extern "C" int gl_mdft_plan_create3(int n, int Kx, int Ky, int n_lambda, const double* scale_x, const double* scale_y,
                                    double center_x, double center_y, const float* weights_rgb, int form, int box,
                                    float red_center, void* stream, gl_mdft_plan** out)
{
    using namespace gl;
    if (!out || !scale_x || !scale_y || !weights_rgb) return fail(GL_ERR_INVALID, "mdft_plan_create: null argument");
    if (box != 0 && box != 1) return fail(GL_ERR_INVALID, "mdft_plan_create: box must be 0 or 1");
    if (!(red_center >= 0.0f) || !(red_center <= (float)n) || red_center != std::floor(2.0f * red_center) * 0.5f)
        return fail(GL_ERR_INVALID, "mdft_plan_create: the reduction centre must be a whole or half index in [0, n]");
    if (n <= 0 || n % 128 || Kx <= 0 || Kx % 128 || Ky <= 0 || Ky % 128)
        return fail(GL_ERR_INVALID, "mdft_plan_create: the pupil side n and output sides Kx, Ky must be multiples of 128");
    if (Kx > 8192 || Ky > 8192 || n > 4096) return fail(GL_ERR_INVALID, "mdft_plan_create: sides above 8192 (4096 for n)");
    if (n_lambda < 1 || n_lambda > 1024) return fail(GL_ERR_INVALID, "mdft_plan_create: 1..1024 wavelengths");
    if (form < 0 || form > 2)
        return fail(GL_ERR_UNSUPPORTED, "mdft_plan_create: form must be 0 (split BF16), 1 (TF32) or 2 (FP32 CUDA cores)");
    // |k - c| < 8192 + 12288 and |j - cj| <= 2048 keep the phase product
    // a (k - c) below 2^26, whose float rounding error the FMA captures exactly
    if (!(std::fabs(center_x) < kMaxCentre) || !(std::fabs(center_y) < kMaxCentre))
        return fail(GL_ERR_INVALID, "mdft_plan_create: centre coordinates must lie within +-12288 pixels");
    cudaStream_t st = (cudaStream_t)stream;
    MdftPlan* p = new MdftPlan();
    p->n = n; p->Kx = Kx; p->Ky = Ky; p->n_lambda = n_lambda; p->form = form;
    p->cx = center_x; p->cy = center_y;
    p->box = box; p->cj = red_center;
    p->Kp = form == 0 ? 3 * n : n;
    p->elem = form == 0 ? 2 : 4;
    const int NBx = Kx / 128;
    const size_t wxbytes = (size_t)n_lambda * 2 * Kx * p->Kp * p->elem;
    const size_t wybytes = (size_t)n_lambda * 2 * Ky * p->Kp * p->elem;
    const size_t mbytes = (size_t)n * p->Kp * p->elem;
    const size_t tbytes = (size_t)n_lambda * NBx * 3 * 128 * p->Kp * p->elem;
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    chk(cudaMalloc(&p->wx, wxbytes));
    chk(cudaMalloc(&p->wy, wybytes));
    chk(cudaMalloc(&p->mask, mbytes));
    chk(cudaMalloc(&p->tprime, tbytes));
    chk(cudaMalloc(&p->weights, sizeof(float4) * n_lambda));
    chk(cudaMalloc(&p->scales, sizeof(float2) * 2 * n_lambda));
    chk(cudaMalloc(&p->err, sizeof(int)));
    chk(cudaMemset(p->err, 0, sizeof(int)));          // a plan never executed reports no error
    int dev = 0;
    chk(cudaGetDevice(&dev));
    chk(cudaDeviceGetAttribute(&p->sms, cudaDevAttrMultiProcessorCount, dev));
    if (e != cudaSuccess)
    {
        mdft_free(p);
        return fail(e == cudaErrorMemoryAllocation ? GL_ERR_OOM : GL_ERR_CUDA, std::string("mdft_plan_create: ") + cudaGetErrorString(e));
    }
    std::vector<float4> w((size_t)n_lambda);
    for (int l = 0; l < n_lambda; ++l) w[l] = make_float4(weights_rgb[3 * l], weights_rgb[3 * l + 1], weights_rgb[3 * l + 2], 0.0f);
    std::vector<float2> sc((size_t)2 * n_lambda);
    for (int l = 0; l < n_lambda; ++l)
    {
        const float xh = (float)scale_x[l], yh = (float)scale_y[l];
        sc[l] = make_float2(xh, (float)(scale_x[l] - (double)xh));
        sc[n_lambda + l] = make_float2(yh, (float)(scale_y[l] - (double)yh));
    }
    chk(cudaMemcpy(p->weights, w.data(), sizeof(float4) * n_lambda, cudaMemcpyHostToDevice));
    chk(cudaMemcpy(p->scales, sc.data(), sizeof(float2) * 2 * n_lambda, cudaMemcpyHostToDevice));
    if (e == cudaSuccess) chk(mdft_build_matrices(p, st));
    chk(cudaStreamSynchronize(st));
    // shared-memory opt-in once here, so execute enqueues kernels only (graph capture)
    {
        const int smem1 = 4 * 3 * kOpTile + 1024, smem2 = 3 * 4 * kOpTile + 1024;
        const int smem2h = 4 * (2 * kOpTile + 2 * 64 * 128) + 1024;
        if (form == 0)
        {
            chk(cudaFuncSetAttribute(mdft_kernel<0, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem1));
            chk(cudaFuncSetAttribute(mdft_kernel<0, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem2));
            chk(cudaFuncSetAttribute(mdft_kernel<0, 2, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem2h));
        }
        else if (form == 1)
        {
            chk(cudaFuncSetAttribute(mdft_kernel<1, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem1));
            chk(cudaFuncSetAttribute(mdft_kernel<1, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem2));
            chk(cudaFuncSetAttribute(mdft_kernel<1, 2, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem2h));
        }
    }
    const CUtensorMapDataType dt = form == 0 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const uint32_t bc = form == 0 ? 64 : 32;
    int rc = GL_OK;
    if (e == cudaSuccess && form != 2)
    {
        rc = make_tmap_2d(&p->t_wx, p->wx, dt, p->elem, (uint64_t)n_lambda * 2 * Kx, (uint64_t)p->Kp, 128, bc);
        if (!rc) rc = make_tmap_2d(&p->t_wy, p->wy, dt, p->elem, (uint64_t)n_lambda * 2 * Ky, (uint64_t)p->Kp, 128, bc);
        if (!rc) rc = make_tmap_2d(&p->t_mask, p->mask, dt, p->elem, (uint64_t)n, (uint64_t)p->Kp, 128, bc);
        if (!rc) rc = make_tmap_2d(&p->t_tp, p->tprime, dt, p->elem, (uint64_t)n_lambda * NBx * 3 * 128, (uint64_t)p->Kp, 128, bc);
        if (!rc) rc = make_tmap_2d(&p->t_tp64, p->tprime, dt, p->elem, (uint64_t)n_lambda * NBx * 3 * 128, (uint64_t)p->Kp, 64, bc);
    }
    if (e != cudaSuccess || rc)
    {
        mdft_free(p);
        if (rc) return rc;
        return fail(GL_ERR_CUDA, std::string("mdft_plan_create: ") + cudaGetErrorString(e));
    }
    *out = new gl_mdft_plan{p};
    return GL_OK;
}

extern "C" int gl_mdft_plan_create2(int n, int Kx, int Ky, int n_lambda, const double* scale_x, const double* scale_y,
                                    double center_x, double center_y, const float* weights_rgb, int form, void* stream,
                                    gl_mdft_plan** out)
{
    return gl_mdft_plan_create3(n, Kx, Ky, n_lambda, scale_x, scale_y, center_x, center_y, weights_rgb, form, 0,
                                0.5f * (float)(n - 1), stream, out);
}

extern "C" int gl_mdft_plan_create(int n, int K_out, int n_lambda, const double* scale_x, const double* scale_y,
                                   double center_x, double center_y, const float* weights_rgb, int form,
                                   void* stream, gl_mdft_plan** out)
{
    return gl_mdft_plan_create2(n, K_out, K_out, n_lambda, scale_x, scale_y, center_x, center_y, weights_rgb, form,
                                stream, out);
}

extern "C" int gl_mdft_plan_set_center(gl_mdft_plan* plan, double center_x, double center_y, void* stream)
{
    using namespace gl;
    if (!plan) return fail(GL_ERR_INVALID, "mdft_plan_set_center: null plan");
    if (!(std::fabs(center_x) < kMaxCentre) || !(std::fabs(center_y) < kMaxCentre))
        return fail(GL_ERR_INVALID, "mdft_plan_set_center: centre coordinates must lie within +-12288 pixels");
    plan->p->cx = center_x;
    plan->p->cy = center_y;
    GL_CUDA_TRY(mdft_build_matrices(plan->p, (cudaStream_t)stream));
    g_last_launches = 2;
    return GL_OK;
}

extern "C" int gl_mdft_plan_execute3(gl_mdft_plan* plan, const float* d_pupil, float* d_out_r, float* d_out_g,
                                     float* d_out_b, int accumulate, int out_w, int out_h, int x0, int y0, int win_w,
                                     int win_h, const float* tint_rgb, void* stream)
{
    using namespace gl;
    if (!plan || !d_pupil || !d_out_r || !d_out_g || !d_out_b) return fail(GL_ERR_INVALID, "mdft_plan_execute: null argument");
    MdftPlan* p = plan->p;
    if (out_w <= 0 || out_h <= 0 || x0 < 0 || y0 < 0 || win_w < 0 || win_h < 0 || win_w > p->Kx || win_h > p->Ky ||
        x0 + win_w > out_w || y0 + win_h > out_h)
        return fail(GL_ERR_INVALID, "mdft_plan_execute: the output window must lie inside the planes and the plan");
    cudaStream_t st = (cudaStream_t)stream;
    const int NBx = p->Kx / 128, NBy = p->Ky / 128, NI = p->n / 128;
    const size_t npx = (size_t)out_w * out_h;
    int launches = 0;
    GL_CUDA_TRY(cudaMemsetAsync(p->err, 0, sizeof(int), st));
    if (p->form == 0) mdft_mask_kernel<0><<<2 * p->sms, 256, 0, st>>>(d_pupil, p->mask, p->n, p->Kp);
    else mdft_mask_kernel<1><<<2 * p->sms, 256, 0, st>>>(d_pupil, p->mask, p->n, p->Kp);
    ++launches;
    if (!accumulate)
    {
        GL_CUDA_TRY(cudaMemsetAsync(d_out_r, 0, npx * sizeof(float), st));
        GL_CUDA_TRY(cudaMemsetAsync(d_out_g, 0, npx * sizeof(float), st));
        GL_CUDA_TRY(cudaMemsetAsync(d_out_b, 0, npx * sizeof(float), st));
    }
    MdftArgs a;
    a.NBt = NBx;
    a.KA = p->Kx; a.Kx = p->Kx; a.NBm = NBx;
    a.n = p->n; a.n_lambda = p->n_lambda; a.Kp = p->Kp;
    a.nkb = p->Kp / (p->form == 0 ? 64 : 32);
    a.NB = NBx; a.NI = NI;
    a.tprime = p->tprime; a.out_r = d_out_r; a.out_g = d_out_g; a.out_b = d_out_b;
    a.weights = p->weights; a.err = p->err;
    a.out_w = out_w; a.x0 = x0; a.y0 = y0; a.win_w = win_w; a.win_h = win_h; a.box = p->box;
    a.tint = tint_rgb ? make_float4(tint_rgb[0], tint_rgb[1], tint_rgb[2], 0.0f) : make_float4(1.0f, 1.0f, 1.0f, 0.0f);
    const size_t smem1 = 4 * 3 * (size_t)kOpTile + 1024, smem2 = 3 * 4 * (size_t)kOpTile + 1024;
    const int l0 = p->lam0, l1 = p->lam1 < 0 ? p->n_lambda : p->lam1, nl = l1 - l0;
    a.lam_base = l0;
    a.n_units = nl * NBx * NI;                          // step 1: (lambda, k block, pupil-row block)
    const int gmax = p->ctas > 0 ? p->ctas : p->sms;
    const int g1 = std::min(a.n_units, gmax);
    MdftArgs a2 = a;
    a2.KA = p->Ky; a2.NBm = NBy;
    const bool half = p->tile_n == 64;
    a2.NBt = p->Kx / p->tile_n;
    a2.n_units = NBy * a2.NBt * nl;                     // step 2: (lambda, output tile)
    const int g2 = std::min(a2.n_units, gmax);
    const size_t smem2h = 4 * (2 * (size_t)kOpTile + 2 * 64 * 128) + 1024;
    if (p->form == 2)
    {
        mdft_simt_step1<<<dim3(NI, NBx, nl), 256, 0, st>>>(static_cast<const float*>(p->wx),
                                                           static_cast<const float*>(p->mask),
                                                           static_cast<float*>(p->tprime), p->Kx, p->n, NBx, l0);
        mdft_simt_step2<<<dim3(NBx, NBy), 256, 0, st>>>(static_cast<const float*>(p->wy), static_cast<const float*>(p->tprime),
                                                       p->weights, d_out_r, d_out_g, d_out_b, p->Ky, p->Kx, p->n, NBx,
                                                       l0, l1, p->box, out_w, x0, y0, win_w, win_h, a.tint);
    }
    else if (p->form == 0)
    {
        mdft_kernel<0, 1><<<g1, kMdftThreads, smem1, st>>>(p->t_wx, p->t_mask, a);
        if (half) mdft_kernel<0, 2, 64><<<g2, kMdftThreads, smem2h, st>>>(p->t_wy, p->t_tp64, a2);
        else mdft_kernel<0, 2><<<g2, kMdftThreads, smem2, st>>>(p->t_wy, p->t_tp, a2);
    }
    else
    {
        mdft_kernel<1, 1><<<g1, kMdftThreads, smem1, st>>>(p->t_wx, p->t_mask, a);
        if (half) mdft_kernel<1, 2, 64><<<g2, kMdftThreads, smem2h, st>>>(p->t_wy, p->t_tp64, a2);
        else mdft_kernel<1, 2><<<g2, kMdftThreads, smem2, st>>>(p->t_wy, p->t_tp, a2);
    }
    GL_CUDA_TRY(cudaGetLastError());
    launches += 2;
    g_last_launches = launches;
    return GL_OK;
}

extern "C" int gl_mdft_plan_execute2(gl_mdft_plan* plan, const float* d_pupil, float* d_out_r, float* d_out_g,
                                     float* d_out_b, int accumulate, void* stream)
{
    if (!plan) return gl::fail(GL_ERR_INVALID, "mdft_plan_execute: null argument");
    const gl::MdftPlan* p = plan->p;
    return gl_mdft_plan_execute3(plan, d_pupil, d_out_r, d_out_g, d_out_b, accumulate, p->Kx, p->Ky, 0, 0, p->Kx, p->Ky,
                                 nullptr, stream);
}

extern "C" int gl_mdft_plan_set_lambda_range(gl_mdft_plan* plan, int lam_begin, int lam_end)
{
    using namespace gl;
    if (!plan) return fail(GL_ERR_INVALID, "mdft_plan_set_lambda_range: null plan");
    MdftPlan* p = plan->p;
    if (lam_begin == 0 && lam_end < 0) { p->lam0 = 0; p->lam1 = -1; return GL_OK; }
    if (lam_begin < 0 || lam_end <= lam_begin || lam_end > p->n_lambda)
        return fail(GL_ERR_INVALID, "mdft_plan_set_lambda_range: need 0 <= begin < end <= n_lambda");
    p->lam0 = lam_begin;
    p->lam1 = lam_end;
    return GL_OK;
}

extern "C" int gl_mdft_plan_set_launch(gl_mdft_plan* plan, int ctas)
{
    using namespace gl;
    if (!plan || ctas < 0) return fail(GL_ERR_INVALID, "mdft_plan_set_launch: bad arguments");
    // one 192-thread CTA with ~161 KB of shared memory fits per SM
    plan->p->ctas = ctas == 0 ? 0 : std::min(ctas, plan->p->sms);
    return GL_OK;
}

extern "C" int gl_mdft_plan_set_tile(gl_mdft_plan* plan, int tile_n)
{
    using namespace gl;
    if (!plan || (tile_n != 64 && tile_n != 128))
        return fail(GL_ERR_INVALID, "mdft_plan_set_tile: the tile width must be 64 or 128 output columns");
    plan->p->tile_n = tile_n;
    return GL_OK;
}

extern "C" int gl_mdft_plan_execute(gl_mdft_plan* plan, const float* d_pupil, float* d_out_r, float* d_out_g,
                                    float* d_out_b, void* stream)
{
    return gl_mdft_plan_execute2(plan, d_pupil, d_out_r, d_out_g, d_out_b, 0, stream);
}

extern "C" int gl_build_pupil2(const gl_surface* surfaces, int n_surfaces, int N, float pupil_fill,
                               int blades_override, float rotation_deg, int aspect_one, const float* d_env, int env_n,
                               float* d_out, void* stream)
{
    using namespace gl;
    if (!surfaces || n_surfaces <= 0 || !d_out) return fail(GL_ERR_INVALID, "build_pupil: bad arguments");
    if (N <= 0 || N > 8192) return fail(GL_ERR_INVALID, "build_pupil: N must be 1..8192");
    if (!(pupil_fill > 0.0f) || pupil_fill > 1.0f) return fail(GL_ERR_INVALID, "build_pupil: pupil_fill must lie in (0, 1]");
    if (d_env && (env_n < 1 || env_n > 4096)) return fail(GL_ERR_INVALID, "build_pupil: envelope side must be 1..4096");
    PupilMask m = resolve_pupil_mask(surfaces, n_surfaces, blades_override, rotation_deg);
    if (aspect_one) m.aspect = 1.0f;
    PupilDev d{m.aspect, m.rot_rad, m.apothem, m.sector, m.n_blades, m.blade};
    const int total = N * N;
    pupil_build_kernel<<<(total + 255) / 256, 256, 0, (cudaStream_t)stream>>>(d_out, N, pupil_fill, d, d_env, env_n);
    GL_CUDA_TRY(cudaGetLastError());
    g_last_launches = 1;
    return GL_OK;
}

extern "C" int gl_build_pupil(const gl_surface* surfaces, int n_surfaces, int N, float pupil_fill,
                              int blades_override, float rotation_deg, float* d_out, void* stream)
{
    return gl_build_pupil2(surfaces, n_surfaces, N, pupil_fill, blades_override, rotation_deg, 0, nullptr, 0, d_out,
                           stream);
}

extern "C" int gl_mdft_plan_status(gl_mdft_plan* plan, int* err_code)
{
    if (!plan || !err_code) return gl::fail(GL_ERR_INVALID, "mdft_plan_status: null argument");
    GL_CUDA_TRY(cudaMemcpy(err_code, plan->p->err, sizeof(int), cudaMemcpyDeviceToHost));
    return GL_OK;
}

extern "C" int gl_mdft_plan_destroy(gl_mdft_plan* plan)
{
    if (!plan) return GL_OK;
    gl::mdft_free(plan->p);
    delete plan;
    return GL_OK;
}
