// gl_mdft.cu — tensor-core matrix products for the matrix-DFT starburst.
//
// This unit holds the tcgen05 machinery shared by the MDFT forms: TMA tensor
// maps built on the host, a warp-specialised CTA (one TMA producer thread,
// one MMA-issuing thread, four epilogue warps reading TMEM) and the plain
// BF16 GEMM C = A * B^T that pins the descriptors against torch.
#include "gl_internal.h"
#include "gl_tc.cuh"

#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
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
