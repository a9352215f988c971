// BF16 GEMM on the 5th-generation tensor cores: C[M][N] (FP32) =
// A[M][K] * B[N][K]^T, both operands K-major. The building block of the
// many-beam beamformer, exported on its own (vgb_gemm_bf16) so it can be
// tested and measured against cuBLAS-free references.
//
// One CTA (4 warps) computes a 128 x 128 tile: warp 0 lane 0 streams 64-wide
// K chunks of A and B through a 4-stage ring with 2-D TMA loads
// (SWIZZLE_128B), warp 1 lane 0 issues four 128x128x16 tcgen05 MMAs per chunk
// into an FP32 accumulator in tensor memory and releases each stage with
// tcgen05.commit, and all four warps read the accumulator back with
// tcgen05.ld for the epilogue. Every wait is bounded; on expiry the CTA flags
// the device status word, frees its tensor memory and returns.
#include <cudaTypedefs.h>

#include "tcgen05.cuh"
#include "vgb_launch.cuh"

namespace vgb {

constexpr int kGemmStages = 4;
constexpr int kTileBytes = 128 * 64 * 2; // one 128-row x 64-column bf16 tile
constexpr uint32_t kWaitPolls = 1u << 24;

struct GemmSmem {
    uint8_t a[kGemmStages][kTileBytes];
    uint8_t b[kGemmStages][kTileBytes];
    uint64_t full[kGemmStages];
    uint64_t empty[kGemmStages];
    uint64_t done;
    uint32_t tmem;
};

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

int make_tmap_bf16(CUtensorMap *map, const void *base, uint64_t rows, uint64_t cols, uint64_t row_bytes,
                   uint32_t box_rows)
{
    auto fn = encode_fn();
    if (!fn) return set_error(VGB_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    if ((reinterpret_cast<uintptr_t>(base) & 15) || (row_bytes & 15) || cols % 64 || box_rows == 0 ||
        box_rows > 256)
        return set_error(VGB_ERR_INVALID, "tensor map: base/stride must be 16-byte aligned, cols a multiple of 64");
    cuuint64_t dims[2] = {cols, rows};
    cuuint64_t strides[1] = {row_bytes};
    cuuint32_t box[2] = {64, box_rows};
    cuuint32_t estr[2] = {1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(VGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return VGB_SUCCESS;
}

__global__ void __launch_bounds__(128, 1)
    gemm_bf16_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, float *C,
                     int N, int K, unsigned *status)
{
    extern __shared__ uint8_t gemm_raw[];
    GemmSmem &sm = *reinterpret_cast<GemmSmem *>((reinterpret_cast<uintptr_t>(gemm_raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * 128, n0 = blockIdx.x * 128;
    const int nk = K / 64;

    if (threadIdx.x == 0) {
        prefetch_tmap(&ta);
        prefetch_tmap(&tb);
        for (int s = 0; s < kGemmStages; s++) {
            mbar_init(&sm.full[s], 1);
            mbar_init(&sm.empty[s], 1);
        }
        mbar_init(&sm.done, 1);
        fence_mbar_init();
    }
    __syncwarp();
    if (warp == 0) {
        tmem_alloc(&sm.tmem, 128);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sm.tmem;

    int issued = 0; // producer: chunks whose loads were issued
    if (warp == 0 && lane == 0) {
        for (int kc = 0; kc < nk; kc++) {
            const int s = kc % kGemmStages;
            if (kc >= kGemmStages &&
                !mbar_wait_bounded(&sm.empty[s], ((kc / kGemmStages) - 1) & 1, kWaitPolls)) {
                atomicOr(status, kErrWaitTimeout);
                break;
            }
            mbar_arrive_expect_tx(&sm.full[s], 2 * kTileBytes);
            tma_load_2d(sm.a[s], &ta, kc * 64, m0, &sm.full[s]);
            tma_load_2d(sm.b[s], &tb, kc * 64, n0, &sm.full[s]);
            issued++;
        }
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_bf16_f32(128);
        for (int kc = 0; kc < nk; kc++) {
            const int s = kc % kGemmStages;
            if (!mbar_wait_bounded(&sm.full[s], (kc / kGemmStages) & 1, kWaitPolls)) {
                atomicOr(status, kErrWaitTimeout);
                break;
            }
            tc_fence_after();
            const uint64_t ad = sdesc_sw128(smem_u32(sm.a[s])), bd = sdesc_sw128(smem_u32(sm.b[s]));
#pragma unroll
            for (int k = 0; k < 4; k++)
                tc_mma(tmem, sdesc_advance_k(ad, k), sdesc_advance_k(bd, k), idesc, (kc | k) != 0);
            tc_commit(&sm.empty[s]);
        }
        tc_commit(&sm.done);
    }
    __syncwarp();

    // epilogue: warp w owns rows 32w..32w+31 of the tile
    const bool done = mbar_wait_bounded(&sm.done, 0, kWaitPolls);
    tc_fence_after();
    if (done) {
        const int row = m0 + warp * 32 + lane;
#pragma unroll
        for (int c = 0; c < 4; c++) {
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + c * 32, v);
            float4 *out = reinterpret_cast<float4 *>(C + (long long)row * N + n0 + c * 32);
#pragma unroll
            for (int j = 0; j < 8; j++) out[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
        }
    } else if (lane == 0) {
        atomicOr(status, kErrWaitTimeout);
    }
    // loads the producer issued must have landed before the CTA leaves
    if (warp == 0 && lane == 0) {
        for (int kc = (issued > kGemmStages ? issued - kGemmStages : 0); kc < issued; kc++)
            mbar_wait_bounded(&sm.full[kc % kGemmStages], (kc / kGemmStages) & 1, kWaitPolls);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 128);
}

} // namespace vgb

using namespace vgb;

extern "C" int vgb_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K, void *stream)
{
    if (!A || !B || !C) return set_error(VGB_ERR_INVALID, "gemm: NULL operand");
    if (M <= 0 || N <= 0 || K <= 0 || M % 128 || N % 128 || K % 64)
        return set_error(VGB_ERR_INVALID, "gemm: M and N must be multiples of 128 and K of 64 (got %d, %d, %d)", M, N,
                         K);
    if ((reinterpret_cast<uintptr_t>(C) & 15)) return set_error(VGB_ERR_INVALID, "gemm: C must be 16-byte aligned");
    CUtensorMap ta, tb;
    int rc = make_tmap_bf16(&ta, A, M, K, (uint64_t)K * 2, 128);
    if (rc) return rc;
    if ((rc = make_tmap_bf16(&tb, B, N, K, (uint64_t)K * 2, 128))) return rc;
    unsigned *status = status_word();
    if (!status) return set_error(VGB_ERR_CUDA, "device status word unavailable");
    const int smem = (int)sizeof(GemmSmem) + 1024;
    if ((rc = check_cuda(cudaFuncSetAttribute(gemm_bf16_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                         "cudaFuncSetAttribute(gemm)")))
        return rc;
    dim3 grid(N / 128, M / 128);
    gemm_bf16_kernel<<<grid, 128, smem, static_cast<cudaStream_t>(stream)>>>(ta, tb, C, N, K, status);
    return check_launch("gemm_bf16_kernel");
}
