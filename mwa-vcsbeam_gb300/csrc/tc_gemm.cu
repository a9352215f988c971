// BF16 GEMM on the 5th-generation tensor cores: C[M][N] (FP32) =
// A[M][K] * B[N][K]^T, both operands K-major. The building block of the
// many-beam beamformer, exported on its own (vgb_gemm_bf16) so it can be
// tested and measured against cuBLAS-free references.
//
// One CTA (4 warps) computes a 128 x BN tile (BN = 128 or 256): warp 0 lane 0
// streams 64-wide K chunks of A and B through a 4-stage ring with 2-D TMA loads
// (SWIZZLE_128B), warp 1 lane 0 issues four 128xBNx16 tcgen05 MMAs per chunk
// into an FP32 accumulator in tensor memory and releases each stage with
// tcgen05.commit, and all four warps read the accumulator back with
// tcgen05.ld for the epilogue. Every wait is bounded; on expiry the CTA flags
// the device status word, frees its tensor memory and returns.
#include <cudaTypedefs.h>

#include <atomic>
#include <map>
#include <mutex>
#include <tuple>

#include "tcgen05.cuh"
#include "vgb_launch.cuh"

namespace vgb {

constexpr int kGemmStages = 4;
constexpr int kTileBytes = 128 * 64 * 2; // one 128-row x 64-column bf16 tile
constexpr uint32_t kWaitPolls = 1u << 24;

template <int BN>
struct GemmSmem {
    uint8_t a[kGemmStages][kTileBytes];
    uint8_t b[kGemmStages][BN * 128];
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
                   uint32_t box_rows, bool fp16)
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
    CUresult r = fn(map, fp16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(base), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(VGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return VGB_SUCCESS;
}

int make_tmap_beam_weights(CUtensorMap *map, const void *W, int nant, int ncc, long long W_cc, int tiles_per_box)
{
    auto fn = encode_fn();
    if (!fn) return set_error(VGB_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    if ((reinterpret_cast<uintptr_t>(W) & 15) || nant <= 0 || ncc <= 0 || W_cc < (long long)nant * kK * 2 ||
        tiles_per_box <= 0 || tiles_per_box > 256)
        return set_error(VGB_ERR_INVALID, "weight tensor map: bad base, sizes or stride");
    // [cc][ant][k][row][4 floats], innermost first
    cuuint64_t dims[5] = {4, 2, (cuuint64_t)kK, (cuuint64_t)nant, (cuuint64_t)ncc};
    cuuint64_t strides[4] = {16, 32, (cuuint64_t)kK * 32, (cuuint64_t)W_cc * 16};
    cuuint32_t box[5] = {4, 1, (cuuint32_t)kK, (cuuint32_t)tiles_per_box, 1};
    cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 5, const_cast<void *>(W), dims, strides, box, estr,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return set_error(VGB_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return VGB_SUCCESS;
}

template <bool kF16, int BN>
__global__ void __launch_bounds__(128, 1)
    gemm_bf16_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, float *C,
                     int M, int N, int K, int Kb, unsigned *status)
{
    extern __shared__ uint8_t gemm_raw[];
    GemmSmem<BN> &sm =
        *reinterpret_cast<GemmSmem<BN> *>((reinterpret_cast<uintptr_t>(gemm_raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * 128, n0 = blockIdx.x * BN;
    const int batch = blockIdx.z; // A rows batch*M.., B rows batch*N.., C batch*M*N..
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
        tmem_alloc(&sm.tmem, BN);
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
            mbar_arrive_expect_tx(&sm.full[s], kTileBytes + BN * 128);
            tma_load_2d(sm.a[s], &ta, kc * 64, batch * M + m0, &sm.full[s]);
            tma_load_2d(sm.b[s], &tb, (kc * 64) % Kb, batch * N + n0, &sm.full[s]);
            issued++;
        }
    } else if (warp == 1 && lane == 0) {
        const uint32_t idesc = idesc_bf16_f32(BN, false, kF16);
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
        for (int c = 0; c < BN / 32; c++) {
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + c * 32, v);
            float4 *out =
                reinterpret_cast<float4 *>(C + ((long long)batch * M + row) * N + n0 + c * 32);
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
    if (warp == 0) tmem_dealloc(tmem, BN);
}


// ---------------------------------------------------------------------------
// Persistent form: one 192-thread CTA per SM walks the (batch, n, m) tiles of
// 128 x 256; warp 0 streams K chunks through a 4-stage TMA ring, warp 1 issues
// the MMAs into one of two 256-column TMEM accumulators, warps 2-5 (TMEM lane
// quarter = warp % 4) store the other one, so a tile's epilogue overlaps the
// next tile's MMAs. Same operands, K order and results as gemm_bf16_kernel.
// ---------------------------------------------------------------------------
constexpr int kPStages = 4;
// kA A planes per K step (2: the A rows hold two K-wide halves, e.g. the hi
// and lo parts of a split operand, both multiplied by the same B tile); the
// ring keeps 192 KB either way.
template <int kA> struct PersistSmem {
    static constexpr int kStages = kA == 2 ? 3 : kPStages;
    uint8_t a[kStages][kA][kTileBytes];
    uint8_t b[kStages][256 * 128];
    float epi[4][32][33];                  // epilogue: each warp's 32 x 32 block, transposed for row-contiguous stores
    uint64_t full[kStages], empty[kStages];
    uint64_t tfull[2], tempty[2], drain;
    uint32_t tmem;
};

template <bool kF16, int kA>
__global__ void __launch_bounds__(192, 1)
    gemm_persist_kernel(const __grid_constant__ CUtensorMap ta, const __grid_constant__ CUtensorMap tb, float *C,
                        int M, int N, int K, int Kb, int batch, unsigned *status)
{
    constexpr int kPStages = PersistSmem<kA>::kStages;
    extern __shared__ uint8_t pg_raw[];
    PersistSmem<kA> &sm =
        *reinterpret_cast<PersistSmem<kA> *>((reinterpret_cast<uintptr_t>(pg_raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int mt = M / 128, ntile = N / 256, nk = K / 64;
    const long long total = (long long)batch * ntile * mt;

    if (threadIdx.x == 0) {
        prefetch_tmap(&ta);
        prefetch_tmap(&tb);
        for (int s = 0; s < kPStages; s++) {
            mbar_init(&sm.full[s], 1);
            mbar_init(&sm.empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&sm.tfull[b], 1);
            mbar_init(&sm.tempty[b], 4);
        }
        mbar_init(&sm.drain, 1);
        fence_mbar_init();
    }
    __syncwarp();
    if (warp == 0) {
        tmem_alloc(&sm.tmem, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sm.tmem;

    if (warp == 0) {
        if (lane == 0) {
            uint32_t it = 0;
            bool ok = true;
            for (long long t = blockIdx.x; t < total && ok; t += gridDim.x) {
                const int m = (int)(t % mt), n = (int)((t / mt) % ntile), b = (int)(t / ((long long)mt * ntile));
                for (int kc = 0; kc < nk; kc++, it++) {
                    const int s = it % kPStages;
                    const uint32_t r = it / kPStages;
                    if (r > 0 && !mbar_wait_bounded(&sm.empty[s], (r - 1) & 1, kWaitPolls)) {
                        atomicOr(status, kErrWaitTimeout);
                        ok = false;
                        break;
                    }
                    mbar_arrive_expect_tx(&sm.full[s], kA * kTileBytes + 256 * 128);
                    tma_load_2d(sm.a[s][0], &ta, kc * 64, b * M + m * 128, &sm.full[s]);
                    if (kA == 2) tma_load_2d(sm.a[s][1], &ta, K + kc * 64, b * M + m * 128, &sm.full[s]);
                    tma_load_2d(sm.b[s], &tb, (kc * 64) % Kb, b * N + n * 256, &sm.full[s]);
                }
            }
            for (uint32_t k = (it > kPStages ? it - kPStages : 0); k < it; k++)
                mbar_wait_bounded(&sm.full[k % kPStages], (k / kPStages) & 1, kWaitPolls);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16_f32(256, false, kF16);
            uint32_t it = 0, tc = 0;
            bool ok = true;
            for (long long t = blockIdx.x; t < total && ok; t += gridDim.x, tc++) {
                const int buf = tc & 1;
                const uint32_t u = tc >> 1;
                if (u > 0 && !mbar_wait_bounded(&sm.tempty[buf], (u - 1) & 1, kWaitPolls)) {
                    atomicOr(status, kErrWaitTimeout);
                    break;
                }
                tc_fence_after();
                const uint32_t d = tmem + buf * 256;
                for (int kc = 0; kc < nk; kc++, it++) {
                    const int s = it % kPStages;
                    if (!mbar_wait_bounded(&sm.full[s], (it / kPStages) & 1, kWaitPolls)) {
                        atomicOr(status, kErrWaitTimeout);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint64_t ad = sdesc_sw128(smem_u32(sm.a[s][0])), bd = sdesc_sw128(smem_u32(sm.b[s]));
                    const uint64_t ad1 = sdesc_sw128(smem_u32(sm.a[s][kA - 1]));
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        tc_mma(d, sdesc_advance_k(ad, k), sdesc_advance_k(bd, k), idesc, (kc | k) != 0);
                        if (kA == 2) tc_mma(d, sdesc_advance_k(ad1, k), sdesc_advance_k(bd, k), idesc, 1);
                    }
                    tc_commit(&sm.empty[s]);
                }
                if (ok) tc_commit(&sm.tfull[buf]);
            }
            tc_commit(&sm.drain);
            mbar_wait_bounded(&sm.drain, 0, kWaitPolls);
        }
    } else {
        const int q4 = warp & 3;
        uint32_t tc = 0;
        for (long long t = blockIdx.x; t < total; t += gridDim.x, tc++) {
            const int buf = tc & 1;
            const int m = (int)(t % mt), n = (int)((t / mt) % ntile), b = (int)(t / ((long long)mt * ntile));
            if (!mbar_wait_bounded(&sm.tfull[buf], (tc >> 1) & 1, kWaitPolls)) {
                if (lane == 0) atomicOr(status, kErrWaitTimeout);
                break;
            }
            tc_fence_after();
            // this warp's 32 rows: each 32-column block goes through shared
            // memory so that a store instruction writes 128 contiguous bytes of one row
            float *out = C + ((long long)b * M + m * 128 + q4 * 32) * N + n * 256;
            float(*stg)[33] = sm.epi[q4];
#pragma unroll 1
            for (int c = 0; c < 8; c++) {
                float v[32];
                tmem_ld32(tmem + ((uint32_t)(q4 * 32) << 16) + buf * 256 + c * 32, v);
#pragma unroll
                for (int j = 0; j < 32; j++) stg[lane][j] = v[j];
                __syncwarp();
#pragma unroll 8
                for (int r = 0; r < 32; r++) out[(long long)r * N + c * 32 + lane] = stg[r][lane];
                __syncwarp();
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&sm.tempty[buf]);
        }
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

} // namespace vgb

using namespace vgb;

namespace vgb {

// Kernel variant for a GEMM shape: the plain kernel with 128- or 256-wide
// tiles, or the persistent kernel (256-wide tiles, overlapped epilogue),
// chosen by timing each on the first call with that shape (3 runs each with
// CUDA events on the caller's stream, after one warm-up) and cached; all give
// identical results (same K order per output). While a stream is being
// captured into a graph the measured choice is used if known, else 256.
static std::atomic<int> g_gemm_variant{0}; // 0: autotuned; else forced (128, 256, 512)

template <class Launch>
int gemm_tile_width(int M, int N, int K, int Kb, int batch, bool fp16, cudaStream_t st, Launch &launch)
{
    if (N % 256) return 128;
    if (const int forced = g_gemm_variant.load()) return forced;
    static std::mutex mu;
    static std::map<std::tuple<int, int, int, int, int, bool>, int> cache;
    const auto key = std::make_tuple(M, N, K, Kb, batch, fp16);
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it != cache.end()) return it->second;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
        cudaGetLastError();
        return 256;
    }
    float best_ms = 0.f;
    int best = 256;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess) return 256;
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return 256;
    }
    for (int bn : {256, 128, 512}) {
        if (launch(bn)) break;
        cudaEventRecord(e0, st);
        for (int i = 0; i < 3; i++) launch(bn);
        cudaEventRecord(e1, st);
        float ms = 0.f;
        if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) break;
        if (bn == 256 || ms < best_ms) {
            best_ms = ms;
            best = bn;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaGetLastError();
    std::lock_guard<std::mutex> lk(mu);
    cache[key] = best;
    return best;
}

// C[b] = A[b] B[b]^T for b < batch: A rows b*M.., B rows b*N.., C rows b*M.. of
// contiguous row-major operands (bf16, or fp16 with `fp16`). B may be
// narrower than A along K (Kb columns, a multiple of 64): column k of A meets
// column k mod Kb of B, i.e. B is read as [B | B | ...] cut to K columns.
int gemm_batched(const void *A, const void *B, float *C, int M, int N, int K, int batch, bool fp16,
                 cudaStream_t st, int Kb)
{
    if (!A || !B || !C) return set_error(VGB_ERR_INVALID, "gemm: NULL operand");
    if (Kb <= 0) Kb = K;
    if (M <= 0 || N <= 0 || K <= 0 || batch <= 0 || M % 128 || N % 128 || K % 64 || Kb % 64)
        return set_error(VGB_ERR_INVALID, "gemm: M and N must be multiples of 128 and K of 64 (got %d, %d, %d)", M, N,
                         K);
    if ((reinterpret_cast<uintptr_t>(C) & 15)) return set_error(VGB_ERR_INVALID, "gemm: C must be 16-byte aligned");
    unsigned *status = status_word();
    if (!status) return set_error(VGB_ERR_CUDA, "device status word unavailable");
    auto launch = [&](int bn) -> int {
        // bn: 128 or 256 = the plain kernel's tile width; 512 = the persistent kernel (256-wide tiles)
        CUtensorMap ta, tb;
        int r = make_tmap_bf16(&ta, A, (uint64_t)M * batch, K, (uint64_t)K * 2, 128, fp16);
        if (!r) r = make_tmap_bf16(&tb, B, (uint64_t)N * batch, Kb, (uint64_t)Kb * 2, bn == 128 ? 128 : 256, fp16);
        if (r) return r;
        if (bn == 512) {
            static int nsm = 0;
            if (!nsm) {
                int dev = 0;
                cudaGetDevice(&dev);
                cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
                if (nsm <= 0) nsm = 1;
            }
            const long long tiles = (long long)batch * (N / 256) * (M / 128);
            const int grid = (int)(tiles < nsm ? tiles : nsm);
            const int smem = (int)sizeof(PersistSmem<1>) + 1024;
            auto kern = fp16 ? gemm_persist_kernel<true, 1> : gemm_persist_kernel<false, 1>;
            int e = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                               "cudaFuncSetAttribute(gemm_persist)");
            if (!e) kern<<<grid, 192, smem, st>>>(ta, tb, C, M, N, K, Kb, batch, status);
            return e ? e : check_launch("gemm_persist_kernel");
        }
        dim3 grid(N / bn, M / 128, batch);
        auto go = [&](auto kern, int smem) {
            int e = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                               "cudaFuncSetAttribute(gemm)");
            if (!e) kern<<<grid, 128, smem, st>>>(ta, tb, C, M, N, K, Kb, status);
            return e ? e : check_launch("gemm_bf16_kernel");
        };
        if (fp16)
            return bn == 256 ? go(gemm_bf16_kernel<true, 256>, (int)sizeof(GemmSmem<256>) + 1024)
                             : go(gemm_bf16_kernel<true, 128>, (int)sizeof(GemmSmem<128>) + 1024);
        return bn == 256 ? go(gemm_bf16_kernel<false, 256>, (int)sizeof(GemmSmem<256>) + 1024)
                         : go(gemm_bf16_kernel<false, 128>, (int)sizeof(GemmSmem<128>) + 1024);
    };
    return launch(gemm_tile_width(M, N, K, Kb, batch, fp16, st, launch));
}

int gemm_batched_planes(const void *A, const void *B, float *C, int M, int N, int K, int batch, bool fp16,
                        cudaStream_t st)
{
    if (!A || !B || !C) return set_error(VGB_ERR_INVALID, "gemm: NULL operand");
    if (M <= 0 || N <= 0 || K <= 0 || batch <= 0 || M % 128 || N % 256 || K % 64)
        return set_error(VGB_ERR_INVALID, "gemm (two A planes): M must be a multiple of 128, N of 256, K of 64 "
                                          "(got %d, %d, %d)", M, N, K);
    if ((reinterpret_cast<uintptr_t>(C) & 15)) return set_error(VGB_ERR_INVALID, "gemm: C must be 16-byte aligned");
    unsigned *status = status_word();
    if (!status) return set_error(VGB_ERR_CUDA, "device status word unavailable");
    CUtensorMap ta, tb;
    int r = make_tmap_bf16(&ta, A, (uint64_t)M * batch, 2 * K, (uint64_t)K * 4, 128, fp16);
    if (!r) r = make_tmap_bf16(&tb, B, (uint64_t)N * batch, K, (uint64_t)K * 2, 256, fp16);
    if (r) return r;
    static int nsm = 0;
    if (!nsm) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
        if (nsm <= 0) nsm = 1;
    }
    const long long tiles = (long long)batch * (N / 256) * (M / 128);
    const int grid = (int)(tiles < nsm ? tiles : nsm);
    const int smem = (int)sizeof(PersistSmem<2>) + 1024;
    auto kern = fp16 ? gemm_persist_kernel<true, 2> : gemm_persist_kernel<false, 2>;
    int e = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                       "cudaFuncSetAttribute(gemm_persist, two planes)");
    if (!e) kern<<<grid, 192, smem, st>>>(ta, tb, C, M, N, K, K, batch, status);
    return e ? e : check_launch("gemm_persist_kernel (two A planes)");
}

} // namespace vgb

extern "C" int vgb_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K, void *stream)
{
    return gemm_batched(A, B, C, M, N, K, 1, false, static_cast<cudaStream_t>(stream), K);
}

extern "C" int vgb_gemm_variant(int v)
{
    if (v != 0 && v != 128 && v != 256 && v != 512)
        return set_error(VGB_ERR_INVALID, "gemm_variant: 0 (autotuned), 128, 256 or 512"), -1;
    const int prev = g_gemm_variant.exchange(v);
    return prev;
}

extern "C" int vgb_gemm_batched(const void *A, const void *B, float *C, int M, int N, int K, int batch, int fp16,
                                void *stream)
{
    return gemm_batched(A, B, C, M, N, K, batch, fp16 != 0, static_cast<cudaStream_t>(stream), K);
}

extern "C" int vgb_gemm_batched_planes(const void *A, const void *B, float *C, int M, int N, int K, int batch,
                                       int fp16, void *stream)
{
    return gemm_batched_planes(A, B, C, M, N, K, batch, fp16 != 0, static_cast<cudaStream_t>(stream));
}
