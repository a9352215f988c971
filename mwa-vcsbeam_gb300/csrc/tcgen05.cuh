// 5th-generation tensor core (tcgen05) and tensor-TMA helpers, sm_100+/sm_103a.
//
// Conventions used by the kernels here:
//  * operands are bf16, K-major (each row of an operand tile holds 64
//    consecutive K elements = 128 bytes), staged by 2-D TMA loads with
//    128-byte swizzling into 1024-byte aligned shared memory; that is the
//    canonical SWIZZLE_128B K-major layout the MMA reads (8-row groups of
//    1 KB, stride 1024 B);
//  * accumulators are FP32 in tensor memory (TMEM), row i of a 128-row tile
//    in TMEM lane i, column j in TMEM column base + j;
//  * one thread issues MMAs; tcgen05.commit arrives on an mbarrier when the
//    MMAs issued before it have completed.
#pragma once

#include <cuda.h>
#include <cstdint>

#include "vgb_internal.cuh"

namespace vgb {

// ---------------------------------------------------------------------------
// TMEM allocation (one full warp executes each of these)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---------------------------------------------------------------------------
// Descriptors
// ---------------------------------------------------------------------------
// Instruction descriptor, kind::f16: FP32 accumulate, BF16 (or, with
// fp16 = true, FP16) A and B, both K-major, M = 128, N (multiple of 16,
// 16..256), optional negation of A.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(uint32_t N, bool negate_a = false, bool fp16 = false)
{
    return (1u << 4)                    // D format: F32
           | ((fp16 ? 0u : 1u) << 7)    // A format: BF16 (1) or F16 (0)
           | ((fp16 ? 0u : 1u) << 10)   // B format: the same type as A
           | ((negate_a ? 1u : 0u) << 13) | (0u << 15) // A K-major
           | (0u << 16)                 // B K-major
           | ((N >> 3) << 17)           // N >> 3
           | ((128u >> 4) << 24);       // M >> 4
}

// The same for an MMA issued over a CTA pair (cta_group::2): M = 256, rows
// 0-127 from the issuing CTA's shared memory and 128-255 from its peer's.
__host__ __device__ constexpr uint32_t idesc_pair_f32(uint32_t N, bool fp16 = false)
{
    return (idesc_bf16_f32(N, false, fp16) & ~(0x1Fu << 24)) | ((256u >> 4) << 24);
}

// Shared-memory matrix descriptor for a SWIZZLE_128B K-major tile whose
// 1024-byte aligned start is `saddr` (shared-space byte address).
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);    // start address
    d |= (uint64_t)1 << 16;                      // leading byte offset (16 B; unused for this layout)
    d |= (uint64_t)(1024u >> 4) << 32;           // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                      // descriptor version for tcgen05
    d |= (uint64_t)2 << 61;                      // 128-byte swizzle
    return d;
}

// Descriptor of the k-th 16-element (32-byte) K slice inside the same tile.
__device__ __forceinline__ uint64_t sdesc_advance_k(uint64_t d, int k) { return d + (uint64_t)((k * 32) >> 4); }

// ---------------------------------------------------------------------------
// MMA, commit, TMEM loads
// ---------------------------------------------------------------------------
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                       uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void tc_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 consecutive FP32 columns of this thread's TMEM lane (warp w of a
// warpgroup reads lanes 32w..32w+31; `taddr` carries the lane in bits 16+).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// 36 consecutive FP32 columns of this thread's TMEM lane (.32x32b: warp w
// reaches lanes 32 (w % 4) .. + 31). The load returns once the values are in
// registers (the wait names the registers, so no use can be scheduled before
// it); the store is asynchronous: tmem_wait_st() before the same columns are
// loaded again or the allocation is released.
__device__ __forceinline__ void tmem_ld36(uint32_t taddr, float (&v)[36])
{
    uint32_t r[36];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35])
                 : "r"(taddr + 32u)
                 : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                   "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                   "+r"(r[29]), "+r"(r[30]), "+r"(r[31]), "+r"(r[32]), "+r"(r[33]), "+r"(r[34]), "+r"(r[35])
                 :
                 : "memory");
#pragma unroll
    for (int i = 0; i < 36; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_st36(uint32_t taddr, const float (&v)[36])
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x32.b32 [%0], "
        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,"
        "%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31,%32};" ::"r"(taddr),
        "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
        "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
        "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
        "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
        "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
        "r"(__float_as_uint(v[15])), "r"(__float_as_uint(v[16])), "r"(__float_as_uint(v[17])),
        "r"(__float_as_uint(v[18])), "r"(__float_as_uint(v[19])), "r"(__float_as_uint(v[20])),
        "r"(__float_as_uint(v[21])), "r"(__float_as_uint(v[22])), "r"(__float_as_uint(v[23])),
        "r"(__float_as_uint(v[24])), "r"(__float_as_uint(v[25])), "r"(__float_as_uint(v[26])),
        "r"(__float_as_uint(v[27])), "r"(__float_as_uint(v[28])), "r"(__float_as_uint(v[29])),
        "r"(__float_as_uint(v[30])), "r"(__float_as_uint(v[31]))
        : "memory");
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(taddr + 32u),
                 "r"(__float_as_uint(v[32])), "r"(__float_as_uint(v[33])), "r"(__float_as_uint(v[34])),
                 "r"(__float_as_uint(v[35]))
                 : "memory");
}

__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// ---------------------------------------------------------------------------
// Tensor TMA (2-D tiled, global -> shared, mbarrier completion)
// ---------------------------------------------------------------------------
// The x coordinate (innermost, in elements) must be a multiple of 8 for bf16
// (16 bytes); callers only pass multiples of 64.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// 5-D tiled load, coordinates innermost first (elements); used for the
// beamformer's weight rows, whose innermost coordinate is always 0.
__device__ __forceinline__ void tma_load_5d(void *dst, const CUtensorMap *map, int c0, int c1, int c2, int c3, int c4,
                                            uint64_t *bar)
{
    asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
                 "%5, %6}], [%7];" ::"r"(smem_u32(dst)),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(c4), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void prefetch_tmap(const CUtensorMap *map)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// ---------------------------------------------------------------------------
// CTA pairs (cta_group::2): the two CTAs of a 2-CTA cluster, which the
// hardware places on the two SMs of one TPC. One thread of the even CTA
// issues MMAs with M = 256 whose A rows and B columns are split between the
// two CTAs' shared memory (same offsets in both) and whose accumulator rows
// are split between their tensor memories (rows 0-127 in the even CTA, 128-255
// in the odd one, same columns). Every tcgen05 instruction of such a kernel
// names cta_group::2; the allocation is made collectively by one warp of each
// CTA.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t cluster_rank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

// Shared::cluster address of the object at shared-space address `saddr` of
// this CTA, in the CTA of cluster rank `rank`.
__device__ __forceinline__ uint32_t mapa_shared(uint32_t saddr, uint32_t rank)
{
    uint32_t d;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(d) : "r"(saddr), "r"(rank));
    return d;
}

// All threads of both CTAs; orders earlier shared-memory writes (barrier
// initialisation included) before the peer's later accesses.
__device__ __forceinline__ void cluster_sync()
{
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

__device__ __forceinline__ void tmem_alloc_pair(uint32_t *dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish_pair()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc_pair(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_mma_pair(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on the mbarrier at the same offset as `bar` in both CTAs of the pair
// once the pair MMAs issued before it have completed.
__device__ __forceinline__ void tc_commit_pair_both(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::
                     "r"(smem_u32(bar)),
                 "h"((uint16_t)0x3)
                 : "memory");
}
// The same on this CTA's own `bar` only.
__device__ __forceinline__ void tc_commit_pair_own(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 2-D tiled load into this CTA's shared memory whose completion is counted on
// the mbarrier at shared::cluster address `bar_cl` (this CTA's or its peer's).
__device__ __forceinline__ void tma_load_2d_pair(void *dst, const CUtensorMap *map, int x, int y, uint32_t bar_cl)
{
    asm volatile("cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, "
                 "{%2, %3}], [%4];" ::"r"(smem_u32(dst)),
                 "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(bar_cl)
                 : "memory");
}

// Arrive on the mbarrier at shared::cluster address `bar_cl` (this CTA's or
// its peer's). What it hands over is tensor memory, whose reads the caller
// has completed (tcgen05.wait::ld) and ordered (tcgen05.fence::before_
// thread_sync) before it, so no cluster-wide memory fence is needed.
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t bar_cl)
{
    asm volatile("mbarrier.arrive.shared::cluster.b64 _, [%0];" ::"r"(bar_cl) : "memory");
}

// Host: build a 2-D tensor map over a row-major bf16 matrix [rows][cols]
// (row stride `row_bytes`), box = 64 columns x `box_rows` rows, 128-byte
// swizzle. Defined in tc_gemm.cu (the driver entry point is looked up at
// run time so the library loads without a driver).
int make_tmap_bf16(CUtensorMap *map, const void *base, uint64_t rows, uint64_t cols, uint64_t row_bytes,
                   uint32_t box_rows, bool fp16 = false);

// Host: 5-D tensor map over the beamformer weights W[cc][ant][k][row]
// (row 0 = (w00, w01), row 1 = (w10, w11), 16 bytes each; `W_cc` float4
// between coarse channels) whose box {4 floats, 1 row, K, tiles_per_box, 1}
// lands as [tile][k] float4 of one row: loading rows 0 and 1 separately
// de-interleaves them, so a warp's reads of one row are contiguous.
int make_tmap_beam_weights(CUtensorMap *map, const void *W, int nant, int ncc, long long W_cc, int tiles_per_box);

} // namespace vgb
