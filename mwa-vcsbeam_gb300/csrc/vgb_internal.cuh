// Shared device/host definitions for the GB300 voltage hot path.
//
// Layout vocabulary follows VCSBeam (include/vcsbeam.h.in:234-268):
//   MWAX voltages   [block][input][sample-in-block] char2, 64000 samples/block
//   fine voltages   v_IDX  [sample][chan][input]
//   Stokes          C_IDX  [pointing][sample][stokes][chan]
//   beam voltages   B_IDX  [pointing][sample][chan][pol]
// A "frame" is the 128 consecutive samples one fine spectrum consumes.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "../../include/vcsbeam_gb300.h"

#include <nvtx3/nvToolsExt.h>

namespace vgb {

// NVTX range for the lifetime of a scope (visible in Nsight timelines; a
// no-op when no tool is attached).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};


constexpr int kVSPVB = 64000;               // samples per MWAX voltage block
constexpr int kK = 128;                     // fine channels (FFT length)
constexpr int kP = 12;                      // taps
constexpr int kFramesPerBlock = kVSPVB / kK; // 500
constexpr int kHistFrames = kP;             // frames of the previous second a second needs

// Error flag bits a kernel may raise in the device status word.
constexpr unsigned kErrWaitTimeout = 1u;    // a bounded mbarrier wait gave up
constexpr unsigned kErrBadFrame = 2u;       // a frame index fell outside the described buffers
constexpr unsigned kErrBadInput = 4u;       // an input index (polQ / polP) fell outside the voltage row

// ---------------------------------------------------------------------------
// Where the frames of one coarse channel's second live.
//
// Window frame w (w = 0 .. nspectra+P-2) is the w-th 128-sample frame of the
// time axis that starts P frames before the second: w < P are the previous
// second's last P frames ("history"), w >= P is frame (w-P) of the second.
// This covers both the reference's single buffer with a one-block margin in
// front (pfb.cpp:149-153) and a compact history array.
// ---------------------------------------------------------------------------
struct VoltView {
    const char2 *hist;     // history frame 0 of input 0
    long long hist_input;  // char2 stride between inputs in the history
    const char2 *cur;      // block 0, input 0, sample 0 of the second
    long long cur_block;   // char2 stride between voltage blocks
    long long cc_hist;     // char2 stride between coarse channels (history)
    long long cc_cur;      // char2 stride between coarse channels (second)
    int ninputs;
    int nblocks;           // voltage blocks in the second
};

// ---------------------------------------------------------------------------
// Host-side status helpers (defined in vgb_api.cu).
// ---------------------------------------------------------------------------
int set_error(int code, const char *fmt, ...);
int check_cuda(cudaError_t e, const char *what);
int check_launch(const char *what);
// Device address of the current device's status word (kernels atomicOr
// kErr* bits into it), or NULL.
unsigned *status_word();

// ---------------------------------------------------------------------------
// PTX helpers: shared-memory addresses, mbarriers, 1-D bulk (TMA) copies.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// Bounded wait on an mbarrier phase. Returns false if the phase did not
// complete within `max_polls` polls (the caller records an error and skips
// the work instead of spinning forever).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t phase, uint32_t max_polls)
{
    uint32_t addr = smem_u32(bar);
    for (uint32_t i = 0; i < max_polls; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n"
            " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// The reference's (uint8_t)(x + 0.5) as its GPU build evaluates it: NaN and
// values <= 0 give 0, larger values keep the low 8 bits of the truncated
// integer (a channel maximum of 256.5 wraps to 0).
__device__ __forceinline__ uint8_t sat_u8(double t)
{
    if (t != t || t <= 0.0) return 0;
    return (uint8_t)((unsigned)t & 0xFFu);
}

// sat_u8((double)v + 0.5) without FP64 arithmetic on the common path: for
// |v| < 2^22 a float's spacing is at most 1/4, so v + 0.5f is exact and equal
// to the double sum; larger magnitudes, infinities and NaN take the FP64 path.
__device__ __forceinline__ uint8_t sat_u8_half(float v)
{
    if (fabsf(v) < 4194304.f) {
        const float t = v + 0.5f;
        return t <= 0.f ? (uint8_t)0 : (uint8_t)((unsigned)t & 0xFFu);
    }
    return sat_u8((double)v + 0.5);
}

// Order-preserving unsigned keys of floats (for atomicMin / atomicMax over
// the extremes of a row); NaN is never passed in.
__device__ __forceinline__ uint32_t fkey(float f)
{
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float fkey_inv(uint32_t k)
{
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// The reference's byte for one value, (uint8_t)((e - off) / scl + 0.5) with
// the division correctly rounded, without a division on the common path.
// With rcp = 1/scl (correctly rounded), q0 = x * rcp is within 1.5 ulp of
// the true quotient, so for |q0| < 512 it differs from the correctly rounded
// quotient q by less than 2^-12. The byte is floor(q + 1/2), which changes
// only at half-integers; when q0 lies further than 2^-12 from every
// half-integer, q lies in the same interval and the byte is q0 rounded to the
// nearest integer (read from the low bits of q0 + 1.5 * 2^23). Otherwise, and
// for out-of-range or non-finite values, the division itself is used.
__device__ __forceinline__ uint8_t quant_u8(float e, float off, float scl, float rcp)
{
    const float x = __fsub_rn(e, off);
    const float q0 = __fmul_rn(x, rcp);
    if (fabsf(q0) < 512.f) {
        const float y = __fadd_rn(q0, 12582912.f);
        const float n = __fsub_rn(y, 12582912.f);
        if (fabsf(__fsub_rn(q0, n)) < 0.499755859375f) { // 1/2 - 2^-12
            const int ni = (int)(__float_as_uint(y) & 0x7FFFFFu) - 4194304;
            return ni > 0 ? (uint8_t)(ni & 0xFF) : (uint8_t)0;
        }
    }
    return sat_u8_half(x / scl);
}

// 1-D bulk copy global -> shared through the TMA unit. dst, src and bytes
// must be multiples of 16 (callers copy whole 256-byte frames).
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// ---------------------------------------------------------------------------
// 128-point DFT building blocks (8 threads per transform).
//
// n = 8q + j (j = thread in group, q = 0..15); k = k1 + 16 k2.
//   pass 1: thread j: Y_j[k1] = sum_q x[8q+j] W16^{q k1}, then * W128^{j k1}
//   pass 2: thread t: for k1 in {2t, 2t+1}: X[k1+16k2] = sum_j Y_j[k1] W8^{j k2}
// The sign of the exponent is a template parameter: -1 forward (cuFFT's
// CUFFT_FORWARD convention), +1 inverse (unnormalised).
// ---------------------------------------------------------------------------
template <int SIGN> __device__ __forceinline__ float2 cmul_tw(float2 a, float c, float s)
{
    // a * (c + i*SIGN*s) where (c, s) = (cos, |sin|) of the positive angle
    const float ss = SIGN * s;
    return make_float2(a.x * c - a.y * ss, a.x * ss + a.y * c);
}

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmulf(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// multiply by SIGN*i  (e^{SIGN i pi/2})
template <int SIGN> __device__ __forceinline__ float2 mul_i(float2 a)
{
    return SIGN > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// Packed FP32x2 arithmetic (sm_100+): one instruction updates both halves of
// a complex value. Rounding is that of the scalar operations (RN per lane;
// a - b is an FMA with -1, exact before its single rounding).
__device__ __forceinline__ float2 padd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }

// In-register DFT of length 4 with exponent sign SIGN (packed butterflies;
// the +-i rotation is folded into scalar adds).
template <int SIGN> __device__ __forceinline__ void dft4(float2 &a0, float2 &a1, float2 &a2, float2 &a3)
{
    const float2 t0 = padd(a0, a2), t1 = psub(a0, a2);
    const float2 t2 = padd(a1, a3), d = psub(a1, a3);
    a0 = padd(t0, t2);
    a2 = psub(t0, t2);
    if (SIGN > 0) {
        a1 = make_float2(t1.x - d.y, t1.y + d.x);
        a3 = make_float2(t1.x + d.y, t1.y - d.x);
    } else {
        a1 = make_float2(t1.x + d.y, t1.y - d.x);
        a3 = make_float2(t1.x - d.y, t1.y + d.x);
    }
}

// Length-8 DFT in registers, natural order in and out.
template <int SIGN> __device__ __forceinline__ void dft8(float2 *x)
{
    const float r = 0.70710678118654752440f;
    float2 a[8];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        a[i] = padd(x[i], x[i + 4]);
        a[i + 4] = psub(x[i], x[i + 4]);
    }
    // twiddles W8^{SIGN*i} on the odd half: i = 1, 2, 3
    a[5] = make_float2(r * (a[5].x - SIGN * a[5].y), r * (a[5].y + SIGN * a[5].x));
    a[6] = mul_i<SIGN>(a[6]);
    a[7] = make_float2(r * (-a[7].x - SIGN * a[7].y), r * (-a[7].y + SIGN * a[7].x));
    dft4<SIGN>(a[0], a[1], a[2], a[3]);
    dft4<SIGN>(a[4], a[5], a[6], a[7]);
    x[0] = a[0];
    x[2] = a[1];
    x[4] = a[2];
    x[6] = a[3];
    x[1] = a[4];
    x[3] = a[5];
    x[5] = a[6];
    x[7] = a[7];
}

// Length-16 DFT in registers (4 x 4 decomposition), natural order.
template <int SIGN> __device__ __forceinline__ void dft16(float2 *x)
{
    // n = 4 n1 + n2, k = k1 + 4 k2
    float2 y[16];
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) {
        float2 a0 = x[n2], a1 = x[n2 + 4], a2 = x[n2 + 8], a3 = x[n2 + 12];
        dft4<SIGN>(a0, a1, a2, a3); // over n1 -> k1
        y[n2 * 4 + 0] = a0;
        y[n2 * 4 + 1] = a1;
        y[n2 * 4 + 2] = a2;
        y[n2 * 4 + 3] = a3;
    }
    // twiddle W16^{n2 k1}
    const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f;
    const float r = 0.70710678118654752440f;
#pragma unroll
    for (int n2 = 1; n2 < 4; n2++) {
#pragma unroll
        for (int k1 = 1; k1 < 4; k1++) {
            const int e = n2 * k1; // 1..9
            float c, s;
            switch (e) {
            case 1: c = c1; s = s1; break;
            case 2: c = r; s = r; break;
            case 3: c = s1; s = c1; break;
            case 4: c = 0.f; s = 1.f; break;
            case 6: c = -r; s = r; break;
            case 9: c = -c1; s = -s1; break;
            default: c = 1.f; s = 0.f; break;
            }
            y[n2 * 4 + k1] = (e == 4) ? mul_i<SIGN>(y[n2 * 4 + k1]) : cmul_tw<SIGN>(y[n2 * 4 + k1], c, s);
        }
    }
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
        float2 a0 = y[k1], a1 = y[4 + k1], a2 = y[8 + k1], a3 = y[12 + k1];
        dft4<SIGN>(a0, a1, a2, a3); // over n2 -> k2
        x[k1] = a0;
        x[k1 + 4] = a1;
        x[k1 + 8] = a2;
        x[k1 + 12] = a3;
    }
}

// Shared-memory row geometry of one 128-point transform (float2 units).
// Pass-1 output Y_j[k1] is stored at k1*9 + j (9 = 8 + 1 pad, conflict-free
// for both passes). Rows are padded so that 4 transforms in one warp land on
// alternating bank halves.
constexpr int kFftRow = 152;

// Slot (float2 units) of the twiddle W128^{j k1} in a 16-byte aligned table
// of 128 float2: pairs k1 = 2i, 2i + 1 of one j sit together, so pass 1 reads
// two twiddles per 16-byte load.
__host__ __device__ __forceinline__ int fft128_tw_slot(int k1, int j) { return ((k1 >> 1) * 8 + j) * 2 + (k1 & 1); }

// Pass 1: the 8 threads of one group read x[8q + j] (row `row`), transform
// over q, twiddle by W128^{j k1} from `tw` (cos/sin pairs of the positive
// angle 2*pi*j*k1/128 at fft128_tw_slot(k1, j)) and write back in place as
// Y_j[k1].
template <int SIGN>
__device__ __forceinline__ void fft128_pass1(float2 *row, const float2 *tw, int j)
{
    float2 x[16];
#pragma unroll
    for (int q = 0; q < 16; q++) x[q] = row[8 * q + j];
    __syncwarp();
    dft16<SIGN>(x);
    const float4 *tw4 = reinterpret_cast<const float4 *>(tw);
#pragma unroll
    for (int i = 0; i < 8; i++) {
        const float4 w = tw4[i * 8 + j]; // W^{j 2i}, W^{j (2i + 1)}
        if (i > 0) x[2 * i] = cmul_tw<SIGN>(x[2 * i], w.x, w.y);
        x[2 * i + 1] = cmul_tw<SIGN>(x[2 * i + 1], w.z, w.w);
    }
#pragma unroll
    for (int k1 = 0; k1 < 16; k1++) row[k1 * 9 + j] = x[k1];
}

// Pass 2: thread t of the group produces X[k1 + 16 k2] for k1 = t, t + 8 and
// all k2, into `out[2][8]` (out[h][k2] for k1 = t + 8h, output index
// fft128_index(t, h, k2)). The 8 threads of a row read at a stride of 9
// float2, which with rows 64 bytes apart modulo 128 (kFftRow) puts a warp's
// four rows on complementary banks: two wavefronts per read, as in pass 1.
template <int SIGN>
__device__ __forceinline__ void fft128_pass2(const float2 *row, int t, float2 (&out)[2][8])
{
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int k1 = t + 8 * h;
#pragma unroll
        for (int j = 0; j < 8; j++) out[h][j] = row[k1 * 9 + j];
        dft8<SIGN>(out[h]);
    }
}

// Frequency index of pass 2's out[h][k2] in thread t.
__device__ __forceinline__ int fft128_index(int t, int h, int k2) { return t + 8 * h + 16 * k2; }

} // namespace vgb
