// Fused forward fine PFB and tied-array / incoherent beamformer for MWAX
// voltages, GB300 (sm_103a).
//
// One CTA (256 threads, ~93 KB of shared memory, two CTAs per SM) owns a
// tile of T = 8 consecutive fine spectra of one coarse channel and walks the
// RF inputs four at a time (two tiles x two pols). Per step:
//   1. the TMA unit copies the 19 voltage frames (T + 11) each input needs
//      (1-D bulk copies) and the two tiles' weights (a 5-D tensor map that
//      splits the two Jones rows apart) into shared memory, double-buffered
//      with mbarriers: step i+1 lands while step i computes;
//   2. weighted overlap-add, exactly (pfb.cpp:121-179): one thread per
//      (input, pair of adjacent samples), the pair's 12 taps in registers,
//      packed FP32x2 FMAs (the even and odd taps summed apart, or int32,
//      when one FP32 sum would not be exact);
//   3. the FPGA rounding (pfb.cpp:202-242) or the 2^-14 scaling
//      (pfb.cpp:256-268);
//   4. a 128-point FFT (16 x 8, eight threads per transform, in place);
//   5. fftshift, 1/K, the (im, re) ordering of pfb.cpp:328-339 and, for the
//      4-bit mode, the round-and-clip of vcsbeam.h.in:453-457;
//   6. beamformer back end: ex/ey = (phi J^-1)[a][c] v (form_beam.cpp:174-177,
//      295-296) accumulated over tiles with the autocorrelation terms
//      (form_beam.cpp:298-315) and the incoherent sum; or the PFB-only back
//      end, which writes the packed legacy-order output (pfb.cpp:316-340).
// The fine-channel voltages never reach HBM on the beamformer path.
#include <atomic>
#include <cstddef>
#include <map>
#include <mutex>
#include <tuple>

#include "tcgen05.cuh"
#include "vgb_launch.cuh"

namespace vgb {

constexpr int kT = 8;                      // spectra per CTA
constexpr int kG = 4;                      // inputs per step (two tiles) of the PFB-only kernel
constexpr int kThreads = 256;
constexpr int kWin = kT + kP - 1;          // frames per input per step
constexpr int kFrameBytes = kK * 2;        // 256

// Shared memory of a front-end CTA taking G inputs (G/2 tiles) per step with
// 64 threads per input: 95 KB for G = 4 (two CTAs per SM), 188 KB for G = 8.
template <int G> struct FrontSmemT {
    char2 stage[2][G][kWin][kK];           // TMA destinations: frames
    float4 wst[2][2][G / 2][kK];           // TMA destinations: weights [row][tile][k'] of the step's tiles
    float2 buf[G * kT][kFftRow];           // WOLA output -> FFT (in place) -> voltages
    float2 tw[128];                        // W128 twiddles at fft128_tw_slot(k1, j) (16-byte aligned)
    uint64_t bar[2];
};
using FrontSmem = FrontSmemT<kG>;
static_assert(offsetof(FrontSmemT<4>, tw) % 16 == 0 && offsetof(FrontSmemT<8>, tw) % 16 == 0,
              "twiddles are read 16 bytes at a time");

// ---------------------------------------------------------------------------
// Copy the frames input `i` needs for spectra [m0, m0 + kT) into `dst`.
// Window frame w = m + p (p = tap). Returns the bytes requested.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t issue_frames(const VoltView &vv, int cc, int i, int w0, int w_end,
                                                 char2 *dst, uint64_t *bar, unsigned *status)
{
    uint32_t bytes = 0;
    int w = w0;
    const char2 *hist = vv.hist + cc * vv.cc_hist + i * vv.hist_input;
    const char2 *cur = vv.cur + cc * vv.cc_cur + (long long)i * kVSPVB;
    while (w < w_end) {
        const char2 *src;
        int cnt;
        if (w < kHistFrames) {
            cnt = min(w_end, kHistFrames) - w;
            src = hist + (long long)w * kK;
        } else {
            const int g = w - kHistFrames;
            const int b = g / kFramesPerBlock, f = g % kFramesPerBlock;
            if (b >= vv.nblocks) {
                atomicOr(status, kErrBadFrame);
                break;
            }
            cnt = min(w_end - w, kFramesPerBlock - f);
            src = cur + b * vv.cur_block + (long long)f * kK;
        }
        bulk_g2s(dst + (w - w0) * kK, src, cnt * kFrameBytes, bar);
        bytes += cnt * kFrameBytes;
        w += cnt;
    }
    return bytes;
}

// Producer: warp 0 queues step `it`'s frames (and, when a weight map is
// given, the two Jones rows of its G/2 tiles, tiles past the last one
// zero-filled) into stage it & 1, one input per lane (lane G the weights), so
// the copy set-up costs the warp about one input's worth. Step position
// it * G + li holds input order[it * G + li] when an order is given, else
// that input itself.
template <int G>
__device__ __forceinline__ void produce(FrontSmemT<G> &sm, const VoltView &vv, int cc, int it, int m0, int nspectra,
                                       const CUtensorMap *wmap, unsigned *status, const int *order = nullptr)
{
    const int lane = threadIdx.x & 31;
    const int s = it & 1;
    const int w_end = min(m0 + kWin, nspectra + kP - 1);
    uint32_t total = 0;
    for (int li = 0; li < G; li++)
        if (it * G + li < vv.ninputs) total += (w_end - m0) * kFrameBytes;
    constexpr uint32_t kWBytes = (G / 2) * kK * 16;   // one Jones row of G/2 tiles
    if (wmap) total += 2 * kWBytes;
    if (lane == 0) mbar_arrive_expect_tx(&sm.bar[s], total);
    __syncwarp();
    uint32_t issued = 0;
    if (lane < G) {
        const int pos = it * G + lane;
        if (pos < vv.ninputs)
            issued = issue_frames(vv, cc, order ? order[pos] : pos, m0, w_end, sm.stage[s][lane][0], &sm.bar[s],
                                  status);
    } else if (lane == G && wmap) {
        tma_load_5d(sm.wst[s][0][0], wmap, 0, 0, 0, (G / 2) * it, cc, &sm.bar[s]);
        tma_load_5d(sm.wst[s][1][0], wmap, 0, 1, 0, (G / 2) * it, cc, &sm.bar[s]);
        issued = 2 * kWBytes;
    }
    // lanes 0..G issue copies: a butterfly over the lowest 8 (G = 4) or 16 lanes
#pragma unroll
    for (int o = G >= 8 ? 8 : 4; o; o >>= 1) issued += __shfl_xor_sync(0xffffffffu, issued, o);
    if (lane == 0 && issued != total) {
        // Some frames were outside the buffers: complete the remaining
        // transaction count so consumers are not left waiting; the status
        // word already records the error.
        asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&sm.bar[s])),
                     "r"(total - issued)
                     : "memory");
    }
}

// Producer of the beamformer kernel, spread over warps so that no warp
// carries all of a step's copy set-up (every warp meets at the step's block
// barriers, where the most loaded one sets the pace): lane 0 of warp li
// (li < G) copies input it * G + li's frames, lane 0 of warp G the two Jones
// rows of the step's tiles, and lane 0 of warp 0 posts the step's expected
// byte count first. Each issuer completes its own shortfall when frames fell
// outside the buffers (the status word records that). The transaction count
// may be consumed before it is posted; the phase still cannot complete before
// warp 0's arrival. Called by every thread after the step's first block
// barrier, as produce() is.
template <int G>
__device__ __forceinline__ void produce_spread(FrontSmemT<G> &sm, const VoltView &vv, int cc, int it, int m0,
                                              int nspectra, const CUtensorMap *wmap, unsigned *status)
{
    if ((threadIdx.x & 31) != 0) return;
    const int warp = threadIdx.x >> 5;
    const int s = it & 1;
    const int w_end = min(m0 + kWin, nspectra + kP - 1);
    const uint32_t per_input = (w_end - m0) * kFrameBytes;
    constexpr uint32_t kWBytes = (G / 2) * kK * 16;   // one Jones row of G/2 tiles
    if (warp == 0) {
        uint32_t total = 2 * kWBytes;
        for (int li = 0; li < G; li++)
            if (it * G + li < vv.ninputs) total += per_input;
        mbar_arrive_expect_tx(&sm.bar[s], total);
    }
    if (warp < G) {
        const int pos = it * G + warp;
        if (pos < vv.ninputs) {
            const uint32_t issued = issue_frames(vv, cc, pos, m0, w_end, sm.stage[s][warp][0], &sm.bar[s], status);
            if (issued != per_input)
                asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&sm.bar[s])),
                             "r"(per_input - issued)
                             : "memory");
        }
    } else if (warp == G) {
        tma_load_5d(sm.wst[s][0][0], wmap, 0, 0, 0, (G / 2) * it, cc, &sm.bar[s]);
        tma_load_5d(sm.wst[s][1][0], wmap, 0, 1, 0, (G / 2) * it, cc, &sm.bar[s]);
    }
}

// Four int8 values (two char2) -> packed floats (re0, re1), (im0, im1), exact,
// via the 2^23 magic number: bytes are offset to unsigned, placed under the
// exponent of 2^23 and the 2^23 + 128 bias subtracted.
__device__ __forceinline__ void c4_to_f(uint32_t w, float2 &re, float2 &im)
{
    const uint32_t u = w ^ 0x80808080u;
    const float2 bias = make_float2(-8388736.0f, -8388736.0f);
    re = padd(make_float2(__uint_as_float(__byte_perm(u, 0x4B000000u, 0x7540)),
                          __uint_as_float(__byte_perm(u, 0x4B000000u, 0x7542))),
              bias);
    im = padd(make_float2(__uint_as_float(__byte_perm(u, 0x4B000000u, 0x7541)),
                          __uint_as_float(__byte_perm(u, 0x4B000000u, 0x7543))),
              bias);
}

// The same four values by the integer-to-float conversion of each signed
// byte (exact). The conversion pipe issues 16 per clock per SM but otherwise
// idles here, while the FMA pipe, which the form above loads with one
// operation per value, is this kernel's busiest: without FPGA rounding this
// form is the faster (full band 21.40 -> 21.12 ms per data-second). With it
// the rounding and 4-bit demotion keep the conversion pipe busy and the form
// above is the faster (24.5 against 25.4 ms).
__device__ __forceinline__ void c4_to_f_cvt(uint32_t w, float2 &re, float2 &im)
{
    re = make_float2((float)(signed char)(w & 0xFFu), (float)(signed char)((w >> 16) & 0xFFu));
    im = make_float2((float)(signed char)((w >> 8) & 0xFFu), (float)(signed char)(w >> 24));
}

template <bool kFpga> __device__ __forceinline__ void widen4(uint32_t w, float2 &re, float2 &im)
{
    if constexpr (kFpga) c4_to_f(w, re, im);
    else c4_to_f_cvt(w, re, im);
}

__device__ __forceinline__ void c4_to_i(uint32_t w, int (&re)[2], int (&im)[2])
{
    re[0] = (int)(signed char)(w & 0xFFu);
    im[0] = (int)(signed char)((w >> 8) & 0xFFu);
    re[1] = (int)(signed char)((w >> 16) & 0xFFu);
    im[1] = (int)(signed char)(w >> 24);
}

// FPGA rounding (pfb.cpp:225-231) of an integer-valued float |X| < 2^24:
// (X + 0x2000) >> 14 for X > 0, X >> 14 otherwise, both exact in FP32.
__device__ __forceinline__ float fpga_round(float X)
{
    return floorf(fmaf(X, 1.0f / 16384.0f, X > 0.f ? 0.5f : 0.f));
}

// ---------------------------------------------------------------------------
// Steps 2-3: weighted overlap-add for thread (li, n0..n0+1) into buf rows.
// ---------------------------------------------------------------------------
// Arithmetic of the sum of 12 products h x (int taps, int8 voltages), each
// giving the exact integer sum rounded once to FP32 -- what the reference's
// int32 sum converted to float gives (pfb.cpp:153-160, 256-268):
//   kWolaFp32   one FP32 sum; exact when every partial sum of the filter
//               times |x| <= 128 stays within 2^24 (vgb_filter_fp32_exact);
//   kWolaSplit  the even and the odd taps summed apart in FP32, each exact
//               within 2^24, and added once (one rounding of the exact sum);
//               the reference's FINEPFB filter (peak tap 117,964) is such a
//               filter. Without FPGA rounding only (that needs the integer);
//   kWolaInt32  int32 sums, any filter.
constexpr int kWolaFp32 = 0, kWolaSplit = 1, kWolaInt32 = 2;

// The taps of samples n0, n0 + 1 in the form the WOLA multiplies by: int32
// pairs, or FP32 pairs carrying the output scale 2^-14 / K when there is no
// FPGA rounding (a power of two: every product and partial sum is the exact
// one scaled, so the result is identical and the final multiply goes).
template <int kW> struct WolaTap {
    using type = float2;
};
template <> struct WolaTap<kWolaInt32> {
    using type = int2;
};

template <int kW, bool kFpga>
__device__ __forceinline__ void make_taps(const int (&hc)[2][kP], typename WolaTap<kW>::type (&t)[kP])
{
#pragma unroll
    for (int p = 0; p < kP; p++) {
        if constexpr (kW == kWolaInt32) {
            t[p] = make_int2(hc[0][p], hc[1][p]);
        } else {
            const float tsc = kFpga ? 1.0f : 1.0f / (16384.0f * kK);
            t[p] = make_float2((float)hc[0][p] * tsc, (float)hc[1][p] * tsc);
        }
    }
}

// stage_in: the input's kWin staged frames [w][kK]; rows: its kT output rows.
template <int kW, bool kFpga>
__device__ __forceinline__ void wola_rows(const char2 *stage_in, float2 (*rows)[kFftRow], int n0,
                                          const typename WolaTap<kW>::type (&t)[kP])
{
    static_assert(kW != kWolaSplit || !kFpga, "the split sum is for the unrounded mode");
    const uint32_t *x = reinterpret_cast<const uint32_t *>(stage_in + n0);
    if constexpr (kW == kWolaInt32) {
        int ar[kT][2], ai[kT][2];
#pragma unroll
        for (int m = 0; m < kT; m++) ar[m][0] = ar[m][1] = ai[m][0] = ai[m][1] = 0;
#pragma unroll
        for (int w = 0; w < kWin; w++) {
            int xr[2], xi[2];
            c4_to_i(x[w * (kK / 2)], xr, xi);
#pragma unroll
            for (int p = 0; p < kP; p++) {
                const int m = w - p;
                if (m >= 0 && m < kT) {
#pragma unroll
                    for (int q = 0; q < 2; q++) {
                        const int h = q ? t[p].y : t[p].x;
                        ar[m][q] += h * xr[q];
                        ai[m][q] += h * xi[q];
                    }
                }
            }
        }
#pragma unroll
        for (int m = 0; m < kT; m++) {
            float4 b;
            if (kFpga) {
                int v[4] = {ar[m][0], ai[m][0], ar[m][1], ai[m][1]};
#pragma unroll
                for (int q = 0; q < 4; q++) v[q] = (v[q] > 0 ? v[q] + 0x2000 : v[q]) >> 14;
                b = make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
            } else {
                const float sc = 1.0f / (16384.0f * kK); // 2^-14 and the FFT's 1/K, exact powers of two
                b = make_float4((float)ar[m][0] * sc, (float)ai[m][0] * sc, (float)ar[m][1] * sc,
                                (float)ai[m][1] * sc);
            }
            *reinterpret_cast<float4 *>(&rows[m][n0]) = b;
        }
    } else if constexpr (kW == kWolaSplit) {
        // Two passes of kT / 2 spectra each keep the even and odd sums within
        // the FP32 path's registers; each pass reads the kT / 2 + kP - 1
        // frames its spectra need.
        constexpr int kH = kT / 2;
#pragma unroll
        for (int half = 0; half < 2; half++) {
            const int mb = half * kH;
            float2 er[kH], ei[kH], od_r[kH], od_i[kH];
#pragma unroll
            for (int m = 0; m < kH; m++) er[m] = ei[m] = od_r[m] = od_i[m] = make_float2(0.f, 0.f);
#pragma unroll
            for (int w = mb; w < mb + kH + kP - 1; w++) {
                float2 xr, xi;
                widen4<kFpga>(x[w * (kK / 2)], xr, xi);
#pragma unroll
                for (int p = 0; p < kP; p++) {
                    const int m = w - p - mb;
                    if (m >= 0 && m < kH) {
                        if (p & 1) {
                            od_r[m] = __ffma2_rn(t[p], xr, od_r[m]);
                            od_i[m] = __ffma2_rn(t[p], xi, od_i[m]);
                        } else {
                            er[m] = __ffma2_rn(t[p], xr, er[m]);
                            ei[m] = __ffma2_rn(t[p], xi, ei[m]);
                        }
                    }
                }
            }
#pragma unroll
            for (int m = 0; m < kH; m++) {
                const float2 r = padd(er[m], od_r[m]), i = padd(ei[m], od_i[m]);
                *reinterpret_cast<float4 *>(&rows[mb + m][n0]) = make_float4(r.x, i.x, r.y, i.y);
            }
        }
    } else {
        float2 ar[kT], ai[kT];
#pragma unroll
        for (int m = 0; m < kT; m++) ar[m] = ai[m] = make_float2(0.f, 0.f);
#pragma unroll
        for (int w = 0; w < kWin; w++) {
            float2 xr, xi;
            widen4<kFpga>(x[w * (kK / 2)], xr, xi);
#pragma unroll
            for (int p = 0; p < kP; p++) {
                const int m = w - p;
                if (m >= 0 && m < kT) {
                    ar[m] = __ffma2_rn(t[p], xr, ar[m]);
                    ai[m] = __ffma2_rn(t[p], xi, ai[m]);
                }
            }
        }
#pragma unroll
        for (int m = 0; m < kT; m++) {
            float4 b;
            if (kFpga) {
                b = make_float4(fpga_round(ar[m].x), fpga_round(ai[m].x), fpga_round(ar[m].y), fpga_round(ai[m].y));
            } else {
                b = make_float4(ar[m].x, ai[m].x, ar[m].y, ai[m].y);
            }
            *reinterpret_cast<float4 *>(&rows[m][n0]) = b;
        }
    }
}

template <int kW, bool kFpga, int G>
__device__ __forceinline__ void wola_step(FrontSmemT<G> &sm, int s, int li, int n0,
                                          const typename WolaTap<kW>::type (&t)[kP])
{
    wola_rows<kW, kFpga>(sm.stage[s][li][0], &sm.buf[li * kT], n0, t);
}

// vcsbeam.h.in:453-456: (int)round(x) clipped to [-8, 7].
__device__ __forceinline__ float demote4(float x)
{
    float r = roundf(x);
    return fminf(fmaxf(r, -8.0f), 7.0f);
}

// Steps 4-5: FFT of row g = (li, m) by the 8 threads of a group, in place;
// the row then holds the shifted, scaled, (im, re)-ordered voltages at k'.
// kScale: apply the 1/K here (after FPGA rounding); without FPGA rounding the
// WOLA output already carries it (scaling by a power of two commutes exactly
// with the FFT's arithmetic).
template <bool kDemote, bool kScale>
__device__ __forceinline__ void fft_rows(float2 (*buf)[kFftRow], const float2 *tw, int tid)
{
    const int g = tid >> 3, j = tid & 7;
    float2 *row = buf[g];
    fft128_pass1<-1>(row, tw, j);
    __syncwarp();
    float2 out[2][8];
    fft128_pass2<-1>(row, j, out);
    __syncwarp();
#pragma unroll
    for (int h = 0; h < 2; h++)
#pragma unroll
        for (int k2 = 0; k2 < 8; k2++) {
            const int k = fft128_index(j, h, k2);
            const int kp = (k + kK / 2) & (kK - 1);
            const float2 X = out[h][k2];
            float vr = kScale ? X.y * (1.0f / kK) : X.y, vi = kScale ? X.x * (1.0f / kK) : X.x;
            if (kDemote) {
                vr = demote4(vr);
                vi = demote4(vi);
            }
            row[kp] = make_float2(vr, vi);
        }
}

template <bool kDemote, bool kScale, int G>
__device__ __forceinline__ void fft_step(FrontSmemT<G> &sm, int tid)
{
    fft_rows<kDemote, kScale>(sm.buf, sm.tw, tid);
}

// W128 twiddles at fft128_tw_slot(k1, j), by threads 0..127.
__device__ __forceinline__ void init_twiddles(float2 *tw, int tid)
{
    if (tid < 128) {
        const int k1 = tid >> 3, j = tid & 7;
        double sn, cs;
        sincospi((double)(j * k1) / 64.0, &sn, &cs);
        tw[fft128_tw_slot(k1, j)] = make_float2((float)cs, (float)sn);
    }
}

template <int G> __device__ __forceinline__ void init_front(FrontSmemT<G> &sm, int tid)
{
    init_twiddles(sm.tw, tid);
    if (tid == 0) {
        mbar_init(&sm.bar[0], 1);
        mbar_init(&sm.bar[1], 1);
        fence_mbar_init();
    }
}

// Taps of samples n0, n0+1: h[K P - K p - n - 1] (pfb.cpp:159).
__device__ __forceinline__ void load_taps(const int *filter, int n0, int (&hc)[2][kP])
{
#pragma unroll
    for (int q = 0; q < 2; q++)
#pragma unroll
        for (int p = 0; p < kP; p++) hc[q][p] = __ldg(filter + kK * kP - kK * p - (n0 + q) - 1);
}

// The rows of input li are written by the WOLA and transformed by the FFT in
// the same 64 threads (two warps: tid / 64 == li in both mappings), so only
// those two warps meet between the two stages (named barrier 1 + li).
__device__ __forceinline__ void input_barrier(int li)
{
    asm volatile("bar.sync %0, 64;" ::"r"(1 + li) : "memory");
}

// Wait for step `it`'s data; every thread learns whether any thread timed
// out, so the CTA leaves together. The barrier also orders the previous
// step's reads of the buffers before this step's writes.
template <int G> __device__ __forceinline__ bool wait_frames(FrontSmemT<G> &sm, int it, unsigned *status)
{
    const bool ok = mbar_wait_bounded(&sm.bar[it & 1], (it >> 1) & 1, 1u << 22);
    const int any_bad = __syncthreads_or(!ok);
    if (any_bad && threadIdx.x == 0) atomicOr(status, kErrWaitTimeout);
    return !any_bad;
}

// Before leaving early, give copies in flight a bounded chance to land.
template <int G> __device__ __forceinline__ void drain(FrontSmemT<G> &sm, int it)
{
    if (threadIdx.x == 0) mbar_wait_bounded(&sm.bar[it & 1], (it >> 1) & 1, 1u << 20);
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Beamformer back end, shared by both beamformer kernels so that they give
// identical results.
// ---------------------------------------------------------------------------
// One tile's contribution to (k', spectrum) (form_beam.cpp:174-177, 295-315):
// ex / ey = the two Jones rows wa = (w00, w01), wb = (w10, w11) times the
// tile's (Q, P) voltages; c[0..3] += ex, ey; c[4..7] += |ex|^2, |ey|^2, ex ey*;
// c[8] += |vq|^2 + |vp|^2 (the incoherent sum).
__device__ __forceinline__ void beam_accumulate(float *c, float4 wa, float4 wb, float2 vq, float2 vp)
{
    const float exr = wa.x * vq.x - wa.y * vq.y + wa.z * vp.x - wa.w * vp.y;
    const float exi = wa.x * vq.y + wa.y * vq.x + wa.z * vp.y + wa.w * vp.x;
    const float eyr = wb.x * vq.x - wb.y * vq.y + wb.z * vp.x - wb.w * vp.y;
    const float eyi = wb.x * vq.y + wb.y * vq.x + wb.z * vp.y + wb.w * vp.x;
    c[0] += exr;
    c[1] += exi;
    c[2] += eyr;
    c[3] += eyi;
    c[4] = fmaf(exr, exr, fmaf(exi, exi, c[4]));
    c[5] = fmaf(eyr, eyr, fmaf(eyi, eyi, c[5]));
    c[6] = fmaf(exr, eyr, fmaf(exi, eyi, c[6]));
    c[7] = fmaf(exi, eyr, fmaf(-exr, eyi, c[7]));
    c[8] = fmaf(vq.x, vq.x, fmaf(vq.y, vq.y, fmaf(vp.x, vp.x, fmaf(vp.y, vp.y, c[8]))));
}

// form_beam.cpp:322-338: Stokes of spectrum m (skipped past the second's
// end), e, the incoherent sum, and the running extremes for the 8-bit stage.
__device__ __forceinline__ void beam_store(const BeamArgs &a, int cc, int m, int kp, const float *c, uint32_t (&kmn)[4],
                                           uint32_t (&kmx)[4])
{
    if (m >= a.nspectra) return;
    const float bnXX = c[0] * c[0] + c[1] * c[1] - c[4];
    const float bnYY = c[2] * c[2] + c[3] * c[3] - c[5];
    const float bxr = c[0] * c[2] + c[1] * c[3] - c[6];
    const float bxi = c[1] * c[2] - c[0] * c[3] - c[7];
    float *S = a.S + cc * a.S_cc + ((long long)m * a.nstokes) * kK + kp;
    const float sv[4] = {a.invw * (bnXX + bnYY), a.invw * (bnXX - bnYY), 2.0f * a.invw * bxr,
                         -2.0f * a.invw * bxi};
    S[0] = sv[0];
    if (a.nstokes == 4) {
        S[kK] = sv[1];
        S[2 * kK] = sv[2];
        S[3 * kK] = sv[3];
    }
    if (a.st_mn) {
#pragma unroll
        for (int st = 0; st < 4; st++) {
            if (st >= a.nstokes) break;
            if (isnan(sv[st])) {
                if (m == 0) a.st_nan0[(long long)(cc * a.nstokes + st) * kK + kp] = 1u;
            } else {
                const uint32_t k = fkey(sv[st]);
                kmn[st] = min(kmn[st], k);
                kmx[st] = max(kmx[st], k);
            }
        }
    }
    if (a.e) a.e[cc * a.e_cc + (long long)m * kK + kp] = make_float4(c[0], c[1], c[2], c[3]);
    if (a.incoh) a.incoh[cc * a.inc_cc + (long long)m * kK + kp] = c[8];
}

// The row extremes for the 8-bit stage (min and max are idempotent, so a
// repeated launch over the same data leaves them unchanged).
__device__ __forceinline__ void beam_store_extremes(const BeamArgs &a, int cc, int kp, const uint32_t (&kmn)[4],
                                                    const uint32_t (&kmx)[4])
{
    if (!a.st_mn) return;
#pragma unroll
    for (int st = 0; st < 4; st++) {
        if (st >= a.nstokes) break;
        const long long r = (long long)(cc * a.nstokes + st) * kK + kp;
        if (kmn[st] != ~0u) atomicMin(&a.st_mn[r], kmn[st]);
        if (kmx[st] != 0u) atomicMax(&a.st_mx[r], kmx[st]);
    }
}

// ---------------------------------------------------------------------------
// Beamformer kernel.
// ---------------------------------------------------------------------------
// G inputs (G/2 tiles) per step, 64 G threads: G = 4 (two CTAs per SM) or
// G = 8 (one CTA of 512 threads, half the steps and block barriers per
// input). Every (k', m) is summed by one thread over the tiles in the same
// order either way, so both give identical results; the host picks by timing.
template <int kW, bool kFpga, bool kDemote, int G>
__global__ void __launch_bounds__(64 * G, G == 4 ? 2 : 1)
    beam_kernel(const BeamArgs a, const __grid_constant__ CUtensorMap wmap)
{
    constexpr int kTiles = G / 2;        // tiles per step
    constexpr int kMh = G / 2;           // threads per k' (spectra m = mh + kMh mi)
    constexpr int kMi = kT / kMh;        // spectra per thread
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    FrontSmemT<G> &sm = *reinterpret_cast<FrontSmemT<G> *>(smem_raw);
    const int tid = threadIdx.x;
    const int cc = blockIdx.y;
    const int m0 = blockIdx.x * kT;
    const int nsteps = (a.vv.ninputs + G - 1) / G;

    if (tid == 0) prefetch_tmap(&wmap);
    init_front(sm, tid);
    typename WolaTap<kW>::type tp[kP];
    const int li = tid >> 6, n0 = 2 * (tid & 63);
    {
        int hc[2][kP];
        load_taps(a.filter, n0, hc);
        make_taps<kW, kFpga>(hc, tp);
    }
    __syncthreads();
    produce_spread(sm, a.vv, cc, 0, m0, a.nspectra, &wmap, a.status);

    // beam accumulators for (k', m = mh + kMh mi)
    const int kp = tid & (kK - 1), mh = tid >> 7;
    float acc[kMi][9];
#pragma unroll
    for (int mi = 0; mi < kMi; mi++)
#pragma unroll
        for (int q = 0; q < 9; q++) acc[mi][q] = 0.f;

    for (int it = 0; it < nsteps; it++) {
        if (!wait_frames(sm, it, a.status)) {
            drain(sm, it);
            return;
        }
        // everyone has finished step it-1, so its buffers may be refilled
        if (it + 1 < nsteps) produce_spread(sm, a.vv, cc, it + 1, m0, a.nspectra, &wmap, a.status);
        wola_step<kW, kFpga>(sm, it & 1, li, n0, tp);
        input_barrier(li);
        fft_step<kDemote, kFpga>(sm, tid);
        __syncthreads();
#pragma unroll
        for (int aa = 0; aa < kTiles; aa++) {
            const int ant = it * kTiles + aa;
            if (ant >= a.nant) break;
            const float4 wa = sm.wst[it & 1][0][aa][kp];
            const float4 wb = sm.wst[it & 1][1][aa][kp];
#pragma unroll
            for (int mi = 0; mi < kMi; mi++) {
                const int m = mh + kMh * mi;
                beam_accumulate(acc[mi], wa, wb, sm.buf[(2 * aa) * kT + m][kp], sm.buf[(2 * aa + 1) * kT + m][kp]);
            }
        }
    }

    uint32_t kmn[4] = {~0u, ~0u, ~0u, ~0u}, kmx[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int mi = 0; mi < kMi; mi++) beam_store(a, cc, m0 + mh + kMh * mi, kp, acc[mi], kmn, kmx);
    beam_store_extremes(a, cc, kp, kmn, kmx);
}

// ---------------------------------------------------------------------------
// Beamformer kernel with three CTAs per SM (variant 5).
// ---------------------------------------------------------------------------
// beam_kernel<..., 4> uses 126-128 registers and 95 KB of shared memory per
// 256-thread CTA, so two CTAs (16 warps) share an SM, and its WOLA, FFT and
// barrier latencies show as idle issue slots. This shape fits three (24
// warps) with the same arithmetic in the same order (identical results):
//   * each thread's 36 beam sums stay in tensor memory between steps
//     (tcgen05.ld at the start of its beam phase, tcgen05.st at its end; one
//     128-column allocation per CTA, warps w and w + 4 sharing a lane
//     quarter at columns 0 and 64), so no register is held across steps;
//   * the taps come from shared memory each step (12 loads per thread);
//   * frames and weights are single-buffered: step it + 1's frames are copied
//     as soon as every thread has finished step it's WOLA (the block barrier
//     after the FFT) and land during its beam sums; step it's weights are
//     copied after step it's first block barrier (every thread has finished
//     step it - 1's sums) and land during its WOLA and FFT.
// 72 KB of shared memory, at most 80 registers per thread.
template <class Tap> struct TmSmem {
    char2 stage[kG][kWin][kK];             // TMA destination: frames
    float4 wst[2][kG / 2][kK];             // TMA destination: weights [row][tile][k']
    float2 buf[kG * kT][kFftRow];          // WOLA output -> FFT (in place) -> voltages
    float2 tw[128];                        // W128 twiddles
    Tap taps[kP][kK / 2];                  // per (tap, sample pair n0 / 2)
    uint64_t bar_f, bar_w;
    uint32_t tmem;
};
static_assert(offsetof(TmSmem<float2>, wst) % 128 == 0 && offsetof(TmSmem<float2>, tw) % 16 == 0,
              "TMA / vector alignment");
constexpr uint32_t kTmCols = 128;          // TMEM columns per CTA (three CTAs: 384 of 512)

// Frames of step `it` into the single stage: lane 0 of warp li (li < kG)
// copies input it * kG + li, lane 0 of warp 0 posts the byte count first
// (completing its own shortfall when frames fell outside the buffers, as
// produce_spread does).
template <class Tap>
__device__ __forceinline__ void tm_frames(TmSmem<Tap> &sm, const VoltView &vv, int cc, int it, int m0, int nspectra,
                                          unsigned *status)
{
    if ((threadIdx.x & 31) != 0) return;
    const int warp = threadIdx.x >> 5;
    if (warp >= kG) return;
    const int w_end = min(m0 + kWin, nspectra + kP - 1);
    const uint32_t per_input = (w_end - m0) * kFrameBytes;
    if (warp == 0) {
        uint32_t total = 0;
        for (int li = 0; li < kG; li++)
            if (it * kG + li < vv.ninputs) total += per_input;
        mbar_arrive_expect_tx(&sm.bar_f, total);
    }
    const int pos = it * kG + warp;
    if (pos < vv.ninputs) {
        const uint32_t issued = issue_frames(vv, cc, pos, m0, w_end, sm.stage[warp][0], &sm.bar_f, status);
        if (issued != per_input)
            asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&sm.bar_f)),
                         "r"(per_input - issued)
                         : "memory");
    }
}

// The two Jones rows of step `it`'s tiles, by lane 0 of warp kG.
template <class Tap> __device__ __forceinline__ void tm_weights(TmSmem<Tap> &sm, const CUtensorMap *wmap, int cc, int it)
{
    if (threadIdx.x != 32 * kG) return;
    constexpr uint32_t kWBytes = (kG / 2) * kK * 16;
    mbar_arrive_expect_tx(&sm.bar_w, 2 * kWBytes);
    tma_load_5d(sm.wst[0][0], wmap, 0, 0, 0, (kG / 2) * it, cc, &sm.bar_w);
    tma_load_5d(sm.wst[1][0], wmap, 0, 1, 0, (kG / 2) * it, cc, &sm.bar_w);
}

template <int kW, bool kFpga, bool kDemote>
__global__ void __launch_bounds__(kThreads, 3)
    beam_tm_kernel(const BeamArgs a, const __grid_constant__ CUtensorMap wmap)
{
    using Tap = typename WolaTap<kW>::type;
    constexpr int kTiles = kG / 2;       // tiles per step
    constexpr int kMh = kG / 2;          // threads per k' (spectra m = mh + kMh mi)
    constexpr int kMi = kT / kMh;        // spectra per thread
    static_assert(kMi * 9 == 36, "36 beam sums per thread");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    TmSmem<Tap> &sm = *reinterpret_cast<TmSmem<Tap> *>(smem_raw);
    const int tid = threadIdx.x, warp = tid >> 5;
    const int cc = blockIdx.y;
    const int m0 = blockIdx.x * kT;
    const int nsteps = (a.vv.ninputs + kG - 1) / kG;
    const int li = tid >> 6, n0 = 2 * (tid & 63);

    if (tid == 0) prefetch_tmap(&wmap);
    init_twiddles(sm.tw, tid);
    if (tid < kK / 2) {
        int hc[2][kP];
        load_taps(a.filter, n0, hc);
        Tap t[kP];
        make_taps<kW, kFpga>(hc, t);
#pragma unroll
        for (int p = 0; p < kP; p++) sm.taps[p][tid] = t[p];
    }
    if (tid == 0) {
        mbar_init(&sm.bar_f, 1);
        mbar_init(&sm.bar_w, 1);
        fence_mbar_init();
    }
    if (warp == 0) {
        tmem_alloc(&sm.tmem, kTmCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    // this thread's 36 sums: lane 32 (warp % 4) + lane, columns 64 (warp / 4) ..
    const uint32_t tacc = sm.tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)(64 * (warp >> 2));
    if (nsteps > 0) {
        tm_frames(sm, a.vv, cc, 0, m0, a.nspectra, a.status);
        tm_weights(sm, &wmap, cc, 0);
    }

    const int kp = tid & (kK - 1), mh = tid >> 7;
    bool wbad = false;                   // a weights wait gave up (leave at the next step's barrier)
    int it = 0;
    for (; it < nsteps; it++) {
        // step it's frames have landed and every thread has finished step it - 1
        const bool got = mbar_wait_bounded(&sm.bar_f, it & 1, 1u << 22);
        if (__syncthreads_or(!got || wbad)) break;
        if (it > 0) tm_weights(sm, &wmap, cc, it);
        {
            Tap t[kP];
#pragma unroll
            for (int p = 0; p < kP; p++) t[p] = sm.taps[p][tid & (kK / 2 - 1)];
            wola_rows<kW, kFpga>(sm.stage[li][0], &sm.buf[li * kT], n0, t);
        }
        input_barrier(li);
        fft_rows<kDemote, kFpga>(sm.buf, sm.tw, tid);
        __syncthreads();
        // every WOLA read of the stage is done: the next step's frames may land
        if (it + 1 < nsteps) tm_frames(sm, a.vv, cc, it + 1, m0, a.nspectra, a.status);
        if (!mbar_wait_bounded(&sm.bar_w, it & 1, 1u << 22)) {
            wbad = true;
            atomicOr(a.status, kErrWaitTimeout);
        }
        __syncwarp(); // the tensor-memory accesses are warp-collective
        float acc[kMi * 9];
        if (it == 0) {
#pragma unroll
            for (int q = 0; q < kMi * 9; q++) acc[q] = 0.f;
        } else {
            tmem_wait_st();
            tmem_ld36(tacc, acc);
        }
#pragma unroll
        for (int aa = 0; aa < kTiles; aa++) {
            const int ant = it * kTiles + aa;
            if (ant >= a.nant) break;
            const float4 wa = sm.wst[0][aa][kp];
            const float4 wb = sm.wst[1][aa][kp];
#pragma unroll
            for (int mi = 0; mi < kMi; mi++) {
                const int m = mh + kMh * mi;
                beam_accumulate(acc + 9 * mi, wa, wb, sm.buf[(2 * aa) * kT + m][kp], sm.buf[(2 * aa + 1) * kT + m][kp]);
            }
        }
        tmem_st36(tacc, acc);
    }

    if (it < nsteps) {
        // left early: the copies in flight (step it's frames, step it - 1's
        // weights) get a bounded chance to land before the CTA exits
        if (tid == 0) {
            atomicOr(a.status, kErrWaitTimeout);
            mbar_wait_bounded(&sm.bar_f, it & 1, 1u << 20);
            if (it > 0) mbar_wait_bounded(&sm.bar_w, (it - 1) & 1, 1u << 20);
        }
    } else {
        // a weights copy whose wait gave up in the last step may still land
        if (tid == 0 && nsteps > 0) mbar_wait_bounded(&sm.bar_w, (nsteps - 1) & 1, 1u << 20);
        __syncwarp();
        float acc[kMi * 9];
        if (nsteps == 0) {
#pragma unroll
            for (int q = 0; q < kMi * 9; q++) acc[q] = 0.f;
        } else {
            tmem_wait_st();
            tmem_ld36(tacc, acc);
        }
        uint32_t kmn[4] = {~0u, ~0u, ~0u, ~0u}, kmx[4] = {0u, 0u, 0u, 0u};
#pragma unroll
        for (int mi = 0; mi < kMi; mi++) beam_store(a, cc, m0 + mh + kMh * mi, kp, acc + 9 * mi, kmn, kmx);
        beam_store_extremes(a, cc, kp, kmn, kmx);
    }
    __syncwarp();
    tmem_wait_st();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(sm.tmem, kTmCols);
}

// ---------------------------------------------------------------------------
// Warp-specialised beamformer kernel (variant 3, selected only when forced
// with vgb_pfb_variant(3): on a GB300 it took 26.0 ms per data-second of the
// full band against beam_kernel<..., 4>'s 21.5 ms -- one 416-thread CTA per
// SM, about three warps per scheduler, hides the WOLA's and FFT's latencies
// worse than two 256-thread CTAs do, and the double-buffered rows leave no
// shared memory for a second CTA). The same arithmetic as
// beam_kernel<..., 4> with the roles split across warps and no block-wide
// barrier inside the loop. One CTA per SM of 416 threads:
//   warps 0-7  front: WOLA + FFT of the step's four inputs (two warps per
//              input, as in beam_kernel), rows into a double-buffered array;
//   warps 8-11 back: one fine channel per thread and all 8 spectra, summing
//              tiles in order as beam_kernel does (identical results);
//   warp 12    producer: lane 0 issues the frames and the weights.
// Six mbarrier rings of two coordinate them: frames full (TMA) / empty
// (front), weights full (TMA) / empty (back), rows full (front) / empty
// (back), so the front works on step it while the back sums step it - 1.
// Every wait is bounded; a wait that gives up raises the status word and an
// abort flag the other roles see at their next wait; the two warps of an
// input agree before either leaves (they share a named barrier), and the
// producer lets its last copies land before the CTA exits.
// ---------------------------------------------------------------------------
constexpr int kWsFront = 64 * kG;               // 256
constexpr int kWsBack = kK;                     // 128
constexpr int kWsThreads = kWsFront + kWsBack + 32;

struct WsSmem {
    char2 stage[2][kG][kWin][kK];               // frames (TMA)
    float4 wst[2][2][kG / 2][kK];               // weights (TMA): [stage][row][tile][k']
    float2 buf[2][kG * kT][kFftRow];            // rows: front -> back, double-buffered
    float2 tw[128];
    uint64_t ffull[2], fempty[2], wfull[2], wempty[2], rfull[2], rempty[2];
    int abort;
};
static_assert(offsetof(WsSmem, wst) % 128 == 0 && offsetof(WsSmem, tw) % 16 == 0, "TMA / vector alignment");

__device__ __forceinline__ bool ws_wait(volatile int *abort, uint64_t *bar, uint32_t parity, unsigned *status)
{
    if (*abort) return false;
    if (mbar_wait_bounded(bar, parity, 1u << 22)) return true;
    *abort = 1;
    atomicOr(status, kErrWaitTimeout);
    return false;
}

// True on all 64 threads of input li's two warps if `pred` holds on any.
__device__ __forceinline__ bool pair_any(int li, bool pred)
{
    uint32_t r;
    asm volatile("{\n .reg .pred p, q;\n setp.ne.u32 p, %1, 0;\n bar.red.or.pred q, %2, 64, p;\n"
                 " selp.u32 %0, 1, 0, q;\n}\n"
                 : "=r"(r)
                 : "r"((uint32_t)pred), "r"(1 + li)
                 : "memory");
    return r != 0;
}

template <int kW, bool kFpga, bool kDemote>
__global__ void __launch_bounds__(kWsThreads, 1)
    beam_ws_kernel(const BeamArgs a, const __grid_constant__ CUtensorMap wmap)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    WsSmem &sm = *reinterpret_cast<WsSmem *>(smem_raw);
    volatile int *abort = &sm.abort;
    const int tid = threadIdx.x, lane = tid & 31;
    const int cc = blockIdx.y;
    const int m0 = blockIdx.x * kT;
    const int nsteps = (a.vv.ninputs + kG - 1) / kG;

    init_twiddles(sm.tw, tid);
    if (tid == 0) {
        for (int s = 0; s < 2; s++) {
            mbar_init(&sm.ffull[s], 1);
            mbar_init(&sm.wfull[s], 1);
            mbar_init(&sm.fempty[s], kWsFront / 32);
            mbar_init(&sm.rfull[s], kWsFront / 32);
            mbar_init(&sm.rempty[s], kWsBack / 32);
            mbar_init(&sm.wempty[s], kWsBack / 32);
        }
        sm.abort = 0;
        fence_mbar_init();
    }
    if (tid == kWsFront + kWsBack) prefetch_tmap(&wmap);
    __syncthreads();

    if (tid >= kWsFront + kWsBack) {
        // ---- producer ----
        int last_it_f = -1, last_it_w = -1; // the last steps whose frames / weights were issued
        if (lane == 0) {
            constexpr uint32_t kWBytes = (kG / 2) * kK * 16;
            for (int it = 0; it < nsteps; it++) {
                const int s = it & 1, k = it >> 1;
                if (k > 0 && !ws_wait(abort, &sm.fempty[s], (k - 1) & 1, a.status)) break;
                const int w_end = min(m0 + kWin, a.nspectra + kP - 1);
                const uint32_t per_input = (w_end - m0) * kFrameBytes;
                uint32_t total = 0;
                for (int li = 0; li < kG; li++)
                    if (it * kG + li < a.vv.ninputs) total += per_input;
                mbar_arrive_expect_tx(&sm.ffull[s], total);
                for (int li = 0; li < kG; li++) {
                    const int pos = it * kG + li;
                    if (pos >= a.vv.ninputs) break;
                    const uint32_t got =
                        issue_frames(a.vv, cc, pos, m0, w_end, sm.stage[s][li][0], &sm.ffull[s], a.status);
                    if (got != per_input)
                        asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&sm.ffull[s])),
                                     "r"(per_input - got)
                                     : "memory");
                }
                last_it_f = it;
                if (k > 0 && !ws_wait(abort, &sm.wempty[s], (k - 1) & 1, a.status)) break;
                mbar_arrive_expect_tx(&sm.wfull[s], 2 * kWBytes);
                tma_load_5d(sm.wst[s][0][0], &wmap, 0, 0, 0, (kG / 2) * it, cc, &sm.wfull[s]);
                tma_load_5d(sm.wst[s][1][0], &wmap, 0, 1, 0, (kG / 2) * it, cc, &sm.wfull[s]);
                last_it_w = it;
            }
        }
        __syncthreads();
        // after an abort, let the copies this CTA issued land before it exits
        // (the two most recent steps' copies, one per stage, may be in flight)
        if (lane == 0 && *abort) {
            for (int it = max(0, last_it_f - 1); it <= last_it_f; it++)
                mbar_wait_bounded(&sm.ffull[it & 1], (it >> 1) & 1, 1u << 20);
            for (int it = max(0, last_it_w - 1); it <= last_it_w; it++)
                mbar_wait_bounded(&sm.wfull[it & 1], (it >> 1) & 1, 1u << 20);
        }
        return;
    }
    if (tid < kWsFront) {
        // ---- front: WOLA + FFT of input li ----
        typename WolaTap<kW>::type tp[kP];
        const int li = tid >> 6, n0 = 2 * (tid & 63);
        {
            int hc[2][kP];
            load_taps(a.filter, n0, hc);
            make_taps<kW, kFpga>(hc, tp);
        }
        for (int it = 0; it < nsteps; it++) {
            const int s = it & 1, k = it >> 1;
            bool ok = ws_wait(abort, &sm.ffull[s], k & 1, a.status);
            if (ok && k > 0) ok = ws_wait(abort, &sm.rempty[s], (k - 1) & 1, a.status);
            if (pair_any(li, !ok)) break;
            wola_rows<kW, kFpga>(sm.stage[s][li][0], &sm.buf[s][li * kT], n0, tp);
            __syncwarp();
            if (lane == 0) mbar_arrive(&sm.fempty[s]);
            input_barrier(li);
            fft_rows<kDemote, kFpga>(sm.buf[s], sm.tw, tid);
            __syncwarp();
            if (lane == 0) mbar_arrive(&sm.rfull[s]);
        }
        __syncthreads();
        return;
    }
    // ---- back: fine channel kp, all kT spectra ----
    const int kp = tid - kWsFront;
    float acc[kT][9];
#pragma unroll
    for (int m = 0; m < kT; m++)
#pragma unroll
        for (int q = 0; q < 9; q++) acc[m][q] = 0.f;
    for (int it = 0; it < nsteps; it++) {
        const int s = it & 1, k = it >> 1;
        bool ok = ws_wait(abort, &sm.rfull[s], k & 1, a.status);
        if (ok) ok = ws_wait(abort, &sm.wfull[s], k & 1, a.status);
        if (!__all_sync(0xffffffffu, ok)) break; // the warp leaves together (it meets at __syncwarp below)
#pragma unroll
        for (int aa = 0; aa < kG / 2; aa++) {
            const int ant = it * (kG / 2) + aa;
            if (ant >= a.nant) break;
            const float4 wa = sm.wst[s][0][aa][kp];
            const float4 wb = sm.wst[s][1][aa][kp];
#pragma unroll
            for (int m = 0; m < kT; m++)
                beam_accumulate(acc[m], wa, wb, sm.buf[s][(2 * aa) * kT + m][kp], sm.buf[s][(2 * aa + 1) * kT + m][kp]);
        }
        __syncwarp();
        if (lane == 0) {
            mbar_arrive(&sm.rempty[s]);
            mbar_arrive(&sm.wempty[s]);
        }
    }
    __syncthreads();
    if (*abort) return;
    uint32_t kmn[4] = {~0u, ~0u, ~0u, ~0u}, kmx[4] = {0u, 0u, 0u, 0u};
#pragma unroll
    for (int m = 0; m < kT; m++) beam_store(a, cc, m0 + m, kp, acc[m], kmn, kmx);
    beam_store_extremes(a, cc, kp, kmn, kmx);
}

// ---------------------------------------------------------------------------
// PFB-only kernel: packed legacy-order output (pfb.cpp:297-343).
// ---------------------------------------------------------------------------
template <int kW, bool kFpga, bool kDemote>
__global__ void __launch_bounds__(kThreads, 2) pack_kernel(const PackArgs a)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    FrontSmem &sm = *reinterpret_cast<FrontSmem *>(smem_raw);
    const int tid = threadIdx.x;
    const int cc = blockIdx.y;
    const int m0 = blockIdx.x * kT;
    const int I = a.vv.ninputs;
    const int nsteps = (I + kG - 1) / kG;

    // Inputs are taken in the order of their output columns (inv[col] = the
    // input written there), so each step fills kG adjacent columns of every
    // (spectrum, channel) row: one 4-byte store in the 4-bit mode, 64
    // contiguous bytes in the complex-double mode. The per-input results do
    // not depend on the order.
    int *inv = reinterpret_cast<int *>(smem_raw + sizeof(FrontSmem));
    for (int j = tid; j < I; j += kThreads) inv[j] = -1;
    __syncthreads();
    for (int i = tid; i < I; i += kThreads) {
        const int io = __ldg(a.i_idx + i);
        if (io >= 0 && io < I) inv[io] = i;
    }
    init_front(sm, tid);
    typename WolaTap<kW>::type tp[kP];
    const int li = tid >> 6, n0 = 2 * (tid & 63);
    {
        int hc[2][kP];
        load_taps(a.filter, n0, hc);
        make_taps<kW, kFpga>(hc, tp);
    }
    __syncthreads();
    // i_idx must be a permutation of the inputs: a column nobody writes means
    // it is not (out of range or repeated)
    int unset = 0;
    for (int j = tid; j < I; j += kThreads) unset |= inv[j] < 0;
    if (__syncthreads_or(unset)) {
        if (tid == 0) atomicOr(a.status, kErrBadInput);
        return;
    }
    if (tid < 32) produce(sm, a.vv, cc, 0, m0, a.nspectra, nullptr, a.status, inv);

    const bool int4 = (a.flags & VGB_PFB_COMPLEX_INT4) != 0;
    const bool imag_first = (a.flags & VGB_PFB_IMAG_PART_FIRST) != 0;
    const int kp = tid & (kK - 1), mh = tid >> 7;
    // 4-bit mode with 16-byte stores: the last four steps' words of each of
    // the thread's spectra, oldest in .x, written together every fourth step
    uint4 held[kT / 2];
#pragma unroll
    for (int mi = 0; mi < kT / 2; mi++) held[mi] = make_uint4(0u, 0u, 0u, 0u);
    for (int it = 0; it < nsteps; it++) {
        if (!wait_frames(sm, it, a.status)) {
            drain(sm, it);
            return;
        }
        if (tid < 32 && it + 1 < nsteps) produce(sm, a.vv, cc, it + 1, m0, a.nspectra, nullptr, a.status, inv);
        wola_step<kW, kFpga>(sm, it & 1, li, n0, tp);
        input_barrier(li);
        fft_step<kDemote, kFpga>(sm, tid);
        __syncthreads();
        const int col0 = it * kG;              // the step's first output column
        const int ncol = min(kG, I - col0);
        if (!int4) {
            // complex double: four adjacent threads write one (spectrum,
            // channel) row's 64 contiguous bytes, so each warp store fills
            // whole sectors
#pragma unroll 4
            for (int e = 0; e < kT * kK * kG / kThreads; e++) {
                const int idx = e * kThreads + tid;
                const int r = idx & (kG - 1), kc = (idx / kG) % kK, ml = idx / (kG * kK);
                const int m = m0 + ml;
                if (r >= ncol || m >= a.nspectra) continue;
                const float2 v = sm.buf[r * kT + ml][kc];
                const float hi = imag_first ? v.y : v.x;
                const float lo = imag_first ? v.x : v.y;
                static_cast<double2 *>(a.out)[cc * a.out_cc + ((long long)m * kK + kc) * I + col0 + r] =
                    make_double2((double)hi, (double)lo);
            }
            continue;
        }
#pragma unroll
        for (int mi = 0; mi < kT / 2; mi++) {
            const int ml = mh + 2 * mi;
            const int m = m0 + ml;
            if (m >= a.nspectra) continue;
            const long long o = cc * a.out_cc + ((long long)m * kK + kp) * I + col0;
            uint32_t word = 0;
#pragma unroll
            for (int r = 0; r < kG; r++) {
                if (r >= ncol) break;
                // buf holds (im, re)/K: the reference's default output order
                const float2 v = sm.buf[r * kT + ml][kp];
                const float hi = imag_first ? v.y : v.x; // first (high / .x) component
                const float lo = imag_first ? v.x : v.y;
                const int h4 = (int)hi & 0xF, l4 = (int)lo & 0xF;
                const uint32_t b = (uint32_t)((h4 << 4) | l4);
                if (a.word_stores) word |= b << (8 * r);
                else static_cast<uint8_t *>(a.out)[o + r] = (uint8_t)b;
            }
            if (a.vec_stores) {
                // I is a multiple of 16, so the steps come in whole groups of
                // four and every fourth step completes 16 aligned columns
                held[mi] = make_uint4(held[mi].y, held[mi].z, held[mi].w, word);
                if ((it & 3) == 3) *reinterpret_cast<uint4 *>(static_cast<uint8_t *>(a.out) + o - 12) = held[mi];
            } else if (a.word_stores) {
                *reinterpret_cast<uint32_t *>(static_cast<uint8_t *>(a.out) + o) = word;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
template <int G = kG> static size_t front_smem() { return sizeof(FrontSmemT<G>); }

template <int G = kG, class K> static int prep(K kern)
{
    return check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)front_smem<G>()),
                      "cudaFuncSetAttribute(front smem)");
}

// Pick the template instance for (WOLA arithmetic, FPGA rounding, 4-bit
// demotion). The split sum is built for the unrounded mode only; a request
// for it with FPGA rounding takes the int32 sums (identical results).
template <template <int, bool, bool> class Sel, class Args>
static int dispatch(const Args &a, dim3 grid, int wola, bool fpga, bool demote, cudaStream_t st)
{
    if (wola == kWolaSplit && fpga) wola = kWolaInt32;
    if (wola == kWolaFp32) {
        const int sel = (fpga ? 2 : 0) | (demote ? 1 : 0);
        switch (sel) {
        case 0: return Sel<kWolaFp32, false, false>::run(a, grid, st);
        case 1: return Sel<kWolaFp32, false, true>::run(a, grid, st);
        case 2: return Sel<kWolaFp32, true, false>::run(a, grid, st);
        default: return Sel<kWolaFp32, true, true>::run(a, grid, st);
        }
    }
    if (wola == kWolaSplit)
        return demote ? Sel<kWolaSplit, false, true>::run(a, grid, st) : Sel<kWolaSplit, false, false>::run(a, grid, st);
    const int sel = (fpga ? 2 : 0) | (demote ? 1 : 0);
    switch (sel) {
    case 0: return Sel<kWolaInt32, false, false>::run(a, grid, st);
    case 1: return Sel<kWolaInt32, false, true>::run(a, grid, st);
    case 2: return Sel<kWolaInt32, true, false>::run(a, grid, st);
    default: return Sel<kWolaInt32, true, true>::run(a, grid, st);
    }
}

// Process-wide switches, read and written from any host thread.
static std::atomic<int> g_pfb_variant{0}; // 0: autotuned; else the forced variant (3, 4, 5 or 8)
static std::atomic<int> g_pfb_last{0};    // inputs per step of the last fused launch

template <int A, bool B, bool C> struct BeamSel {
    static int run_g(const BeamArgs &a, dim3 grid, cudaStream_t st, int g)
    {
        CUtensorMap wmap;
        int rc = make_tmap_beam_weights(&wmap, a.W, a.nant, (int)grid.y, a.W_cc, (g == 3 || g == 5) ? kG / 2 : g / 2);
        if (rc) return rc;
        g_pfb_last = g;
        if (g == 5) {
            auto kern = beam_tm_kernel<A, B, C>;
            constexpr int kSmem = (int)sizeof(TmSmem<typename WolaTap<A>::type>);
            if ((rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmem),
                                 "cudaFuncSetAttribute(tm smem)")))
                return rc;
            // three CTAs' shared memory per SM
            if ((rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100),
                                 "cudaFuncSetAttribute(tm carveout)")))
                return rc;
            kern<<<grid, kThreads, kSmem, st>>>(a, wmap);
        } else if (g == 3) {
            auto kern = beam_ws_kernel<A, B, C>;
            if ((rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                      (int)sizeof(WsSmem)),
                                 "cudaFuncSetAttribute(ws smem)")))
                return rc;
            kern<<<grid, kWsThreads, sizeof(WsSmem), st>>>(a, wmap);
        } else if (g == 8) {
            if ((rc = prep<8>(beam_kernel<A, B, C, 8>))) return rc;
            beam_kernel<A, B, C, 8><<<grid, 512, front_smem<8>(), st>>>(a, wmap);
        } else {
            if ((rc = prep<4>(beam_kernel<A, B, C, 4>))) return rc;
            beam_kernel<A, B, C, 4><<<grid, 256, front_smem<4>(), st>>>(a, wmap);
        }
        return check_launch("beam_kernel");
    }
    // Inputs per step for this shape: timed once per shape (one warm-up and
    // two timed launches of each variant with CUDA events on the caller's
    // stream; the outputs are the same either way) and cached. While the
    // stream is being captured the cached choice is used if known, else 4.
    static int run(const BeamArgs &a, dim3 grid, cudaStream_t st)
    {
        if (const int forced = g_pfb_variant.load()) return run_g(a, grid, st, forced);
        static std::mutex mu;
        static std::map<std::tuple<int, int, int, int, int, bool, bool>, int> cache;
        const auto key = std::make_tuple((int)grid.x, (int)grid.y, a.vv.ninputs, a.nant, a.nstokes, a.e != nullptr,
                                         a.incoh != nullptr);
        {
            std::lock_guard<std::mutex> lk(mu);
            auto it = cache.find(key);
            if (it != cache.end()) return run_g(a, grid, st, it->second);
        }
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        cudaStreamIsCapturing(st, &cs);
        if (cs != cudaStreamCaptureStatusNone) return run_g(a, grid, st, 4);
        cudaEvent_t e0, e1;
        int rc = check_cuda(cudaEventCreate(&e0), "cudaEventCreate");
        if (!rc) rc = check_cuda(cudaEventCreate(&e1), "cudaEventCreate");
        float best = 0.f;
        int pick = 4;
        for (int g : {4, 8, 5}) { // variant 3 measured slower on every shape tried; forced only
            if (rc) break;
            rc = run_g(a, grid, st, g);
            if (!rc) rc = check_cuda(cudaEventRecord(e0, st), "cudaEventRecord");
            for (int r = 0; r < 2 && !rc; r++) rc = run_g(a, grid, st, g);
            if (!rc) rc = check_cuda(cudaEventRecord(e1, st), "cudaEventRecord");
            if (!rc) rc = check_cuda(cudaEventSynchronize(e1), "cudaEventSynchronize");
            float ms = 0.f;
            if (!rc) rc = check_cuda(cudaEventElapsedTime(&ms, e0, e1), "cudaEventElapsedTime");
            if (!rc && (g == 4 || ms < best)) {
                best = ms;
                pick = g;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc) return rc;
        {
            std::lock_guard<std::mutex> lk(mu);
            cache[key] = pick;
        }
        return run_g(a, grid, st, pick);
    }
};

template <int A, bool B, bool C> struct PackSel {
    static int run(const PackArgs &a, dim3 grid, cudaStream_t st)
    {
        const size_t smem = front_smem<kG>() + sizeof(int) * (size_t)kPackMaxInputs;
        int rc = check_cuda(cudaFuncSetAttribute(pack_kernel<A, B, C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)smem),
                            "cudaFuncSetAttribute(pack smem)");
        if (rc) return rc;
        pack_kernel<A, B, C><<<grid, kThreads, smem, st>>>(a);
        return check_launch("pack_kernel");
    }
};

int pfb_variant_last() { return g_pfb_last; }

int pfb_variant(int g)
{
    if (g != 0 && g != 3 && g != 4 && g != 5 && g != 8) return -1;
    return g_pfb_variant.exchange(g);
}

// WOLA arithmetic requested by the pfb_flags bits: VGB_WOLA_INT32, else
// VGB_WOLA_FP32, else VGB_WOLA_FP32_SPLIT, else int32.
static int wola_mode(unsigned flags)
{
    if (flags & VGB_WOLA_INT32) return kWolaInt32;
    if (flags & VGB_WOLA_FP32) return kWolaFp32;
    if (flags & VGB_WOLA_FP32_SPLIT) return kWolaSplit;
    return kWolaInt32;
}

int launch_beam(const BeamArgs &a, int ncc, unsigned flags, cudaStream_t st)
{
    if (a.nspectra <= 0 || ncc <= 0) return VGB_SUCCESS;
    dim3 grid((a.nspectra + kT - 1) / kT, ncc);
    return dispatch<BeamSel>(a, grid, wola_mode(flags), (flags & VGB_PFB_EMULATE_FPGA) != 0,
                             (flags & VGB_PFB_COMPLEX_INT4) != 0, st);
}

int launch_pack(const PackArgs &a, int ncc, unsigned flags, cudaStream_t st)
{
    if (a.nspectra <= 0 || ncc <= 0) return VGB_SUCCESS;
    dim3 grid((a.nspectra + kT - 1) / kT, ncc);
    return dispatch<PackSel>(a, grid, wola_mode(flags), (flags & VGB_PFB_EMULATE_FPGA) != 0,
                             (flags & VGB_PFB_COMPLEX_INT4) != 0, st);
}

// Gather the last P frames of a second into the compact history layout
// [cc][input][P][K] char2 that the next second reads (the reference keeps a
// whole voltage block for this, buffer.c:106-124; only 12 frames are used).
__global__ void hist_gather_kernel(const char2 *cur, long long cur_block, long long cc_cur, int ninputs,
                                   int nblocks, char2 *hist, long long cc_hist)
{
    const int cc = blockIdx.z, i = blockIdx.y;
    const int idx = blockIdx.x * blockDim.x + threadIdx.x; // 16-byte word within the 3072 bytes
    if (idx >= kHistFrames * kK / 8) return;
    const long long last_frame = (long long)nblocks * kFramesPerBlock - kHistFrames;
    const int b = (int)(last_frame / kFramesPerBlock), f = (int)(last_frame % kFramesPerBlock);
    const uint4 *src = reinterpret_cast<const uint4 *>(cur + cc * cc_cur + b * cur_block + (long long)i * kVSPVB +
                                                       (long long)f * kK);
    uint4 *dst = reinterpret_cast<uint4 *>(hist + cc * cc_hist + (long long)i * kHistFrames * kK);
    dst[idx] = src[idx];
}

int launch_hist_gather(const char2 *cur, long long cur_block, long long cc_cur, int ninputs, int nblocks, int ncc,
                       char2 *hist, long long cc_hist, cudaStream_t st)
{
    dim3 grid(1, ninputs, ncc);
    hist_gather_kernel<<<grid, kHistFrames * kK / 8, 0, st>>>(cur, cur_block, cc_cur, ninputs, nblocks, hist,
                                                              cc_hist);
    return check_launch("hist_gather_kernel");
}

} // namespace vgb
