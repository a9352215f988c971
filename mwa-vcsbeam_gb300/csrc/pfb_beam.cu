// Fused forward fine PFB and tied-array / incoherent beamformer for MWAX
// voltages, GB300 (sm_103a).
//
// One CTA owns a tile of T = 16 consecutive fine spectra of one coarse
// channel and walks the RF inputs four at a time (two tiles x two pols). Per
// step:
//   1. the TMA unit copies the 27 voltage frames (T + 11) each input needs
//      into shared memory (1-D bulk copies, double-buffered with mbarriers:
//      the next step's frames land while this step computes);
//   2. weighted overlap-add, exactly (pfb.cpp:121-179), one thread per
//      (input, sample-in-frame) with its 12 filter taps in registers;
//   3. the FPGA rounding (pfb.cpp:202-242) or the 2^-14 scaling
//      (pfb.cpp:256-268);
//   4. a 128-point FFT (16 x 8, eight threads per transform);
//   5. fftshift, 1/K, the (im, re) ordering of pfb.cpp:328-339 and, for the
//      4-bit mode, the round-and-clip of vcsbeam.h.in:453-457;
//   6. beamformer back end: ex/ey = (phi J^-1)[a][c] v (form_beam.cpp:174-177,
//      295-296) accumulated over tiles with the autocorrelation terms
//      (form_beam.cpp:298-315) and the incoherent sum; or the PFB-only back
//      end, which writes the packed legacy-order output (pfb.cpp:316-340).
// The fine-channel voltages never reach HBM on the beamformer path.
#include "vgb_launch.cuh"

namespace vgb {

constexpr int kT = 16;                     // spectra per CTA
constexpr int kG = 4;                      // inputs per step
constexpr int kThreads = 512;              // = kG * kK
constexpr int kWin = kT + kP - 1;          // frames per input per step
constexpr int kFrameBytes = kK * 2;        // 256
constexpr int kStageBytes = kG * kWin * kFrameBytes;
constexpr int kXRow = kK + 8;              // bufX row (float2), padded

struct FrontSmem {
    char2 stage[2][kG][kWin][kK];          // TMA destinations
    float2 bufB[kG * kT][kFftRow];         // WOLA output / FFT work rows
    float2 bufX[kG * kT][kXRow];           // fine-channel voltages (shifted order)
    float2 tw[128];                        // W128 twiddles, [k1][j]
    uint64_t bar[2];
};

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

// Producer: one thread queues the frames of step `it` into stage `s`.
__device__ __forceinline__ void produce(FrontSmem &sm, const VoltView &vv, int cc, int it, int m0,
                                       int nspectra, unsigned *status)
{
    const int s = it & 1;
    const int w_end = min(m0 + kWin, nspectra + kP - 1);
    // Count first so expect_tx is armed before any copy can complete.
    uint32_t total = 0;
    for (int li = 0; li < kG; li++) {
        const int i = it * kG + li;
        if (i < vv.ninputs) total += (w_end - m0) * kFrameBytes;
    }
    mbar_arrive_expect_tx(&sm.bar[s], total);
    uint32_t issued = 0;
    for (int li = 0; li < kG; li++) {
        const int i = it * kG + li;
        if (i < vv.ninputs) issued += issue_frames(vv, cc, i, m0, w_end, sm.stage[s][li][0], &sm.bar[s], status);
    }
    if (issued != total) {
        // Some frames were outside the buffers: complete the remaining
        // transaction count so consumers are not left waiting; the status
        // word already records the error.
        asm volatile("mbarrier.complete_tx.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&sm.bar[s])),
                     "r"(total - issued)
                     : "memory");
    }
}

// char2 (as a 16-bit word) -> two exact floats, via the 2^23 magic number.
__device__ __forceinline__ void c2_to_f(uint32_t v, float &re, float &im)
{
    const uint32_t u = v ^ 0x8080u; // offset binary: byte + 128
    re = __uint_as_float(0x4B000000u | (u & 0xFFu)) - 8388736.0f;
    im = __uint_as_float(0x4B000000u | ((u >> 8) & 0xFFu)) - 8388736.0f;
}
__device__ __forceinline__ void c2_to_i(uint32_t v, int &re, int &im)
{
    re = (int)(signed char)(v & 0xFFu);
    im = (int)(signed char)((v >> 8) & 0xFFu);
}

// ---------------------------------------------------------------------------
// Steps 2-3: weighted overlap-add for thread (li, n) into bufB rows.
// kInt32: accumulate in int32 (any filter); else FP32, exact when every
// partial sum stays below 2^24 (the host checks the filter).
// ---------------------------------------------------------------------------
template <bool kInt32, bool kFpga>
__device__ __forceinline__ void wola_step(FrontSmem &sm, int s, int li, int n, const int (&hc)[kP])
{
    const uint16_t *x = reinterpret_cast<const uint16_t *>(sm.stage[s][li][0]) + n;
    if (kInt32) {
        int ar[kT], ai[kT];
#pragma unroll
        for (int m = 0; m < kT; m++) ar[m] = ai[m] = 0;
#pragma unroll
        for (int w = 0; w < kWin; w++) {
            int xr, xi;
            c2_to_i(x[w * kK], xr, xi);
#pragma unroll
            for (int p = 0; p < kP; p++) {
                const int m = w - p;
                if (m >= 0 && m < kT) {
                    ar[m] += hc[p] * xr;
                    ai[m] += hc[p] * xi;
                }
            }
        }
#pragma unroll
        for (int m = 0; m < kT; m++) {
            float2 b;
            if (kFpga) {
                int X = ar[m], Y = ai[m];
                if (X > 0) X += 0x2000;
                if (Y > 0) Y += 0x2000;
                b = make_float2((float)(X >> 14), (float)(Y >> 14));
            } else {
                b = make_float2((float)ar[m] * (1.0f / 16384.0f), (float)ai[m] * (1.0f / 16384.0f));
            }
            sm.bufB[li * kT + m][n] = b;
        }
    } else {
        float hf[kP];
#pragma unroll
        for (int p = 0; p < kP; p++) hf[p] = (float)hc[p];
        float ar[kT], ai[kT];
#pragma unroll
        for (int m = 0; m < kT; m++) ar[m] = ai[m] = 0.f;
#pragma unroll
        for (int w = 0; w < kWin; w++) {
            float xr, xi;
            c2_to_f(x[w * kK], xr, xi);
#pragma unroll
            for (int p = 0; p < kP; p++) {
                const int m = w - p;
                if (m >= 0 && m < kT) {
                    ar[m] = fmaf(hf[p], xr, ar[m]);
                    ai[m] = fmaf(hf[p], xi, ai[m]);
                }
            }
        }
#pragma unroll
        for (int m = 0; m < kT; m++) {
            float2 b;
            if (kFpga) {
                // (X + 0x2000) >> 14 for X > 0, X >> 14 otherwise; exact in
                // FP32 because |X| < 2^24.
                const float X = ar[m] * (1.0f / 16384.0f), Y = ai[m] * (1.0f / 16384.0f);
                b = make_float2(ar[m] > 0.f ? floorf(X + 0.5f) : floorf(X),
                                ai[m] > 0.f ? floorf(Y + 0.5f) : floorf(Y));
            } else {
                b = make_float2(ar[m] * (1.0f / 16384.0f), ai[m] * (1.0f / 16384.0f));
            }
            sm.bufB[li * kT + m][n] = b;
        }
    }
}

// vcsbeam.h.in:453-456: (int)round(x) clipped to [-8, 7].
__device__ __forceinline__ float demote4(float x)
{
    float r = roundf(x);
    return fminf(fmaxf(r, -8.0f), 7.0f);
}

// Steps 4-5: FFT of row (li, m) by the 8 threads of a group; writes the
// shifted, scaled, (im, re)-ordered voltages into bufX.
template <bool kDemote>
__device__ __forceinline__ void fft_step(FrontSmem &sm, int tid)
{
    const int g = tid >> 3, j = tid & 7;
    float2 *row = sm.bufB[g];
    fft128_pass1<-1>(row, sm.tw, j);
    __syncwarp();
    float2 out[2][8];
    fft128_pass2<-1>(row, j, out);
#pragma unroll
    for (int h = 0; h < 2; h++)
#pragma unroll
        for (int k2 = 0; k2 < 8; k2++) {
            const int k = 2 * j + h + 16 * k2;
            const int kp = (k + kK / 2) & (kK - 1);
            const float2 X = out[h][k2];
            float vr = X.y * (1.0f / kK), vi = X.x * (1.0f / kK);
            if (kDemote) {
                vr = demote4(vr);
                vi = demote4(vi);
            }
            sm.bufX[g][kp] = make_float2(vr, vi);
        }
}

__device__ __forceinline__ void init_front(FrontSmem &sm, int tid)
{
    if (tid < 128) {
        const int k1 = tid >> 3, j = tid & 7;
        double sn, cs;
        sincospi((double)(j * k1) / 64.0, &sn, &cs);
        sm.tw[tid] = make_float2((float)cs, (float)sn);
    }
    if (tid == 0) {
        mbar_init(&sm.bar[0], 1);
        mbar_init(&sm.bar[1], 1);
        fence_mbar_init();
    }
}

__device__ __forceinline__ void load_taps(const int *filter, int n, int (&hc)[kP])
{
#pragma unroll
    for (int p = 0; p < kP; p++) hc[p] = __ldg(filter + kK * kP - kK * p - n - 1);
}

// Wait for step `it`'s frames; every thread learns whether any thread timed
// out, so the CTA leaves together.
__device__ __forceinline__ bool wait_frames(FrontSmem &sm, int it, unsigned *status)
{
    const bool ok = mbar_wait_bounded(&sm.bar[it & 1], (it >> 1) & 1, 1u << 22);
    const int any_bad = __syncthreads_or(!ok);
    if (any_bad && threadIdx.x == 0) atomicOr(status, kErrWaitTimeout);
    return !any_bad;
}

// Before leaving early, give copies in flight a bounded chance to land.
__device__ __forceinline__ void drain(FrontSmem &sm, int it, int nsteps)
{
    if (threadIdx.x == 0) {
        mbar_wait_bounded(&sm.bar[it & 1], (it >> 1) & 1, 1u << 20);
        if (it + 1 < nsteps) mbar_wait_bounded(&sm.bar[(it + 1) & 1], ((it + 1) >> 1) & 1, 1u << 20);
    }
    __syncthreads();
}

// ---------------------------------------------------------------------------
// Beamformer kernel.
// ---------------------------------------------------------------------------

template <bool kInt32, bool kFpga, bool kDemote>
__global__ void __launch_bounds__(kThreads, 1) beam_kernel(const BeamArgs a)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    FrontSmem &sm = *reinterpret_cast<FrontSmem *>(smem_raw);
    const int tid = threadIdx.x;
    const int cc = blockIdx.y;
    const int m0 = blockIdx.x * kT;
    const int nsteps = (a.vv.ninputs + kG - 1) / kG;

    init_front(sm, tid);
    int hc[kP];
    const int n = tid & (kK - 1), li = tid >> 7;
    load_taps(a.filter, n, hc);
    __syncthreads();
    if (tid == 0) produce(sm, a.vv, cc, 0, m0, a.nspectra, a.status);

    // beam accumulators for (k', m = mq + 4 mi)
    const int kp = tid & (kK - 1), mq = tid >> 7;
    float acc[4][9];
#pragma unroll
    for (int mi = 0; mi < 4; mi++)
#pragma unroll
        for (int q = 0; q < 9; q++) acc[mi][q] = 0.f;

    const float4 *Wcc = a.W + cc * a.W_cc;
    for (int it = 0; it < nsteps; it++) {
        if (tid == 0 && it + 1 < nsteps) produce(sm, a.vv, cc, it + 1, m0, a.nspectra, a.status);
        if (!wait_frames(sm, it, a.status)) {
            drain(sm, it, nsteps);
            return;
        }
        wola_step<kInt32, kFpga>(sm, it & 1, li, n, hc);
        __syncthreads();
        fft_step<kDemote>(sm, tid);
        __syncthreads();
#pragma unroll
        for (int aa = 0; aa < 2; aa++) {
            const int ant = it * 2 + aa;
            if (ant >= a.nant) break;
            const float4 wa = __ldg(Wcc + ((long long)ant * kK + kp) * 2);
            const float4 wb = __ldg(Wcc + ((long long)ant * kK + kp) * 2 + 1);
#pragma unroll
            for (int mi = 0; mi < 4; mi++) {
                const int m = mq + 4 * mi;
                const float2 vq = sm.bufX[(2 * aa) * kT + m][kp];
                const float2 vp = sm.bufX[(2 * aa + 1) * kT + m][kp];
                const float exr = wa.x * vq.x - wa.y * vq.y + wa.z * vp.x - wa.w * vp.y;
                const float exi = wa.x * vq.y + wa.y * vq.x + wa.z * vp.y + wa.w * vp.x;
                const float eyr = wb.x * vq.x - wb.y * vq.y + wb.z * vp.x - wb.w * vp.y;
                const float eyi = wb.x * vq.y + wb.y * vq.x + wb.z * vp.y + wb.w * vp.x;
                float *c = acc[mi];
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
        }
    }

    // form_beam.cpp:322-338
#pragma unroll
    for (int mi = 0; mi < 4; mi++) {
        const int m = m0 + mq + 4 * mi;
        if (m >= a.nspectra) continue;
        const float *c = acc[mi];
        const float bnXX = c[0] * c[0] + c[1] * c[1] - c[4];
        const float bnYY = c[2] * c[2] + c[3] * c[3] - c[5];
        const float bxr = c[0] * c[2] + c[1] * c[3] - c[6];
        const float bxi = c[1] * c[2] - c[0] * c[3] - c[7];
        float *S = a.S + cc * a.S_cc + ((long long)m * a.nstokes) * kK + kp;
        S[0] = a.invw * (bnXX + bnYY);
        if (a.nstokes == 4) {
            S[kK] = a.invw * (bnXX - bnYY);
            S[2 * kK] = 2.0f * a.invw * bxr;
            S[3 * kK] = -2.0f * a.invw * bxi;
        }
        if (a.e) a.e[cc * a.e_cc + (long long)m * kK + kp] = make_float4(c[0], c[1], c[2], c[3]);
        if (a.incoh) a.incoh[cc * a.inc_cc + (long long)m * kK + kp] = c[8];
    }
}

// ---------------------------------------------------------------------------
// PFB-only kernel: packed legacy-order output (pfb.cpp:297-343).
// ---------------------------------------------------------------------------

template <bool kInt32, bool kFpga, bool kDemote>
__global__ void __launch_bounds__(kThreads, 1) pack_kernel(const PackArgs a)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    FrontSmem &sm = *reinterpret_cast<FrontSmem *>(smem_raw);
    const int tid = threadIdx.x;
    const int cc = blockIdx.y;
    const int m0 = blockIdx.x * kT;
    const int I = a.vv.ninputs;
    const int nsteps = (I + kG - 1) / kG;

    init_front(sm, tid);
    int hc[kP];
    const int n = tid & (kK - 1), li = tid >> 7;
    load_taps(a.filter, n, hc);
    __syncthreads();
    if (tid == 0) produce(sm, a.vv, cc, 0, m0, a.nspectra, a.status);

    const bool int4 = (a.flags & VGB_PFB_COMPLEX_INT4) != 0;
    const bool imag_first = (a.flags & VGB_PFB_IMAG_PART_FIRST) != 0;
    for (int it = 0; it < nsteps; it++) {
        if (tid == 0 && it + 1 < nsteps) produce(sm, a.vv, cc, it + 1, m0, a.nspectra, a.status);
        if (!wait_frames(sm, it, a.status)) {
            drain(sm, it, nsteps);
            return;
        }
        wola_step<kInt32, kFpga>(sm, it & 1, li, n, hc);
        __syncthreads();
        fft_step<kDemote>(sm, tid);
        __syncthreads();
        // thread -> (k', spectrum row) pairs; one input per pass
#pragma unroll
        for (int r = 0; r < kG; r++) {
            const int i = it * kG + r;
            if (i >= I) break;
            const int io = __ldg(a.i_idx + i);
            const int kp = tid & (kK - 1);
#pragma unroll
            for (int mi = 0; mi < kT / 4; mi++) {
                const int ml = (tid >> 7) + 4 * mi;
                const int m = m0 + ml;
                if (m >= a.nspectra) continue;
                // bufX holds (im, re)/K: the reference's default output order
                const float2 v = sm.bufX[r * kT + ml][kp];
                const float hi = imag_first ? v.y : v.x; // first (high / .x) component
                const float lo = imag_first ? v.x : v.y;
                const long long o = cc * a.out_cc + ((long long)m * kK + kp) * I + io;
                if (int4) {
                    const int h4 = (int)hi & 0xF, l4 = (int)lo & 0xF;
                    static_cast<uint8_t *>(a.out)[o] = (uint8_t)((h4 << 4) | l4);
                } else {
                    static_cast<double2 *>(a.out)[o] = make_double2((double)hi, (double)lo);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
static size_t front_smem() { return sizeof(FrontSmem); }

template <class K> static int prep(K kern)
{
    return check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)front_smem()),
                      "cudaFuncSetAttribute(front smem)");
}

// Pick the template instance for (int32 WOLA, FPGA rounding, 4-bit demotion).
template <template <bool, bool, bool> class Sel, class Args>
static int dispatch(const Args &a, dim3 grid, bool i32, bool fpga, bool demote, cudaStream_t st)
{
    const int sel = (i32 ? 4 : 0) | (fpga ? 2 : 0) | (demote ? 1 : 0);
    switch (sel) {
    case 0: return Sel<false, false, false>::run(a, grid, st);
    case 1: return Sel<false, false, true>::run(a, grid, st);
    case 2: return Sel<false, true, false>::run(a, grid, st);
    case 3: return Sel<false, true, true>::run(a, grid, st);
    case 4: return Sel<true, false, false>::run(a, grid, st);
    case 5: return Sel<true, false, true>::run(a, grid, st);
    case 6: return Sel<true, true, false>::run(a, grid, st);
    default: return Sel<true, true, true>::run(a, grid, st);
    }
}

template <bool A, bool B, bool C> struct BeamSel {
    static int run(const BeamArgs &a, dim3 grid, cudaStream_t st)
    {
        int rc = prep(beam_kernel<A, B, C>);
        if (rc) return rc;
        beam_kernel<A, B, C><<<grid, kThreads, front_smem(), st>>>(a);
        return check_launch("beam_kernel");
    }
};

template <bool A, bool B, bool C> struct PackSel {
    static int run(const PackArgs &a, dim3 grid, cudaStream_t st)
    {
        int rc = prep(pack_kernel<A, B, C>);
        if (rc) return rc;
        pack_kernel<A, B, C><<<grid, kThreads, front_smem(), st>>>(a);
        return check_launch("pack_kernel");
    }
};

int launch_beam(const BeamArgs &a, int ncc, bool int32_wola, bool fpga, bool demote, cudaStream_t st)
{
    if (a.nspectra <= 0 || ncc <= 0) return VGB_SUCCESS;
    dim3 grid((a.nspectra + kT - 1) / kT, ncc);
    return dispatch<BeamSel>(a, grid, int32_wola, fpga, demote, st);
}

int launch_pack(const PackArgs &a, int ncc, bool int32_wola, bool fpga, bool demote, cudaStream_t st)
{
    if (a.nspectra <= 0 || ncc <= 0) return VGB_SUCCESS;
    dim3 grid((a.nspectra + kT - 1) / kT, ncc);
    return dispatch<PackSel>(a, grid, int32_wola, fpga, demote, st);
}

} // namespace vgb

namespace vgb {

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
