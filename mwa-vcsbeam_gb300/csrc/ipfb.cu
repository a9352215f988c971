// Inverse (synthesis) PFB fused with VDIF quantisation, and the staged
// forward-PFB kernels behind the reference's per-stage API.
//
// Inverse PFB. The reference evaluates, per output sample n and pol
// (pfb.cpp:842-907),
//     x^[n] = 1/K sum_m f[n - mK] sum_k X_k[m] e^{2 pi i ((k + K/2) n mod K)/K}
// as 12 x 128 complex multiply-adds per sample. With n = fK + r the inner sum
// does not depend on f:
//     sum_k X_k[m] e^{2 pi i (k + K/2)(fK + r)/K} = (-1)^r IDFT(X[m])[r],
// so one 128-point inverse FFT per fine sample m and pol, reused by the 12
// frames it overlaps, followed by a 12-tap polyphase sum per output sample
// computes the same quantity with ~100x fewer operations. The tap range is
// m = f-11 .. f (floor division), which equals the reference's range for
// every n >= 12*128 and every n % 128 == 0; for the other 1,524 samples of
// the first 1,536 the reference truncates toward zero and reads outside its
// filter table (pfb.cpp:863, 884), which is not reproduced.
//
// Each output frame of 128 samples x 2 pols is one VDIF frame
// (beam_vdif.c:52-92): 32-byte header, then (re, im) int8 per (sample, pol),
// clamped to [-126, 127], rounded to nearest even, XOR 0x80
// (beam_vdif.c:29-38, 254-260).
#include "vgb_launch.cuh"

namespace vgb {

// The seconds / frame words of the header template (w0, w1) advanced by n
// frames at kVdifFramesPerSecond (nextVDIFHeader applied n times,
// beam_vdif.c:80): word `which` (0 or 1) of the result. n < 2^31, so the
// frame total (< 2^24 + 2^31) and its division by the constant stay 32-bit.
__device__ __forceinline__ uint32_t vdif_advanced_word(uint32_t w0, uint32_t w1, uint32_t n, int which)
{
    const uint32_t total = (w1 & 0xFFFFFFu) + n;
    const uint32_t sec = total / (uint32_t)kVdifFramesPerSecond;
    if (which == 0) return (w0 & 0xC0000000u) | ((w0 + sec) & 0x3FFFFFFFu);
    return (w1 & 0xFF000000u) | (total - sec * (uint32_t)kVdifFramesPerSecond);
}

constexpr int kIFT = 32;                 // frames per CTA
constexpr int kIThreads = 512;           // two halves of 256: 16 frames each in the polyphase sum

constexpr int kIRowsPad = 88;            // 2 x (kIFT + 11) = 86 rows, padded to whole warps of
                                         // 8-thread groups; ~108 KB: two CTAs per SM
static_assert(kIRowsPad >= 2 * (kIFT + kP - 1) && kIRowsPad % 4 == 0, "FFT rows");


struct IpfbSmem {
    float2 y[kIRowsPad][kFftRow];
    float2 tw[128];
};
static_assert(sizeof(float2) * kIRowsPad * kFftRow % 16 == 0, "twiddles are read 16 bytes at a time");

__global__ void __launch_bounds__(kIThreads, 2) ipfb_kernel(const IpfbArgs a)
{
    extern __shared__ __align__(16) unsigned char ism_raw[];
    IpfbSmem &sm = *reinterpret_cast<IpfbSmem *>(ism_raw);
    const int tid = threadIdx.x;
    const int job = blockIdx.y;
    const int f0 = blockIdx.x * kIFT;
    const int mlo = f0 - (kP - 1);

    if (tid < 128) {
        const int k1 = tid >> 3, j = tid & 7;
        double sn, cs;
        sincospi((double)(j * k1) / 64.0, &sn, &cs);
        sm.tw[fft128_tw_slot(k1, j)] = make_float2((float)cs, (float)sn);
    }
    // load X_k[m] for m in [f0 - 11, f0 + kIFT), de-interleaving the pols
    const float4 *e = a.e + job * a.e_job;
    const float4 *hist = a.hist ? a.hist + job * a.hist_job : nullptr;
    // asynchronous 8-byte copies, all in flight before one wait; samples with
    // no source (outside the second and its history) are zero-filled
    for (int idx = tid; idx < (kIFT + kP - 1) * kK; idx += kIThreads) {
        const int ml = idx / kK, k = idx % kK;
        const int m = mlo + ml;
        const float4 *src = e;
        uint32_t bytes = 0;
        if (m >= 0 && m < a.nsamples) {
            src = e + (long long)m * kK + k;
            bytes = 8;
        } else if (m < 0 && hist && m >= -kP) {
            src = hist + (long long)(m + kP) * kK + k;
            bytes = 8;
        }
        const float2 *s2 = reinterpret_cast<const float2 *>(src);
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(smem_u32(&sm.y[2 * ml][k])), "l"(s2),
                     "r"(bytes)
                     : "memory");
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(smem_u32(&sm.y[2 * ml + 1][k])),
                     "l"(s2 + 1), "r"(bytes)
                     : "memory");
    }
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
    __syncthreads();

    // inverse FFTs, 64 transforms per pass (whole warps past the padded rows
    // sit the last pass out), (-1)^r applied on the way out
    {
        const int g = tid >> 3, j = tid & 7;
        for (int base = 0; base < kIRowsPad; base += kIThreads / 8) {
            if (base + g >= kIRowsPad) break;
            float2 *row = sm.y[base + g];
            fft128_pass1<+1>(row, sm.tw, j);
            __syncwarp();
            float2 out[2][8];
            fft128_pass2<+1>(row, j, out);
            __syncwarp();
#pragma unroll
            for (int h = 0; h < 2; h++)
#pragma unroll
                for (int k2 = 0; k2 < 8; k2++) {
                    const int r = fft128_index(j, h, k2);
                    const float2 v = out[h][k2];
                    row[r] = (r & 1) ? make_float2(-v.x, -v.y) : v;
                }
        }
    }
    __syncthreads();

    // polyphase sum: thread (r, pol) of half h sums frames 16 h .. 16 h + 15
    const int r = (tid & 255) >> 1, pol = tid & 1, half = tid >> 8;
    float fr[kP];
#pragma unroll
    for (int p = 0; p < kP; p++) fr[p] = __ldg(a.coeffs + p * kK + r);
    const float invK = 1.0f / kK;
    float *outf = a.out_f ? a.out_f + job * a.outf_job : nullptr;
    uint8_t *vd = a.vdif ? a.vdif + job * a.vdif_job : nullptr;
    // frame headers: one word per thread (kIFT frames x 8 words = 256)
    if (vd && tid < kIFT * 8) {
        const int f = f0 + (tid >> 3), wi = tid & 7;
        if (f < a.nsamples) {
            uint32_t wv = a.hdr ? __ldg(a.hdr + job * 8 + wi) : 0u;
            if (wi < 2) {
                const uint32_t w0 = a.hdr ? __ldg(a.hdr + job * 8) : 0u;
                const uint32_t w1 = a.hdr ? __ldg(a.hdr + job * 8 + 1) : 0u;
                wv = vdif_advanced_word(w0, w1, (uint32_t)a.frame_offset + (uint32_t)f, wi);
            }
            reinterpret_cast<uint32_t *>(vd + (long long)f * 544)[wi] = wv;
        }
    }
    static_assert(kIThreads == 512 && kIFT == 32, "two halves of 16 frames");
    {
        const int chunk = 16 * half;
        float ar[16], ai[16];
#pragma unroll
        for (int q = 0; q < 16; q++) ar[q] = ai[q] = 0.f;
        // frame fl = chunk + q uses local m index (chunk + q) + 11 - p
#pragma unroll
        for (int w = 0; w < 16 + kP - 1; w++) {
            const float2 y = sm.y[2 * (chunk + w) + pol][r];
#pragma unroll
            for (int p = 0; p < kP; p++) {
                const int q = w - (kP - 1) + p;
                if (q >= 0 && q < 16) {
                    ar[q] = fmaf(fr[p], y.x, ar[q]);
                    ai[q] = fmaf(fr[p], y.y, ai[q]);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 16; q++) {
            const int f = f0 + chunk + q;
            if (f >= a.nsamples) break;
            const float xr = ar[q] * invK, xi = ai[q] * invK;
            const long long n = (long long)f * kK + r;
            if (outf) reinterpret_cast<float2 *>(outf)[n * 2 + pol] = make_float2(xr, xi);
            if (vd) {
                uint8_t *frame = vd + (long long)f * 544;
                float cr = xr > 127.f ? 127.f : xr;
                cr = cr < -126.f ? -126.f : cr;
                float ci = xi > 127.f ? 127.f : xi;
                ci = ci < -126.f ? -126.f : ci;
                const uint32_t br = ((uint32_t)__float2int_rn(cr) ^ 0x80u) & 0xFFu;
                const uint32_t bi = ((uint32_t)__float2int_rn(ci) ^ 0x80u) & 0xFFu;
                reinterpret_cast<uint16_t *>(frame + 32)[r * 2 + pol] = (uint16_t)(br | (bi << 8));
            }
        }
    }
}

int launch_ipfb(const IpfbArgs &a, int njobs, cudaStream_t st)
{
    if (a.nsamples <= 0 || njobs <= 0) return VGB_SUCCESS;
    const int smem = (int)sizeof(IpfbSmem);
    int rc = check_cuda(cudaFuncSetAttribute(ipfb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                        "cudaFuncSetAttribute(ipfb)");
    if (rc) return rc;
    dim3 grid((a.nsamples + kIFT - 1) / kIFT, njobs);
    ipfb_kernel<<<grid, kIThreads, smem, st>>>(a);
    return check_launch("ipfb_kernel");
}

// Advance each job's header template [job][8] by n frames.
__global__ void vdif_advance_kernel(uint32_t *hdr, int njobs, int n)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= njobs) return;
    uint32_t *h = hdr + j * 8;
    const uint32_t w0 = h[0], w1 = h[1];
    h[0] = vdif_advanced_word(w0, w1, (uint32_t)n, 0);
    h[1] = vdif_advanced_word(w0, w1, (uint32_t)n, 1);
}

int launch_vdif_advance(uint32_t *hdr, int njobs, int nframes, cudaStream_t st)
{
    if (njobs <= 0) return VGB_SUCCESS;
    vdif_advance_kernel<<<(njobs + 127) / 128, 128, 0, st>>>(hdr, njobs, nframes);
    return check_launch("vdif_advance_kernel");
}

// ===========================================================================
// Staged forward-PFB kernels (one reference stage each).
// ===========================================================================

// vmWOLA_kernel's result, computed directly (no memset, no atomics):
// b[m][i][n] = sum_p h[K P - K p - n - 1] x[frame m + p][n], int32.
__global__ void wola_staged_kernel(VoltView vv, const int *filter, int nspectra, int2 *b)
{
    const int n = threadIdx.x;
    const int i = blockIdx.y;
    const int m = blockIdx.x;
    const char2 *hist = vv.hist + (long long)i * vv.hist_input;
    const char2 *cur = vv.cur + (long long)i * kVSPVB;
    int X = 0, Y = 0;
#pragma unroll
    for (int p = 0; p < kP; p++) {
        const int w = m + p;
        char2 x;
        if (w < kHistFrames) {
            x = hist[(long long)w * kK + n];
        } else {
            const int g = w - kHistFrames;
            x = cur[(g / kFramesPerBlock) * vv.cur_block + (long long)(g % kFramesPerBlock) * kK + n];
        }
        const int h = __ldg(filter + kK * kP - kK * p - n - 1);
        X += h * (int)x.x;
        Y += h * (int)x.y;
    }
    b[((long long)m * vv.ninputs + i) * kK + n] = make_int2(X, Y);
}

// pfb.cpp:202-242 (fpga) or pfb.cpp:256-268 (scale), in place.
__global__ void round_staged_kernel(int *data, long long n, int fpga)
{
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= n) return;
    int X = data[idx];
    float f;
    if (fpga) {
        if (X > 0) X += 0x2000;
        f = (float)(X >> 14);
    } else {
        f = (float)X * (1.0f / 16384.0f);
    }
    reinterpret_cast<float *>(data)[idx] = f;
}

// In-place batched 128-point forward FFT of rows [nrows][128] float2
// (replaces the reference's cuFFT calls, pfb.cpp:637-644). 32 rows per CTA.
__global__ void __launch_bounds__(256) fft_staged_kernel(float2 *rows, long long nrows)
{
    __shared__ float2 buf[32][kFftRow];
    __shared__ __align__(16) float2 tw[128];
    const int tid = threadIdx.x;
    const long long r0 = blockIdx.x * 32LL;
    if (tid < 128) {
        const int k1 = tid >> 3, j = tid & 7;
        double sn, cs;
        sincospi((double)(j * k1) / 64.0, &sn, &cs);
        tw[fft128_tw_slot(k1, j)] = make_float2((float)cs, (float)sn);
    }
    for (int idx = tid; idx < 32 * kK; idx += 256) {
        const int r = idx / kK, n = idx % kK;
        buf[r][n] = (r0 + r < nrows) ? rows[(r0 + r) * kK + n] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int g = tid >> 3, j = tid & 7;
    fft128_pass1<-1>(buf[g], tw, j);
    __syncwarp();
    float2 out[2][8];
    fft128_pass2<-1>(buf[g], j, out);
    if (r0 + g < nrows) {
#pragma unroll
        for (int h = 0; h < 2; h++)
#pragma unroll
            for (int k2 = 0; k2 < 8; k2++) rows[(r0 + g) * kK + fft128_index(j, h, k2)] = out[h][k2];
    }
}

// pfb.cpp:297-343 from FFT output rows [m][i][k] to [m][k'][i_idx[i]].
__global__ void pack_staged_kernel(const float2 *ffted, int nspectra, int ninputs, const int *i_idx,
                                   unsigned flags, void *out)
{
    const int i = threadIdx.x + blockIdx.z * blockDim.x;
    const int k = blockIdx.y;
    const int m = blockIdx.x;
    if (i >= ninputs) return;
    const int kp = (k + kK / 2) % kK;
    const float2 X = ffted[((long long)m * ninputs + i) * kK + k];
    const float re = X.x / kK, im = X.y / kK;
    const long long o = ((long long)m * kK + kp) * ninputs + i_idx[i];
    const bool imag_first = (flags & VGB_PFB_IMAG_PART_FIRST) != 0;
    const float hi = imag_first ? re : im, lo = imag_first ? im : re;
    if (flags & VGB_PFB_COMPLEX_INT4) {
        const int h4 = (int)fminf(fmaxf(roundf(hi), -8.f), 7.f) & 0xF;
        const int l4 = (int)fminf(fmaxf(roundf(lo), -8.f), 7.f) & 0xF;
        static_cast<uint8_t *>(out)[o] = (uint8_t)((h4 << 4) | l4);
    } else {
        static_cast<double2 *>(out)[o] = make_double2((double)hi, (double)lo);
    }
}

int launch_wola_staged(const VoltView &vv, const int *filter, int nspectra, int2 *b, cudaStream_t st)
{
    if (nspectra <= 0) return VGB_SUCCESS;
    wola_staged_kernel<<<dim3(nspectra, vv.ninputs), kK, 0, st>>>(vv, filter, nspectra, b);
    return check_launch("wola_staged_kernel");
}

int launch_round_staged(int *data, long long n, int fpga, cudaStream_t st)
{
    if (n <= 0) return VGB_SUCCESS;
    round_staged_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(data, n, fpga);
    return check_launch("round_staged_kernel");
}

int launch_fft_staged(float2 *rows, long long nrows, cudaStream_t st)
{
    if (nrows <= 0) return VGB_SUCCESS;
    fft_staged_kernel<<<(unsigned)((nrows + 31) / 32), 256, 0, st>>>(rows, nrows);
    return check_launch("fft_staged_kernel");
}

int launch_pack_staged(const float2 *ffted, int nspectra, int ninputs, const int *i_idx, unsigned flags,
                       void *out, cudaStream_t st)
{
    if (nspectra <= 0) return VGB_SUCCESS;
    const int bx = ninputs < 256 ? ninputs : 256;
    dim3 grid(nspectra, kK, (ninputs + bx - 1) / bx);
    pack_staged_kernel<<<grid, bx, 0, st>>>(ffted, nspectra, ninputs, i_idx, flags, out);
    return check_launch("pack_staged_kernel");
}

} // namespace vgb
