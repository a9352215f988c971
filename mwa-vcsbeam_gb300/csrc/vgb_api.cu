// The plain C ABI (include/vcsbeam_gb300.h): argument checks, status
// reporting and the one-second streaming pipeline.
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include <vector>

#include "vgb_launch.cuh"

namespace vgb {

static thread_local char t_err[512] = "";

int set_error(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(t_err, sizeof(t_err), fmt, ap);
    va_end(ap);
    return code;
}

int check_cuda(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return VGB_SUCCESS;
    return set_error(VGB_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

int check_launch(const char *what) { return check_cuda(cudaGetLastError(), what); }

// One status word per device, raised by kernels with atomicOr.
__device__ unsigned g_status;

unsigned *status_word()
{
    static unsigned *ptrs[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    if (!ptrs[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_status) != cudaSuccess) return nullptr;
        ptrs[dev] = static_cast<unsigned *>(p);
    }
    return ptrs[dev];
}

static bool aligned16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

static int to_view(const vgb_voltages *v, int ncc, int nspectra, VoltView &vv)
{
    if (!v) return set_error(VGB_ERR_INVALID, "voltages descriptor is NULL");
    if (v->ninputs <= 0 || v->nblocks <= 0)
        return set_error(VGB_ERR_INVALID, "ninputs (%d) and nblocks (%d) must be positive", v->ninputs, v->nblocks);
    if (!v->cur || !v->hist) return set_error(VGB_ERR_INVALID, "voltage pointers must not be NULL");
    if (!aligned16(v->cur) || !aligned16(v->hist))
        return set_error(VGB_ERR_INVALID, "voltage pointers must be 16-byte aligned");
    if ((v->hist_input_stride | v->cur_block_stride) & 15 || (ncc > 1 && ((v->hist_cc_stride | v->cur_cc_stride) & 15)))
        return set_error(VGB_ERR_INVALID, "voltage strides must be multiples of 16 bytes");
    if (v->cur_block_stride < (long long)v->ninputs * kVSPVB * 2)
        return set_error(VGB_ERR_INVALID, "cur_block_stride smaller than one voltage block");
    if (v->hist_input_stride < kHistFrames * kK * 2)
        return set_error(VGB_ERR_INVALID, "hist_input_stride smaller than 12 frames");
    if (nspectra < 0 || nspectra > v->nblocks * kFramesPerBlock)
        return set_error(VGB_ERR_INVALID, "nspectra %d exceeds the %d frames in %d blocks", nspectra,
                         v->nblocks * kFramesPerBlock, v->nblocks);
    vv.hist = static_cast<const char2 *>(v->hist);
    vv.hist_input = v->hist_input_stride / 2;
    vv.cc_hist = v->hist_cc_stride / 2;
    vv.cur = static_cast<const char2 *>(v->cur);
    vv.cur_block = v->cur_block_stride / 2;
    vv.cc_cur = v->cur_cc_stride / 2;
    vv.ninputs = v->ninputs;
    vv.nblocks = v->nblocks;
    return VGB_SUCCESS;
}

static int check_geometry(int ntaps, int nchan)
{
    if (ntaps != kP || nchan != kK)
        return set_error(VGB_ERR_UNSUPPORTED, "kernels are built for %d taps x %d channels (got %d x %d)", kP, kK,
                         ntaps, nchan);
    return VGB_SUCCESS;
}

static cudaStream_t S(void *s) { return static_cast<cudaStream_t>(s); }

} // namespace vgb

using namespace vgb;

extern "C" {

const char *vgb_last_error(void) { return t_err; }

int vgb_version(void) { return 1; }

// Largest sum of |h| over the taps p = first, first + step, ... of one
// sample position n (the taps h[p * nchan + n] that one output sums).
static long long worst_tap_sum(const int32_t *filter, int ntaps, int nchan, int first, int step)
{
    long long worst = 0;
    for (int n = 0; n < nchan; n++) {
        long long s = 0;
        for (int p = first; p < ntaps; p += step) {
            const long long h = filter[p * nchan + n];
            s += h < 0 ? -h : h;
        }
        if (s > worst) worst = s;
    }
    return worst;
}

// |x| <= 128 for int8 voltages: a sum is exact in FP32 when the largest
// possible partial sum stays within 2^24.
int vgb_filter_fp32_exact(const int32_t *filter, int ntaps, int nchan)
{
    if (!filter || ntaps <= 0 || nchan <= 0) return 0;
    return worst_tap_sum(filter, ntaps, nchan, 0, 1) * 128 <= (1LL << 24) ? 1 : 0;
}

unsigned vgb_filter_wola_flags(const int32_t *filter, int ntaps, int nchan)
{
    if (!filter || ntaps <= 0 || nchan <= 0) return 0u;
    if (vgb_filter_fp32_exact(filter, ntaps, nchan)) return VGB_WOLA_FP32;
    const long long even = worst_tap_sum(filter, ntaps, nchan, 0, 2), odd = worst_tap_sum(filter, ntaps, nchan, 1, 2);
    return (even > odd ? even : odd) * 128 <= (1LL << 24) ? VGB_WOLA_FP32_SPLIT : 0u;
}

// A wait on an mbarrier that nothing arrives on, limited to `polls` polls:
// the kernel gives up, records kErrWaitTimeout in the status word and
// returns, as every bounded wait in the library does on expiry.
__global__ void selftest_wait_kernel(uint32_t polls, unsigned *status)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0 && !mbar_wait_bounded(&bar, 0, polls)) atomicOr(status, kErrWaitTimeout);
}

int vgb_selftest_bounded_wait(int polls, void *stream)
{
    if (polls <= 0 || polls > (1 << 24)) return set_error(VGB_ERR_INVALID, "selftest_bounded_wait: polls 1..2^24");
    unsigned *status = status_word();
    if (!status) return set_error(VGB_ERR_CUDA, "device status word unavailable");
    selftest_wait_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>((uint32_t)polls, status);
    return check_launch("selftest_wait_kernel");
}

int vgb_check_device_status(void *stream, unsigned *flags_out)
{
    unsigned *p = status_word();
    if (!p) return set_error(VGB_ERR_CUDA, "device status word unavailable");
    int rc = check_cuda(cudaStreamSynchronize(S(stream)), "cudaStreamSynchronize");
    if (rc) return rc;
    unsigned h = 0;
    rc = check_cuda(cudaMemcpy(&h, p, sizeof(h), cudaMemcpyDeviceToHost), "read device status");
    if (rc) return rc;
    if (h) {
        unsigned z = 0;
        rc = check_cuda(cudaMemcpy(p, &z, sizeof(z), cudaMemcpyHostToDevice), "clear device status");
        if (rc) return rc;
    }
    if (flags_out) *flags_out = h;
    if (h)
        return set_error(VGB_ERR_DEVICE, "kernel status 0x%x%s%s%s", h,
                         (h & kErrWaitTimeout) ? " (bounded wait expired)" : "",
                         (h & kErrBadFrame) ? " (frame outside the voltage buffers)" : "",
                         (h & kErrBadInput) ? " (an input index outside the voltage row, or an input map that is not a permutation)"
                                              : "");
    return VGB_SUCCESS;
}

} // extern "C"

namespace {

// vgb_beamform_mwax, optionally gathering the per-(cc, stokes, channel)
// extremes of S for the 8-bit stage (rstat: min keys, max keys, NaN flags,
// [ncc][nstokes][128] each, or NULL).
int beamform_mwax_impl(const vgb_voltages *v, int ncc, int nspectra, const int32_t *filter, int ntaps, int nchan,
                       unsigned pfb_flags, const void *W, int nant, float invw, int nstokes, float *S_, void *e,
                       float *incoh, uint32_t *rstat, void *stream)
{
    int rc = check_geometry(ntaps, nchan);
    if (rc) return rc;
    BeamArgs a{};
    if ((rc = to_view(v, ncc, nspectra, a.vv))) return rc;
    if (ncc <= 0) return set_error(VGB_ERR_INVALID, "ncc must be positive");
    if (nant <= 0 || v->ninputs != 2 * nant)
        return set_error(VGB_ERR_INVALID, "ninputs (%d) must equal 2*nant (nant=%d)", v->ninputs, nant);
    if (nstokes != 1 && nstokes != 4) return set_error(VGB_ERR_INVALID, "nstokes must be 1 or 4");
    if (!filter || !W || !S_) return set_error(VGB_ERR_INVALID, "filter, W and S must not be NULL");
    if (!aligned16(W) || (e && !aligned16(e))) return set_error(VGB_ERR_INVALID, "W and e must be 16-byte aligned");
    a.filter = filter;
    a.W = static_cast<const float4 *>(W);
    a.W_cc = (long long)nant * kK * 2;
    a.nspectra = nspectra;
    a.nant = nant;
    a.invw = invw;
    a.nstokes = nstokes;
    a.S = S_;
    a.S_cc = (long long)nspectra * nstokes * kK;
    a.e = static_cast<float4 *>(e);
    a.e_cc = (long long)nspectra * kK;
    a.incoh = incoh;
    a.inc_cc = (long long)nspectra * kK;
    a.status = status_word();
    if (!a.status) return set_error(VGB_ERR_CUDA, "device status word unavailable");
    if (rstat) {
        const long long n = (long long)ncc * nstokes * kK;
        a.st_mn = rstat;
        a.st_mx = rstat + n;
        a.st_nan0 = rstat + 2 * n;
    }
    return launch_beam(a, ncc, pfb_flags, S(stream));
}

} // namespace

extern "C" {

int vgb_beamform_mwax(const vgb_voltages *v, int ncc, int nspectra, const int32_t *filter, int ntaps, int nchan,
                      unsigned pfb_flags, const void *W, int nant, float invw, int nstokes, float *S_, void *e,
                      float *incoh, void *stream)
{
    return beamform_mwax_impl(v, ncc, nspectra, filter, ntaps, nchan, pfb_flags, W, nant, invw, nstokes, S_, e, incoh,
                              nullptr, stream);
}

int vgb_pfb_variant_last(void) { return pfb_variant_last(); }

int vgb_pfb_variant(int inputs_per_step)
{
    const int prev = pfb_variant(inputs_per_step);
    if (prev < 0) set_error(VGB_ERR_INVALID, "pfb_variant: 0 (timed choice), 3, 4, 5 or 8");
    return prev;
}

int vgb_fpfb(const vgb_voltages *v, int ncc, int nspectra, const int32_t *filter, int ntaps, int nchan,
             const int32_t *i_idx, unsigned pfb_flags, void *out, void *stream)
{
    int rc = check_geometry(ntaps, nchan);
    if (rc) return rc;
    PackArgs a{};
    if ((rc = to_view(v, ncc, nspectra, a.vv))) return rc;
    if (ncc <= 0) return set_error(VGB_ERR_INVALID, "ncc must be positive");
    if (!filter || !i_idx || !out) return set_error(VGB_ERR_INVALID, "filter, i_idx and out must not be NULL");
    if (v->ninputs > kPackMaxInputs)
        return set_error(VGB_ERR_UNSUPPORTED, "fpfb: at most %d inputs (got %d)", kPackMaxInputs, v->ninputs);
    a.filter = filter;
    a.i_idx = i_idx;
    a.word_stores = v->ninputs % 4 == 0 && (reinterpret_cast<uintptr_t>(out) & 3) == 0;
    a.vec_stores = v->ninputs % 16 == 0 && (reinterpret_cast<uintptr_t>(out) & 15) == 0;
    a.nspectra = nspectra;
    a.flags = pfb_flags;
    a.out = out;
    a.out_cc = (long long)nspectra * kK * v->ninputs;
    a.status = status_word();
    if (!a.status) return set_error(VGB_ERR_CUDA, "device status word unavailable");
    return launch_pack(a, ncc, pfb_flags, S(stream));
}

int vgb_wola(const vgb_voltages *v, int nspectra, const int32_t *filter, int ntaps, int nchan, int32_t *b,
             void *stream)
{
    int rc = check_geometry(ntaps, nchan);
    if (rc) return rc;
    VoltView vv{};
    if ((rc = to_view(v, 1, nspectra, vv))) return rc;
    if (!filter || !b) return set_error(VGB_ERR_INVALID, "filter and b must not be NULL");
    return launch_wola_staged(vv, filter, nspectra, reinterpret_cast<int2 *>(b), S(stream));
}

int vgb_round(int32_t *b, long long nvalues, int emulate_fpga, void *stream)
{
    if (!b || nvalues < 0) return set_error(VGB_ERR_INVALID, "bad buffer");
    return launch_round_staged(b, nvalues, emulate_fpga, S(stream));
}

int vgb_fft128(void *rows, long long nrows, void *stream)
{
    if (!rows || nrows < 0) return set_error(VGB_ERR_INVALID, "bad buffer");
    return launch_fft_staged(static_cast<float2 *>(rows), nrows, S(stream));
}

int vgb_pack(const void *ffted, int nspectra, int ninputs, const int32_t *i_idx, unsigned pfb_flags, void *out,
             void *stream)
{
    if (!ffted || !i_idx || !out || ninputs <= 0) return set_error(VGB_ERR_INVALID, "bad arguments");
    return launch_pack_staged(static_cast<const float2 *>(ffted), nspectra, ninputs, i_idx, pfb_flags, out,
                              S(stream));
}

int vgb_phase(const double *unit, const double *east, const double *north, const double *height,
              const double *cable, const double *chan_freqs_hz, int npointing, int nant, int nchan, double href,
              void *phi, void *stream)
{
    if (!unit || !east || !north || !height || !cable || !chan_freqs_hz || !phi)
        return set_error(VGB_ERR_INVALID, "NULL table pointer");
    return launch_phase(unit, east, north, height, cable, chan_freqs_hz, npointing, nant, nchan, href,
                        static_cast<double2 *>(phi), S(stream));
}

int vgb_array_factor(const double *look, const double *dirs, int npix, double freq_hz, const double *east,
                     const double *north, const double *height, const double *cable, double href, int nant, double *af,
                     void *stream)
{
    if (!look || !dirs || !east || !north || !height || !cable || !af)
        return set_error(VGB_ERR_INVALID, "array_factor: NULL argument");
    if (npix < 0 || nant <= 0 || nant > 6000) return set_error(VGB_ERR_INVALID, "array_factor: bad sizes");
    return launch_array_factor(look, dirs, npix, freq_hz, east, north, height, cable, href, nant, af, S(stream));
}

int vgb_jones(const void *D, const void *B, int npointing, int nant, int nchan, void *J, void *stream)
{
    if (!D || !B || !J) return set_error(VGB_ERR_INVALID, "NULL table pointer");
    return launch_jones(static_cast<const double2 *>(D), static_cast<const double2 *>(B), npointing, nant, nchan,
                        static_cast<double2 *>(J), S(stream));
}

int vgb_weights(const void *J, const void *phi, long long n, void *W, void *stream)
{
    if (!J || !phi || !W) return set_error(VGB_ERR_INVALID, "NULL table pointer");
    return launch_weights(static_cast<const double2 *>(J), static_cast<const double2 *>(phi), n,
                          static_cast<float4 *>(W), S(stream));
}

int vgb_beamform_legacy(const void *v, int datatype, int nsamples, int nchan, int nant, const uint32_t *polQ,
                        const uint32_t *polP, const void *W, int npointing, float invw, int nstokes, float *S_,
                        void *e, float *incoh, void *stream)
{
    if (!v || !polQ || !polP || !W || !S_) return set_error(VGB_ERR_INVALID, "NULL pointer");
    if (datatype != VGB_INT4 && datatype != VGB_DBL) return set_error(VGB_ERR_INVALID, "bad datatype");
    if (nstokes != 1 && nstokes != 4) return set_error(VGB_ERR_INVALID, "nstokes must be 1 or 4");
    if (nant <= 0 || nchan <= 0 || npointing <= 0 || nsamples < 0) return set_error(VGB_ERR_INVALID, "bad sizes");
    if (datatype == VGB_INT4 && !aligned16(v)) return set_error(VGB_ERR_INVALID, "v must be 16-byte aligned");
    LegacyArgs a{};
    a.v = v;
    a.datatype = datatype;
    a.nsamples = nsamples;
    a.nchan = nchan;
    a.nant = nant;
    a.polQ = polQ;
    a.polP = polP;
    a.W = static_cast<const float4 *>(W);
    a.npointing = npointing;
    a.invw = invw;
    a.nstokes = nstokes;
    a.S = S_;
    a.e = static_cast<float4 *>(e);
    a.incoh = datatype == VGB_INT4 ? incoh : nullptr;
    a.status = status_word();
    if (!a.status) return set_error(VGB_ERR_CUDA, "device status word unavailable");
    return launch_legacy_beam(a, S(stream));
}

int vgb_incoh_beam(const uint8_t *data, long long nrows, int ninput, float *incoh, void *stream)
{
    if (!data || !incoh || ninput <= 0 || nrows < 0) return set_error(VGB_ERR_INVALID, "bad arguments");
    if ((ninput & 31) == 0 && !aligned16(data)) return set_error(VGB_ERR_INVALID, "data must be 16-byte aligned");
    return launch_incoh(data, nrows, ninput, incoh, S(stream));
}

} // extern "C"

namespace {

// vgb_renormalise, optionally from extremes the beam kernel gathered (rstat
// as in beamform_mwax_impl, one pointing) instead of its own first pass.
int renormalise_impl(const float *S_, int ncc, int npointing, int nstep, int nstokes, int nchan, uint8_t *out,
                     long long out_cc, long long out_p, long long out_s, long long out_st, float *offsets,
                     float *scales, const uint32_t *rstat, void *stream)
{
    if (!S_ || !out || !offsets || !scales) return set_error(VGB_ERR_INVALID, "NULL pointer");
    if (rstat && npointing != 1) return set_error(VGB_ERR_INVALID, "gathered extremes cover one pointing");
    if (ncc <= 0 || npointing <= 0 || nstokes <= 0 || nchan <= 0 || nstep < 0)
        return set_error(VGB_ERR_INVALID, "bad sizes");
    RenormArgs a{};
    a.S = S_;
    a.S_cc = (long long)npointing * nstep * nstokes * nchan;
    a.npointing = npointing;
    a.nstep = nstep;
    a.nstokes = nstokes;
    a.nchan = nchan;
    a.out = out;
    a.out_cc = out_cc;
    a.out_p = out_p;
    a.out_s = out_s;
    a.out_st = out_st;
    a.offsets = offsets;
    a.scales = scales;
    a.stat_cc = (long long)npointing * nstokes * nchan;
    if (rstat) {
        const long long n = (long long)ncc * nstokes * nchan;
        a.st_mn = rstat;
        a.st_mx = rstat + n;
        a.st_nan0 = rstat + 2 * n;
    }
    return launch_renorm(a, ncc, S(stream));
}

} // namespace

extern "C" {

int vgb_renormalise(const float *S_, int ncc, int npointing, int nstep, int nstokes, int nchan, uint8_t *out,
                    long long out_cc, long long out_p, long long out_s, long long out_st, float *offsets,
                    float *scales, void *stream)
{
    return renormalise_impl(S_, ncc, npointing, nstep, nstokes, nchan, out, out_cc, out_p, out_s, out_st, offsets,
                            scales, nullptr, stream);
}

int vgb_ipfb(const void *e, long long e_job_stride, const void *hist, long long hist_job_stride, const float *coeffs,
             int ntaps, int nchan, int nsamples, int njobs, float *out_f, uint8_t *vdif, const uint32_t *hdr,
             int frame_offset, void *stream)
{
    int rc = check_geometry(ntaps, nchan);
    if (rc) return rc;
    if (!e || !coeffs || (!out_f && !vdif)) return set_error(VGB_ERR_INVALID, "NULL pointer");
    if (frame_offset < 0 || (long long)frame_offset + nsamples >= (1LL << 31))
        return set_error(VGB_ERR_INVALID, "frame_offset must be >= 0 and frame_offset + nsamples < 2^31");
    if (!aligned16(e) || (hist && !aligned16(hist)) || (e_job_stride & 15) || (hist_job_stride & 15))
        return set_error(VGB_ERR_INVALID, "e/hist must be 16-byte aligned with 16-byte job strides");
    IpfbArgs a{};
    a.e = static_cast<const float4 *>(e);
    a.e_job = e_job_stride / 16;
    a.hist = static_cast<const float4 *>(hist);
    a.hist_job = hist_job_stride / 16;
    a.coeffs = coeffs;
    a.nsamples = nsamples;
    a.out_f = out_f;
    a.outf_job = (long long)nsamples * kK * 4;
    a.vdif = vdif;
    a.vdif_job = (long long)nsamples * 544;
    a.hdr = hdr;
    a.frame_offset = frame_offset;
    return launch_ipfb(a, njobs, S(stream));
}

int vgb_vdif_advance(uint32_t *d_hdr, int njobs, int nframes, void *stream)
{
    if (!d_hdr || njobs < 0 || nframes < 0) return set_error(VGB_ERR_INVALID, "vdif_advance: bad argument");
    return launch_vdif_advance(d_hdr, njobs, nframes, S(stream));
}

} // extern "C"

// ===========================================================================
// Streaming pipeline
// ===========================================================================
struct vgb_pipeline {
    vgb_pipeline_config cfg{};
    int ninputs = 0, nspectra = 0;
    long long second_bytes = 0;      // one coarse channel's second, bytes
    unsigned wola_flags = 0;         // VGB_WOLA_FP32 / VGB_WOLA_FP32_SPLIT for the loaded filter
    cudaStream_t s_comp = nullptr, s_copy = nullptr;
    cudaEvent_t ev_copied[2] = {}, ev_consumed[2] = {};
    int32_t *d_filter = nullptr;
    float *d_coeffs = nullptr;
    float4 *d_W = nullptr;
    char2 *d_volt[2] = {};           // host-mode staging, [cc][block][input][sample]
    char2 *d_hist[2] = {};           // [cc][input][12][128]
    float *d_S = nullptr;
    float4 *d_e = nullptr;
    float *d_incoh = nullptr;
    float4 *d_ehist[2] = {};         // [cc][12][128]
    uint8_t *d_psrfits = nullptr;    // [ns][nstokes][ncc*128]
    float *d_off = nullptr, *d_scl = nullptr;
    uint8_t *d_ipsr = nullptr;       // incoherent beam, Stokes I: [ns][ncc*128]
    float *d_ioff = nullptr, *d_iscl = nullptr; // [ncc][128]
    uint8_t *d_vdif = nullptr;       // [cc][ns][544]
    uint32_t *d_hdr = nullptr;
    uint32_t *d_rstat = nullptr;     // [3][cc][stokes][128]: Stokes min / max keys, first-value NaN flags
    long long second = 0;            // seconds completed
    int launches = 0;
    int host_buf = 0;
    // asynchronous host outputs
    uint8_t *h_psrfits = nullptr, *h_vdif = nullptr;
    float *h_off = nullptr, *h_scl = nullptr;
    uint8_t *h_ipsr = nullptr;
    float *h_ioff = nullptr, *h_iscl = nullptr;
    // per-second tracking (vmCalcJonesAndDelays): caller's device tables and
    // the pipeline's own second counter, pointing, B and beam-model scratch
    bool tracking = false;
    vgb_tracking trk{};
    long long *d_trk_counter = nullptr;
    double *d_trk_cur = nullptr;     // az, za, unit E, N, H of the current second
    double2 *d_trk_B = nullptr;      // [cc][nant][2][2]
    int *d_trk_scratch = nullptr;    // 2*nant + 1
    // per-stage timing: events 0..4 bound the four stages, event 5 precedes
    // the tracking tables
    bool timing = false;
    cudaEvent_t ev_stage[6] = {};
    // CUDA graphs of one second, keyed by what the captured launches bake in
    struct Graph {
        const void *volt;
        long long stride;
        int parity;
        bool first;
        const void *hout;
        cudaGraphExec_t exec;
        int launches;
    };
    std::vector<Graph> graphs;
    bool use_graphs = true;
    bool front_timed = false; // the fused front end's inputs-per-step choice has been timed
};

// The configured pfb_flags with the WOLA arithmetic: the configuration's own
// WOLA bits if it has any, else the exact choice derived from the filter.
static unsigned pipeline_pfb_flags(const vgb_pipeline *p)
{
    constexpr unsigned kWolaBits = VGB_WOLA_FP32 | VGB_WOLA_FP32_SPLIT | VGB_WOLA_INT32;
    return p->cfg.pfb_flags | ((p->cfg.pfb_flags & kWolaBits) ? 0u : p->wola_flags);
}

namespace {

template <class T> int dalloc(T **p, size_t bytes)
{
    if (cudaMalloc(reinterpret_cast<void **>(p), bytes) != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return set_error(VGB_ERR_ALLOC, "cudaMalloc of %zu bytes failed", bytes);
    }
    return VGB_SUCCESS;
}

// The voltage view of one second: history of the previous second + `volt`.
vgb_voltages pipeline_voltages(const vgb_pipeline *p, const char2 *volt, long long cc_stride_bytes)
{
    vgb_voltages v{};
    v.hist = p->d_hist[(int)(p->second & 1)];
    v.hist_input_stride = (long long)kHistFrames * kK * 2;
    v.hist_cc_stride = (long long)p->ninputs * kHistFrames * kK * 2;
    v.cur = volt;
    v.cur_block_stride = (long long)p->ninputs * kVSPVB * 2;
    v.cur_cc_stride = cc_stride_bytes;
    v.ninputs = p->ninputs;
    v.nblocks = p->cfg.nblocks;
    return v;
}

// Empty extremes (min keys all ones, max keys and NaN flags zero) for the
// next second's beam kernel to gather into.
int reset_rstat(vgb_pipeline *p)
{
    const size_t n = (size_t)p->cfg.ncc * p->cfg.nstokes * kK;
    int rc = check_cuda(cudaMemsetAsync(p->d_rstat, 0xFF, n * sizeof(uint32_t), p->s_comp), "reset extremes");
    return rc ? rc : check_cuda(cudaMemsetAsync(p->d_rstat + n, 0, 2 * n * sizeof(uint32_t), p->s_comp),
                                "reset extremes");
}

// One second of compute on s_comp with the voltages at `volt`.
int pipeline_second(vgb_pipeline *p, const char2 *volt, long long cc_stride_bytes)
{
    NvtxRange range("vgb: pipeline second");
    const vgb_pipeline_config &c = p->cfg;
    const int cur = (int)(p->second & 1), nxt = cur ^ 1;
    int rc;
    p->launches = 0;
    const vgb_voltages v = pipeline_voltages(p, volt, cc_stride_bytes);
    const unsigned flags = pipeline_pfb_flags(p);
    auto mark = [&](int i) {
        return p->timing ? check_cuda(cudaEventRecord(p->ev_stage[i], p->s_comp), "stage event") : VGB_SUCCESS;
    };
    if ((rc = mark(5))) return rc;
    if (p->tracking) {
        // the second's pointing, B at each coarse channel's beam frequency,
        // then J^-1, phi and W for every (cc, tile, channel)
        const vgb_tracking &t = p->trk;
        rc = launch_track_select(t.az, t.za, t.nseconds, p->d_trk_counter, p->d_trk_cur, p->s_comp);
        if (rc) return rc;
        PbArgs pb{p->d_trk_cur, p->d_trk_cur + 1, 1, t.beam_freqs_hz, c.ncc, t.delays, c.nant, t.latitude,
                  t.pa_correction, p->d_trk_B};
        rc = launch_beam_model(pb, p->s_comp, p->d_trk_scratch);
        if (rc) return rc;
        rc = launch_track_weights(reinterpret_cast<const double2 *>(t.D), p->d_trk_B, p->d_trk_cur + 2, t.east,
                                  t.north, t.height, t.cable, t.chan_freqs_hz, c.ncc, c.nant, kK, t.href, p->d_W,
                                  p->s_comp);
        if (rc) return rc;
        p->launches += 5;
    }
    if ((rc = mark(0))) return rc;
    rc = beamform_mwax_impl(&v, c.ncc, p->nspectra, p->d_filter, kP, kK, flags, p->d_W, c.nant, c.invw, c.nstokes,
                            p->d_S, p->d_e, p->d_incoh, p->d_rstat, p->s_comp);
    if (rc) return rc;
    p->launches++;
    if ((rc = mark(1))) return rc;
    // spliced PSRFITS rows: [s][st][cc*128 + c]
    const long long row = (long long)c.nstokes * c.ncc * kK;
    rc = renormalise_impl(p->d_S, c.ncc, 1, p->nspectra, c.nstokes, kK, p->d_psrfits, kK, 0, row,
                          (long long)c.ncc * kK, p->d_off, p->d_scl, p->d_rstat, p->s_comp);
    if (rc) return rc;
    p->launches++;
    // the incoherent beam's 8-bit rows (Stokes I, spliced the same way; its
    // renormalise as cu_form_incoh_beam's, form_beam.cpp:495-497)
    rc = renormalise_impl(p->d_incoh, c.ncc, 1, p->nspectra, 1, kK, p->d_ipsr, kK, 0, (long long)c.ncc * kK,
                          (long long)c.ncc * kK, p->d_ioff, p->d_iscl, nullptr, p->s_comp);
    if (rc) return rc;
    p->launches++;
    // the next second's extremes start empty
    rc = reset_rstat(p);
    if (rc) return rc;
    if ((rc = mark(2))) return rc;
    if (c.do_ipfb) {
        const long long ejob = (long long)p->nspectra * kK * 16;
        rc = vgb_ipfb(p->d_e, ejob, p->second > 0 ? p->d_ehist[cur] : nullptr, (long long)kHistFrames * kK * 16,
                      p->d_coeffs, kP, kK, p->nspectra, c.ncc, nullptr, p->d_vdif, p->d_hdr, 0, p->s_comp);
        if (rc) return rc;
        p->launches++;
        // the next second's headers start where this second's end
        rc = launch_vdif_advance(p->d_hdr, c.ncc, p->nspectra, p->s_comp);
        if (rc) return rc;
        p->launches++;
        // carry the last 12 beam samples of each coarse channel
        rc = check_cuda(cudaMemcpy2DAsync(p->d_ehist[nxt], (size_t)kHistFrames * kK * 16,
                                          p->d_e + (long long)(p->nspectra - kHistFrames) * kK, (size_t)ejob,
                                          (size_t)kHistFrames * kK * 16, c.ncc, cudaMemcpyDeviceToDevice,
                                          p->s_comp),
                        "carry beam history");
        if (rc) return rc;
    }
    if ((rc = mark(3))) return rc;
    // carry the last 12 voltage frames of each input
    rc = launch_hist_gather(volt, (long long)p->ninputs * kVSPVB, cc_stride_bytes / 2, p->ninputs, c.nblocks, c.ncc,
                            p->d_hist[nxt], (long long)p->ninputs * kHistFrames * kK, p->s_comp);
    if (rc) return rc;
    p->launches++;
    if ((rc = mark(4))) return rc;
    p->second++;
    // asynchronous copies of the products into the caller's host buffers
    const size_t ns = p->nspectra;
    if (p->h_psrfits)
        rc = check_cuda(cudaMemcpyAsync(p->h_psrfits, p->d_psrfits, ns * c.nstokes * c.ncc * kK,
                                        cudaMemcpyDeviceToHost, p->s_comp),
                        "D2H psrfits");
    if (!rc && p->h_off)
        rc = check_cuda(cudaMemcpyAsync(p->h_off, p->d_off, sizeof(float) * c.ncc * c.nstokes * kK,
                                        cudaMemcpyDeviceToHost, p->s_comp),
                        "D2H offsets");
    if (!rc && p->h_scl)
        rc = check_cuda(cudaMemcpyAsync(p->h_scl, p->d_scl, sizeof(float) * c.ncc * c.nstokes * kK,
                                        cudaMemcpyDeviceToHost, p->s_comp),
                        "D2H scales");
    if (!rc && p->h_vdif && c.do_ipfb)
        rc = check_cuda(cudaMemcpyAsync(p->h_vdif, p->d_vdif, (size_t)c.ncc * ns * 544, cudaMemcpyDeviceToHost,
                                        p->s_comp),
                        "D2H vdif");
    if (!rc && p->h_ipsr)
        rc = check_cuda(cudaMemcpyAsync(p->h_ipsr, p->d_ipsr, ns * c.ncc * kK, cudaMemcpyDeviceToHost, p->s_comp),
                        "D2H incoherent psrfits");
    if (!rc && p->h_ioff)
        rc = check_cuda(cudaMemcpyAsync(p->h_ioff, p->d_ioff, sizeof(float) * c.ncc * kK, cudaMemcpyDeviceToHost,
                                        p->s_comp),
                        "D2H incoherent offsets");
    if (!rc && p->h_iscl)
        rc = check_cuda(cudaMemcpyAsync(p->h_iscl, p->d_iscl, sizeof(float) * c.ncc * kK, cudaMemcpyDeviceToHost,
                                        p->s_comp),
                        "D2H incoherent scales");
    return rc;
}

void drop_graphs(vgb_pipeline *p)
{
    for (auto &g : p->graphs) cudaGraphExecDestroy(g.exec);
    p->graphs.clear();
}

// One second, replayed from a captured CUDA graph (captured on first use for
// this input buffer, second parity and output set); eager while timing.
int pipeline_second_graph(vgb_pipeline *p, const char2 *volt, long long cc_stride_bytes)
{
    if (!p->use_graphs || p->timing) return pipeline_second(p, volt, cc_stride_bytes);
    const int parity = (int)(p->second & 1);
    const bool first = p->second == 0;
    const void *hout = p->h_psrfits ? (const void *)p->h_psrfits
                                    : p->h_vdif ? (const void *)p->h_vdif : (const void *)p->h_ipsr;
    for (auto &g : p->graphs)
        if (g.volt == volt && g.stride == cc_stride_bytes && g.parity == parity && g.first == first && g.hout == hout) {
            int rc = check_cuda(cudaGraphLaunch(g.exec, p->s_comp), "cudaGraphLaunch");
            if (!rc) {
                p->second++;
                p->launches = g.launches;
            }
            return rc;
        }
    if (p->graphs.size() >= 8) drop_graphs(p);
    const long long saved = p->second;
    // one eager fused PFB + beamformer pass first, so the front end's
    // inputs-per-step choice is timed (and cached) outside the capture; it
    // writes only the Stokes and beam buffers the second then rewrites
    int rc = VGB_SUCCESS;
    if (!p->front_timed) {
        const vgb_pipeline_config &c = p->cfg;
        const vgb_voltages v = pipeline_voltages(p, volt, cc_stride_bytes);
        rc = vgb_beamform_mwax(&v, c.ncc, p->nspectra, p->d_filter, kP, kK,
                               pipeline_pfb_flags(p), p->d_W, c.nant, c.invw, c.nstokes,
                               p->d_S, p->d_e, p->d_incoh, p->s_comp);
        if (rc) return rc;
        p->front_timed = true; // one shape per pipeline
    }
    rc = check_cuda(cudaStreamBeginCapture(p->s_comp, cudaStreamCaptureModeRelaxed), "cudaStreamBeginCapture");
    if (rc) return rc;
    rc = pipeline_second(p, volt, cc_stride_bytes);
    cudaGraph_t graph = nullptr;
    const int rc_end = check_cuda(cudaStreamEndCapture(p->s_comp, &graph), "cudaStreamEndCapture");
    p->second = saved;
    if (!rc) rc = rc_end;
    cudaGraphExec_t exec = nullptr;
    if (!rc) rc = check_cuda(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
    if (graph) cudaGraphDestroy(graph);
    if (rc) return rc;
    p->graphs.push_back({volt, cc_stride_bytes, parity, first, hout, exec, p->launches});
    rc = check_cuda(cudaGraphLaunch(exec, p->s_comp), "cudaGraphLaunch");
    if (!rc) p->second++;
    return rc;
}

} // namespace

extern "C" {

int vgb_pipeline_create(const vgb_pipeline_config *cfg, vgb_pipeline **out)
{
    if (!cfg || !out) return set_error(VGB_ERR_INVALID, "NULL argument");
    if (cfg->ncc <= 0 || cfg->nant <= 0 || cfg->nblocks <= 0 || (cfg->nstokes != 1 && cfg->nstokes != 4))
        return set_error(VGB_ERR_INVALID, "bad pipeline configuration");
    vgb_pipeline *p = new vgb_pipeline();
    p->cfg = *cfg;
    p->ninputs = 2 * cfg->nant;
    p->nspectra = cfg->nblocks * kFramesPerBlock;
    p->second_bytes = (long long)cfg->nblocks * p->ninputs * kVSPVB * 2;
    const long long ncc = cfg->ncc, ns = p->nspectra;
    int rc = VGB_SUCCESS;
    rc = rc ? rc : check_cuda(cudaStreamCreateWithFlags(&p->s_comp, cudaStreamNonBlocking), "stream");
    rc = rc ? rc : check_cuda(cudaStreamCreateWithFlags(&p->s_copy, cudaStreamNonBlocking), "stream");
    for (int i = 0; i < 6 && !rc; i++) rc = check_cuda(cudaEventCreate(&p->ev_stage[i]), "event");
    for (int b = 0; b < 2 && !rc; b++) {
        rc = check_cuda(cudaEventCreateWithFlags(&p->ev_copied[b], cudaEventDisableTiming), "event");
        rc = rc ? rc : check_cuda(cudaEventCreateWithFlags(&p->ev_consumed[b], cudaEventDisableTiming), "event");
    }
    rc = rc ? rc : dalloc(&p->d_filter, sizeof(int32_t) * kK * kP);
    rc = rc ? rc : dalloc(&p->d_coeffs, sizeof(float) * kK * kP);
    rc = rc ? rc : dalloc(&p->d_W, sizeof(float4) * 2 * ncc * cfg->nant * kK);
    for (int b = 0; b < 2 && !rc; b++) {
        rc = dalloc(&p->d_hist[b], (size_t)ncc * p->ninputs * kHistFrames * kK * 2);
        rc = rc ? rc : dalloc(&p->d_ehist[b], sizeof(float4) * ncc * kHistFrames * kK);
    }
    rc = rc ? rc : dalloc(&p->d_S, sizeof(float) * ncc * ns * cfg->nstokes * kK);
    rc = rc ? rc : dalloc(&p->d_e, sizeof(float4) * ncc * ns * kK);
    rc = rc ? rc : dalloc(&p->d_incoh, sizeof(float) * ncc * ns * kK);
    rc = rc ? rc : dalloc(&p->d_psrfits, (size_t)ns * cfg->nstokes * ncc * kK);
    rc = rc ? rc : dalloc(&p->d_ipsr, (size_t)ns * ncc * kK);
    rc = rc ? rc : dalloc(&p->d_ioff, sizeof(float) * ncc * kK);
    rc = rc ? rc : dalloc(&p->d_iscl, sizeof(float) * ncc * kK);
    rc = rc ? rc : dalloc(&p->d_off, sizeof(float) * ncc * cfg->nstokes * kK);
    rc = rc ? rc : dalloc(&p->d_scl, sizeof(float) * ncc * cfg->nstokes * kK);
    if (cfg->do_ipfb) rc = rc ? rc : dalloc(&p->d_vdif, (size_t)ncc * ns * 544);
    rc = rc ? rc : dalloc(&p->d_hdr, sizeof(uint32_t) * 8 * ncc);
    rc = rc ? rc : dalloc(&p->d_rstat, sizeof(uint32_t) * 3 * ncc * cfg->nstokes * kK);
    rc = rc ? rc : dalloc(&p->d_trk_counter, sizeof(long long));
    rc = rc ? rc : dalloc(&p->d_trk_cur, sizeof(double) * 8);
    rc = rc ? rc : dalloc(&p->d_trk_B, sizeof(double2) * 4 * ncc * cfg->nant);
    rc = rc ? rc : dalloc(&p->d_trk_scratch, sizeof(int) * (2 * (size_t)cfg->nant + 1));
    if (!rc) {
        for (int b = 0; b < 2 && !rc; b++)
            rc = check_cuda(cudaMemsetAsync(p->d_hist[b], 0, (size_t)ncc * p->ninputs * kHistFrames * kK * 2,
                                            p->s_comp),
                            "memset history");
        rc = rc ? rc : check_cuda(cudaMemsetAsync(p->d_hdr, 0, sizeof(uint32_t) * 8 * ncc, p->s_comp), "memset hdr");
        rc = rc ? rc : reset_rstat(p);
        rc = rc ? rc : check_cuda(cudaMemsetAsync(p->d_trk_counter, 0, sizeof(long long), p->s_comp), "memset");
        rc = rc ? rc : check_cuda(cudaStreamSynchronize(p->s_comp), "sync");
    }
    if (rc) {
        vgb_pipeline_destroy(p);
        return rc;
    }
    // resolve the device status word now, not inside a graph capture
    if (!status_word()) {
        vgb_pipeline_destroy(p);
        return set_error(VGB_ERR_CUDA, "device status word unavailable");
    }
    *out = p;
    return VGB_SUCCESS;
}

int vgb_pipeline_destroy(vgb_pipeline *p)
{
    if (!p) return VGB_SUCCESS;
    if (p->s_comp) cudaStreamSynchronize(p->s_comp);
    if (p->s_copy) cudaStreamSynchronize(p->s_copy);
    drop_graphs(p);
    void *bufs[] = {p->d_filter, p->d_coeffs, p->d_W, p->d_volt[0], p->d_volt[1], p->d_hist[0], p->d_hist[1],
                    p->d_S, p->d_e, p->d_incoh, p->d_ehist[0], p->d_ehist[1], p->d_psrfits, p->d_off, p->d_scl,
                    p->d_vdif, p->d_hdr, p->d_rstat, p->d_trk_counter, p->d_trk_cur, p->d_trk_B,
                    p->d_trk_scratch, p->d_ipsr, p->d_ioff, p->d_iscl};
    for (void *b : bufs)
        if (b) cudaFree(b);
    for (int i = 0; i < 6; i++)
        if (p->ev_stage[i]) cudaEventDestroy(p->ev_stage[i]);
    for (int b = 0; b < 2; b++) {
        if (p->ev_copied[b]) cudaEventDestroy(p->ev_copied[b]);
        if (p->ev_consumed[b]) cudaEventDestroy(p->ev_consumed[b]);
    }
    if (p->s_comp) cudaStreamDestroy(p->s_comp);
    if (p->s_copy) cudaStreamDestroy(p->s_copy);
    delete p;
    return VGB_SUCCESS;
}

int vgb_pipeline_set_filters(vgb_pipeline *p, const int32_t *analysis, const float *synthesis)
{
    if (!p || !analysis) return set_error(VGB_ERR_INVALID, "NULL argument");
    if (p->cfg.do_ipfb && !synthesis) return set_error(VGB_ERR_INVALID, "synthesis filter required for the IPFB");
    p->wola_flags = vgb_filter_wola_flags(analysis, kP, kK);
    int rc = check_cuda(cudaMemcpyAsync(p->d_filter, analysis, sizeof(int32_t) * kK * kP, cudaMemcpyHostToDevice,
                                        p->s_comp),
                        "upload analysis filter");
    if (!rc && synthesis)
        rc = check_cuda(cudaMemcpyAsync(p->d_coeffs, synthesis, sizeof(float) * kK * kP, cudaMemcpyHostToDevice,
                                        p->s_comp),
                        "upload synthesis filter");
    return rc ? rc : check_cuda(cudaStreamSynchronize(p->s_comp), "sync");
}

int vgb_pipeline_set_tracking(vgb_pipeline *p, const vgb_tracking *t)
{
    if (!p) return set_error(VGB_ERR_INVALID, "NULL pipeline");
    int rc = check_cuda(cudaStreamSynchronize(p->s_comp), "sync");
    if (rc) return rc;
    drop_graphs(p); // the captured seconds did (or did not) rebuild W
    if (!t) {
        p->tracking = false;
        return VGB_SUCCESS;
    }
    if (!t->D || !t->delays || !t->east || !t->north || !t->height || !t->cable || !t->chan_freqs_hz ||
        !t->beam_freqs_hz || !t->az || !t->za)
        return set_error(VGB_ERR_INVALID, "pipeline_set_tracking: NULL table");
    if (t->nseconds <= 0) return set_error(VGB_ERR_INVALID, "pipeline_set_tracking: nseconds %d", t->nseconds);
    if ((reinterpret_cast<uintptr_t>(t->delays) | reinterpret_cast<uintptr_t>(t->D)) & 15)
        return set_error(VGB_ERR_INVALID, "pipeline_set_tracking: D and delays must be 16-byte aligned");
    p->trk = *t;
    p->tracking = true;
    // the table index follows the pipeline's second counter
    const long long s = p->second;
    return check_cuda(cudaMemcpy(p->d_trk_counter, &s, sizeof(s), cudaMemcpyHostToDevice), "tracking counter");
}

int vgb_pipeline_set_weights(vgb_pipeline *p, const void *W, int on_device)
{
    if (!p || !W) return set_error(VGB_ERR_INVALID, "NULL argument");
    if (p->tracking) {
        int rc = vgb_pipeline_set_tracking(p, nullptr);
        if (rc) return rc;
    }
    const size_t bytes = sizeof(float4) * 2 * p->cfg.ncc * p->cfg.nant * kK;
    return check_cuda(cudaMemcpyAsync(p->d_W, W, bytes, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice,
                                      p->s_comp),
                      "upload weights");
}

int vgb_pipeline_set_vdif_header(vgb_pipeline *p, const uint32_t *hdr)
{
    if (!p || !hdr) return set_error(VGB_ERR_INVALID, "NULL argument");
    int rc = check_cuda(cudaMemcpyAsync(p->d_hdr, hdr, sizeof(uint32_t) * 8 * p->cfg.ncc, cudaMemcpyHostToDevice,
                                        p->s_comp),
                        "upload VDIF header");
    return rc ? rc : check_cuda(cudaStreamSynchronize(p->s_comp), "sync");
}

int vgb_pipeline_run_device(vgb_pipeline *p, const void *d_voltages, long long cur_cc_stride)
{
    if (!p || !d_voltages) return set_error(VGB_ERR_INVALID, "NULL argument");
    if (cur_cc_stride < p->second_bytes && p->cfg.ncc > 1)
        return set_error(VGB_ERR_INVALID, "coarse-channel stride smaller than one second");
    return pipeline_second_graph(p, static_cast<const char2 *>(d_voltages), cur_cc_stride);
}

// Carry-over state between seconds: a header, the 12 voltage frames of each
// input and the 12 beam samples of each coarse channel the next second reads.
struct PipelineStateHeader {
    uint32_t magic, version;
    int32_t ncc, ninputs, nblocks, do_ipfb;
    int64_t second;
};
constexpr uint32_t kStateMagic = 0x56474253u; // "VGBS"

static long long state_hist_bytes(const vgb_pipeline *p)
{
    return (long long)p->cfg.ncc * p->ninputs * kHistFrames * kK * 2;
}
static long long state_ehist_bytes(const vgb_pipeline *p) { return (long long)sizeof(float4) * p->cfg.ncc * kHistFrames * kK; }
static long long state_hdr_bytes(const vgb_pipeline *p) { return (long long)sizeof(uint32_t) * 8 * p->cfg.ncc; }
constexpr uint32_t kStateVersion = 2; // version 2 adds the VDIF header templates

long long vgb_pipeline_state_bytes(const vgb_pipeline *p)
{
    return p ? (long long)sizeof(PipelineStateHeader) + state_hist_bytes(p) + state_ehist_bytes(p) + state_hdr_bytes(p)
             : 0;
}

int vgb_pipeline_save_state(vgb_pipeline *p, void *host, long long bytes)
{
    if (!p || !host) return set_error(VGB_ERR_INVALID, "pipeline_save_state: NULL argument");
    if (bytes < vgb_pipeline_state_bytes(p)) return set_error(VGB_ERR_INVALID, "pipeline_save_state: buffer too small");
    int rc = check_cuda(cudaStreamSynchronize(p->s_comp), "sync");
    if (rc) return rc;
    PipelineStateHeader h{kStateMagic, kStateVersion, p->cfg.ncc, p->ninputs, p->cfg.nblocks, p->cfg.do_ipfb,
                          p->second};
    char *out = static_cast<char *>(host);
    std::memcpy(out, &h, sizeof(h));
    const int cur = (int)(p->second & 1);
    rc = check_cuda(cudaMemcpy(out + sizeof(h), p->d_hist[cur], state_hist_bytes(p), cudaMemcpyDeviceToHost),
                    "save voltage history");
    if (!rc)
        rc = check_cuda(cudaMemcpy(out + sizeof(h) + state_hist_bytes(p), p->d_ehist[cur], state_ehist_bytes(p),
                                   cudaMemcpyDeviceToHost),
                        "save beam history");
    if (!rc)
        rc = check_cuda(cudaMemcpy(out + sizeof(h) + state_hist_bytes(p) + state_ehist_bytes(p), p->d_hdr,
                                   state_hdr_bytes(p), cudaMemcpyDeviceToHost),
                        "save VDIF headers");
    return rc;
}

int vgb_pipeline_load_state(vgb_pipeline *p, const void *host, long long bytes)
{
    if (!p || !host) return set_error(VGB_ERR_INVALID, "pipeline_load_state: NULL argument");
    if (bytes < vgb_pipeline_state_bytes(p)) return set_error(VGB_ERR_INVALID, "pipeline_load_state: buffer too small");
    PipelineStateHeader h;
    std::memcpy(&h, host, sizeof(h));
    if (h.magic != kStateMagic || h.version != kStateVersion || h.ncc != p->cfg.ncc || h.ninputs != p->ninputs ||
        h.nblocks != p->cfg.nblocks || h.do_ipfb != p->cfg.do_ipfb || h.second < 0)
        return set_error(VGB_ERR_INVALID, "pipeline_load_state: state is from a different pipeline configuration");
    int rc = check_cuda(cudaStreamSynchronize(p->s_comp), "sync");
    if (rc) return rc;
    drop_graphs(p);
    p->second = h.second;
    const int cur = (int)(p->second & 1);
    const char *in = static_cast<const char *>(host);
    rc = check_cuda(cudaMemcpy(p->d_hist[cur], in + sizeof(h), state_hist_bytes(p), cudaMemcpyHostToDevice),
                    "load voltage history");
    if (!rc)
        rc = check_cuda(cudaMemcpy(p->d_ehist[cur], in + sizeof(h) + state_hist_bytes(p), state_ehist_bytes(p),
                                   cudaMemcpyHostToDevice),
                        "load beam history");
    if (!rc)
        rc = check_cuda(cudaMemcpy(p->d_hdr, in + sizeof(h) + state_hist_bytes(p) + state_ehist_bytes(p),
                                   state_hdr_bytes(p), cudaMemcpyHostToDevice),
                        "load VDIF headers");
    if (!rc)
        rc = check_cuda(cudaMemcpy(p->d_trk_counter, &h.second, sizeof(long long), cudaMemcpyHostToDevice),
                        "load tracking counter");
    return rc;
}

int vgb_pipeline_enable_graphs(vgb_pipeline *p, int on)
{
    if (!p) return set_error(VGB_ERR_INVALID, "NULL pipeline");
    int rc = check_cuda(cudaStreamSynchronize(p->s_comp), "sync");
    drop_graphs(p);
    p->use_graphs = on != 0;
    return rc;
}

int vgb_pipeline_run_host(vgb_pipeline *p, const void *h_voltages, long long cur_cc_stride)
{
    if (!p || !h_voltages) return set_error(VGB_ERR_INVALID, "NULL argument");
    if (cur_cc_stride < p->second_bytes && p->cfg.ncc > 1)
        return set_error(VGB_ERR_INVALID, "coarse-channel stride smaller than one second");
    const size_t total = (size_t)p->second_bytes * p->cfg.ncc;
    const int b = p->host_buf;
    int rc;
    if (!p->d_volt[b] && (rc = dalloc(&p->d_volt[b], total))) return rc;
    // the buffer is free once the compute that last read it has finished
    rc = check_cuda(cudaStreamWaitEvent(p->s_copy, p->ev_consumed[b], 0), "wait consumed");
    if (rc) return rc;
    if (cur_cc_stride == p->second_bytes || p->cfg.ncc == 1) {
        rc = check_cuda(cudaMemcpyAsync(p->d_volt[b], h_voltages, total, cudaMemcpyHostToDevice, p->s_copy), "H2D");
    } else {
        rc = check_cuda(cudaMemcpy2DAsync(p->d_volt[b], (size_t)p->second_bytes, h_voltages, (size_t)cur_cc_stride,
                                          (size_t)p->second_bytes, p->cfg.ncc, cudaMemcpyHostToDevice, p->s_copy),
                        "H2D");
    }
    if (rc) return rc;
    rc = check_cuda(cudaEventRecord(p->ev_copied[b], p->s_copy), "record copied");
    rc = rc ? rc : check_cuda(cudaStreamWaitEvent(p->s_comp, p->ev_copied[b], 0), "wait copied");
    if (rc) return rc;
    rc = pipeline_second_graph(p, p->d_volt[b], p->second_bytes);
    if (rc) return rc;
    rc = check_cuda(cudaEventRecord(p->ev_consumed[b], p->s_comp), "record consumed");
    p->host_buf ^= 1;
    return rc;
}

int vgb_pipeline_fetch(vgb_pipeline *p, uint8_t *psrfits, float *offsets, float *scales, uint8_t *vdif)
{
    if (!p) return set_error(VGB_ERR_INVALID, "NULL pipeline");
    const vgb_pipeline_config &c = p->cfg;
    const size_t ns = p->nspectra;
    int rc = VGB_SUCCESS;
    if (psrfits)
        rc = check_cuda(cudaMemcpyAsync(psrfits, p->d_psrfits, ns * c.nstokes * c.ncc * kK, cudaMemcpyDeviceToHost,
                                        p->s_comp),
                        "D2H psrfits");
    if (!rc && offsets)
        rc = check_cuda(cudaMemcpyAsync(offsets, p->d_off, sizeof(float) * c.ncc * c.nstokes * kK,
                                        cudaMemcpyDeviceToHost, p->s_comp),
                        "D2H offsets");
    if (!rc && scales)
        rc = check_cuda(cudaMemcpyAsync(scales, p->d_scl, sizeof(float) * c.ncc * c.nstokes * kK,
                                        cudaMemcpyDeviceToHost, p->s_comp),
                        "D2H scales");
    if (!rc && vdif) {
        if (!c.do_ipfb) return set_error(VGB_ERR_STATE, "pipeline was created without the IPFB");
        rc = check_cuda(cudaMemcpyAsync(vdif, p->d_vdif, (size_t)c.ncc * ns * 544, cudaMemcpyDeviceToHost, p->s_comp),
                        "D2H vdif");
    }
    if (rc) return rc;
    rc = check_cuda(cudaStreamSynchronize(p->s_comp), "sync");
    if (rc) return rc;
    return vgb_check_device_status(p->s_comp, nullptr);
}

int vgb_pipeline_fetch_incoh(vgb_pipeline *p, uint8_t *psrfits, float *offsets, float *scales)
{
    if (!p) return set_error(VGB_ERR_INVALID, "NULL pipeline");
    const size_t ns = p->nspectra, ncc = p->cfg.ncc;
    int rc = VGB_SUCCESS;
    if (psrfits)
        rc = check_cuda(cudaMemcpyAsync(psrfits, p->d_ipsr, ns * ncc * kK, cudaMemcpyDeviceToHost, p->s_comp),
                        "D2H incoherent psrfits");
    if (!rc && offsets)
        rc = check_cuda(cudaMemcpyAsync(offsets, p->d_ioff, sizeof(float) * ncc * kK, cudaMemcpyDeviceToHost,
                                        p->s_comp),
                        "D2H incoherent offsets");
    if (!rc && scales)
        rc = check_cuda(cudaMemcpyAsync(scales, p->d_iscl, sizeof(float) * ncc * kK, cudaMemcpyDeviceToHost,
                                        p->s_comp),
                        "D2H incoherent scales");
    if (rc) return rc;
    return check_cuda(cudaStreamSynchronize(p->s_comp), "sync");
}

int vgb_pipeline_set_host_incoh(vgb_pipeline *p, uint8_t *psrfits, float *offsets, float *scales)
{
    if (!p) return set_error(VGB_ERR_INVALID, "NULL pipeline");
    int rc = check_cuda(cudaStreamSynchronize(p->s_comp), "sync");
    if (rc) return rc;
    drop_graphs(p); // graphs captured the previous destinations
    p->h_ipsr = psrfits;
    p->h_ioff = offsets;
    p->h_iscl = scales;
    return VGB_SUCCESS;
}

int vgb_pipeline_fetch_raw(vgb_pipeline *p, float *S_, void *e, float *incoh)
{
    if (!p) return set_error(VGB_ERR_INVALID, "NULL pipeline");
    const size_t n = (size_t)p->cfg.ncc * p->nspectra * kK;
    int rc = VGB_SUCCESS;
    if (S_)
        rc = check_cuda(cudaMemcpyAsync(S_, p->d_S, sizeof(float) * n * p->cfg.nstokes, cudaMemcpyDeviceToHost,
                                        p->s_comp),
                        "D2H S");
    if (!rc && e)
        rc = check_cuda(cudaMemcpyAsync(e, p->d_e, sizeof(float4) * n, cudaMemcpyDeviceToHost, p->s_comp), "D2H e");
    if (!rc && incoh)
        rc = check_cuda(cudaMemcpyAsync(incoh, p->d_incoh, sizeof(float) * n, cudaMemcpyDeviceToHost, p->s_comp),
                        "D2H incoh");
    if (rc) return rc;
    return check_cuda(cudaStreamSynchronize(p->s_comp), "sync");
}

int vgb_pipeline_device_products(vgb_pipeline *p, const float **S_, const void **e, const float **incoh,
                                 const uint8_t **psrfits, const uint8_t **vdif)
{
    if (!p) return set_error(VGB_ERR_INVALID, "NULL pipeline");
    int rc = check_cuda(cudaStreamSynchronize(p->s_comp), "sync");
    if (rc) return rc;
    if (S_) *S_ = p->d_S;
    if (e) *e = p->d_e;
    if (incoh) *incoh = p->d_incoh;
    if (psrfits) *psrfits = p->d_psrfits;
    if (vdif) *vdif = p->d_vdif;
    return VGB_SUCCESS;
}

int vgb_pipeline_launch_count(vgb_pipeline *p) { return p ? p->launches : 0; }

void *vgb_pipeline_stream(vgb_pipeline *p) { return p ? (void *)p->s_comp : nullptr; }

int vgb_pipeline_set_host_outputs(vgb_pipeline *p, uint8_t *psrfits, float *offsets, float *scales, uint8_t *vdif)
{
    if (!p) return set_error(VGB_ERR_INVALID, "NULL pipeline");
    if (vdif && !p->cfg.do_ipfb) return set_error(VGB_ERR_STATE, "pipeline was created without the IPFB");
    // graphs captured the previous destinations
    int rc = check_cuda(cudaStreamSynchronize(p->s_comp), "sync");
    if (rc) return rc;
    drop_graphs(p);
    p->h_psrfits = psrfits;
    p->h_off = offsets;
    p->h_scl = scales;
    p->h_vdif = vdif;
    return VGB_SUCCESS;
}

int vgb_pipeline_sync(vgb_pipeline *p)
{
    if (!p) return set_error(VGB_ERR_INVALID, "NULL pipeline");
    int rc = check_cuda(cudaStreamSynchronize(p->s_copy), "sync copy stream");
    rc = rc ? rc : check_cuda(cudaStreamSynchronize(p->s_comp), "sync compute stream");
    return rc ? rc : vgb_check_device_status(p->s_comp, nullptr);
}

int vgb_pipeline_enable_timing(vgb_pipeline *p, int on)
{
    if (!p) return set_error(VGB_ERR_INVALID, "NULL pipeline");
    p->timing = on != 0;
    return VGB_SUCCESS;
}

int vgb_pipeline_stage_ms(vgb_pipeline *p, float *ms, int n)
{
    if (!p || !ms) return set_error(VGB_ERR_INVALID, "NULL argument");
    if (!p->timing || p->second == 0) return set_error(VGB_ERR_STATE, "timing not enabled or nothing run");
    int rc = check_cuda(cudaEventSynchronize(p->ev_stage[4]), "sync stage events");
    for (int i = 0; i < n && i < 4 && !rc; i++)
        rc = check_cuda(cudaEventElapsedTime(&ms[i], p->ev_stage[i], p->ev_stage[i + 1]), "stage time");
    if (!rc && n > 4) rc = check_cuda(cudaEventElapsedTime(&ms[4], p->ev_stage[5], p->ev_stage[0]), "stage time");
    return rc;
}

} // extern "C"
