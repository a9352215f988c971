// The VCSBeam library's own GPU entry points (the vm* / cu_* functions of
// src/pfb.cpp and src/form_beam.cpp, declared in include/vcsbeam.h.in), with
// the same names, arguments and vcsbeam_context fields, implemented on this
// library's GB300 kernels (vcsbeam_gb300.h). A VCSBeam build links this in
// place of pfb.cpp and form_beam.cpp and its app/ programs run unchanged.
//
// This file has no declaration of its own for the context: it is compiled
// against the VCSBeam installation's configured vcsbeam.h and the dependency
// headers that header includes (mwalib, PAL, psrfits_utils, vdifio,
// hyperbeam, MPI), so every field it touches sits where that build puts it.
//
// Two groups of functions:
//  * strong: every function pfb.cpp and form_beam.cpp define;
//  * weak: the device-memory, upload and read-buffer helpers of metadata.c,
//    geometry.c and buffer.c that the per-second loop calls around them
//    (vmMalloc*/vmFree*, vmSetMaxGPUMem, vmPushChunk, vmPushJ, vmPushPhi,
//    vmCreateStatistics, vmCreateCudaStreams, vmInitReadBuffer, ...). A build
//    that keeps those source files gets theirs (a strong definition wins at
//    link time); a program linked without them gets these, which do the same.
//
// Differences a caller can see, all in what is not computed rather than in
// results:
//  * the forward PFB is one fused pass (weighted overlap-add, rounding, FFT,
//    packing): vmWOLAChunk, vmFPGARoundingChunk and vmFFTChunk only record
//    their stage and vmPackChunk runs the pass, so fpfb->d_weighted_overlap_add
//    (2.75 GB in the reference) is NULL and fpfb->plan is unused;
//  * vmBeamformSecond on MWAX voltages runs the fused PFB + beamformer per
//    pointing straight from the uploaded voltages (the packed fine channels
//    in fpfb->d_vcs_data are not formed); vmApplyJChunk only records its
//    stage and vmBeamformChunk applies J^-1 and forms the beam in one pass,
//    so the Jv_P / Jv_Q buffers are not used;
//  * cu_invert_pfb uses the floor-correct tap range for the first 1,536
//    output samples of each second, where the reference's truncating index
//    (pfb.cpp:863) shifts the tap set;
//  * the kernels work in FP32 (the reference's beamformer in FP64); e and S
//    are written in the reference's layouts and types.
// Errors end the process with a message, as the reference's GPU macros do
// (gpu_macros.h:27-35); vgb_last_error() holds the library's own message.
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <unordered_map>

#include "vcsbeam.h"
#include "vcsbeam_gb300.h"

#define VGB_WEAK __attribute__((weak))

namespace {

constexpr int kK = 128, kP = 12, kFrames = 500, kSamplesPerBlock = 64000;

[[noreturn]] void fail(const char *fn, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    std::fprintf(stderr, "error: %s: ", fn);
    std::vfprintf(stderr, fmt, ap);
    std::fprintf(stderr, "\n");
    va_end(ap);
    std::exit(EXIT_FAILURE);
}

void ck(cudaError_t e, const char *fn, const char *what)
{
    if (e != cudaSuccess) fail(fn, "%s: %s", what, cudaGetErrorString(e));
}

void vk(int rc, const char *fn)
{
    if (rc != VGB_SUCCESS) fail(fn, "%s", vgb_last_error());
}

// Per-context state this library keeps beside the reference's struct.
struct CtxState {
    float4 *d_W = nullptr;           // [p][a][c] two float4 (W = phi J^-1)
    size_t W_n = 0;
    float4 *d_ef = nullptr;          // complex float beam voltages of one chunk, [s][c][pol]
    size_t ef_bytes = 0;
    unsigned wola_flags = 0; // VGB_WOLA_FP32 / VGB_WOLA_FP32_SPLIT for the loaded filter
    unsigned stages = 0;             // forward-PFB / ApplyJ stages recorded since the last pass
};
struct IpfbState {
    float *d_coeffs = nullptr;       // ncoeffs synthesis taps
    float2 *h_x = nullptr, *d_x = nullptr;  // (ntaps + nsamples) rows of [c][pol] complex float
    size_t x_bytes = 0;
};
std::mutex g_mu;
std::unordered_map<const void *, CtxState> g_ctx;
std::unordered_map<const void *, IpfbState> g_ipfb;

CtxState &state(const vcsbeam_context *vm)
{
    std::lock_guard<std::mutex> lk(g_mu);
    return g_ctx[vm];
}

template <class T> void dmalloc(T **p, size_t bytes, const char *fn)
{
    ck(cudaMalloc(reinterpret_cast<void **>(p), bytes), fn, "cudaMalloc");
}
template <class T> void hmalloc(T **p, size_t bytes, const char *fn)
{
    ck(cudaMallocHost(reinterpret_cast<void **>(p), bytes), fn, "cudaMallocHost");
}

// The reference's read buffer / upload chunk as this library's voltage view:
// one margin block, then `nblocks` blocks of [input][64000] char2.
vgb_voltages chunk_view(const void *base, int ninputs, int nblocks)
{
    const long long block = (long long)ninputs * kSamplesPerBlock * 2;
    vgb_voltages v{};
    v.hist = static_cast<const char *>(base) + (long long)(kFrames - kP) * kK * 2;
    v.hist_input_stride = (long long)kSamplesPerBlock * 2;
    v.cur = static_cast<const char *>(base) + block;
    v.cur_block_stride = block;
    v.ninputs = ninputs;
    v.nblocks = nblocks;
    return v;
}

// complex float [n] -> complex double [n] (the reference's e type)
__global__ void widen_kernel(const float2 *in, double2 *out, long long n)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = make_double2(in[i].x, in[i].y);
}

void widen(const void *in, void *out, long long n, const char *fn)
{
    if (n <= 0) return;
    widen_kernel<<<(unsigned)((n + 255) / 256), 256>>>(static_cast<const float2 *>(in), static_cast<double2 *>(out),
                                                        n);
    ck(cudaGetLastError(), fn, "widen_kernel");
}

int nant_of(const vcsbeam_context *vm) { return (int)vm->obs_metadata->num_ants; }

// W = phi J^-1 for every pointing from the pushed tables (vmPushJ, vmPushPhi).
void build_weights(vcsbeam_context *vm, CtxState &s, const char *fn)
{
    const size_t n = (size_t)vm->npointing * nant_of(vm) * vm->nfine_chan;
    if (!vm->d_J || !vm->gdelays.d_phi) fail(fn, "J and phi must be on the device (vmPushJ, vmPushPhi)");
    if (s.W_n < n) {
        if (s.d_W) cudaFree(s.d_W);
        dmalloc(&s.d_W, n * 2 * sizeof(float4), fn);
        s.W_n = n;
    }
    vk(vgb_weights(vm->d_J, vm->gdelays.d_phi, (long long)n, s.d_W, nullptr), fn);
}

void ensure_ef(CtxState &s, size_t bytes, const char *fn)
{
    if (s.ef_bytes >= bytes) return;
    if (s.d_ef) cudaFree(s.d_ef);
    dmalloc(&s.d_ef, bytes, fn);
    s.ef_bytes = bytes;
}

float inverse_weight(const vcsbeam_context *vm, const char *fn)
{
    if (vm->num_not_flagged <= 0) fail(fn, "no unflagged RF inputs");
    return (float)(1.0 / vm->num_not_flagged);
}

enum : unsigned { kStageWola = 1, kStageRound = 2, kStageFft = 4, kStageApplyJ = 8 };

} // namespace

extern "C" {

// ===========================================================================
// Forward PFB (pfb.cpp)
// ===========================================================================

// pfb.cpp:378-496. Same fields as the reference, without the WOLA scratch
// buffer and the cuFFT plan (the pass is fused).
void vmInitForwardPFB(vcsbeam_context *vm, int M, pfb_flags flags)
{
    const char *fn = "vmInitForwardPFB";
    vm->fpfb = static_cast<forward_pfb *>(std::calloc(1, sizeof(forward_pfb)));
    forward_pfb *f = vm->fpfb;
    f->flags = flags;
    const unsigned nsamples = (unsigned)(vm->vcs_metadata->num_samples_per_voltage_block *
                                         vm->vcs_metadata->num_voltage_blocks_per_second);
    f->nspectra = nsamples / M;
    f->M = M;
    f->K = vm->analysis_filter->nchans;
    f->I = (int)vm->obs_metadata->num_rf_inputs;
    f->P = vm->analysis_filter->ncoeffs / f->K;
    if (f->K != kK || f->P != kP || M != kK || vm->vcs_metadata->num_samples_per_voltage_block != kSamplesPerBlock)
        fail(fn, "the GB300 kernels take 128 channels, 12 taps, M = K and 64000-sample blocks (got K %d, P %d, "
                 "M %d, %llu samples per block)",
             f->K, f->P, M, (unsigned long long)vm->vcs_metadata->num_samples_per_voltage_block);

    hmalloc(&f->i_output_idx, sizeof(int) * f->I, fn);
    dmalloc(&f->d_i_output_idx, sizeof(int) * f->I, fn);
    for (int i = 0; i < f->I; i++) {
        const Rfinput &r = vm->obs_metadata->rf_inputs[i];
        const int mwax = 2 * (int)r.ant + (*r.pol - 'X');
        if (mwax < 0 || mwax >= f->I) fail(fn, "RF input %d maps outside the MWAX order", i);
        f->i_output_idx[mwax] = (int)r.vcs_order;
    }
    ck(cudaMemcpy(f->d_i_output_idx, f->i_output_idx, sizeof(int) * f->I, cudaMemcpyHostToDevice), fn, "H2D");

    while (f->nspectra % vm->chunks_per_second != 0) vm->chunks_per_second++;
    f->nspectra_per_chunk = f->nspectra / vm->chunks_per_second;
    const uint64_t nblk = vm->vcs_metadata->num_voltage_blocks_per_second;
    const uint64_t block_bytes = vm->vcs_metadata->voltage_block_size_bytes;
    if (nblk % vm->chunks_per_second != 0)
        fail(fn, "%u chunks per second do not divide the %llu voltage blocks", (unsigned)vm->chunks_per_second,
             (unsigned long long)nblk);
    const uint64_t blocks_per_chunk = nblk / vm->chunks_per_second;
    f->d_htr_size = (blocks_per_chunk + 1) * block_bytes;
    if (flags & PFB_COMPLEX_INT4) {
        f->vcs_size = (size_t)f->nspectra * f->I * f->K;
        vm->datatype = VM_INT4;
    } else {
        f->vcs_size = (size_t)f->nspectra * f->I * f->K * sizeof(gpuDoubleComplex);
        vm->datatype = VM_DBL;
    }
    f->d_vcs_size = f->vcs_size / vm->chunks_per_second;
    f->htr_stride = nblk * block_bytes / vm->chunks_per_second;
    f->vcs_stride = f->d_vcs_size;
    f->char2s_per_second = nblk * block_bytes / 2;
    f->bytes_per_block = block_bytes;
    f->d_weighted_overlap_add = nullptr; // fused: no overlap-add buffer
    f->weighted_overlap_add_size = 0;

    const size_t filter_size = sizeof(int) * vm->analysis_filter->ncoeffs;
    hmalloc(&f->filter_coeffs, filter_size, fn);
    dmalloc(&f->d_filter_coeffs, filter_size, fn);
    for (int i = 0; i < vm->analysis_filter->ncoeffs; i++)
        f->filter_coeffs[i] = (int)vm->analysis_filter->coeffs[i]; // the reference's cast to int
    ck(cudaMemcpy(f->d_filter_coeffs, f->filter_coeffs, filter_size, cudaMemcpyHostToDevice), fn, "H2D");
    f->vcs_data = nullptr;
    if (flags & PFB_MALLOC_HOST_OUTPUT) hmalloc(&f->vcs_data, f->vcs_size, fn);
    if (flags & PFB_MALLOC_DEVICE_INPUT) dmalloc(&f->d_htr_data, f->d_htr_size, fn);
    if (flags & PFB_MALLOC_DEVICE_OUTPUT) dmalloc(&f->d_vcs_data, f->d_vcs_size, fn);
    f->ninputs_per_cufft_batch = 32;
    f->cufft_batch_size = f->nspectra_per_chunk * f->ninputs_per_cufft_batch;
    std::memset(&f->plan, 0, sizeof(f->plan));
    state(vm).wola_flags = vgb_filter_wola_flags(f->filter_coeffs, kP, kK);

    vm->fine_sample_rate = f->nspectra;
    vm->nfine_chan = f->K;
}

// pfb.cpp:506-518
void vmFreeForwardPFB(forward_pfb *f)
{
    if (!f) return;
    cudaFreeHost(f->filter_coeffs);
    cudaFreeHost(f->vcs_data);
    cudaFreeHost(f->i_output_idx);
    cudaFree(f->d_filter_coeffs);
    cudaFree(f->d_htr_data);
    cudaFree(f->d_vcs_data);
    cudaFree(f->d_i_output_idx);
    std::free(f);
}

// pfb.cpp:544-561: the chunk's blocks (one margin block + the chunk) from
// the read buffer; the buffer unlocks after the second's last chunk.
void vmUploadForwardPFBChunk(vcsbeam_context *vm)
{
    const char *fn = "vmUploadForwardPFBChunk";
    forward_pfb *f = vm->fpfb;
    const int chunk = vm->chunk_to_load % vm->chunks_per_second;
    ck(cudaMemcpy(f->d_htr_data, static_cast<char *>(vm->v->buffer) + chunk * f->htr_stride, f->d_htr_size,
                  cudaMemcpyHostToDevice),
       fn, "H2D");
    if (chunk == (int)vm->chunks_per_second - 1) vm->v->locked = false;
}

// pfb.cpp:569-649: the three stages before packing, fused into vmPackChunk.
void vmWOLAChunk(vcsbeam_context *vm) { state(vm).stages |= kStageWola; }
void vmFPGARoundingChunk(vcsbeam_context *vm) { state(vm).stages |= kStageRound; }
void vmFFTChunk(vcsbeam_context *vm) { state(vm).stages |= kStageFft; }

// pfb.cpp:657-673: the whole forward PFB of the uploaded chunk into
// fpfb->d_vcs_data (legacy order, 4+4-bit or complex double).
void vmPackChunk(vcsbeam_context *vm)
{
    const char *fn = "vmPackChunk";
    forward_pfb *f = vm->fpfb;
    CtxState &s = state(vm);
    s.stages &= ~(kStageWola | kStageRound | kStageFft);
    const vgb_voltages v = chunk_view(f->d_htr_data, f->I, (int)(f->nspectra_per_chunk / kFrames));
    const unsigned fl = ((unsigned)f->flags & (VGB_PFB_COMPLEX_INT4 | VGB_PFB_COMPLEX_FLOAT64 |
                                               VGB_PFB_IMAG_PART_FIRST | VGB_PFB_EMULATE_FPGA)) |
                        s.wola_flags;
    vk(vgb_fpfb(&v, 1, f->nspectra_per_chunk, f->d_filter_coeffs, kP, kK, f->d_i_output_idx, fl, f->d_vcs_data,
                nullptr),
       fn);
    ck(cudaDeviceSynchronize(), fn, "synchronise");
    vk(vgb_check_device_status(nullptr, nullptr), fn);
}

// pfb.cpp:699-715
void vmDownloadForwardPFBChunk(vcsbeam_context *vm)
{
    forward_pfb *f = vm->fpfb;
    const int chunk = vm->chunk_to_load % vm->chunks_per_second;
    ck(cudaMemcpy(static_cast<char *>(f->vcs_data) + chunk * f->vcs_stride, f->d_vcs_data, f->d_vcs_size,
                  cudaMemcpyDeviceToHost),
       "vmDownloadForwardPFBChunk", "D2H");
}

// pfb.cpp:730-773
void vmExecuteForwardPFB(vcsbeam_context *vm)
{
    if (!vm->v || !vm->v->buffer) fail("vmExecuteForwardPFB", "Input data buffer have not been set");
    for (unsigned chunk = 0; chunk < vm->chunks_per_second; chunk++) {
        vmUploadForwardPFBChunk(vm);
        vmWOLAChunk(vm);
        vmFPGARoundingChunk(vm);
        vmFFTChunk(vm);
        vmPackChunk(vm);
        if (vm->fpfb->vcs_data) vmDownloadForwardPFBChunk(vm);
        vm->chunk_to_load++;
    }
}

// pfb.cpp:781-796 (the file name comes from metadata.c's vmGetLegacyVoltFilename)
void vmGetLegacyVoltFilename(vcsbeam_context *, unsigned int, uint64_t, char *) VGB_WEAK;
void vmWritePFBOutputToFile(vcsbeam_context *vm)
{
    const char *fn = "vmWritePFBOutputToFile";
    if (!vmGetLegacyVoltFilename) fail(fn, "vmGetLegacyVoltFilename (metadata.c) is not linked");
    char filename[128];
    vmGetLegacyVoltFilename(vm, vm->coarse_chan_idxs_to_process[0],
                            vm->gps_seconds_to_process[vm->current_gps_idx - 1], filename);
    FILE *out = std::fopen(filename, "w");
    if (!out) fail(fn, "cannot open %s", filename);
    std::fwrite(vm->fpfb->vcs_data, vm->fpfb->vcs_size, 1, out);
    std::fclose(out);
}

// ===========================================================================
// Inverse PFB (pfb.cpp:940-1102)
// ===========================================================================

// pfb.cpp:1054-1085: the reference's sizes and buffers, plus this library's
// packed complex input and its synthesis taps.
void malloc_ipfb(struct gpu_ipfb_arrays *g, pfb_filter *filter, int nsamples, int npol, int npointing)
{
    const char *fn = "malloc_ipfb";
    const int ntaps = filter->ntaps, nchan = filter->nchans, fil_size = filter->ncoeffs;
    if (ntaps != kP || nchan != kK || npol != 2)
        fail(fn, "the GB300 inverse PFB takes 12 taps, 128 channels, 2 pols (got %d, %d, %d)", ntaps, nchan, npol);
    g->ntaps = ntaps;
    g->in_size = npointing * ((nsamples + ntaps) * nchan * npol) * (int)sizeof(float);
    g->ft_size = fil_size * nchan * (int)sizeof(float);
    g->out_size = npointing * nsamples * nchan * npol * 2 * (int)sizeof(float);
    dmalloc(&g->d_in_real, g->in_size, fn);
    dmalloc(&g->d_in_imag, g->in_size, fn);
    dmalloc(&g->d_ft_real, g->ft_size, fn);
    dmalloc(&g->d_ft_imag, g->ft_size, fn);
    dmalloc(&g->d_out, g->out_size, fn);
    g->in_real = static_cast<float *>(std::malloc(g->in_size));
    g->in_imag = static_cast<float *>(std::malloc(g->in_size));
    g->ft_real = static_cast<float *>(std::malloc(g->ft_size));
    g->ft_imag = static_cast<float *>(std::malloc(g->ft_size));
    IpfbState st;
    dmalloc(&st.d_coeffs, sizeof(float) * fil_size, fn);
    st.x_bytes = (size_t)(nsamples + ntaps) * nchan * npol * sizeof(float2);
    hmalloc(&st.h_x, st.x_bytes, fn);
    dmalloc(&st.d_x, st.x_bytes, fn);
    std::lock_guard<std::mutex> lk(g_mu);
    g_ipfb[g] = st;
}

// pfb.cpp:1025-1041: the reference's filter x twiddle tables (host and
// device), and the scaled taps this library's FFT-factorised synthesis uses.
void cu_load_ipfb_filter(pfb_filter *filter, struct gpu_ipfb_arrays *g)
{
    const char *fn = "cu_load_ipfb_filter";
    for (int f = 0; f < filter->ncoeffs; f++)
        for (int ch = 0; ch < filter->nchans; ch++) {
            const int i = filter->ncoeffs * ch + f;
            const gpuDoubleComplex tw =
                filter->twiddles ? filter->twiddles[ch] : make_cuDoubleComplex(1.0, 0.0);
            g->ft_real[i] = (float)(cuCreal(tw) * filter->coeffs[f]);
            g->ft_imag[i] = (float)(cuCimag(tw) * filter->coeffs[f]);
        }
    ck(cudaMemcpy(g->d_ft_real, g->ft_real, g->ft_size, cudaMemcpyHostToDevice), fn, "H2D");
    ck(cudaMemcpy(g->d_ft_imag, g->ft_imag, g->ft_size, cudaMemcpyHostToDevice), fn, "H2D");
    IpfbState st;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        st = g_ipfb[g];
    }
    if (!st.d_coeffs) fail(fn, "call malloc_ipfb first");
    float taps[kK * kP];
    for (int f = 0; f < kK * kP; f++) taps[f] = (float)filter->coeffs[f];
    ck(cudaMemcpy(st.d_coeffs, taps, sizeof(taps), cudaMemcpyHostToDevice), fn, "H2D");
}

// pfb.cpp:940-1003: the second's beam voltages and the 12 samples before
// them out of the two-second ring (zeros for file 0), synthesised to
// data_buffer_vdif [nsamples*128][pol][re, im].
void cu_invert_pfb(gpuDoubleComplex *data_buffer_fine, int file_no, int npointing, int nsamples, int nchan,
                   int npol, int sizeof_buffer, struct gpu_ipfb_arrays *g, float *data_buffer_vdif)
{
    (void)sizeof_buffer;
    const char *fn = "cu_invert_pfb";
    if (npointing > 1) fail(fn, "PFB inversion currently only supports a single pointing");
    IpfbState st;
    {
        std::lock_guard<std::mutex> lk(g_mu);
        st = g_ipfb[g];
    }
    if (!st.d_x) fail(fn, "call malloc_ipfb first");
    const int ntaps = g->ntaps;
    const int start_s = (file_no % 2 == 0 ? 2 * nsamples - ntaps : nsamples - ntaps);
    const size_t row = (size_t)nchan * npol;
    for (int s_in = 0; s_in < nsamples + ntaps; s_in++) {
        float2 *dst = st.h_x + s_in * row;
        if (file_no == 0 && s_in < ntaps) {
            std::memset(dst, 0, row * sizeof(float2));
            continue;
        }
        const int s = (start_s + s_in) % (2 * nsamples);
        const gpuDoubleComplex *src = data_buffer_fine + (size_t)s * row;
        for (size_t k = 0; k < row; k++) dst[k] = make_float2((float)cuCreal(src[k]), (float)cuCimag(src[k]));
    }
    ck(cudaMemcpy(st.d_x, st.h_x, st.x_bytes, cudaMemcpyHostToDevice), fn, "H2D");
    const long long hist_bytes = (long long)ntaps * row * sizeof(float2);
    vk(vgb_ipfb(reinterpret_cast<char *>(st.d_x) + hist_bytes, (long long)nsamples * row * sizeof(float2), st.d_x,
                hist_bytes, st.d_coeffs, kP, kK, nsamples, 1, g->d_out, nullptr, nullptr, 0, nullptr),
       fn);
    ck(cudaMemcpy(data_buffer_vdif, g->d_out, g->out_size, cudaMemcpyDeviceToHost), fn, "D2H");
}

// pfb.cpp:1090-1102
void free_ipfb(struct gpu_ipfb_arrays *g)
{
    std::free(g->in_real);
    std::free(g->in_imag);
    std::free(g->ft_real);
    std::free(g->ft_imag);
    cudaFree(g->d_in_real);
    cudaFree(g->d_in_imag);
    cudaFree(g->d_ft_real);
    cudaFree(g->d_ft_imag);
    cudaFree(g->d_out);
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_ipfb.find(g);
    if (it != g_ipfb.end()) {
        cudaFree(it->second.d_coeffs);
        cudaFree(it->second.d_x);
        cudaFreeHost(it->second.h_x);
        g_ipfb.erase(it);
    }
}

// ===========================================================================
// Beamformer (form_beam.cpp)
// ===========================================================================

// form_beam.cpp:463-505: incoherent sum of 4+4-bit legacy voltages
// [nsample][nchan][ninput], then its 8-bit renormalise (one Stokes).
void cu_form_incoh_beam(uint8_t *data, uint8_t *d_data, size_t data_size, float *d_incoh, unsigned int nsample,
                        int nchan, int ninput, float *offsets, float *d_offsets, float *scales, float *d_scales,
                        uint8_t *Iscaled, uint8_t *d_Iscaled, size_t Iscaled_size)
{
    const char *fn = "cu_form_incoh_beam";
    ck(cudaMemcpy(d_data, data, data_size, cudaMemcpyHostToDevice), fn, "H2D");
    vk(vgb_incoh_beam(d_data, (long long)nsample * nchan, ninput, d_incoh, nullptr), fn);
    vk(vgb_renormalise(d_incoh, 1, 1, (int)nsample, 1, nchan, d_Iscaled, 0, 0, nchan, nchan, d_offsets, d_scales,
                       nullptr),
       fn);
    ck(cudaMemcpy(offsets, d_offsets, nchan * sizeof(float), cudaMemcpyDeviceToHost), fn, "D2H");
    ck(cudaMemcpy(scales, d_scales, nchan * sizeof(float), cudaMemcpyDeviceToHost), fn, "D2H");
    ck(cudaMemcpy(Iscaled, d_Iscaled, Iscaled_size, cudaMemcpyDeviceToHost), fn, "D2H");
}

// form_beam.cpp:510-533: J^-1 is applied inside vmBeamformChunk's pass.
void vmApplyJChunk(vcsbeam_context *vm) { state(vm).stages |= kStageApplyJ; }

// form_beam.cpp:541-582: beam of the chunk of legacy-layout fine channels in
// vm->d_v (4+4-bit or complex double, v_IDX) for every pointing: S and e at
// the chunk's samples of the second (C_IDX, B_IDX).
void vmBeamformChunk(vcsbeam_context *vm)
{
    const char *fn = "vmBeamformChunk";
    CtxState &s = state(vm);
    s.stages &= ~kStageApplyJ;
    const int nant = nant_of(vm), K = (int)vm->nfine_chan, nst = vm->out_nstokes;
    const int nsc = vm->fine_sample_rate / (int)vm->chunks_per_second;
    const int chunk = vm->chunk_to_load % vm->chunks_per_second;
    const int soff = chunk * nsc;
    build_weights(vm, s, fn);
    ensure_ef(s, (size_t)nsc * K * 2 * sizeof(float2), fn);
    const float invw = inverse_weight(vm, fn);
    for (unsigned p = 0; p < vm->npointing; p++) {
        float *S = static_cast<float *>(vm->d_S) + ((size_t)p * vm->fine_sample_rate + soff) * nst * K;
        vk(vgb_beamform_legacy(vm->d_v, vm->datatype == VM_INT4 ? VGB_INT4 : VGB_DBL, nsc, K, nant, vm->d_polQ_idxs,
                               vm->d_polP_idxs, s.d_W + (size_t)p * nant * K * 2, 1, invw, nst, S, s.d_ef, nullptr,
                               nullptr),
           fn);
        widen(s.d_ef, vm->d_e + ((size_t)p * vm->fine_sample_rate + soff) * K * 2, (long long)nsc * K * 2, fn);
    }
    ck(cudaDeviceSynchronize(), fn, "synchronise");
    vk(vgb_check_device_status(nullptr, nullptr), fn);
}

void vmPushChunk(vcsbeam_context *vm);

// form_beam.cpp:587-627. MWAX: per chunk, upload and one fused PFB +
// beamformer pass per pointing; legacy: per chunk, vmPushChunk then
// vmBeamformChunk. Unlocks the read buffer at the end.
void vmBeamformSecond(vcsbeam_context *vm)
{
    const char *fn = "vmBeamformSecond";
    if (vm->obs_metadata->mwa_version == VCSLegacyRecombined) {
        for (unsigned chunk = 0; chunk < vm->chunks_per_second; chunk++) {
            vmPushChunk(vm);
            vmApplyJChunk(vm);
            vmBeamformChunk(vm);
            vm->chunk_to_load++;
        }
        ck(cudaDeviceSynchronize(), fn, "synchronise");
        vm->v->locked = false;
        return;
    }
    forward_pfb *f = vm->fpfb;
    if (!f) fail(fn, "vmInitForwardPFB has not been called");
    CtxState &s = state(vm);
    const int nant = nant_of(vm), K = kK, nst = vm->out_nstokes;
    if (f->I != 2 * nant) fail(fn, "%d RF inputs for %d antennas", f->I, nant);
    // the fused pass takes antenna a's X / Y inputs as MWAX inputs 2a / 2a+1;
    // the pol index lists (vmSetPolIdxLists) must name the same inputs
    if (vm->polQ_idxs && vm->polP_idxs)
        for (int a = 0; a < nant; a++)
            if ((int)vm->polQ_idxs[a] != f->i_output_idx[2 * a] || (int)vm->polP_idxs[a] != f->i_output_idx[2 * a + 1])
                fail(fn, "antenna %d: pol index lists disagree with the PFB's input order", a);
    build_weights(vm, s, fn);
    const int nsc = f->nspectra_per_chunk;
    ensure_ef(s, (size_t)nsc * K * 2 * sizeof(float2), fn);
    const float invw = inverse_weight(vm, fn);
    const unsigned fl = ((unsigned)f->flags & (VGB_PFB_COMPLEX_INT4 | VGB_PFB_EMULATE_FPGA)) |
                        s.wola_flags;
    for (unsigned chunk = 0; chunk < vm->chunks_per_second; chunk++) {
        vmUploadForwardPFBChunk(vm);
        const vgb_voltages v = chunk_view(f->d_htr_data, f->I, nsc / kFrames);
        const int soff = (vm->chunk_to_load % vm->chunks_per_second) * nsc;
        for (unsigned p = 0; p < vm->npointing; p++) {
            float *S = static_cast<float *>(vm->d_S) + ((size_t)p * vm->fine_sample_rate + soff) * nst * K;
            vk(vgb_beamform_mwax(&v, 1, nsc, f->d_filter_coeffs, kP, kK, fl, s.d_W + (size_t)p * nant * K * 2, nant,
                                 invw, nst, S, s.d_ef, nullptr, nullptr),
               fn);
            widen(s.d_ef, vm->d_e + ((size_t)p * vm->fine_sample_rate + soff) * K * 2, (long long)nsc * K * 2, fn);
        }
        vm->chunk_to_load++;
    }
    ck(cudaDeviceSynchronize(), fn, "synchronise");
    vk(vgb_check_device_status(nullptr, nullptr), fn);
    vm->v->locked = false;
}

// form_beam.cpp:632-644. The reference queues these copies asynchronously
// and its programs read vm->e / vm->S on the host right after
// (app/make_mwa_tied_array_beam.c:280-283); here the copy has finished when
// the call returns.
void vmPullE(vcsbeam_context *vm)
{
    ck(cudaMemcpy(vm->e, vm->d_e, vm->e_size_bytes, cudaMemcpyDeviceToHost), "vmPullE", "D2H");
}
void vmPullS(vcsbeam_context *vm)
{
    ck(cudaMemcpy(vm->S, vm->d_S, vm->S_size_bytes, cudaMemcpyDeviceToHost), "vmPullS", "D2H");
}

// form_beam.cpp:653-673: 8-bit renormalise of every pointing's Stokes into
// the PSRFITS sub-integration of mpfs[p] (data [s][stokes][chan], offsets and
// scales [stokes][chan]).
void vmSendSToFits(vcsbeam_context *vm, mpi_psrfits *mpfs)
{
    const char *fn = "vmSendSToFits";
    const int K = (int)vm->nfine_chan, nst = vm->out_nstokes, ns = vm->fine_sample_rate;
    cudaStream_t st = vm->streams ? vm->streams[0] : nullptr;
    vk(vgb_renormalise(static_cast<const float *>(vm->d_S), 1, (int)vm->npointing, ns, nst, K, vm->d_Cscaled, 0,
                       (long long)ns * nst * K, (long long)nst * K, K, vm->d_offsets, vm->d_scales, st),
       fn);
    ck(cudaDeviceSynchronize(), fn, "synchronise");
    ck(cudaMemcpy(vm->offsets, vm->d_offsets, vm->offsets_size, cudaMemcpyDeviceToHost), fn, "D2H");
    ck(cudaMemcpy(vm->scales, vm->d_scales, vm->scales_size, cudaMemcpyDeviceToHost), fn, "D2H");
    ck(cudaMemcpy(vm->Cscaled, vm->d_Cscaled, vm->Cscaled_size, cudaMemcpyDeviceToHost), fn, "D2H");
    for (unsigned p = 0; p < vm->npointing; p++) {
        std::memcpy(mpfs[p].coarse_chan_pf.sub.dat_offsets, vm->offsets + (size_t)p * K * nst, sizeof(float) * K * nst);
        std::memcpy(mpfs[p].coarse_chan_pf.sub.dat_scales, vm->scales + (size_t)p * K * nst, sizeof(float) * K * nst);
        std::memcpy(mpfs[p].coarse_chan_pf.sub.data, vm->Cscaled + (size_t)p * ns * K * nst, (size_t)ns * K * nst);
    }
}

// form_beam.cpp:679-683
void vmPushPolIdxLists(vcsbeam_context *vm)
{
    const char *fn = "vmPushPolIdxLists";
    ck(cudaMemcpy(vm->d_polQ_idxs, vm->polQ_idxs, vm->pol_idxs_size_bytes, cudaMemcpyHostToDevice), fn, "H2D");
    ck(cudaMemcpy(vm->d_polP_idxs, vm->polP_idxs, vm->pol_idxs_size_bytes, cudaMemcpyHostToDevice), fn, "H2D");
}

// form_beam.cpp:690-700
float *create_pinned_data_buffer(size_t size)
{
    float *p = nullptr;
    hmalloc(&p, size, "create_pinned_data_buffer");
    std::memset(p, 0, size);
    return p;
}

// form_beam.cpp:707-727 (deprecated in the reference)
gpuDoubleComplex ****create_detected_beam(int npointing, int nsamples, int nchan, int npol)
{
    auto a = static_cast<gpuDoubleComplex ****>(std::malloc(npointing * sizeof(gpuDoubleComplex ***)));
    for (int p = 0; p < npointing; p++) {
        a[p] = static_cast<gpuDoubleComplex ***>(std::malloc(nsamples * sizeof(gpuDoubleComplex **)));
        for (int s = 0; s < nsamples; s++) {
            a[p][s] = static_cast<gpuDoubleComplex **>(std::malloc(nchan * sizeof(gpuDoubleComplex *)));
            for (int c = 0; c < nchan; c++)
                a[p][s][c] = static_cast<gpuDoubleComplex *>(std::malloc(npol * sizeof(gpuDoubleComplex)));
        }
    }
    return a;
}

// form_beam.cpp:734-746
gpuDoubleComplex *create_data_buffer_fine(int npointing, int nsamples, int nchan, int npol)
{
    const size_t bytes = (size_t)npointing * nsamples * nchan * npol * sizeof(gpuDoubleComplex);
    auto *b = static_cast<gpuDoubleComplex *>(std::malloc(bytes));
    std::memset(b, 0, bytes);
    return b;
}

// form_beam.cpp:753-780: vm->e into the half of the two-second ring this
// timestep owns (the reference's indexing, pointing stride included).
void prepare_data_buffer_fine(gpuDoubleComplex *data_buffer_fine, vcsbeam_context *vm, uintptr_t timestep_idx)
{
    const size_t nchan = vm->nfine_chan, npol = vm->obs_metadata->num_ant_pols, ns = vm->fine_sample_rate;
    const size_t offset = (timestep_idx % 2) * ns;
    for (unsigned p = 0; p < vm->npointing; p++)
        std::memcpy(data_buffer_fine + (p * ns + offset) * nchan * npol, vm->e + p * ns * nchan * npol,
                    ns * nchan * npol * sizeof(gpuDoubleComplex));
}

// form_beam.cpp:787-805 (deprecated in the reference)
void allocate_input_output_arrays(void **data, void **d_data, size_t size)
{
    ck(cudaMallocHost(data, size), "allocate_input_output_arrays", "cudaMallocHost");
    ck(cudaMalloc(d_data, size), "allocate_input_output_arrays", "cudaMalloc");
}
void free_input_output_arrays(void *data, void *d_data)
{
    cudaFreeHost(data);
    cudaFree(d_data);
}

// ===========================================================================
// Weak: device memory, uploads and the read buffer (metadata.c, geometry.c,
// buffer.c), the same sizes and copies as the reference's
// ===========================================================================

// buffer.c:52-77, 86-91, 106-124
VGB_WEAK host_buffer *vmInitReadBuffer(size_t read_size, size_t copy_size)
{
    if (read_size == 0) return nullptr;
    auto *rb = static_cast<host_buffer *>(std::malloc(sizeof(host_buffer)));
    rb->buffer_size = read_size + copy_size;
    hmalloc(&rb->buffer, rb->buffer_size, "vmInitReadBuffer");
    rb->read_size = read_size;
    rb->copy_size = copy_size;
    rb->read_ptr = static_cast<char *>(rb->buffer) + copy_size;
    rb->copy_from_ptr = static_cast<char *>(rb->buffer) + read_size;
    rb->copy_to_ptr = rb->buffer;
    rb->locked = false;
    return rb;
}
VGB_WEAK void vmFreeReadBuffer(host_buffer *rb)
{
    if (!rb) return;
    cudaFreeHost(rb->buffer);
    std::free(rb);
}
VGB_WEAK vm_error vmReadBufferCopyMargin(host_buffer *rb)
{
    if (!rb || !rb->buffer) return VM_READ_BUFFER_NOT_SET;
    if (!rb->copy_from_ptr || !rb->copy_to_ptr || rb->copy_size == 0) return VM_SUCCESS;
    std::memcpy(rb->copy_to_ptr, rb->copy_from_ptr, rb->copy_size);
    return VM_SUCCESS;
}

// metadata.c:448-454
VGB_WEAK void vmMallocVHost(vcsbeam_context *vm)
{
    if (vm->obs_metadata->mwa_version == VCSLegacyRecombined)
        vm->v = vmInitReadBuffer(vm->bytes_per_second, 0);
    else if (vm->obs_metadata->mwa_version == VCSMWAXv2)
        vm->v = vmInitReadBuffer(vm->bytes_per_second, vm->vcs_metadata->voltage_block_size_bytes);
}
VGB_WEAK void vmFreeVHost(vcsbeam_context *vm) { vmFreeReadBuffer(vm->v); }

// metadata.c:464-476, 683-708: sizes as the reference's; this library's
// beamformer applies J^-1 inside its pass, so no Jv buffers are allocated.
VGB_WEAK void vmMallocJVHost(vcsbeam_context *vm)
{
    vm->Jv_size_bytes = vm->npointing * vm->obs_metadata->num_ants * vm->nfine_chan * vm->fine_sample_rate *
                        sizeof(gpuDoubleComplex);
    vm->Jv_P = vm->Jv_Q = nullptr;
}
VGB_WEAK void vmFreeJVHost(vcsbeam_context *) {}
VGB_WEAK void vmMallocJVDevice(vcsbeam_context *vm)
{
    vm->d_Jv_size_bytes = vm->npointing * vm->obs_metadata->num_ants * vm->nfine_chan * vm->fine_sample_rate *
                          sizeof(gpuDoubleComplex) / vm->chunks_per_second;
    vm->d_Jv_P = vm->d_Jv_Q = nullptr;
}
VGB_WEAK void vmFreeJVDevice(vcsbeam_context *) {}

// metadata.c:484-559, 717-807
VGB_WEAK void vmMallocEHost(vcsbeam_context *vm)
{
    vm->e_size_bytes = vm->npointing * vm->fine_sample_rate * vm->nfine_chan * vm->obs_metadata->num_ant_pols *
                       sizeof(gpuDoubleComplex);
    hmalloc(&vm->e, vm->e_size_bytes, "vmMallocEHost");
}
VGB_WEAK void vmFreeEHost(vcsbeam_context *vm) { cudaFreeHost(vm->e); }
VGB_WEAK void vmMallocEDevice(vcsbeam_context *vm)
{
    vm->d_e_size_bytes = vm->npointing * vm->fine_sample_rate * vm->nfine_chan * vm->obs_metadata->num_ant_pols *
                         sizeof(gpuDoubleComplex);
    dmalloc(&vm->d_e, vm->d_e_size_bytes, "vmMallocEDevice");
}
VGB_WEAK void vmFreeEDevice(vcsbeam_context *vm) { cudaFree(vm->d_e); }
VGB_WEAK void vmMallocSHost(vcsbeam_context *vm)
{
    vm->S_size_bytes = vm->npointing * vm->nfine_chan * vm->out_nstokes * vm->fine_sample_rate * sizeof(float);
    hmalloc(&vm->S, vm->S_size_bytes, "vmMallocSHost");
}
VGB_WEAK void vmFreeSHost(vcsbeam_context *vm) { cudaFreeHost(vm->S); }
VGB_WEAK void vmMallocSDevice(vcsbeam_context *vm)
{
    vm->d_S_size_bytes = vm->npointing * vm->nfine_chan * vm->out_nstokes * vm->fine_sample_rate * sizeof(float);
    dmalloc(&vm->d_S, vm->d_S_size_bytes, "vmMallocSDevice");
}
VGB_WEAK void vmFreeSDevice(vcsbeam_context *vm) { cudaFree(vm->d_S); }
VGB_WEAK void vmMallocJHost(vcsbeam_context *vm)
{
    vm->J_size_bytes = vm->npointing * vm->obs_metadata->num_ants * vm->nfine_chan *
                       vm->obs_metadata->num_visibility_pols * sizeof(gpuDoubleComplex);
    hmalloc(&vm->J, vm->J_size_bytes, "vmMallocJHost");
}
VGB_WEAK void vmFreeJHost(vcsbeam_context *vm) { cudaFreeHost(vm->J); }
VGB_WEAK void vmMallocJDevice(vcsbeam_context *vm)
{
    vm->d_J_size_bytes = vm->npointing * vm->obs_metadata->num_ants * vm->nfine_chan *
                         vm->obs_metadata->num_visibility_pols * sizeof(gpuDoubleComplex);
    dmalloc(&vm->d_J, vm->d_J_size_bytes, "vmMallocJDevice");
}
VGB_WEAK void vmFreeJDevice(vcsbeam_context *vm) { cudaFree(vm->d_J); }
VGB_WEAK void vmMallocDHost(vcsbeam_context *vm)
{
    vm->D_size_bytes = vm->obs_metadata->num_ants * vm->nfine_chan * vm->obs_metadata->num_visibility_pols *
                       sizeof(gpuDoubleComplex);
    hmalloc(&vm->D, vm->D_size_bytes, "vmMallocDHost");
}
VGB_WEAK void vmFreeDHost(vcsbeam_context *vm) { cudaFreeHost(vm->D); }
VGB_WEAK void vmMallocDDevice(vcsbeam_context *vm)
{
    vm->d_D_size_bytes = vm->obs_metadata->num_ants * vm->nfine_chan * vm->obs_metadata->num_visibility_pols *
                         sizeof(gpuDoubleComplex);
    dmalloc(&vm->d_D, vm->d_D_size_bytes, "vmMallocDDevice");
}
VGB_WEAK void vmFreeDDevice(vcsbeam_context *vm) { cudaFree(vm->d_D); }
VGB_WEAK void vmMallocPQIdxsHost(vcsbeam_context *vm)
{
    vm->pol_idxs_size_bytes = vm->obs_metadata->num_ants * sizeof(uint32_t);
    hmalloc(&vm->polP_idxs, vm->pol_idxs_size_bytes, "vmMallocPQIdxsHost");
    hmalloc(&vm->polQ_idxs, vm->pol_idxs_size_bytes, "vmMallocPQIdxsHost");
}
VGB_WEAK void vmFreePQIdxsHost(vcsbeam_context *vm)
{
    cudaFreeHost(vm->polP_idxs);
    cudaFreeHost(vm->polQ_idxs);
}
VGB_WEAK void vmMallocPQIdxsDevice(vcsbeam_context *vm)
{
    vm->d_pol_idxs_size_bytes = vm->obs_metadata->num_ants * sizeof(uint32_t);
    dmalloc(&vm->d_polP_idxs, vm->d_pol_idxs_size_bytes, "vmMallocPQIdxsDevice");
    dmalloc(&vm->d_polQ_idxs, vm->d_pol_idxs_size_bytes, "vmMallocPQIdxsDevice");
}
VGB_WEAK void vmFreePQIdxsDevice(vcsbeam_context *vm)
{
    cudaFree(vm->d_polP_idxs);
    cudaFree(vm->d_polQ_idxs);
}

// metadata.c:656-671, 811-817: MWAX fine channels live in the PFB's output
VGB_WEAK void vmMallocVDevice(vcsbeam_context *vm)
{
    if (vm->obs_metadata->mwa_version == VCSLegacyRecombined) {
        vm->d_v_size_bytes = vm->bytes_per_second / vm->chunks_per_second;
        dmalloc(reinterpret_cast<char **>(&vm->d_v), vm->d_v_size_bytes, "vmMallocVDevice");
    } else {
        vm->d_v = vm->fpfb->d_vcs_data;
        vm->d_v_size_bytes = vm->fpfb->d_vcs_size;
    }
}
VGB_WEAK void vmFreeVDevice(vcsbeam_context *vm)
{
    if (vm->obs_metadata->mwa_version == VCSLegacyRecombined) cudaFree(vm->d_v);
}

// metadata.c:892-906
VGB_WEAK void vmSetMaxGPUMem(vcsbeam_context *vm, int nchunks)
{
    vm->chunks_per_second = nchunks;
    if (nchunks <= 0 || vm->sample_rate % nchunks != 0)
        fail("vmSetMaxGPUMem", "Bad number of chunks requested: must divide number of samples per second of data.");
    vm->d_v_size_bytes = vm->bytes_per_second / vm->chunks_per_second;
    vm->d_Jv_size_bytes = vm->Jv_size_bytes / vm->chunks_per_second;
}

// metadata.c:913-923
VGB_WEAK void vmPushChunk(vcsbeam_context *vm)
{
    const int chunk = vm->chunk_to_load % vm->chunks_per_second;
    ck(cudaMemcpy(vm->d_v, static_cast<char *>(vm->v->buffer) + chunk * vm->d_v_size_bytes, vm->d_v_size_bytes,
                  cudaMemcpyHostToDevice),
       "vmPushChunk", "H2D");
}

// metadata.c:1000-1014, geometry.c:192-198
VGB_WEAK void vmPushJ(vcsbeam_context *vm)
{
    ck(cudaMemcpy(vm->d_J, vm->J, vm->J_size_bytes, cudaMemcpyHostToDevice), "vmPushJ", "H2D");
}
VGB_WEAK void vmPushPhi(vcsbeam_context *vm)
{
    const size_t bytes = vm->gdelays.npointings * vm->gdelays.nant * vm->gdelays.nchan * sizeof(gpuDoubleComplex);
    ck(cudaMemcpy(vm->gdelays.d_phi, vm->gdelays.phi, bytes, cudaMemcpyHostToDevice), "vmPushPhi", "H2D");
}

// metadata.c:1023-1050
VGB_WEAK void vmCreateCudaStreams(vcsbeam_context *vm)
{
    vm->streams = static_cast<gpuStream_t *>(std::malloc(vm->npointing * sizeof(gpuStream_t)));
    for (unsigned p = 0; p < vm->npointing; p++) ck(cudaStreamCreate(&vm->streams[p]), "vmCreateCudaStreams", "stream");
}
VGB_WEAK void vmDestroyCudaStreams(vcsbeam_context *vm)
{
    for (unsigned p = 0; p < vm->npointing; p++) cudaStreamDestroy(vm->streams[p]);
    std::free(vm->streams);
    vm->streams = nullptr;
}

// metadata.c:1061-1099
VGB_WEAK void vmCreateStatistics(vcsbeam_context *vm, mpi_psrfits *mpfs)
{
    const char *fn = "vmCreateStatistics";
    vm->offsets_size = vm->npointing * vm->nfine_chan * vm->out_nstokes * sizeof(float);
    vm->scales_size = vm->npointing * vm->nfine_chan * vm->out_nstokes * sizeof(float);
    vm->Cscaled_size = vm->npointing * mpfs[0].coarse_chan_pf.sub.bytes_per_subint;
    dmalloc(&vm->d_offsets, vm->offsets_size, fn);
    dmalloc(&vm->d_scales, vm->scales_size, fn);
    dmalloc(&vm->d_Cscaled, vm->Cscaled_size, fn);
    hmalloc(&vm->offsets, vm->offsets_size, fn);
    hmalloc(&vm->scales, vm->scales_size, fn);
    hmalloc(&vm->Cscaled, vm->Cscaled_size, fn);
}
VGB_WEAK void vmDestroyStatistics(vcsbeam_context *vm)
{
    cudaFreeHost(vm->offsets);
    cudaFreeHost(vm->scales);
    cudaFreeHost(vm->Cscaled);
    cudaFree(vm->d_offsets);
    cudaFree(vm->d_scales);
    cudaFree(vm->d_Cscaled);
}

// The per-context state this library keeps for `vm` (no reference
// counterpart: call after the context's buffers are freed).
void vgb_compat_release(vcsbeam_context *vm)
{
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_ctx.find(vm);
    if (it == g_ctx.end()) return;
    cudaFree(it->second.d_W);
    cudaFree(it->second.d_ef);
    g_ctx.erase(it);
}

} // extern "C"
