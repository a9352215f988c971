/*
 * vcsbeam_gb300.h -- plain C ABI of the GB300 voltage hot path.
 *
 * Every entry point takes device pointers, sizes and a CUDA stream (as
 * void *, NULL = the legacy default stream), returns VGB_SUCCESS or an error
 * code, and never exits the process. vgb_last_error() describes the last
 * failure on the calling thread. Launches are asynchronous on the given
 * stream; vgb_check_device_status() reports errors kernels raised (a bounded
 * wait that expired, a frame outside the described buffers, an input index
 * outside the voltage row).
 *
 * VCSBeam's own GPU API (the vm* / cu_* functions of its src/pfb.cpp and
 * src/form_beam.cpp, over its vcsbeam_context) is implemented on top of these
 * calls in mwa-vcsbeam_gb300/csrc/compat/vm_compat.cu (libvcsbeam_compat.so),
 * compiled against the VCSBeam build's own configured vcsbeam.h.
 * Each entry point below names the reference routine(s) it replaces;
 * file:line references are to the VCSBeam source tree.
 *
 * Layouts use the reference's index macros (include/vcsbeam.h.in:234-268):
 *   MWAX voltages  [block][input][sample] char2, 64000 samples per block,
 *                  input = 2*antenna + pol (pol 0 = X = "Q", 1 = Y = "P")
 *   legacy/fine    v_IDX [sample][chan][input]
 *   Stokes         C_IDX [pointing][sample][stokes][chan]
 *   beam voltages  B_IDX [pointing][sample][chan][pol] complex float
 * Batched calls add a leading coarse-channel dimension ("cc").
 */
#ifndef VCSBEAM_GB300_H
#define VCSBEAM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define VGB_SUCCESS 0
#define VGB_ERR_INVALID 1     /* an argument is out of range or misaligned */
#define VGB_ERR_CUDA 2        /* a CUDA runtime call failed */
#define VGB_ERR_DEVICE 3      /* a kernel raised its device status word */
#define VGB_ERR_UNSUPPORTED 4 /* a shape the kernels are not built for */
#define VGB_ERR_ALLOC 5       /* device or pinned host allocation failed */
#define VGB_ERR_STATE 6       /* call out of order (e.g. buffer locked) */

/* ---- pfb_flags bits (include/vcsbeam.h.in:459-480) ---- */
#define VGB_PFB_COMPLEX_INT4 0x10
#define VGB_PFB_COMPLEX_FLOAT64 0x20
#define VGB_PFB_IMAG_PART_FIRST 0x100
#define VGB_PFB_EMULATE_FPGA 0x200

/* Not reference bits: the arithmetic of the weighted overlap-add. Neither
 * bit: int32 sums (any filter). VGB_WOLA_FP32: one FP32 sum, exact (identical
 * results) only when every partial sum of the filter times int8 voltages
 * stays within 2^24; vgb_filter_fp32_exact() checks that. VGB_WOLA_FP32_SPLIT:
 * the even and the odd taps summed apart in FP32 and added once, exact when
 * each half's partial sums stay within 2^24 (the reference's FINEPFB filter,
 * peak tap 117,964, is such a filter); ignored with VGB_PFB_EMULATE_FPGA,
 * whose rounding takes the int32 sums. vgb_filter_wola_flags() picks the
 * fastest exact one for a filter. */
#define VGB_WOLA_FP32 0x10000
#define VGB_WOLA_FP32_SPLIT 0x20000
/* Force the int32 sums (takes precedence over the two bits above). In a
 * pipeline's configured pfb_flags any of the three WOLA bits overrides the
 * choice it derives from the filter. */
#define VGB_WOLA_INT32 0x40000

/* ---- vcsbeam_datatype (include/vcsbeam.h.in:346-350) ---- */
#define VGB_INT4 0
#define VGB_DBL 1

/* Fine-PFB geometry the kernels are built for: 128 channels, 12 taps,
 * 64000-sample MWAX blocks (pfb.cpp:153 hard-codes the 500 frames/block). */
#define VGB_NCHAN 128
#define VGB_NTAPS 12
#define VGB_SAMPLES_PER_BLOCK 64000

const char *vgb_last_error(void);
int vgb_version(void);
/* 1 if FP32 accumulation of the weighted overlap-add is exact for this
 * host-side filter (K*P taps) and int8 voltages, else 0. */
int vgb_filter_fp32_exact(const int32_t *filter, int ntaps, int nchan);
/* VGB_WOLA_FP32 when one FP32 sum is exact for this host-side filter (K*P
 * taps) and int8 voltages, else VGB_WOLA_FP32_SPLIT when the even/odd split
 * sums are, else 0 (int32). The pipeline and the VCSBeam API layer apply it
 * to the filter they are given. */
unsigned vgb_filter_wola_flags(const int32_t *filter, int ntaps, int nchan);
/* Copies and clears the device status word of the current device (after
 * synchronising `stream`). Returns VGB_ERR_DEVICE if any bit was set. */
int vgb_check_device_status(void *stream, unsigned *flags_out);
/* Self-test of the bounded waits: one kernel waits on an mbarrier that
 * nothing arrives on for `polls` polls, gives up and flags the device status
 * word (VGB_ERR_DEVICE from vgb_check_device_status; the context stays
 * usable). */
int vgb_selftest_bounded_wait(int polls, void *stream);

/*
 * Where one second of MWAX voltages lives, per coarse channel. Window frame
 * w (128 samples) of the second is history frame w for w < 12 (the last 12
 * frames of the previous second) and frame w-12 of the second otherwise.
 * The reference's read buffer (one margin block, then the second,
 * buffer.c:52-77, metadata.c:448-454) is hist = buffer + 488*256 bytes,
 * hist_input_stride = 128000, cur = buffer + block_bytes,
 * cur_block_stride = block_bytes. All pointers and strides in bytes and
 * multiples of 16 (the frames are copied by the TMA unit).
 */
typedef struct vgb_voltages {
    const void *hist;
    long long hist_input_stride;
    long long hist_cc_stride;
    const void *cur;
    long long cur_block_stride;
    long long cur_cc_stride;
    int ninputs;
    int nblocks;
} vgb_voltages;

/*
 * Fused forward fine PFB + tied-array beam + incoherent sum + Stokes
 * detection for `ncc` coarse channels of MWAX voltages. Replaces, per second:
 * vmUploadForwardPFBChunk..vmPackChunk (pfb.cpp:544-673) followed by
 * vmApplyJChunk and vmBeamformChunk (form_beam.cpp:510-582), i.e.
 * vmBeamformSecond (form_beam.cpp:587-627) for one pointing.
 *   filter      K*P int32 analysis taps (pfb.cpp:459-460 cast)
 *   pfb_flags   VGB_PFB_EMULATE_FPGA and/or VGB_PFB_COMPLEX_INT4 select the
 *               rounding (pfb.cpp:602-616) and the 4-bit demotion the
 *               reference's beamformer input carries (pfb.cpp:325-332);
 *               a VGB_WOLA_* bit the overlap-add arithmetic (none: int32)
 *   W           [ncc][nant][128][2][2] complex float: phi * J^-1
 *               (vgb_weights)
 *   invw        1 / number of unflagged RF inputs (metadata.c:1554-1561)
 *   S           [ncc][nspectra][nstokes][128] float (nstokes 1 or 4)
 *   e           [ncc][nspectra][128][2] complex float, or NULL
 *   incoh       [ncc][nspectra][128] float, or NULL
 */
int vgb_beamform_mwax(const vgb_voltages *v, int ncc, int nspectra, const int32_t *filter, int ntaps,
                      int nchan, unsigned pfb_flags, const void *W, int nant, float invw, int nstokes,
                      float *S, void *e, float *incoh, void *stream);
/* The fused front end has four variants, all giving identical results:
 * 4 inputs (two tiles) per step in 256-thread CTAs (two per SM); 8 inputs per
 * step in 512-thread CTAs (one per SM); 5, the 4-input shape at three CTAs
 * per SM (each thread's beam sums kept in tensor memory between steps, taps
 * read from shared memory, frames and weights single-buffered); and 3,
 * warp-specialised: one 416-thread CTA per SM whose front warps run the PFB
 * of step i while its back warps sum step i - 1, handing rows over through
 * mbarriers instead of block-wide barriers (measured slower: 26.0 against
 * 21.5 ms per data-second of the full band, so it runs only when forced).
 * The first call for a shape times variants 4, 8 and 5 and keeps the fastest
 * (a call made while the stream is being captured uses the known choice,
 * else 4). Force one with 3, 4, 5 or 8, or 0 for the timed choice; returns
 * the previous setting, -1 on a bad value. */
int vgb_pfb_variant(int inputs_per_step);
/* Variant of the last fused front-end launch (3, 4, 5 or 8; 0 before the first). */
int vgb_pfb_variant_last(void);

/*
 * Forward fine PFB only, packed to the legacy recombined layout (the output
 * of vmExecuteForwardPFB, pfb.cpp:730-773): out [ncc][nspectra][128][ninputs]
 * uint8 (4+4-bit, VGB_PFB_COMPLEX_INT4) or complex double, input i written at
 * column i_idx[i] (the VCS order, pfb.cpp:410-419). i_idx must be a
 * permutation of 0 .. ninputs-1 (the reference's map is; otherwise nothing is
 * written and the device status word reports bad input); at most 1024 inputs.
 * The inputs are processed in the order of their output columns, so each row
 * of the output is written in whole adjacent groups.
 */
int vgb_fpfb(const vgb_voltages *v, int ncc, int nspectra, const int32_t *filter, int ntaps, int nchan,
             const int32_t *i_idx, unsigned pfb_flags, void *out, void *stream);

/* The reference's four forward-PFB stages, one call each (pfb.cpp:569-673):
 * vgb_wola: b[m][i][n] int32 pairs (vmWOLAChunk, without memset/atomics);
 * vgb_round: in place int32 -> float, FPGA rounding or 2^-14 (vmFPGARoundingChunk);
 * vgb_fft128: in-place forward 128-point FFTs of nrows float2 rows (vmFFTChunk);
 * vgb_pack: rows [m][i][k] -> legacy layout (vmPackChunk). */
int vgb_wola(const vgb_voltages *v, int nspectra, const int32_t *filter, int ntaps, int nchan, int32_t *b,
             void *stream);
int vgb_round(int32_t *b, long long nvalues, int emulate_fpga, void *stream);
int vgb_fft128(void *rows, long long nrows, void *stream);
int vgb_pack(const void *ffted, int nspectra, int ninputs, const int32_t *i_idx, unsigned pfb_flags,
             void *out, void *stream);

/*
 * Table builders on the device in FP64 (replacing the host loops
 * vmCalcPhi geometry.c:111-135 and vmCalcJ jones.c:97-157, and the pushes
 * vmPushPhi geometry.c:192-198 / vmPushJ metadata.c:1000-1014):
 *   vgb_phase:   phi[p][a][c] complex double from tile E/N/H/cable (m),
 *                pointing unit vectors unit[p][3] = (E, N, H) and channel
 *                frequencies (Hz); href = array reference height (m)
 *   vgb_jones:   J[p][a][c][2][2] = inv(norm_F(D[a][c] B[p][a]))
 *   vgb_weights: W[n][2][2] complex float = phi[n] * J[n] (n = p*nant*nchan + ...)
 */
int vgb_phase(const double *unit, const double *east, const double *north, const double *height,
              const double *cable, const double *chan_freqs_hz, int npointing, int nant, int nchan,
              double href, void *phi, void *stream);
int vgb_jones(const void *D, const void *B, int npointing, int nant, int nchan, void *J, void *stream);
int vgb_weights(const void *J, const void *phi, long long n, void *W, void *stream);

/*
 * Beamformer for fine voltages already in the legacy layout v_IDX
 * [nsamples][nchan][2*nant], 4+4-bit (VGB_INT4) or complex double (VGB_DBL)
 * (vmApplyJChunk + vmBeamformChunk, form_beam.cpp:510-582, for legacy
 * recombined input, form_beam.cpp:593-596). polQ/polP: vcs_order of each
 * antenna's X/Y input (jones.c:40-64). W [npointing][nant][nchan][2][2].
 * S [npointing][nsamples][nstokes][nchan]; e (nullable) [npointing][nsamples][nchan][2]
 * complex float; incoh (nullable, VGB_INT4 only) [nsamples][nchan].
 */
int vgb_beamform_legacy(const void *v, int datatype, int nsamples, int nchan, int nant, const uint32_t *polQ,
                        const uint32_t *polP, const void *W, int npointing, float invw, int nstokes, float *S,
                        void *e, float *incoh, void *stream);

/* Incoherent beam of 4+4-bit voltages [nrows][ninput] -> [nrows] float
 * (incoh_beam, form_beam.cpp:60-87, nrows = nsample*nchan). */
int vgb_incoh_beam(const uint8_t *data, long long nrows, int ninput, float *incoh, void *stream);

/*
 * Per-channel 8-bit scale-and-offset (renormalise_channels_kernel,
 * form_beam.cpp:408-449, launched by vmSendSToFits form_beam.cpp:653-663 and
 * cu_form_incoh_beam form_beam.cpp:495-497) for ncc coarse channels.
 * S [ncc][npointing][nstep][nstokes][nchan] float. The 8-bit output element
 * (cc, p, s, st, c) goes to out[cc*out_cc + p*out_p + s*out_s + st*out_st + c]
 * (the per-channel layout, or a spliced multi-channel PSRFITS row layout
 * with no MPI gather, beam_psrfits.c:608-628). offsets/scales:
 * [ncc][npointing][nstokes][nchan].
 */
int vgb_renormalise(const float *S, int ncc, int npointing, int nstep, int nstokes, int nchan, uint8_t *out,
                    long long out_cc, long long out_p, long long out_s, long long out_st, float *offsets,
                    float *scales, void *stream);

/*
 * Inverse PFB to 1.28 MHz complex samples and/or VDIF frames for njobs
 * (coarse channel, pointing) pairs (ipfb_kernel + cu_invert_pfb,
 * pfb.cpp:842-1003, and the quantisation of vdif_write_second,
 * beam_vdif.c:29-92).
 *   e       [job][nsamples][128][2] complex float (B_IDX, one pointing)
 *   hist    [job][12][128][2] complex float: the previous second's last 12
 *           samples, or NULL for the first second (zeros, pfb.cpp:972-976)
 *   coeffs  12*128 float synthesis taps, already scaled (vmScaleFilterCoeffs)
 *   out_f   [job][nsamples*128][2][2] float (data_buffer_vdif layout), or NULL
 *   vdif    [job][nsamples][544] bytes: 32-byte header + 512 payload, or NULL
 *   hdr     [job][8] uint32 DEVICE header template, or NULL for zeros;
 *           frame f carries it advanced by frame_offset + f frames (see the
 *           VDIF header functions below); frame_offset >= 0
 */
int vgb_ipfb(const void *e, long long e_job_stride, const void *hist, long long hist_job_stride,
             const float *coeffs, int ntaps, int nchan, int nsamples, int njobs, float *out_f, uint8_t *vdif,
             const uint32_t *hdr, int frame_offset, void *stream);

/*
 * Voltage files on the host, one second of one coarse channel into a caller's
 * (ideally pinned) buffer, for vgb_pipeline_run_host or an upload. They
 * replace mwalib_voltage_context_read_second (metadata.c:973-985) and
 * mwalib_metafits_get_expected_volt_filename (metadata.c:1214-1226); mwalib
 * itself is not used. Reads are split over `nthreads` positioned reads.
 *
 * MWAX subfile: an ASCII "KEY value" header (HDR_SIZE bytes, default 4096;
 * NINPUTS required; NBIT must be 8 if given; SECS_PER_SUBOBS default 8;
 * OBS_ID, SUBOBS_ID = GPS second of the first block, COARSE_CHANNEL), one
 * metadata block, then 20 blocks of [ninputs][64000] char2 per second.
 * vgb_subfile_read_second writes the second's 20 blocks, [block][input]
 * [sample] (the layout of one coarse channel of the pipeline's input).
 * Legacy recombined file: the whole file (one second, v_IDX 4+4-bit bytes).
 * vgb_volt_filename: <obsid>_<gps>_<rec_chan>.sub (gps rounded down to a
 * multiple of 8, metadata.c:1152) or <obsid>_<gps>_ch<rec_chan>.dat.
 */
typedef struct vgb_subfile_info {
    long long header_bytes;     /* HDR_SIZE */
    long long block_bytes;      /* ninputs * 64000 * 2 */
    long long file_bytes;
    long long obs_id;           /* OBS_ID (0 if absent) */
    long long subobs_id;        /* SUBOBS_ID: GPS second of the first voltage block */
    int ninputs;
    int samples_per_block;      /* 64000 */
    int secs_per_subobs;
    int coarse_channel;         /* COARSE_CHANNEL (-1 if absent) */
    int metadata_blocks;        /* blocks before the voltages (1) */
    int complete;               /* 1 if the file holds every second it names */
} vgb_subfile_info;
int vgb_subfile_info_read(const char *path, vgb_subfile_info *info);
int vgb_subfile_read_second(const char *path, long long gps_second, void *dst, long long dst_bytes, int nthreads);
int vgb_legacy_read_second(const char *path, void *dst, long long dst_bytes, int nthreads);
int vgb_volt_filename(char *out, int out_len, long long obs_id, long long gps_second, int rec_chan, int mwax);

/*
 * VDIF frame headers (8 uint32 words, VDIF 1.0 layout; host memory unless
 * noted). Frame f of a vgb_ipfb call carries the template hdr advanced by
 * frame_offset + f frames at 10000 frames per second, the MWA fine sample
 * rate (nextVDIFHeader applied f times, beam_vdif.c:80): the frame number
 * rolls over to 0 and the seconds field steps on at each whole second.
 *
 * vgb_vdif_header_create     createVDIFHeader (beam_vdif.c:201-202): zero the
 *                            header, set frame length ((bytes + 32) / 8),
 *                            log2(nchan), bits - 1, complex flag, thread id
 *                            and the two-character station id
 * vgb_vdif_header_set_epoch_mjd  setVDIFEpochMJD (beam_vdif.c:209): reference
 *                            epoch = half-years from 2000 to the MJD's date
 * vgb_vdif_header_epoch_mjd  MJD of the header's reference epoch
 * vgb_vdif_header_set_mjdsec setVDIFFrameMJDSec (beam_vdif.c:210): seconds
 *                            since the reference epoch from MJD x 86400 + s
 * vgb_vdif_header_set_frame  setVDIFFrameNumber (beam_vdif.c:211)
 * vgb_vdif_header_next       nextVDIFHeader (beam_vdif.c:80)
 * vgb_vdif_populate_header   the header part of vmPopulateVDIFHeader
 *                            (beam_vdif.c:178-211): 8-bit complex, 2
 *                            channels (one per pol), 512 data bytes, epoch
 *                            and seconds of intmjd + roundf(fracmjd x 86400),
 *                            frame 0; stationid NULL = "mw"
 * vgb_vdif_advance           DEVICE templates d_hdr [njobs][8]: advance each
 *                            by nframes frames (the second-to-second step
 *                            the pipeline takes after every second)
 */
int vgb_vdif_header_create(uint32_t *hdr, int dataarraylength, int threadid, int bits, int nchan, int iscomplex,
                           const char *stationid);
int vgb_vdif_header_set_epoch_mjd(uint32_t *hdr, int mjd);
int vgb_vdif_header_epoch_mjd(const uint32_t *hdr, int *mjd);
int vgb_vdif_header_set_mjdsec(uint32_t *hdr, long long mjdsec);
int vgb_vdif_header_set_frame(uint32_t *hdr, int frame);
int vgb_vdif_header_next(uint32_t *hdr, int frames_per_second);
int vgb_vdif_populate_header(uint32_t *hdr, int intmjd, double fracmjd, int threadid, const char *stationid);
int vgb_vdif_advance(uint32_t *d_hdr, int njobs, int nframes, void *stream);

/*
 * MWAX voltages to 8-bit PSRFITS bytes without allocating any memory. This
 * entry point has no counterpart in the reference. It is for callers that
 * cannot allocate device memory while they run, such as a real-time
 * observing pipeline that reserves all GPU memory at start-up and must not
 * fail or stall on an allocation mid-observation. It runs the fused PFB +
 * beamformer (vgb_beamform_mwax) and then the per-channel renormalise
 * (vgb_renormalise). The full-resolution Stokes passed between them live in a
 * fixed 24 MiB array inside the library, which every GPU that loads the
 * library holds until the process exits. The limit is
 * ncc x nspectra x nstokes x 128 float values <= 6,291,456, i.e. one
 * full-Stokes second of one coarse channel; larger requests are rejected
 * with VGB_ERR_INVALID.
 *   out      [ncc][nspectra][nstokes][128] bytes (C_IDX per channel)
 *   offsets, scales  [ncc][nstokes][128]
 * The array is placed on a device when the library's module holding it is
 * first used there, which (under CUDA's default lazy module loading) is the
 * first call on that device: make one call on each device before reserving
 * the GPU's memory and before any stream capture. A call with nspectra = 0
 * does only that set-up (its other pointers may be NULL). Setting
 * CUDA_MODULE_LOADING=EAGER places the array when the library loads instead.
 * The first call for each new shape also times the fused front end's two
 * tile shapes once (extra launches and a wait on CUDA events, see
 * vgb_pfb_variant); force one with vgb_pfb_variant(4) to skip that.
 * All calls share the one array, which keeps the last call's contents.
 * Nothing in it needs to start at zero, because each call writes every
 * value it reads. Calls that overlap on the GPU (e.g. on different streams)
 * race on it.
 */
int vgb_beamform_mwax_psrfits_noalloc(const vgb_voltages *v, int ncc, int nspectra, const int32_t *filter,
                                      int ntaps, int nchan, unsigned pfb_flags, const void *W, int nant,
                                      float invw, int nstokes, uint8_t *out, float *offsets, float *scales,
                                      void *stream);

/*
 * BF16 GEMM on the tensor cores (tcgen05, accumulators in tensor memory):
 * C[M][N] (FP32, row-major) = A[M][K] * B[N][K]^T, A and B row-major bf16
 * ("K-major"). M, N multiples of 128, K a multiple of 64. The building block
 * of the many-beam beamformer; no reference counterpart (the reference has
 * no tensor-core path, form_beam.cpp:239-371 sums tiles with one thread).
 * The CTA tile width (128 or 256 columns) is chosen per shape by timing both
 * on the first call with that shape (an autotuner; results are identical).
 */
int vgb_gemm_bf16(const void *A, const void *B, float *C, int M, int N, int K, void *stream);

/*
 * Batched form: C[b] = A[b] B[b]^T for b < batch, A[b] at A + b*M*K elements,
 * B[b] at B + b*N*K, C[b] at C + b*M*N. fp16 != 0 selects FP16 operands
 * instead of BF16 (both operands the same type). Same shape rules.
 */
int vgb_gemm_batched(const void *A, const void *B, float *C, int M, int N, int K, int batch, int fp16,
                     void *stream);
/* Split-operand form: C[b] = (A0[b] + A1[b]) B[b]^T where each row of A holds
 * A0 then A1 (K elements each, 2K in all; A[b] at A + b*M*2K) and B[b] at
 * B + b*N*K: the hi + lo product of a split operand with B read once per K
 * step (persistent kernel). M a multiple of 128, N of 256, K of 64. */
int vgb_gemm_batched_planes(const void *A, const void *B, float *C, int M, int N, int K, int batch, int fp16,
                            void *stream);
/* Force the GEMM kernel variant for shapes whose N is a multiple of 256 (128
 * or 256: the plain kernel's tile width; 512: the persistent kernel), or 0 for
 * the autotuned choice. Returns the previous setting (-1 on a bad value). */
int vgb_gemm_variant(int v);

/* Tied-array array factor (calc_array_factor, geometry.c:440-467; Eq. A4 of
 * Meyers et al. 2017) of the look direction at npix test directions, FP64 on
 * the device: af[i] = |sum_a conj(w_a) psi_a|^2 / nant^2 with the geometric
 * phases of vgb_phase at frequency freq_hz (cast to whole Hz as the
 * reference does). look [3], dirs [npix][3] (E, N, H direction cosines),
 * tile east/north/height/cable [nant], af [npix]: device pointers. The
 * building block of the PSF tool (app/mwa_tied_array_beam_psf.c). */
int vgb_array_factor(const double *look, const double *dirs, int npix, double freq_hz, const double *east,
                     const double *north, const double *height, const double *cable, double href, int nant,
                     double *af, void *stream);

/* ---- table inputs on the host: calibration solutions, filter files ----
 * D layout: [nant][nfine][2][2] complex double (D_IDX, vcsbeam.h.in:242-251). */

/* Offringa binary solution of one coarse channel (vmLoadOffringaSolution,
 * calibration.c:426-582). ncc = coarse channels in the solution's request
 * (mpi_size there); nchan_cal = calibration fine channels per coarse channel
 * (the file's own count wins when it differs); each calibration channel fills
 * nfine / nchan_cal fine channels; NaN matrices become zero. counts (nullable)
 * receives the header's interval, antenna, channel and polarisation counts. */
int vgb_cal_load_offringa(const char *path, int coarse_chan_idx, int ncc, int nant, int nchan_cal, int nfine,
                          double *D, uint32_t *counts);

/* RTS solution of one coarse channel (vmLoadRTSSolution, calibration.c:51-225):
 * DIJones file, optional Bandpass file (NULL: DIJones only), D = Dd Db A^-1
 * reversed into the (q, p) basis. cal_ant[a] = index of observation antenna
 * a in the calibration solution (matching tile, calibration.c:165-166). */
int vgb_cal_load_rts(const char *dijones_path, const char *bandpass_path, int nant_cal, int nchan_cal,
                     int chan_width_hz, const int *cal_ant, int nant, int nfine, double *D);

/* vmApplyCalibrationCorrections (calibration.c:747-882): rotate phases
 * against antenna ref_ant (< 0: off), zero PQ/QP unless keep_cross_terms,
 * multiply the first column by exp(i (slope f + offset)). */
int vgb_cal_apply_corrections(double *D, int nant, int nfine, int ref_ant, int keep_cross_terms,
                              double phase_slope, double phase_offset, long long chan_start_hz,
                              int coarse_chan_width_hz);

/* pq_phase_correction.txt lookup for a GPS second
 * (parse_calibration_correction_file, calibration.c:663-745); ref_tile gets
 * the reference tile name or "NONE". */
int vgb_cal_pq_correction(const char *path, uint32_t gpstime, double *slope, double *offset, char *ref_tile,
                          int ref_tile_len, int *found);

/* Zero D of the listed antennas (vmSetCustomTileFlags, calibration.c:952-1013). */
int vgb_cal_flag_tiles(double *D, int nant, int nfine, const int *ants, int nflags);

/* Filter coefficients from an ASCII file, scaled (vmLoadFilter +
 * vmScaleFilterCoeffs, filter.c:62-165). coeffs may be NULL to count. */
int vgb_load_filter(const char *path, int nchans, double scale, double *coeffs, int max_coeffs, int *ncoeffs,
                    int *ntaps);

/* ---- primary beam (vmCalcB, primary_beam.c:79-191) ----
 * B [nfreq][npointing][ntile][2][2] complex double = J P on the device, FP64:
 * J the analytic MWA tile model (4 x 4 dipoles over a ground plane with the
 * tile beamformer delays; the reference's FEE model is not available to this
 * build), P the parallactic-angle rotation at `latitude` (primary_beam.c:
 * 436-456) when pa_correction != 0. az, za [npointing] radians; freq_hz
 * [nfreq]; delays [ntile][16] (0..31, 32 = dead dipole). All device pointers;
 * delays and B 16-byte aligned. Tiles with identical delays share one
 * evaluation (vmCalcB's per-configuration cache), copied to each tile. */
int vgb_primary_beam(const double *az, const double *za, int npointing, const double *freq_hz, int nfreq,
                     const uint32_t *delays, int ntile, double latitude, int pa_correction, void *B, void *stream);
/* Index of a live/dead dipole pattern (amps[16], 0 = dead) among the 138
 * cached configurations of primary_beam.c:355-414; -1 for more than two (but
 * not all) dead dipoles; -2 on a NULL argument. */
int vgb_hash_dipole_config(const double *amps);

/* ---- learned primary-beam surrogate ----
 * An MLP (6 inputs: sin az, cos az, za, frequency, a learned 2-d embedding of
 * the delay set; 4 hidden layers of 256, GELU; 8 outputs: re/im of the 2x2
 * Jones matrix) with BF16 weights and FP32 accumulation on the tensor cores,
 * trained on the device by the library's own forward/backward/Adam kernels on
 * Jones matrices of the plain model (vgb_primary_beam without the
 * parallactic rotation). After validation, queries in sky cells whose error
 * exceeded the tolerance (and tiles whose delays are not a trained set) are
 * answered by the plain model. No reference counterpart: it replaces the
 * beam-model calls of vmCalcB (primary_beam.c:79-191). */
typedef struct vgb_surrogate vgb_surrogate;
/* batch: training / inference rows per GEMM pass, a multiple of 512. */
int vgb_surrogate_create(int nsets, int batch, unsigned long long seed, vgb_surrogate **out);
void vgb_surrogate_destroy(vgb_surrogate *s);
int vgb_surrogate_param_count(const vgb_surrogate *s);
/* FP32 master parameters, host buffers of vgb_surrogate_param_count floats:
 * W0 [256][6], W1..W3 [256][256], W4 [8][256], b0..b3 [256], b4 [8],
 * embeddings [nsets][2]. */
int vgb_surrogate_get_params(vgb_surrogate *s, float *host, int n);
int vgb_surrogate_set_params(vgb_surrogate *s, const float *host, int n);
/* Training table on the device: delay_sets [nsets][16] (host), freqs_hz
 * [nfreq] (host), ndir random directions above 10 degrees elevation. */
int vgb_surrogate_set_training(vgb_surrogate *s, const uint32_t *delay_sets, const double *freqs_hz, int nfreq,
                               int ndir, unsigned long long seed);
/* Adam steps with a cosine learning-rate schedule; loss_host (nullable)
 * receives the mean squared error of each step. */
int vgb_surrogate_train(vgb_surrogate *s, int steps, float lr_max, float lr_min, float *loss_host);
/* One forward/backward pass without an update on a given batch (host
 * arrays, batch rows): feat [batch][4] (sin az, cos az, scaled za, scaled f),
 * set [batch], target [batch][8]; returns the gradient of the mean squared
 * error for every parameter and the loss. For checking the kernels. */
int vgb_surrogate_gradients(vgb_surrogate *s, const float *feat_host, const int *set_host, const float *y_host,
                            float *grad_host, float *loss_host);
/* Validation over nval random (delay set, direction, trained frequency) queries;
 * builds the per-cell error map used for fallback decisions. */
int vgb_surrogate_validate(vgb_surrogate *s, long long nval, float tol, float *max_err, float *frac_cells_ok);
/* B [nfreq][npointing][ntile][2][2] complex double, as vgb_primary_beam, from
 * the surrogate (tile_set[t] = trained delay-set index of tile t, < 0 = none)
 * with plain-model fallback; nfallback (host, nullable) receives the number
 * of (frequency, pointing, tile) entries the plain model answered. The
 * network runs once per (frequency, pointing) for each delay set some tile
 * uses; tile_set and za are read back to the host on `stream` (the call waits
 * for them) to skip work whose answers would be discarded. When no sky cell
 * of any trained set passed the last validation's tolerance, the call is the
 * plain model on `stream` (nothing read back, nothing waited for). */
int vgb_surrogate_beam(vgb_surrogate *s, const double *az, const double *za, int npointing, const double *freq_hz,
                       int nfreq, const int *tile_set, const uint32_t *delays, int ntile, double latitude,
                       int pa_correction, void *B, unsigned *nfallback, void *stream);

/* ---- many-beam beamformer on the tensor cores ----
 *
 * Replaces, for npointing > 1, the per-pointing loop of vmBeamformChunk
 * (vmApplyJ_kernel + vmBeamform_kernel, form_beam.cpp:510-582, 122-371)
 * and the host tables it consumes (vmCalcJ, jones.c:97-188; vmCalcPhi /
 * calc_geometric_delays, geometry.c:40-213), followed by the per-channel
 * 8-bit scale-and-offset of vmSendSToFits (form_beam.cpp:408-449, 653-673).
 * Output Stokes are integrated over 10 samples (1 ms at 10 kHz); a value is
 * the sum of the reference's 10 per-sample Stokes values.
 *
 * Precision modes: split BF16 weights (hi + lo, FP32 accumulate; within 1e-3
 * of the FP64 chain), single BF16, single FP16 on the tensor cores, and FP32
 * weights on the CUDA cores. Voltages are exact in all. */
#define VGB_MB_SPLIT_BF16 0
#define VGB_MB_BF16 1
#define VGB_MB_FP16 2
#define VGB_MB_FP32 3 /* FP32 weights on the CUDA cores (no tensor cores): the plain baseline */
#define VGB_MB_INT4 0 /* legacy 4+4-bit bytes, high nibble real (v_IDX order) */
#define VGB_MB_INT8 1 /* int8 re, im pairs, same order */

typedef struct vgb_multibeam vgb_multibeam;

typedef struct vgb_multibeam_config {
    int ncc;        /* coarse channels per call */
    int nfine;      /* fine channels per coarse channel (128) */
    int nant;       /* tiles, a multiple of 16; ninput = 2*nant */
    int npointing;  /* beams */
    int nsamples;   /* samples per channel per call, a multiple of 10 */
    int nstokes;    /* 1 (I) or 4 (I, Q, U, V) */
    int precision;  /* VGB_MB_* precision mode */
    int input;      /* VGB_MB_INT4 or VGB_MB_INT8 */
    float invw;     /* 1 / unflagged RF inputs */
} vgb_multibeam_config;

int vgb_multibeam_create(const vgb_multibeam_config *cfg, vgb_multibeam **out);
void vgb_multibeam_destroy(vgb_multibeam *mb);
/* Device pointers: unit [npointing][3] (E, N, H direction cosines), tile
 * east/north/height/cable [nant] in metres; href the array reference height. */
int vgb_multibeam_set_geometry(vgb_multibeam *mb, const double *unit, const double *east, const double *north,
                               const double *height, const double *cable, double href, void *stream);
/* Device pointers: D [ncc][nant][nfine][2][2] and B [ncc][npointing][nant][2][2]
 * complex double (calibration and primary-beam Jones, D_IDX / PB order);
 * freqs [ncc][nfine] Hz (lower channel edges); polQ/polP [nant] input indices
 * (vmSetPolIdxLists, jones.c:40-64). */
int vgb_multibeam_set_jones(vgb_multibeam *mb, const double *D, const double *B, const double *freqs,
                            const uint32_t *polQ, const uint32_t *polP, void *stream);
/* v: device [ncc][nsamples][nfine][2*nant] voltages. S (nullable): device
 * float [ncc][nfine][npointing][nstokes][nsamples/10]. out (nullable):
 * device uint8 [ncc][npointing][nsamples/10][nstokes][nfine] with offsets and
 * scales [ncc][npointing][nstokes][nfine]. */
int vgb_multibeam_run(vgb_multibeam *mb, const void *v, float *S, uint8_t *out, float *offsets, float *scales,
                      void *stream);
/* The same from pinned host memory, double-buffered: v_host [ncc][nsamples]
 * [nfine][2*nant] voltages are uploaded one coarse channel ahead of the
 * compute and each channel's PSRFITS bytes, offsets and scales (same layouts
 * as vgb_multibeam_run) are downloaded while the next one computes. Returns
 * once enqueued; `stream` completes after every product is on the host
 * (replaces the synchronous vmPushChunk / vmPullS pattern, metadata.c:
 * 913-923, form_beam.cpp:632-644). */
int vgb_multibeam_run_host(vgb_multibeam *mb, const void *v_host, uint8_t *out_host, float *off_host,
                           float *scl_host, void *stream);
/* Kernels the last vgb_multibeam_run launched. */
int vgb_multibeam_launches(const vgb_multibeam *mb);
/* The beam GEMM's kernel, for all multibeam objects (results are identical):
 * 0 (default) automatic: where the beam tiles of 32 beams pair up, an
 * object's first run (outside stream capture) times the CTA-pair kernel
 * (cta_group::2: the two SMs of a TPC share one 256-row MMA and each stages
 * half of the voltage tile) against the single-CTA kernel on its first coarse
 * channel, two launches each, waits for them, and keeps the faster (a first
 * run inside a capture takes the pair kernel); otherwise the single-CTA
 * kernel. 1 the single-CTA kernel; 2 the pair kernel or an error. Returns the
 * previous setting (-1 on a bad value). */
int vgb_multibeam_beam_variant(int v);
/* CTA pairs (2-CTA clusters) the last beam GEMM ran on; 0 if it ran the
 * single-CTA kernel. */
int vgb_multibeam_last_pair(const vgb_multibeam *mb);
/* Stage timing with CUDA events (off by default): ms[0..4] = weights,
 * voltage conversion, autocorrelation GEMM, beam GEMM, renormalise of the
 * last run, summed over coarse channels (waits for the run to finish). */
int vgb_multibeam_enable_timing(vgb_multibeam *mb, int on);
int vgb_multibeam_stage_ms(vgb_multibeam *mb, float *ms, int n);

/* ---- streaming pipeline: one second of all coarse channels per step ---- */
typedef struct vgb_pipeline vgb_pipeline;

typedef struct vgb_pipeline_config {
    int ncc;                 /* coarse channels processed together */
    int nant;                /* tiles; ninputs = 2*nant */
    int nblocks;             /* MWAX voltage blocks per second (20) */
    int nstokes;             /* 1 or 4 */
    unsigned pfb_flags;      /* rounding / demotion of the beamformer input;
                                no VGB_WOLA_* bit: the exact arithmetic
                                vgb_filter_wola_flags() picks for the filter */
    int do_ipfb;             /* inverse PFB + VDIF */
    float invw;              /* 1 / unflagged RF inputs */
} vgb_pipeline_config;

int vgb_pipeline_create(const vgb_pipeline_config *cfg, vgb_pipeline **out);
int vgb_pipeline_destroy(vgb_pipeline *p);
/* Analysis taps (K*P int32) and, when do_ipfb, synthesis taps (K*P float). */
int vgb_pipeline_set_filters(vgb_pipeline *p, const int32_t *analysis, const float *synthesis);
/* W [ncc][nant][128][2][2] complex float on the host or device (fixed
 * weights; turns per-second tracking off). */
int vgb_pipeline_set_weights(vgb_pipeline *p, const void *W, int on_device);
/*
 * Per-second tracking: every second, before its beamformer, the pipeline
 * rebuilds W on the device from these tables, as vmCalcJonesAndDelays does
 * on the host each second (jones.c:170-188, called from
 * app/make_mwa_tied_array_beam.c:256-262): the second's pointing (the
 * per-second az/za the caller derives from RA/Dec, e.g. with calc_beam_geom,
 * geometry.c:226-286; the unit vector is formed from az and el = pi/2 - za
 * as there), B = vgb_primary_beam at each coarse channel's beam frequency,
 * J^-1 = inv(norm_F(D B)) (vmCalcJ), phi at the fine-channel frequencies
 * (vmCalcPhi) and W = phi J^-1, all FP64 with the arithmetic of vgb_phase /
 * vgb_jones / vgb_weights, W rounded to FP32. Five small launches inside each
 * captured second. Second s of the pipeline (counting from 0, including
 * seconds restored by vgb_pipeline_load_state) uses entry min(s, nseconds-1).
 * All pointers are device pointers that must stay valid while tracking is
 * on; NULL `t` turns tracking off (so does vgb_pipeline_set_weights).
 */
typedef struct vgb_tracking {
    const double *D;             /* [ncc][nant][128][2][2] complex double (D_IDX per coarse channel) */
    const uint32_t *delays;      /* [nant][16] dipole delays 0..31, 32 = dead dipole */
    const double *east, *north, *height, *cable;  /* [nant] metres */
    const double *chan_freqs_hz; /* [ncc][128] fine-channel frequencies for phi (geometry.c:152-163) */
    const double *beam_freqs_hz; /* [ncc] frequency B is evaluated at (the coarse channel's, primary_beam.c:224) */
    const double *az, *za;       /* [nseconds] pointing of each second, radians */
    int nseconds;
    int pa_correction;           /* parallactic-angle rotation of B (primary_beam.c:436-456) */
    double href;                 /* array reference height, metres */
    double latitude;             /* array latitude, radians */
} vgb_tracking;
int vgb_pipeline_set_tracking(vgb_pipeline *p, const vgb_tracking *t);
/* VDIF header template of the next second's first frame, [ncc][8] uint32 on
 * the host (optional; zeros by default). After every second the pipeline
 * advances the templates by that second's frames (vgb_vdif_advance), so the
 * headers run on across seconds as nextVDIFHeader's do (beam_vdif.c:80); the
 * templates are part of the saved state. */
int vgb_pipeline_set_vdif_header(vgb_pipeline *p, const uint32_t *hdr);
/* Process one second whose voltages are already on the device, laid out
 * [cc][block][input][sample] char2 (cc stride cur_cc_stride bytes). The
 * previous second's last 12 frames are carried inside the pipeline. */
int vgb_pipeline_run_device(vgb_pipeline *p, const void *d_voltages, long long cur_cc_stride);
/* The same from host memory (pinned is fastest): copies the second to the
 * device on a copy stream, double-buffered so the next second's copy can
 * overlap this second's compute. */
int vgb_pipeline_run_host(vgb_pipeline *p, const void *h_voltages, long long cur_cc_stride);
/* Copy the last completed second's products to host buffers (each nullable):
 * psrfits [nspectra][nstokes][ncc*128] bytes (channel-spliced rows),
 * offsets/scales [ncc][nstokes][128], vdif [ncc][nspectra][544]. */
int vgb_pipeline_fetch(vgb_pipeline *p, uint8_t *psrfits, float *offsets, float *scales, uint8_t *vdif);
/* The incoherent beam of the last completed second as 8-bit PSRFITS rows
 * (Stokes I; each coarse channel's incoherent sum renormalised per channel
 * as cu_form_incoh_beam does, form_beam.cpp:463-505): psrfits
 * [nspectra][ncc*128] bytes (channel-spliced), offsets/scales [ncc][128]
 * (each nullable). Synchronises. */
int vgb_pipeline_fetch_incoh(vgb_pipeline *p, uint8_t *psrfits, float *offsets, float *scales);
/* Host buffers (each nullable) every following vgb_pipeline_run_* fills
 * asynchronously with the incoherent beam's rows, offsets and scales, as
 * vgb_pipeline_set_host_outputs does for the tied-array beam. */
int vgb_pipeline_set_host_incoh(vgb_pipeline *p, uint8_t *psrfits, float *offsets, float *scales);
/* Copy the last second's unquantised products to host buffers (each
 * nullable), as vmPullS / vmPullE do (form_beam.cpp:632-644):
 * S [ncc][nspectra][nstokes][128] float, e [ncc][nspectra][128][2] complex
 * float, incoh [ncc][nspectra][128] float. */
int vgb_pipeline_fetch_raw(vgb_pipeline *p, float *S, void *e, float *incoh);
/* Device pointers to the last second's products, for chaining further
 * device work (valid until the next vgb_pipeline_run_*). */
int vgb_pipeline_device_products(vgb_pipeline *p, const float **S, const void **e, const float **incoh,
                                 const uint8_t **psrfits, const uint8_t **vdif);
/* Kernel launches the last vgb_pipeline_run_* issued. */
int vgb_pipeline_launch_count(vgb_pipeline *p);
/* The CUDA stream the pipeline computes on (cudaStream_t as void *). */
void *vgb_pipeline_stream(vgb_pipeline *p);
/* Host buffers (pinned for speed; each nullable) that every following
 * vgb_pipeline_run_* fills asynchronously, on the compute stream right after
 * the second's kernels: the vgb_pipeline_fetch products without a
 * synchronisation, so the next second's host-to-device copy overlaps this
 * second's compute. Call vgb_pipeline_sync() before reading them. */
int vgb_pipeline_set_host_outputs(vgb_pipeline *p, uint8_t *psrfits, float *offsets, float *scales,
                                  uint8_t *vdif);
/* Wait for everything the pipeline has queued; reports kernel status. */
int vgb_pipeline_sync(vgb_pipeline *p);
/* Record CUDA events around each stage of every second (off by default). */
int vgb_pipeline_enable_timing(vgb_pipeline *p, int on);
/* Replay each second from a CUDA graph captured on its first occurrence (per
 * input buffer, second parity and output set); on by default, bypassed while
 * stage timing is on. */
int vgb_pipeline_enable_graphs(vgb_pipeline *p, int on);
/* Checkpoint / resume at a second boundary: the state the next second needs
 * (the last 12 voltage frames of each input, the last 12 beam samples of each
 * coarse channel for the inverse PFB, the second counter) to / from a host
 * buffer of vgb_pipeline_state_bytes bytes. A pipeline of the same
 * configuration that loads it continues bit-identically (the reference
 * carries the same state in its read-buffer margin and IPFB buffer,
 * buffer.c:106-124, pfb.cpp:950-976). */
long long vgb_pipeline_state_bytes(const vgb_pipeline *p);
int vgb_pipeline_save_state(vgb_pipeline *p, void *host, long long bytes);
int vgb_pipeline_load_state(vgb_pipeline *p, const void *host, long long bytes);
/* Diagnostic (no reference counterpart): this GPU's FP32 FMA throughput in
 * TFLOP/s (2 flops per FMA), from independent FMA chains on every SM timed
 * with CUDA events; packed != 0 issues them as FFMA2. The compute
 * denominator of the fused PFB + beamformer's roofline. */
int vgb_fp32_peak(int packed, int iters, double *tflops, void *stream);

/* The PSRFITS channel splice across processes (the reference's MPI_Igather
 * into the spliced sub-integration, beam_psrfits.c:608-628), host memory:
 * one process's spliced rows part [nspectra][nstokes][ncc_part*nchan] (its
 * pipeline's vgb_pipeline_fetch output) placed at coarse channels
 * [cc_offset, cc_offset + ncc_part) of the full rows out
 * [nspectra][nstokes][ncc_total*nchan]. The offsets and scales
 * ([ncc][nstokes][nchan]) and VDIF frames ([ncc][...]) of consecutive
 * channels are contiguous and join by concatenation. */
int vgb_splice_psrfits(const uint8_t *part, int nspectra, int nstokes, int nchan, int ncc_part, int cc_offset,
                       int ncc_total, uint8_t *out);
/* Milliseconds per stage of the last second: [0] fused PFB + beamformer,
 * [1] renormalise, [2] inverse PFB + VDIF, [3] history carry, [4] tracking
 * tables (n = 5; 0 when tracking is off). Synchronises. */
int vgb_pipeline_stage_ms(vgb_pipeline *p, float *ms, int n);

#ifdef __cplusplus
}
#endif
#endif
