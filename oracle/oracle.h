/*
 * oracle.h -- CPU restatement of the VCSBeam voltage hot path.
 *
 * TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load this library, and only as the checker (or, for
 * bench.py, as the timed CPU baseline). The shipped library never links it.
 *
 * Two families:
 *   orc_*    FP64 restatements of each reference kernel / host routine, one
 *            function per reference routine, each citing the file:line it
 *            follows (paths relative to the VCSBeam source tree).
 *   orc32_*  An OpenMP FP32 transcription of the same arithmetic, used as the
 *            timed CPU baseline (the reference has no CPU path for its
 *            kernels: src/gpu_macros.h:128).
 *
 * Complex values are interleaved (re, im) doubles or floats.
 */
#ifndef VGB_ORACLE_H
#define VGB_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* MWAX voltage block geometry (include/vcsbeam.h.in:238-240). */
#define ORC_VSPVB 64000

/* pfb_flags bits (include/vcsbeam.h.in:459-480). */
#define ORC_PFB_COMPLEX_INT4 0x10
#define ORC_PFB_COMPLEX_FLOAT64 0x20
#define ORC_PFB_IMAG_PART_FIRST 0x100
#define ORC_PFB_EMULATE_FPGA 0x200

/* ---- deterministic synthetic inputs (integer arithmetic only, so the same
 *      seed gives the same bytes on every machine) ---- */
uint64_t orc_hash64(uint64_t seed, uint64_t idx);
/* Irwin-Hall(12) approximation of N(0,1), an exact multiple of 2^-16. */
double orc_gauss(uint64_t seed, uint64_t idx);
/* round(N(0,1) * sigma_num / sigma_den) clipped to [lo, hi], integer math. */
void orc_gen_int8(uint64_t seed, int8_t *out, size_t n, int sigma_num,
                  int sigma_den, int lo, int hi);
/* Legacy 4+4-bit bytes: high nibble and low nibble each an independent
 * draw of the above (include/vcsbeam.h.in:997-1003 packing). */
void orc_gen_int4_bytes(uint64_t seed, uint8_t *out, size_t n, int sigma_num,
                        int sigma_den);

/* ---- forward fine PFB (src/pfb.cpp) ---- */
/* pfb.cpp:121-179 vmWOLA_kernel. htr is the MWAX char2 buffer
 * [nblocks][I][VSPVB][2] including the one-block margin at its front.
 * b (out) is int32 [nspectra][I][K][2] (pfb.cpp:161 b_idx). */
void orc_wola(const int8_t *htr, int I, int nspectra, const int32_t *h,
              int K, int P, int32_t *b);
/* pfb.cpp:202-242: X>0 ? (X+0x2000)>>14 : X>>14, as float. */
void orc_fpga_round(const int32_t *b, size_t nvals, float *out);
/* pfb.cpp:256-268 with scale 1/16384 (pfb.cpp:614). */
void orc_int2float(const int32_t *b, size_t nvals, float *out);
/* Forward DFT X[k] = sum_n x[n] e^{-2 pi i k n / K} in FP64, nfft rows.
 * (The reference calls cuFFT, pfb.cpp:639-643; this is its definition.) */
void orc_fft_forward(const double *in, double *out, int K, size_t nfft);
/* pfb.cpp:297-343 pack_into_recombined_format. X is complex FP64
 * [nspectra][I][K]; i_idx maps MWAX input -> legacy input (pfb.cpp:410-419).
 * int4 mode: out is uint8 [nspectra][K][I]; else complex double. */
void orc_pack(const double *X, int nspectra, int I, int K,
              const int32_t *i_idx, uint32_t flags, void *out);
/* pfb.cpp:730-773 for one chunk: WOLA, rounding, FFT, pack. */
void orc_fpfb(const int8_t *htr, int I, int nspectra, const int32_t *h,
              int K, int P, const int32_t *i_idx, uint32_t flags, void *out);

/* ---- beamformer (src/form_beam.cpp) ---- */
/* vcsbeam.h.in:997-1003 UCMPLX4_TO_CMPLX_FLT: high nibble is "real". */
void orc_unpack_int4(const uint8_t *in, size_t n, double *out);
/* form_beam.cpp:122-204 (vmApplyJ_kernel) followed by form_beam.cpp:239-371
 * (vmBeamform_kernel), for every pointing. v is [nsamples][nchan][2*nant]
 * (v_IDX), int4 bytes (datatype 0) or complex double (datatype 1).
 * J: complex [npointing][nant][nchan][2][2]; phi: complex
 * [npointing][nant][nchan]. S (out): float [npointing][nsamples][nstokes][nchan]
 * (C_IDX); e (out, nullable): complex [npointing][nsamples][nchan][2] (B_IDX). */
void orc_beamform(const void *v, int datatype, int nsamples, int nchan,
                  int nant, const double *J, const double *phi,
                  const uint32_t *polQ, const uint32_t *polP, int npointing,
                  double invw, int nstokes, float *S, double *e);
/* form_beam.cpp:408-449 renormalise_channels_kernel. */
void orc_renormalise(const float *S, int npointing, int nstep, int nstokes,
                     int nchan, float *offsets, float *scales, uint8_t *out);
/* The float->uint8 conversion of form_beam.cpp:443 as the reference GPU
 * build performs it: truncate, keep the low 8 bits (so 256.5 -> 0), NaN -> 0.
 * Exposed for tests. */
uint8_t orc_sat_u8(double x);
/* form_beam.cpp:60-87 incoh_beam: I[s][c] = sum_i |v|^2 over int4 bytes. */
void orc_incoh_beam(const uint8_t *data, int nsample, int nchan, int ninput,
                    float *incoh);

/* ---- inverse PFB (src/pfb.cpp:842-1046) ---- */
/* x^[n] = (1/K) sum_m sum_k X_k[m] f[n-mK] e^{2 pi i ((k+K/2) n mod K)/K}.
 * in: complex [(nsamples + ntaps)][nchan][npol] where rows 0..ntaps-1 are the
 * previous second's last ntaps samples (zeros for the first second,
 * pfb.cpp:950-984). f: ntaps*nchan synthesis coefficients (already scaled).
 * out: float-valued FP64 [nsamples*nchan][npol][2].
 * reference_taps = 0: the tap range m in [floor(n/K)-ntaps+1, floor(n/K)].
 * reference_taps = 1: the reference's own range m0 = (n-F)/K + 1 with C
 * truncation (pfb.cpp:863); terms whose filter index is negative read the
 * previous twiddle row (pfb.cpp:884), or 0 where the reference reads before
 * the table (row 0). */
void orc_ipfb(const double *in, int nsamples, int nchan, int npol,
              const double *f, int ntaps, int reference_taps, double *out);
/* pfb.cpp:1025-1046 filter x twiddle table, FP64 then rounded to float:
 * ft[ch*F + i] = coeff[i] * e^{2 pi i ch / nchan}. */
void orc_ipfb_table(const double *coeffs, int ncoeffs, int nchan,
                    float *ft_real, float *ft_imag);

/* ---- VDIF bytes (src/beam_vdif.c) ---- */
/* beam_vdif.c:29-38 clamp to [-126,127], rint, int8; beam_vdif.c:254-260
 * XOR 0x80. */
void orc_vdif_quantise(const float *in, size_t n, uint8_t *out);

/* ---- table builders (src/jones.c, src/geometry.c, src/filter.c) ---- */
/* jones.c:97-157 vmCalcJ: J = inv2x2S(norm2x2(D[a][c] B[p][a])). */
void orc_calc_j(int npointing, int nant, int nchan, const double *D,
                const double *B, double *J);
/* geometry.c:40-101 + 111-135: phi[p][a][c] = e^{i 2 pi dt f_c},
 * dt = (E uE + N uN + (H-Href) uH - L)/c. unit: [npointing][3] (E,N,H). */
void orc_calc_phi(int npointing, int nant, int nchan, const double *unit,
                  const double *east, const double *north,
                  const double *height, const double *cable,
                  const double *chan_freqs_hz, double *phi);
/* filter.c:21-48 roots_of_unity: e^{2 pi i n / N}. */
void orc_roots_of_unity(int N, double *out);
/* jones.c:215-330, 404-424 2x2 helpers (complex [4]). */
void orc_mult2x2d(const double *M1, const double *M2, double *Mout);
double orc_norm2x2(const double *M, double *Mout);
void orc_inv2x2S(const double *Min, double *Mout);

/* ---- FP32 OpenMP transcription (timed CPU baseline) ---- */
/* One coarse-channel pass over spectra [m_begin, m_end): the forward PFB
 * (int32 WOLA, rounding, radix-2 FP32 FFT, pack to float), Jones x phase x
 * tile sum, Stokes with autocorrelation removal, and the incoherent sum.
 * W is the per-(antenna, channel) 2x2 weight phi*J^-1 in FP32
 * [nant][nchan][2][2] complex. S: [m][4][nchan]; e: [m][nchan][2] complex;
 * incoh: [m][nchan]. Returns the number of threads used. */
int orc32_pfb_beam(const int8_t *htr, int I, int m_begin, int m_end,
                   const int32_t *h, int K, int P, int emulate_fpga,
                   const float *W, float invw, float *S, float *e,
                   float *incoh);
/* Reference-algorithm inverse PFB (direct sum, pfb.cpp:842-907) in FP32 for
 * output samples [n_begin, n_end), followed by VDIF quantisation. */
int orc32_ipfb_vdif(const float *in, int nsamples, int nchan, int npol,
                    const float *ft_real, const float *ft_imag, int ntaps,
                    long n_begin, long n_end, uint8_t *vdif_out);
/* form_beam.cpp:408-449 with one thread per (stokes, channel). */
int orc32_renormalise(const float *S, int nstep, int nstokes, int nchan,
                      float *offsets, float *scales, uint8_t *out);
int orc32_max_threads(void);

#ifdef __cplusplus
}
#endif
#endif
