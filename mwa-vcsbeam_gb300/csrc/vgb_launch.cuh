// Kernel argument blocks and launchers shared by the kernel files and the
// C-ABI layer (vgb_api.cu). Every launcher returns a VGB_* status.
#pragma once

#include "vgb_internal.cuh"

namespace vgb {

struct BeamArgs {
    VoltView vv;
    const int *filter;      // K*P taps, reference order
    const float4 *W;        // [cc][nant][K][2]: (w00, w01), (w10, w11)
    long long W_cc;         // float4 stride between coarse channels
    int nspectra;
    int nant;
    float invw;
    int nstokes;            // 1 or 4
    float *S;               // [cc][s][nstokes][K]
    long long S_cc;
    float4 *e;              // [cc][s][K] (ex, ey), nullable
    long long e_cc;
    float *incoh;           // [cc][s][K], nullable
    long long inc_cc;
    unsigned *status;
    // nullable: per (cc, stokes, channel) extremes of S over the spectra, as
    // order-preserving keys (atomicMin / atomicMax; reset to ~0 / 0 / 0), and
    // whether spectrum 0's value is NaN: [cc][nstokes][K] each (the index of
    // the 8-bit stage's offsets for one pointing)
    uint32_t *st_mn, *st_mx, *st_nan0;
};

struct PackArgs {
    VoltView vv;
    const int *filter;
    const int *i_idx;       // MWAX input -> legacy input (pfb.cpp:410-419)
    int nspectra;
    unsigned flags;         // PFB_COMPLEX_INT4 / PFB_IMAG_PART_FIRST
    void *out;              // [cc][s][K][I] uint8 or double2
    long long out_cc;       // elements between coarse channels
    unsigned *status;       // kErrBadInput when i_idx is not a permutation of the inputs
    bool word_stores;       // 4-bit mode: out and I allow one aligned 4-byte store per 4 columns
    bool vec_stores;        // ... and one aligned 16-byte store per 16 columns
};
// Largest input count of the packing PFB (its inverse input map lives in
// shared memory).
constexpr int kPackMaxInputs = 1024;

struct RenormArgs {
    const float *S;        // [cc][p][nstep][nstokes][nchan]
    long long S_cc;
    int npointing, nstep, nstokes, nchan;
    uint8_t *out;          // out + cc*out_cc + p*out_p + s*out_s + st*out_st + c
    long long out_cc, out_p, out_s, out_st;
    float *offsets, *scales; // + cc*stat_cc + (p*nstokes + st)*nchan + c
    long long stat_cc;
    // nullable: the extremes gathered by the beam kernel (same index as
    // offsets); with them the samples are read once instead of twice
    const uint32_t *st_mn, *st_mx, *st_nan0;
};

struct LegacyArgs {
    const void *v;           // [s][c][ni] uint8 (int4) or double2
    int datatype;            // VGB_INT4 or VGB_DBL
    int nsamples, nchan, nant;
    const uint32_t *polQ, *polP;
    const float4 *W;         // [p][nant][nchan][2]
    int npointing;
    float invw;
    int nstokes;
    float *S;                // [p][s][nstokes][nchan]
    float4 *e;               // [p][s][nchan] nullable
    float *incoh;            // [s][nchan] nullable (int4 only)
    unsigned *status;        // kErrBadInput when polQ / polP name an input outside the row
};

struct IpfbArgs {
    const float4 *e;        // [job][ns][K] (ex, ey) beamformed voltages
    long long e_job;
    const float4 *hist;     // [job][P][K] previous second's last P samples; null = zeros
    long long hist_job;
    const float *coeffs;    // [P*K] synthesis filter (scaled)
    int nsamples;           // fine samples in the second
    float *out_f;           // [job][ns*K][2][2] nullable (cu_invert_pfb output)
    long long outf_job;
    uint8_t *vdif;          // [job][ns][544] nullable
    long long vdif_job;
    const uint32_t *hdr;    // [job][8] header of frame 0; nullable = zero header
    int frame_offset;
};

// flags: the pfb_flags bits (FPGA rounding, 4-bit demotion) and the WOLA
// arithmetic bits VGB_WOLA_FP32 / VGB_WOLA_FP32_SPLIT (neither: int32).
int launch_beam(const BeamArgs &a, int ncc, unsigned flags, cudaStream_t st);
// VDIF frames per second (the MWA fine sample rate, 1.28 MHz / 128): where a
// header's frame number rolls over to the next second.
constexpr int kVdifFramesPerSecond = 10000;
int launch_vdif_advance(uint32_t *hdr, int njobs, int nframes, cudaStream_t st);
// Force the fused front end's inputs per step (4 or 8), or 0 for the timed
// choice; returns the previous setting, -1 for a bad value.
int pfb_variant_last();
int pfb_variant(int g);
int launch_pack(const PackArgs &a, int ncc, unsigned flags, cudaStream_t st);
int launch_phase(const double *unit, const double *east, const double *north, const double *height,
                 const double *cable, const double *freqs, int npointing, int nant, int nchan, double href,
                 double2 *phi, cudaStream_t st);
int launch_jones(const double2 *D, const double2 *B, int npointing, int nant, int nchan, double2 *J,
                 cudaStream_t st);
int launch_weights(const double2 *J, const double2 *phi, long long n, float4 *W, cudaStream_t st);
// Per-second tracking: the second's pointing cur[5] = (az, za, E, N, H) from
// the per-second tables at *counter (then stepped), and W [cc][a][c] from
// D [cc][a][c], B [cc][a] and freqs [cc][c].
int launch_track_select(const double *az_tab, const double *za_tab, int nseconds, long long *counter, double *cur,
                        cudaStream_t st);
int launch_track_weights(const double2 *D, const double2 *B, const double *unit, const double *east,
                         const double *north, const double *height, const double *cable, const double *freqs,
                         int ncc, int nant, int nchan, double href, float4 *W, cudaStream_t st);
int launch_renorm(const RenormArgs &a, int ncc, cudaStream_t st);
int launch_incoh(const uint8_t *data, long long nrows, int ninput, float *incoh, cudaStream_t st);
int launch_legacy_beam(const LegacyArgs &a, cudaStream_t st);
int launch_ipfb(const IpfbArgs &a, int njobs, cudaStream_t st);
int launch_wola_staged(const VoltView &vv, const int *filter, int nspectra, int2 *b, cudaStream_t st);
int launch_round_staged(int *data, long long n, int fpga, cudaStream_t st);
int launch_fft_staged(float2 *rows, long long nrows, cudaStream_t st);
int launch_hist_gather(const char2 *cur, long long cur_block, long long cc_cur, int ninputs, int nblocks, int ncc,
                       char2 *hist, long long cc_hist, cudaStream_t st);
struct PbArgs { // primary-beam model evaluation
    const double *az, *za;       // [npointing] radians
    int npointing;
    const double *freq;          // [nfreq] Hz
    int nfreq;
    const uint32_t *delays;      // [ntile][16]
    int ntile;
    double lat;                  // radians
    int pa;                      // apply the parallactic-angle rotation
    double2 *B;                  // [nfreq][npointing][ntile][4]
};
// `scratch` (nullable): 2*ntile + 1 ints of device memory for the
// configuration lists; NULL takes them from the stream-ordered allocator.
int launch_beam_model(const PbArgs &a, cudaStream_t st, int *scratch = nullptr);
int launch_array_factor(const double *look, const double *dirs, int npix, double freq, const double *east,
                        const double *north, const double *height, const double *cable, double href, int nant,
                        double *af, cudaStream_t st);
int gemm_batched(const void *A, const void *B, float *C, int M, int N, int K, int batch, bool fp16,
                 cudaStream_t st, int Kb);
// C[b] = (A0[b] + A1[b]) B[b]^T where each A row holds A0 then A1 (K wide
// each, 2K in all) and B rows are K wide: the split-operand product of the
// K-concatenated form with B read once per K step (persistent kernel; M a
// multiple of 128, N of 256).
int gemm_batched_planes(const void *A, const void *B, float *C, int M, int N, int K, int batch, bool fp16,
                        cudaStream_t st);
int launch_pack_staged(const float2 *ffted, int nspectra, int ninputs, const int *i_idx, unsigned flags,
                       void *out, cudaStream_t st);

} // namespace vgb
