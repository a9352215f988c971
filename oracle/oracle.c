/*
 * oracle.c -- CPU restatement of the VCSBeam voltage hot path.
 *
 * TEST INFRASTRUCTURE (see oracle.h): the checker for the CUDA library and
 * the timed CPU baseline. Every orc_* routine follows the reference routine
 * cited beside it (paths relative to the VCSBeam source tree). Complex
 * arithmetic follows cuComplex.h's cuCmul ordering, as the reference does.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MWA_ALTITUDE_METRES 377.827
#define ORC_SPEED_OF_LIGHT 299792458.0

/* ------------------------------------------------------------------------ */
/* deterministic generators                                                  */
/* ------------------------------------------------------------------------ */

static uint64_t splitmix64(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}

uint64_t orc_hash64(uint64_t seed, uint64_t idx)
{
    return splitmix64(splitmix64(seed) ^ (idx * 0xD1B54A32D192ED03ull));
}

/* Sum of twelve uniform 16-bit draws minus their mean: an integer whose
 * distribution approximates N(0, 65536^2). */
static int64_t irwin_hall12(uint64_t seed, uint64_t idx)
{
    int64_t s = 0;
    for (int j = 0; j < 3; j++) {
        uint64_t h = orc_hash64(seed, 3 * idx + j);
        s += (int64_t)(h & 0xFFFF) + (int64_t)((h >> 16) & 0xFFFF) +
             (int64_t)((h >> 32) & 0xFFFF) + (int64_t)((h >> 48) & 0xFFFF);
    }
    return s - 393210;
}

double orc_gauss(uint64_t seed, uint64_t idx)
{
    return (double)irwin_hall12(seed, idx) / 65536.0;
}

static int64_t round_div(int64_t num, int64_t den)
{
    /* round half away from zero, den > 0 */
    if (num >= 0) return (num + den / 2) / den;
    return -((-num + den / 2) / den);
}

static int draw_int(uint64_t seed, uint64_t idx, int sn, int sd, int lo, int hi)
{
    int64_t v = round_div(irwin_hall12(seed, idx) * sn, (int64_t)65536 * sd);
    if (v < lo) v = lo;
    if (v > hi) v = hi;
    return (int)v;
}

void orc_gen_int8(uint64_t seed, int8_t *out, size_t n, int sigma_num,
                  int sigma_den, int lo, int hi)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; i++)
        out[i] = (int8_t)draw_int(seed, (uint64_t)i, sigma_num, sigma_den, lo, hi);
}

void orc_gen_int4_bytes(uint64_t seed, uint8_t *out, size_t n, int sigma_num,
                        int sigma_den)
{
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)n; i++) {
        int hi = draw_int(seed, 2 * (uint64_t)i, sigma_num, sigma_den, -8, 7);
        int lo = draw_int(seed, 2 * (uint64_t)i + 1, sigma_num, sigma_den, -8, 7);
        out[i] = (uint8_t)(((hi & 0xF) << 4) | (lo & 0xF));
    }
}

/* ------------------------------------------------------------------------ */
/* complex helpers (cuComplex.h semantics)                                   */
/* ------------------------------------------------------------------------ */

typedef struct { double x, y; } cplx;

static inline cplx cmk(double x, double y) { cplx r = {x, y}; return r; }
static inline cplx cmul(cplx a, cplx b)
{
    return cmk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
static inline cplx cadd(cplx a, cplx b) { return cmk(a.x + b.x, a.y + b.y); }
static inline cplx csub(cplx a, cplx b) { return cmk(a.x - b.x, a.y - b.y); }
static inline cplx cconj(cplx a) { return cmk(a.x, -a.y); }
static inline double detect(cplx a) { return cmul(a, cconj(a)).x; }
static inline cplx cld(const double *p) { return cmk(p[0], p[1]); }
static inline void cst(double *p, cplx a) { p[0] = a.x; p[1] = a.y; }

/* ------------------------------------------------------------------------ */
/* forward fine PFB                                                          */
/* ------------------------------------------------------------------------ */

/* vcsbeam.h.in:240 vMWAX_IDX(s,i,ni) in char2 units. */
static inline size_t mwax_idx(size_t s, size_t i, size_t ni)
{
    return ((s / ORC_VSPVB) * ni + i) * ORC_VSPVB + (s % ORC_VSPVB);
}

void orc_wola(const int8_t *htr, int I, int nspectra, const int32_t *h,
              int K, int P, int32_t *b)
{
    const int M = K; /* critically sampled, pfb.cpp:142 */
#pragma omp parallel for collapse(2) schedule(static)
    for (int m = 0; m < nspectra; m++)
        for (int i = 0; i < I; i++) {
            /* pfb.cpp:153: the buffer starts with one whole voltage block */
            long mprime = (long)m + ORC_VSPVB / M - P;
            for (int n = 0; n < K; n++) {
                int32_t X = 0, Y = 0;
                for (int p = 0; p < P; p++) {
                    int hv = h[K * P - K * p - n - 1]; /* pfb.cpp:159 */
                    size_t xi = mwax_idx((size_t)(mprime * M + p * K + n), i, I);
                    X += hv * (int32_t)htr[2 * xi];
                    Y += hv * (int32_t)htr[2 * xi + 1];
                }
                size_t bi = (size_t)m * K * I + (size_t)i * K + n; /* pfb.cpp:161 */
                b[2 * bi] = X;
                b[2 * bi + 1] = Y;
            }
        }
}

void orc_fpga_round(const int32_t *b, size_t nvals, float *out)
{
    for (size_t j = 0; j < nvals; j++) {
        int32_t X = b[j];
        if (X > 0) X += 0x2000; /* pfb.cpp:226 */
        X >>= 14;               /* pfb.cpp:230 (arithmetic shift) */
        out[j] = (float)X;
    }
}

void orc_int2float(const int32_t *b, size_t nvals, float *out)
{
    const double scale = 1.0 / 16384.0; /* pfb.cpp:614 */
    for (size_t j = 0; j < nvals; j++)
        out[j] = (float)((double)(float)b[j] * scale);
}

static int is_pow2(int K) { return K > 0 && (K & (K - 1)) == 0; }

void orc_fft_forward(const double *in, double *out, int K, size_t nfft)
{
    double *tw = (double *)malloc(sizeof(double) * 2 * K);
    for (int j = 0; j < K; j++) {
        double th = -2.0 * M_PI * (double)j / (double)K;
        tw[2 * j] = cos(th);
        tw[2 * j + 1] = sin(th);
    }
    int logK = 0;
    while ((1 << logK) < K) logK++;
#pragma omp parallel for schedule(static)
    for (long f = 0; f < (long)nfft; f++) {
        const double *x = in + 2 * (size_t)f * K;
        double *X = out + 2 * (size_t)f * K;
        if (!is_pow2(K)) {
            for (int k = 0; k < K; k++) {
                double sr = 0, si = 0;
                for (int n = 0; n < K; n++) {
                    int j = (int)(((long)k * n) % K);
                    sr += x[2 * n] * tw[2 * j] - x[2 * n + 1] * tw[2 * j + 1];
                    si += x[2 * n] * tw[2 * j + 1] + x[2 * n + 1] * tw[2 * j];
                }
                X[2 * k] = sr;
                X[2 * k + 1] = si;
            }
            continue;
        }
        /* bit-reversed copy, then iterative radix-2 decimation in time */
        for (int n = 0; n < K; n++) {
            int r = 0;
            for (int q = 0; q < logK; q++)
                if (n & (1 << q)) r |= 1 << (logK - 1 - q);
            X[2 * r] = x[2 * n];
            X[2 * r + 1] = x[2 * n + 1];
        }
        for (int len = 2; len <= K; len <<= 1) {
            int half = len / 2, step = K / len;
            for (int s = 0; s < K; s += len)
                for (int j = 0; j < half; j++) {
                    double wr = tw[2 * j * step], wi = tw[2 * j * step + 1];
                    double *a = X + 2 * (s + j), *c = X + 2 * (s + j + half);
                    double tr = c[0] * wr - c[1] * wi, ti = c[0] * wi + c[1] * wr;
                    c[0] = a[0] - tr;
                    c[1] = a[1] - ti;
                    a[0] += tr;
                    a[1] += ti;
                }
        }
    }
    free(tw);
}

/* vcsbeam.h.in:453-457 CLIP / INT_TO_UINT8 / DEMOTE / PACK_NIBBLES */
static inline int clip8(int x) { return x < -8 ? -8 : (x > 7 ? 7 : x); }
static inline int int_to_uint8(int x) { return x < 0 ? clip8(x) + 0x10 : clip8(x); }
static inline int demote(double x) { return int_to_uint8((int)round(x)); }

void orc_pack(const double *X, int nspectra, int I, int K,
              const int32_t *i_idx, uint32_t flags, void *out)
{
#pragma omp parallel for collapse(2) schedule(static)
    for (int m = 0; m < nspectra; m++)
        for (int k = 0; k < K; k++)
            for (int i = 0; i < I; i++) {
                int kprime = (k + K / 2) % K; /* pfb.cpp:310 */
                size_t bi = (size_t)m * K * I + (size_t)i * K + k;
                size_t Xi = (size_t)m * I * K + (size_t)kprime * I + i_idx[i];
                /* pfb.cpp:321-322: float / int in the reference (exact for
                 * power-of-two K); the oracle keeps FP64. */
                double re = X[2 * bi] / K, im = X[2 * bi + 1] / K;
                if (flags & ORC_PFB_COMPLEX_INT4) {
                    uint8_t *o = (uint8_t *)out;
                    if (flags & ORC_PFB_IMAG_PART_FIRST)
                        o[Xi] = (uint8_t)((demote(re) << 4) + demote(im));
                    else
                        o[Xi] = (uint8_t)((demote(im) << 4) + demote(re));
                } else {
                    double *o = (double *)out;
                    if (flags & ORC_PFB_IMAG_PART_FIRST) {
                        o[2 * Xi] = re;
                        o[2 * Xi + 1] = im;
                    } else {
                        o[2 * Xi] = im;
                        o[2 * Xi + 1] = re;
                    }
                }
            }
}

void orc_fpfb(const int8_t *htr, int I, int nspectra, const int32_t *h,
              int K, int P, const int32_t *i_idx, uint32_t flags, void *out)
{
    size_t nv = (size_t)2 * nspectra * I * K;
    int32_t *b = (int32_t *)malloc(sizeof(int32_t) * nv);
    float *bf = (float *)malloc(sizeof(float) * nv);
    double *bd = (double *)malloc(sizeof(double) * nv);
    double *X = (double *)malloc(sizeof(double) * nv);
    orc_wola(htr, I, nspectra, h, K, P, b);
    if (flags & ORC_PFB_EMULATE_FPGA)
        orc_fpga_round(b, nv, bf);
    else
        orc_int2float(b, nv, bf);
    for (size_t j = 0; j < nv; j++) bd[j] = bf[j];
    orc_fft_forward(bd, X, K, (size_t)nspectra * I);
    orc_pack(X, nspectra, I, K, i_idx, flags, out);
    free(b);
    free(bf);
    free(bd);
    free(X);
}

/* ------------------------------------------------------------------------ */
/* beamformer                                                                */
/* ------------------------------------------------------------------------ */

static inline int uint8_to_int(int x) { return x >= 0x8 ? x - 0x10 : x; }

static inline cplx unpack4(uint8_t b)
{
    /* vcsbeam.h.in:997-1003 */
    return cmk((double)(float)uint8_to_int((b >> 4) & 0xf),
               (double)(float)uint8_to_int(b & 0xf));
}

void orc_unpack_int4(const uint8_t *in, size_t n, double *out)
{
    for (size_t j = 0; j < n; j++) cst(out + 2 * j, unpack4(in[j]));
}

void orc_beamform(const void *v, int datatype, int nsamples, int nchan,
                  int nant, const double *J, const double *phi,
                  const uint32_t *polQ, const uint32_t *polP, int npointing,
                  double invw, int nstokes, float *S, double *e)
{
    const int ni = 2 * nant;
#pragma omp parallel for collapse(3) schedule(static)
    for (int p = 0; p < npointing; p++)
        for (int s = 0; s < nsamples; s++)
            for (int c = 0; c < nchan; c++) {
                cplx exs = cmk(0, 0), eys = cmk(0, 0);
                cplx Nxx = cmk(0, 0), Nxy = cmk(0, 0), Nyy = cmk(0, 0);
                for (int a = 0; a < nant; a++) {
                    size_t iq = (size_t)s * ni * nchan + (size_t)c * ni + polQ[a];
                    size_t ip = (size_t)s * ni * nchan + (size_t)c * ni + polP[a];
                    cplx vq, vp;
                    if (datatype == 0) { /* VM_INT4, form_beam.cpp:156-161 */
                        vq = unpack4(((const uint8_t *)v)[iq]);
                        vp = unpack4(((const uint8_t *)v)[ip]);
                    } else {             /* VM_DBL, form_beam.cpp:162-167 */
                        vq = cld((const double *)v + 2 * iq);
                        vp = cld((const double *)v + 2 * ip);
                    }
                    /* form_beam.cpp:174-177 */
                    const double *Jp = J + 2 * 4 * (((size_t)p * nant + a) * nchan + c);
                    cplx JvQ = cadd(cmul(cld(Jp + 0), vq), cmul(cld(Jp + 2), vp));
                    cplx JvP = cadd(cmul(cld(Jp + 4), vq), cmul(cld(Jp + 6), vp));
                    /* form_beam.cpp:295-300 */
                    cplx ph = cld(phi + 2 * (((size_t)p * nant + a) * nchan + c));
                    cplx ex = cmul(ph, JvQ), ey = cmul(ph, JvP);
                    cplx nxx = cmul(ex, cconj(ex)), nxy = cmul(ex, cconj(ey));
                    cplx nyy = cmul(ey, cconj(ey));
                    /* form_beam.cpp:305-315: sequential sum from antenna 0 */
                    if (a == 0) {
                        exs = ex; eys = ey; Nxx = nxx; Nxy = nxy; Nyy = nyy;
                    } else {
                        exs = cadd(exs, ex); eys = cadd(eys, ey);
                        Nxx = cadd(Nxx, nxx); Nxy = cadd(Nxy, nxy); Nyy = cadd(Nyy, nyy);
                    }
                }
                /* form_beam.cpp:322-338 (bnXX, bnYY are floats there) */
                float bnXX = (float)(detect(exs) - Nxx.x);
                float bnYY = (float)(detect(eys) - Nyy.x);
                cplx bnXY = csub(cmul(exs, cconj(eys)), Nxy);
                size_t base = (((size_t)p * nsamples + s) * nstokes) * nchan + c;
                S[base] = (float)(invw * (float)(bnXX + bnYY));
                if (nstokes == 4) {
                    S[base + 1 * nchan] = (float)(invw * (float)(bnXX - bnYY));
                    S[base + 2 * nchan] = (float)(2.0 * invw * bnXY.x);
                    S[base + 3 * nchan] = (float)(-2.0 * invw * bnXY.y);
                }
                if (e) {
                    size_t eb = (((size_t)p * nsamples + s) * nchan + c) * 2;
                    cst(e + 2 * eb, exs);
                    cst(e + 2 * (eb + 1), eys);
                }
            }
}

uint8_t orc_sat_u8(double x)
{
    /* Measured on the reference's own kernel (tests/golden/ref_golden.npz):
     * the value is truncated to an integer and only its low 8 bits are
     * kept, so a channel's maximum (256.5) becomes 0; NaN becomes 0. The
     * argument is never negative on this path. */
    if (x != x) return 0;
    if (x <= 0.0) return 0;
    return (uint8_t)((uint32_t)x & 0xFFu);
}

void orc_renormalise(const float *S, int npointing, int nstep, int nstokes,
                     int nchan, float *offsets, float *scales, uint8_t *out)
{
    for (int p = 0; p < npointing; p++)
        for (int st = 0; st < nstokes; st++)
            for (int c = 0; c < nchan; c++) {
#define CIDX(i) ((((size_t)p * nstep + (i)) * nstokes + st) * nchan + c)
                float mn = S[CIDX(0)], mx = S[CIDX(0)];
                for (int i = 0; i < nstep; i++) {
                    float val = S[CIDX(i)];
                    mn = (val < mn ? val : mn);
                    mx = (val > mx ? val : mx);
                }
                float scale = (float)((mx - mn) / 256.0); /* form_beam.cpp:437 */
                float offset = mn;
                for (int i = 0; i < nstep; i++) {
                    float val = (S[CIDX(i)] - offset) / scale;
                    out[CIDX(i)] = orc_sat_u8((double)val + 0.5);
                }
                scales[(size_t)p * nstokes * nchan + st * nchan + c] = scale;
                offsets[(size_t)p * nstokes * nchan + st * nchan + c] = offset;
#undef CIDX
            }
}

void orc_incoh_beam(const uint8_t *data, int nsample, int nchan, int ninput,
                    float *incoh)
{
    for (int s = 0; s < nsample; s++)
        for (int c = 0; c < nchan; c++) {
            float acc = 0.0f;
            for (int i = 0; i < ninput; i++)
                acc += (float)detect(unpack4(data[((size_t)s * nchan + c) * ninput + i]));
            incoh[(size_t)s * nchan + c] = acc;
        }
}

/* ------------------------------------------------------------------------ */
/* inverse PFB                                                               */
/* ------------------------------------------------------------------------ */

static long floor_div(long a, long b)
{
    long q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) q--;
    return q;
}

void orc_ipfb(const double *in, int nsamples, int nchan, int npol,
              const double *f, int ntaps, int reference_taps, double *out)
{
    const int K = nchan, M = nchan, P = ntaps, F = ntaps * nchan;
    double *tw = (double *)malloc(sizeof(double) * 2 * K);
    orc_roots_of_unity(K, tw);
    long nout = (long)nsamples * K;
#pragma omp parallel for schedule(static)
    for (long n = 0; n < nout; n++)
        for (int pol = 0; pol < npol; pol++) {
            long m0 = reference_taps ? (n - F) / M + 1    /* pfb.cpp:863 */
                                     : floor_div(n - F, M) + 1;
            double sr = 0.0, si = 0.0;
            for (long m = m0; m < m0 + P; m++) {
                long fi = n - m * M;
                for (int k = 0; k < K; k++) {
                    int t = (int)(((long)(k + K / 2) * n) % K); /* pfb.cpp:880 */
                    double fr, fim;
                    if (fi >= 0) {
                        fr = f[fi] * tw[2 * t];
                        fim = f[fi] * tw[2 * t + 1];
                    } else if (t > 0) {
                        /* reference reads the previous row of the table */
                        fr = f[F + fi] * tw[2 * (t - 1)];
                        fim = f[F + fi] * tw[2 * (t - 1) + 1];
                    } else {
                        fr = 0.0; /* before the table: taken as zero */
                        fim = 0.0;
                    }
                    size_t ii = ((size_t)(m + P) * K + k) * npol + pol; /* pfb.cpp:890 */
                    double xr = in[2 * ii], xi = in[2 * ii + 1];
                    sr += xr * fr - xi * fim;
                    si += xr * fim + xi * fr;
                }
            }
            out[2 * ((size_t)n * npol + pol)] = sr / K;
            out[2 * ((size_t)n * npol + pol) + 1] = si / K;
        }
    free(tw);
}

void orc_ipfb_table(const double *coeffs, int ncoeffs, int nchan,
                    float *ft_real, float *ft_imag)
{
    double *tw = (double *)malloc(sizeof(double) * 2 * nchan);
    orc_roots_of_unity(nchan, tw);
    for (int f = 0; f < ncoeffs; f++)
        for (int ch = 0; ch < nchan; ch++) {
            cplx ft = cmul(cld(tw + 2 * ch), cmk(coeffs[f], 0.0));
            ft_real[(size_t)ncoeffs * ch + f] = (float)ft.x;
            ft_imag[(size_t)ncoeffs * ch + f] = (float)ft.y;
        }
    free(tw);
}

/* ------------------------------------------------------------------------ */
/* VDIF bytes                                                                */
/* ------------------------------------------------------------------------ */

void orc_vdif_quantise(const float *in, size_t n, uint8_t *out)
{
    for (size_t j = 0; j < n; j++) {
        float v = in[j];
        v = (v > 127.0f) ? 127.0f : v;
        v = (v < -126.0f) ? -126.0f : v;
        int8_t q = (int8_t)rint(v);
        out[j] = (uint8_t)(q ^ 0x80);
    }
}

/* ------------------------------------------------------------------------ */
/* table builders                                                            */
/* ------------------------------------------------------------------------ */

void orc_roots_of_unity(int N, double *out)
{
    for (int n = 0; n < N; n++) {
        double th = 2 * M_PI * (double)n / (double)N;
        out[2 * n] = cos(th);
        out[2 * n + 1] = sin(th);
    }
}

void orc_mult2x2d(const double *M1, const double *M2, double *Mout)
{
    cplx a0 = cld(M1), a1 = cld(M1 + 2), a2 = cld(M1 + 4), a3 = cld(M1 + 6);
    cplx b0 = cld(M2), b1 = cld(M2 + 2), b2 = cld(M2 + 4), b3 = cld(M2 + 6);
    cplx m00 = cmul(a0, b0), m12 = cmul(a1, b2), m01 = cmul(a0, b1), m13 = cmul(a1, b3);
    cplx m20 = cmul(a2, b0), m32 = cmul(a3, b2), m21 = cmul(a2, b1), m33 = cmul(a3, b3);
    cst(Mout, cadd(m00, m12));
    cst(Mout + 2, cadd(m01, m13));
    cst(Mout + 4, cadd(m20, m32));
    cst(Mout + 6, cadd(m21, m33));
}

double orc_norm2x2(const double *M, double *Mout)
{
    double F = 0.0;
    for (int i = 0; i < 4; i++) F += detect(cld(M + 2 * i));
    F = sqrt(F);
    for (int i = 0; i < 4; i++) {
        if (F == 0.0)
            cst(Mout + 2 * i, cmk(0.0, 0.0));
        else
            cst(Mout + 2 * i, cmk(M[2 * i] / F, M[2 * i + 1] / F));
    }
    return F;
}

void orc_inv2x2S(const double *Min, double *Mout)
{
    cplx a0 = cld(Min), a1 = cld(Min + 2), a2 = cld(Min + 4), a3 = cld(Min + 6);
    cplx det = csub(cmul(a0, a3), cmul(a1, a2));
    double scale = 1.0 / (det.x * det.x + det.y * det.y); /* jones.c:215-219 */
    cplx inv = cmk(scale * det.x, -scale * det.y);
    cplx ninv = cmk(-inv.x, -inv.y);
    cst(Mout, cmul(inv, a3));
    cst(Mout + 2, cmul(ninv, a1));
    cst(Mout + 4, cmul(ninv, a2));
    cst(Mout + 6, cmul(inv, a0));
}

void orc_calc_j(int npointing, int nant, int nchan, const double *D,
                const double *B, double *J)
{
    for (int p = 0; p < npointing; p++)
        for (int ch = 0; ch < nchan; ch++)
            for (int a = 0; a < nant; a++) {
                double Ji[8];
                const double *Dp = D + 8 * ((size_t)a * nchan + ch);
                const double *Bp = B + 8 * ((size_t)p * nant + a);
                double *Jp = J + 8 * (((size_t)p * nant + a) * nchan + ch);
                orc_mult2x2d(Dp, Bp, Ji);
                double F = orc_norm2x2(Ji, Ji);
                if (F != 0.0)
                    orc_inv2x2S(Ji, Jp);
                else
                    memset(Jp, 0, 8 * sizeof(double));
            }
}

void orc_calc_phi(int npointing, int nant, int nchan, const double *unit,
                  const double *east, const double *north,
                  const double *height, const double *cable,
                  const double *chan_freqs_hz, double *phi)
{
    for (int p = 0; p < npointing; p++)
        for (int c = 0; c < nchan; c++) {
            uint32_t freq_hz = (uint32_t)chan_freqs_hz[c];
            for (int a = 0; a < nant; a++) {
                double L = cable[a] - 0.0;
                double w = (east[a] - 0.0) * unit[3 * p + 0] +
                           (north[a] - 0.0) * unit[3 * p + 1] +
                           (height[a] - ORC_MWA_ALTITUDE_METRES) * unit[3 * p + 2];
                double dt = (w - L) / ORC_SPEED_OF_LIGHT;
                double phase = 2.0 * M_PI * dt * freq_hz;
                double *o = phi + 2 * (((size_t)p * nant + a) * nchan + c);
                o[0] = cos(phase);
                o[1] = sin(phase);
            }
        }
}

/* ------------------------------------------------------------------------ */
/* FP32 OpenMP transcription (timed CPU baseline)                            */
/* ------------------------------------------------------------------------ */

int orc32_max_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

static void fft32_inplace(float *X, int K, int logK, const float *tw)
{
    for (int n = 0; n < K; n++) {
        int r = 0;
        for (int q = 0; q < logK; q++)
            if (n & (1 << q)) r |= 1 << (logK - 1 - q);
        if (r > n) {
            float t0 = X[2 * n], t1 = X[2 * n + 1];
            X[2 * n] = X[2 * r];
            X[2 * n + 1] = X[2 * r + 1];
            X[2 * r] = t0;
            X[2 * r + 1] = t1;
        }
    }
    for (int len = 2; len <= K; len <<= 1) {
        int half = len / 2, step = K / len;
        for (int s = 0; s < K; s += len)
            for (int j = 0; j < half; j++) {
                float wr = tw[2 * j * step], wi = tw[2 * j * step + 1];
                float *a = X + 2 * (s + j), *c = X + 2 * (s + j + half);
                float tr = c[0] * wr - c[1] * wi, ti = c[0] * wi + c[1] * wr;
                c[0] = a[0] - tr;
                c[1] = a[1] - ti;
                a[0] += tr;
                a[1] += ti;
            }
    }
}

int orc32_pfb_beam(const int8_t *htr, int I, int m_begin, int m_end,
                   const int32_t *h, int K, int P, int emulate_fpga,
                   const float *W, float invw, float *S, float *e,
                   float *incoh)
{
    const int nant = I / 2;
    int logK = 0;
    while ((1 << logK) < K) logK++;
    float *tw = (float *)malloc(sizeof(float) * 2 * K);
    for (int j = 0; j < K; j++) {
        tw[2 * j] = (float)cos(-2.0 * M_PI * j / K);
        tw[2 * j + 1] = (float)sin(-2.0 * M_PI * j / K);
    }
    int nthreads = 1;
#pragma omp parallel
    {
#ifdef _OPENMP
#pragma omp single
        nthreads = omp_get_num_threads();
#endif
        float *X = (float *)malloc(sizeof(float) * 4 * K); /* two inputs */
        float *acc = (float *)malloc(sizeof(float) * 9 * K);
#pragma omp for schedule(dynamic, 4)
        for (int m = m_begin; m < m_end; m++) {
            memset(acc, 0, sizeof(float) * 9 * K);
            long mprime = (long)m + ORC_VSPVB / K - P;
            for (int a = 0; a < nant; a++) {
                for (int pol = 0; pol < 2; pol++) {
                    int i = 2 * a + pol;
                    float *x = X + 2 * K * pol;
                    for (int n = 0; n < K; n++) {
                        int32_t re = 0, im = 0;
                        for (int p = 0; p < P; p++) {
                            int hv = h[K * P - K * p - n - 1];
                            size_t xi = mwax_idx((size_t)(mprime * K + p * K + n), i, I);
                            re += hv * (int32_t)htr[2 * xi];
                            im += hv * (int32_t)htr[2 * xi + 1];
                        }
                        if (emulate_fpga) {
                            if (re > 0) re += 0x2000;
                            if (im > 0) im += 0x2000;
                            x[2 * n] = (float)(re >> 14);
                            x[2 * n + 1] = (float)(im >> 14);
                        } else {
                            x[2 * n] = (float)re * (1.0f / 16384.0f);
                            x[2 * n + 1] = (float)im * (1.0f / 16384.0f);
                        }
                    }
                    fft32_inplace(x, K, logK, tw);
                }
                for (int k = 0; k < K; k++) {
                    int kp = (k + K / 2) % K;
                    /* (im, re) / K ordering of pfb.cpp:328-339 */
                    float vq_r = X[2 * k + 1] / K, vq_i = X[2 * k] / K;
                    float vp_r = X[2 * (K + k) + 1] / K, vp_i = X[2 * (K + k)] / K;
                    if (emulate_fpga) {
                        vq_r = (float)uint8_to_int(demote(vq_r));
                        vq_i = (float)uint8_to_int(demote(vq_i));
                        vp_r = (float)uint8_to_int(demote(vp_r));
                        vp_i = (float)uint8_to_int(demote(vp_i));
                    }
                    const float *w = W + 8 * ((size_t)a * K + kp);
                    float exr = w[0] * vq_r - w[1] * vq_i + w[2] * vp_r - w[3] * vp_i;
                    float exi = w[0] * vq_i + w[1] * vq_r + w[2] * vp_i + w[3] * vp_r;
                    float eyr = w[4] * vq_r - w[5] * vq_i + w[6] * vp_r - w[7] * vp_i;
                    float eyi = w[4] * vq_i + w[5] * vq_r + w[6] * vp_i + w[7] * vp_r;
                    float *ac = acc + 9 * kp;
                    ac[0] += exr; ac[1] += exi; ac[2] += eyr; ac[3] += eyi;
                    ac[4] += exr * exr + exi * exi;
                    ac[5] += eyr * eyr + eyi * eyi;
                    ac[6] += exr * eyr + exi * eyi;
                    ac[7] += exi * eyr - exr * eyi;
                    ac[8] += vq_r * vq_r + vq_i * vq_i + vp_r * vp_r + vp_i * vp_i;
                }
            }
            size_t row = (size_t)(m - m_begin);
            for (int c = 0; c < K; c++) {
                const float *ac = acc + 9 * c;
                float bnXX = ac[0] * ac[0] + ac[1] * ac[1] - ac[4];
                float bnYY = ac[2] * ac[2] + ac[3] * ac[3] - ac[5];
                float bxr = ac[0] * ac[2] + ac[1] * ac[3] - ac[6];
                float bxi = ac[1] * ac[2] - ac[0] * ac[3] - ac[7];
                S[(row * 4 + 0) * K + c] = invw * (bnXX + bnYY);
                S[(row * 4 + 1) * K + c] = invw * (bnXX - bnYY);
                S[(row * 4 + 2) * K + c] = 2.0f * invw * bxr;
                S[(row * 4 + 3) * K + c] = -2.0f * invw * bxi;
                e[(row * K + c) * 4 + 0] = ac[0];
                e[(row * K + c) * 4 + 1] = ac[1];
                e[(row * K + c) * 4 + 2] = ac[2];
                e[(row * K + c) * 4 + 3] = ac[3];
                incoh[row * K + c] = ac[8];
            }
        }
        free(X);
        free(acc);
    }
    free(tw);
    return nthreads;
}

int orc32_ipfb_vdif(const float *in, int nsamples, int nchan, int npol,
                    const float *ft_real, const float *ft_imag, int ntaps,
                    long n_begin, long n_end, uint8_t *vdif_out)
{
    const int K = nchan, M = nchan, P = ntaps, F = ntaps * nchan;
    (void)nsamples;
    int nthreads = 1;
#pragma omp parallel
    {
#ifdef _OPENMP
#pragma omp single
        nthreads = omp_get_num_threads();
#endif
#pragma omp for schedule(static)
        for (long n = n_begin; n < n_end; n++)
            for (int pol = 0; pol < npol; pol++) {
                long m0 = floor_div(n - F, M) + 1;
                float sr = 0.0f, si = 0.0f;
                for (long m = m0; m < m0 + P; m++) {
                    long fi = n - m * M;
                    for (int k = 0; k < K; k++) {
                        int t = (int)(((long)(k + K / 2) * n) % K);
                        size_t ii = ((size_t)(m + P) * K + k) * npol + pol;
                        float fr = ft_real[(size_t)F * t + fi], fim = ft_imag[(size_t)F * t + fi];
                        sr += in[2 * ii] * fr - in[2 * ii + 1] * fim;
                        si += in[2 * ii] * fim + in[2 * ii + 1] * fr;
                    }
                }
                float v[2] = {sr / K, si / K};
                orc_vdif_quantise(v, 2, vdif_out + 2 * ((size_t)(n - n_begin) * npol + pol));
            }
    }
    return nthreads;
}

int orc32_renormalise(const float *S, int nstep, int nstokes, int nchan,
                      float *offsets, float *scales, uint8_t *out)
{
    int nthreads = 1;
#pragma omp parallel
    {
#ifdef _OPENMP
#pragma omp single
        nthreads = omp_get_num_threads();
#endif
#pragma omp for collapse(2) schedule(static)
        for (int st = 0; st < nstokes; st++)
            for (int c = 0; c < nchan; c++) {
                size_t stride = (size_t)nstokes * nchan, b = (size_t)st * nchan + c;
                float mn = S[b], mx = S[b];
                for (int i = 0; i < nstep; i++) {
                    float val = S[b + i * stride];
                    mn = val < mn ? val : mn;
                    mx = val > mx ? val : mx;
                }
                float scale = (float)((mx - mn) / 256.0), offset = mn;
                for (int i = 0; i < nstep; i++)
                    out[b + i * stride] = orc_sat_u8((double)((S[b + i * stride] - offset) / scale) + 0.5);
                scales[b] = scale;
                offsets[b] = offset;
            }
    }
    return nthreads;
}
