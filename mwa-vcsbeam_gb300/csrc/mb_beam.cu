// Many-beam tied-array beamformer on the 5th-generation tensor cores.
//
// The reference forms each pointing separately: vmApplyJ_kernel multiplies
// every tile's dual-pol voltage by that tile's inverse Jones matrix and
// vmBeamform_kernel sums phi * Jv over tiles with one thread, then detects
// (form_beam.cpp:122-204, 239-371). For B pointings that is, per fine
// channel, a complex contraction (beams x 2 pols) x (tiles x 2 pols) x time:
//
//   E[p, x](s) = sum_{a, q} W[p, x, a, q] v[a, q](s),  W = phi[p, a, c] J^-1[p, a, c]
//
// Here it runs as a real GEMM per fine channel on tcgen05:
//   rows    m = 4 p + 2 x + rho       (beam, output pol, re/im of E)
//   columns s                         (samples; 256 per tile, 250 used)
//   K       k = 4 a + 2 q + sigma     (tile, input pol, re/im of v)
// with A = [[Wr, -Wi], [Wi, Wr]] (the real embedding of W) and B the
// voltages, which are exact in bf16/fp16. In the split precision mode the
// weights are two bf16 planes, A = A_hi + A_lo (|A - A_hi - A_lo| <= 2^-17
// |A|), both multiplied into the same FP32 accumulator in tensor memory.
//
// Detection (form_beam.cpp:300-371) removes each tile's own power:
//   bnXX = |sum_a ex_a|^2 - sum_a |ex_a|^2, bnYY likewise, bnXY = ... ex ey*.
// The subtracted sum is linear in the per-tile coherency C_a = v_a v_a^H and
// does not depend on phi:  sum_a |ex_a|^2 = sum_a w_x C_a w_x^H with w_x the
// x row of J^-1. Summed over the 10 samples of an integration it is a second,
// much smaller GEMM,
//   R[(p, st)](t) = sum_{a, j} Q[(p, st), (a, j)] Cint[(a, j)](t),
// j in {C_QQ, C_PP, Re C_QP, Im C_QP}, st the Stokes parameter. It runs on the
// FP16 tensor path (tc_gemm.cu): integrated coherencies of 4-bit voltages are
// exact in FP16, those of 8-bit voltages are split into exact hi + lo halves,
// and Q carries a power-of-two scale per row (and, in the split mode, an FP16
// lo half).
//
// The beam GEMM's epilogue reads the accumulators back with tcgen05.ld,
// forms XX, YY, XY per sample across the four lanes that hold one beam,
// integrates 10 samples, subtracts R and writes Stokes
//   I = w (XX + YY), Q = w (XX - YY), U = 2 w Re XY, V = -2 w Im XY
// (w = 1 / unflagged inputs, metadata.c:1554-1561), 1 ms per value.
//
// Weights: J^-1 = inv(D B / |D B|_F) (jones.c:97-157) is evaluated as
// |D B|_F B^-1 D^-1, with D^-1 (per tile, channel) and B^-1 (per beam, tile)
// inverted in FP64 and |D B|_F^2 = tr(D^H D B B^H); the geometric delay and
// the wrap of the phase turns dt * f (geometry.c:40-101) are FP64; the
// per-(beam, tile, channel) product and the sine/cosine of the wrapped phase
// are FP32 (relative error ~1e-7, below the 2^-17 of the split weights).
#include <atomic>

#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "tcgen05.cuh"
#include "vgb_launch.cuh"

namespace vgb {

constexpr int kMbN = 256;      // samples per MMA tile
constexpr int kMbInt = 10;     // samples per integration (1 ms at 10 kHz)
constexpr int kMbUsed = 250;   // samples of a tile that are used: 25 integrations
constexpr int kMbNint = kMbUsed / kMbInt;
constexpr int kMbBeamsPerTile = 32;  // 128 rows / 4
constexpr int kMbEpq = 3;            // epilogue warps per TMEM lane quarter
constexpr int kMbEpiWarps = 4 * kMbEpq;
constexpr int kMbThreads = 64 + 32 * kMbEpiWarps; // warp 0 TMA, warp 1 MMA, warps 2.. epilogue
constexpr uint32_t kMbPolls = 1u << 26;

// Per-row statistics for the 8-bit stage, gathered by the beam epilogues: the
// minimum and maximum as order-preserving unsigned keys (atomicMin/Max), and
// whether the row's first value is NaN. The reference's sequential scan
// (form_beam.cpp:408-449) starts from the first value and compares with <, >:
// a NaN there makes the result NaN, any other NaN is skipped; fminf/fmaxf over
// the rest give the same extremes.
struct MbStats {
    uint32_t *mn, *mx; // [nfine][B][nst] keys
    uint32_t *nan0;    // [nfine][B][nst]: the row's first value is NaN
};

// ---------------------------------------------------------------------------
// Tables
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 zmul2(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// 2x2 complex inverse in FP64 (same formula as jones.c's inv2x2S).
__device__ __forceinline__ void zinv2x2(const double2 (&m)[4], double2 (&o)[4])
{
    const double2 det = make_double2(m[0].x * m[3].x - m[0].y * m[3].y - (m[1].x * m[2].x - m[1].y * m[2].y),
                                     m[0].x * m[3].y + m[0].y * m[3].x - (m[1].x * m[2].y + m[1].y * m[2].x));
    const double scale = 1.0 / (det.x * det.x + det.y * det.y);
    const double2 inv = make_double2(scale * det.x, -scale * det.y);
    const double2 ninv = make_double2(-inv.x, -inv.y);
    o[0] = zmul2(inv, m[3]);
    o[1] = zmul2(ninv, m[1]);
    o[2] = zmul2(ninv, m[2]);
    o[3] = zmul2(inv, m[0]);
}

// Per (beam, tile): geometric delay (geometry.c:40-101, same operation order
// as the single-beam phase kernel), B^-1 and H = B B^H. Beams >= npointing are
// zero (their weights vanish).
__global__ void mb_pa_kernel(const double *unit, const double *east, const double *north, const double *height,
                             const double *cable, double href, const double2 *Bj, int npointing, int Bp, int nant,
                             double *dt, float4 *Binv, float4 *H)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= Bp * nant) return;
    const int a = idx % nant, p = idx / nant;
    if (p >= npointing) {
        dt[idx] = 0.0;
        Binv[2 * idx] = Binv[2 * idx + 1] = make_float4(0.f, 0.f, 0.f, 0.f);
        H[idx] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    if (unit) {
        const double L = cable[a] - 0.0;
        const double w = (east[a] - 0.0) * unit[3 * p + 0] + (north[a] - 0.0) * unit[3 * p + 1] +
                         (height[a] - href) * unit[3 * p + 2];
        dt[idx] = (w - L) / 299792458.0;
    }
    if (Bj) {
        double2 b[4], bi[4];
        for (int i = 0; i < 4; i++) b[i] = Bj[4 * (long long)idx + i];
        zinv2x2(b, bi);
        Binv[2 * idx] = make_float4((float)bi[0].x, (float)bi[0].y, (float)bi[1].x, (float)bi[1].y);
        Binv[2 * idx + 1] = make_float4((float)bi[2].x, (float)bi[2].y, (float)bi[3].x, (float)bi[3].y);
        // H = B B^H: H11 = |b00|^2 + |b01|^2, H22 = |b10|^2 + |b11|^2, H12 = b00 b10* + b01 b11*
        const double h11 = b[0].x * b[0].x + b[0].y * b[0].y + b[1].x * b[1].x + b[1].y * b[1].y;
        const double h22 = b[2].x * b[2].x + b[2].y * b[2].y + b[3].x * b[3].x + b[3].y * b[3].y;
        const double h12r = b[0].x * b[2].x + b[0].y * b[2].y + b[1].x * b[3].x + b[1].y * b[3].y;
        const double h12i = b[0].y * b[2].x - b[0].x * b[2].y + b[1].y * b[3].x - b[1].x * b[3].y;
        H[idx] = make_float4((float)h11, (float)h22, (float)h12r, (float)h12i);
    }
}

// Per (channel, tile) of one coarse channel: D^-1 and G = D^H D, from the
// calibration solution D [tile][channel][2][2] (D_IDX order).
__global__ void mb_ca_kernel(const double2 *D, int nant, int nfine, float4 *Dinv, float4 *G)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= nant * nfine) return;
    const int a = idx % nant, c = idx / nant; // output order [c][a]
    double2 d[4], di[4];
    for (int i = 0; i < 4; i++) d[i] = D[4 * ((long long)a * nfine + c) + i];
    zinv2x2(d, di);
    Dinv[2 * idx] = make_float4((float)di[0].x, (float)di[0].y, (float)di[1].x, (float)di[1].y);
    Dinv[2 * idx + 1] = make_float4((float)di[2].x, (float)di[2].y, (float)di[3].x, (float)di[3].y);
    // G = D^H D: G11 = |d00|^2 + |d10|^2, G22 = |d01|^2 + |d11|^2, G12 = d00* d01 + d10* d11
    const double g11 = d[0].x * d[0].x + d[0].y * d[0].y + d[2].x * d[2].x + d[2].y * d[2].y;
    const double g22 = d[1].x * d[1].x + d[1].y * d[1].y + d[3].x * d[3].x + d[3].y * d[3].y;
    const double g12r = d[0].x * d[1].x + d[0].y * d[1].y + d[2].x * d[3].x + d[2].y * d[3].y;
    const double g12i = d[0].x * d[1].y - d[0].y * d[1].x + d[2].x * d[3].y - d[2].y * d[3].x;
    G[idx] = make_float4((float)g11, (float)g22, (float)g12r, (float)g12i);
}

struct MbWeightArgs {
    const double *dt;     // [Bp][A]
    const float4 *Binv;   // [Bp][A][2]
    const float4 *H;      // [Bp][A]
    const float4 *Dinv;   // [nfine][A][2]
    const float4 *G;      // [nfine][A]
    const double *freq;   // [nfine] Hz
    int A, Bp, nfine, nst, planes, fp16, int8;
    int Mrows, Mq, KA, Kq;
    uint16_t *Aw;         // [planes][nfine][Mrows][KA]
    __half *Aq;           // [nfine][Mq][Kq]
    float *qscale;        // [nfine][Mq]
    float2 *W32;          // FP32 mode instead: W [nfine][Bp][2][A][2] complex
    float *Q32;           //                    Q [nfine][Mq][4A]
    MbStats stats;        // reset here for the run's rows
    int B;
};

__device__ __forceinline__ float2 cmul32(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cmulc32(float2 a, float2 b) // a * conj(b)
{
    return make_float2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}

// J^-1 from the beam's (B^-1, Gram of B) and the channel's (D^-1, Gram of D);
// zero when |D B|_F = 0 (jones.c:144-147).
__device__ __forceinline__ void mb_jinv_from(const float4 h, const float4 g, const float4 b0, const float4 b1,
                                             const float4 d0, const float4 d1, float2 (&J)[4])
{
    const float tr = g.x * h.x + g.y * h.y + 2.f * (g.z * h.z + g.w * h.w);
    if (!(tr > 0.f)) {
        J[0] = J[1] = J[2] = J[3] = make_float2(0.f, 0.f);
        return;
    }
    const float n = sqrtf(tr);
    const float2 b[4] = {make_float2(b0.x, b0.y), make_float2(b0.z, b0.w), make_float2(b1.x, b1.y),
                         make_float2(b1.z, b1.w)};
    const float2 d[4] = {make_float2(d0.x, d0.y), make_float2(d0.z, d0.w), make_float2(d1.x, d1.y),
                         make_float2(d1.z, d1.w)};
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
        for (int col = 0; col < 2; col++) {
            const float2 t = cmul32(b[2 * r], d[col]);
            const float2 u = cmul32(b[2 * r + 1], d[2 + col]);
            J[2 * r + col] = make_float2(n * (t.x + u.x), n * (t.y + u.y));
        }
}

// J^-1 for (channel c, beam p, tile a).
__device__ __forceinline__ void mb_jinv(const MbWeightArgs &w, int c, int p, int a, float2 (&J)[4])
{
    const long long pa = (long long)p * w.A + a, ca = (long long)c * w.A + a;
    mb_jinv_from(w.H[pa], w.G[ca], w.Binv[2 * pa], w.Binv[2 * pa + 1], w.Dinv[2 * ca], w.Dinv[2 * ca + 1], J);
}

// Autocorrelation coefficients of Stokes st over (C_QQ, C_PP, Re C_QP, Im C_QP).
__device__ __forceinline__ void mb_qrow(const float2 (&J)[4], int st, float (&q)[4])
{
    const float2 al = J[0], be = J[1], ga = J[2], de = J[3];
    const float2 ab = cmulc32(al, be), gd = cmulc32(ga, de);
    const float2 ag = cmulc32(al, ga), bd = cmulc32(be, de), ad = cmulc32(al, de), bg = cmulc32(be, ga);
    const float xx[4] = {al.x * al.x + al.y * al.y, be.x * be.x + be.y * be.y, 2.f * ab.x, -2.f * ab.y};
    const float yy[4] = {ga.x * ga.x + ga.y * ga.y, de.x * de.x + de.y * de.y, 2.f * gd.x, -2.f * gd.y};
    const float rexy[4] = {ag.x, bd.x, ad.x + bg.x, bg.y - ad.y};
    const float imxy[4] = {ag.y, bd.y, ad.y + bg.y, ad.x - bg.x};
#pragma unroll
    for (int j = 0; j < 4; j++)
        q[j] = st == 0 ? xx[j] + yy[j] : st == 1 ? xx[j] - yy[j] : st == 2 ? 2.f * rexy[j] : -2.f * imxy[j];
}

__device__ __forceinline__ uint16_t to_bits(float x, bool fp16)
{
    return fp16 ? __half_as_ushort(__float2half_rn(x)) : __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ float from_bits(uint16_t b, bool fp16)
{
    return fp16 ? __half2float(__ushort_as_half(b)) : __bfloat162float(__ushort_as_bfloat16(b));
}

// One block per (beam, channel); the threads step over tiles. Pass 1 finds the
// largest |Q| of each Stokes row (its power-of-two scale), pass 2 writes the
// embedded weights (hi, lo planes) and the scaled, split Q rows.
constexpr int kMbWeightThreads = 128;
constexpr int kMbPairMaxTiles = 512; // arrays the pair kernel covers (2 tiles per thread, 256 threads)
constexpr int kMbWeightBeams = 8;    // beams per block in the pair kernel

// Phase (cos, sin) of tile a for beam p at frequency f: turns dt * f in FP64,
// wrapped to [-1/2, 1/2], then sin/cos in FP32.
__device__ __forceinline__ float2 mb_phase(const MbWeightArgs &w, int p, int a, double f)
{
    const double turns = w.dt[(long long)p * w.A + a] * f;
    const float r = (float)(turns - rint(turns));
    float sn, cs;
    sincospif(2.f * r, &sn, &cs);
    return make_float2(cs, sn);
}

// The embedded real rows (x, rho) of W = phase J^-1: four values per tile,
// split into a hi part and the remainder (lo) in the GEMM's 16-bit type.
__device__ __forceinline__ void mb_weight_halves(const float2 ph, const float2 (&J)[4], int x, int rho, bool h16,
                                                 uint2 &hi2, uint2 &lo2)
{
    float val[4];
    for (int q = 0; q < 2; q++) {
        const float2 v = cmul32(ph, J[2 * x + q]);
        val[2 * q + 0] = rho == 0 ? v.x : v.y;
        val[2 * q + 1] = rho == 0 ? -v.y : v.x;
    }
    uint16_t hi[4], lo[4];
    for (int j = 0; j < 4; j++) {
        hi[j] = to_bits(val[j], h16);
        lo[j] = to_bits(val[j] - from_bits(hi[j], h16), h16);
    }
    hi2 = make_uint2(hi[0] | ((uint32_t)hi[1] << 16), hi[2] | ((uint32_t)hi[3] << 16));
    lo2 = make_uint2(lo[0] | ((uint32_t)lo[1] << 16), lo[2] | ((uint32_t)lo[3] << 16));
}

// Q row values scaled by inv_scale, split into FP16 hi and lo.
__device__ __forceinline__ void mb_q_halves(const float (&q)[4], float inv_scale, uint2 &hi2, uint2 &lo2)
{
    uint16_t hi[4], lo[4];
    for (int j = 0; j < 4; j++) {
        const float s = q[j] * inv_scale;
        const __half h = __float2half_rn(s);
        hi[j] = __half_as_ushort(h);
        lo[j] = __half_as_ushort(__float2half_rn(s - __half2float(h)));
    }
    hi2 = make_uint2(hi[0] | ((uint32_t)hi[1] << 16), hi[2] | ((uint32_t)hi[3] << 16));
    lo2 = make_uint2(lo[0] | ((uint32_t)lo[1] << 16), lo[2] | ((uint32_t)lo[3] << 16));
}

// Power-of-two scale of each Stokes row of Q from the block's per-warp maxima.
__device__ __forceinline__ void mb_q_scales(const MbWeightArgs &w, int c, int p, float (&mx)[4],
                                            float (&smax)[8][4], float (&inv_scale)[4])
{
    for (int st = 0; st < 4; st++) {
        for (int o = 16; o; o >>= 1) mx[st] = fmaxf(mx[st], __shfl_xor_sync(0xffffffffu, mx[st], o));
        if ((threadIdx.x & 31) == 0) smax[threadIdx.x >> 5][st] = mx[st];
    }
    __syncthreads();
    for (int st = 0; st < 4; st++) {
        float m = 0.f;
        for (int k = 0; k < (int)(blockDim.x >> 5); k++) m = fmaxf(m, smax[k][st]);
        int e = 0;
        if (m > 0.f && isfinite(m)) frexpf(m, &e); // m = f 2^e, f in [0.5, 1)
        inv_scale[st] = ldexpf(1.f, -e);
        if (threadIdx.x == 0 && st < w.nst) w.qscale[(long long)c * w.Mq + p * w.nst + st] = ldexpf(1.f, e);
    }
}

__device__ __forceinline__ void mb_reset_stats(const MbWeightArgs &w, int c, int p)
{
    if ((int)threadIdx.x < w.nst && p < w.B) {
        const long long r = ((long long)c * w.B + p) * w.nst + threadIdx.x;
        w.stats.mn[r] = 0xFFFFFFFFu;
        w.stats.mx[r] = 0u;
    }
}

// Any array size: one block per (beam, channel), threads stepping over tiles.
// The first pass finds each Stokes row's largest |Q| (its power-of-two scale),
// the second forms J^-1 again and writes the weight and Q rows. Also the FP32
// CUDA-core mode's complex weights and unscaled Q rows.
__global__ void __launch_bounds__(kMbWeightThreads) mb_weights_kernel(const MbWeightArgs w)
{
    const int p = blockIdx.x, c = blockIdx.y;
    __shared__ float smax[8][4];
    mb_reset_stats(w, c, p);
    const double f = (double)(uint32_t)w.freq[c];
    if (w.W32) {
        for (int a = threadIdx.x; a < w.A; a += blockDim.x) {
            float2 J[4];
            mb_jinv(w, c, p, a, J);
            const float2 ph = mb_phase(w, p, a, f);
            for (int x = 0; x < 2; x++) {
                float4 *d = reinterpret_cast<float4 *>(w.W32 + ((((long long)c * w.Bp + p) * 2 + x) * w.A + a) * 2);
                const float2 w0 = cmul32(ph, J[2 * x]), w1 = cmul32(ph, J[2 * x + 1]);
                *d = make_float4(w0.x, w0.y, w1.x, w1.y);
            }
            for (int st = 0; st < w.nst; st++) {
                float q[4];
                mb_qrow(J, st, q);
                *reinterpret_cast<float4 *>(w.Q32 + ((long long)c * w.Mq + p * w.nst + st) * w.KA + 4 * a) =
                    make_float4(q[0], q[1], q[2], q[3]);
            }
        }
        return;
    }
    float mx[4] = {0.f, 0.f, 0.f, 0.f};
    for (int a = threadIdx.x; a < w.A; a += blockDim.x) {
        float2 J[4];
        mb_jinv(w, c, p, a, J);
        for (int st = 0; st < w.nst; st++) {
            float q[4];
            mb_qrow(J, st, q);
            for (int j = 0; j < 4; j++) mx[st] = fmaxf(mx[st], fabsf(q[j]));
        }
    }
    float inv_scale[4];
    mb_q_scales(w, c, p, mx, smax, inv_scale);
    const bool h16 = w.fp16 != 0;
    for (int a = threadIdx.x; a < w.A; a += blockDim.x) {
        float2 J[4];
        mb_jinv(w, c, p, a, J);
        const float2 ph = mb_phase(w, p, a, f);
        for (int x = 0; x < 2; x++)
            for (int rho = 0; rho < 2; rho++) {
                uint2 hi, lo;
                mb_weight_halves(ph, J, x, rho, h16, hi, lo);
                const long long row = (long long)c * w.Mrows + 4 * p + 2 * x + rho;
                *reinterpret_cast<uint2 *>(w.Aw + row * w.KA + 4 * a) = hi;
                if (w.planes == 2)
                    *reinterpret_cast<uint2 *>(w.Aw + ((long long)w.nfine * w.Mrows + row) * w.KA + 4 * a) = lo;
            }
        for (int st = 0; st < w.nst; st++) {
            float q[4];
            mb_qrow(J, st, q);
            uint2 hi, lo;
            mb_q_halves(q, inv_scale[st], hi, lo);
            // 4-bit voltages: [Q_hi (| Q_lo)] against [C]; 8-bit: [Q_hi | Q_hi (| Q_lo)] against [C_hi | C_lo]
            __half *qrow = w.Aq + ((long long)c * w.Mq + p * w.nst + st) * w.Kq;
            *reinterpret_cast<uint2 *>(qrow + 4 * a) = hi;
            int k = w.KA;
            if (w.int8) {
                *reinterpret_cast<uint2 *>(qrow + k + 4 * a) = hi;
                k += w.KA;
            }
            if (w.planes == 2) *reinterpret_cast<uint2 *>(qrow + k + 4 * a) = lo;
        }
    }
}

// Up to 512 tiles: one block per (channel, kMbWeightBeams beams), thread t owning
// tiles 2t and 2t+1. The channel's D^-1 and its Gram terms stay in registers
// across the block's beams, each J^-1 is formed once (and held while the
// block finds the Q rows' scales), and every row is written with 16-byte
// stores covering both tiles.
__global__ void __launch_bounds__(256, 4) mb_weights_pair_kernel(const MbWeightArgs w)
{
    __shared__ float smax[8][4];
    const int c = blockIdx.y;
    const int a0 = 2 * threadIdx.x;
    const bool live = a0 < w.A;
    float4 dv[2][2], gv[2];
    for (int u = 0; u < 2; u++) {
        const long long ca = (long long)c * w.A + (live ? a0 + u : 0);
        dv[u][0] = w.Dinv[2 * ca];
        dv[u][1] = w.Dinv[2 * ca + 1];
        gv[u] = w.G[ca];
    }
    const double f = (double)(uint32_t)w.freq[c];
    const bool h16 = w.fp16 != 0;
    const int p_end = min(w.Bp, ((int)blockIdx.x + 1) * kMbWeightBeams);
    for (int p = blockIdx.x * kMbWeightBeams; p < p_end; p++) {
        mb_reset_stats(w, c, p);
        float mx[4] = {0.f, 0.f, 0.f, 0.f};
        float2 J[2][4];
        if (live) {
            float2 ph[2];
            for (int u = 0; u < 2; u++) {
                const long long pa = (long long)p * w.A + a0 + u;
                mb_jinv_from(w.H[pa], gv[u], w.Binv[2 * pa], w.Binv[2 * pa + 1], dv[u][0], dv[u][1], J[u]);
                ph[u] = mb_phase(w, p, a0 + u, f);
            }
            for (int x = 0; x < 2; x++)
                for (int rho = 0; rho < 2; rho++) {
                    uint2 hi0, lo0, hi1, lo1;
                    mb_weight_halves(ph[0], J[0], x, rho, h16, hi0, lo0);
                    mb_weight_halves(ph[1], J[1], x, rho, h16, hi1, lo1);
                    const long long row = (long long)c * w.Mrows + 4 * p + 2 * x + rho;
                    *reinterpret_cast<uint4 *>(w.Aw + row * w.KA + 4 * a0) = make_uint4(hi0.x, hi0.y, hi1.x, hi1.y);
                    if (w.planes == 2)
                        *reinterpret_cast<uint4 *>(w.Aw + ((long long)w.nfine * w.Mrows + row) * w.KA + 4 * a0) =
                            make_uint4(lo0.x, lo0.y, lo1.x, lo1.y);
                }
#pragma unroll
            for (int st = 0; st < 4; st++)
                if (st < w.nst)
#pragma unroll
                    for (int u = 0; u < 2; u++) {
                        float q[4];
                        mb_qrow(J[u], st, q);
                        for (int j = 0; j < 4; j++) mx[st] = fmaxf(mx[st], fabsf(q[j]));
                    }
        }
        float inv_scale[4];
        mb_q_scales(w, c, p, mx, smax, inv_scale);
        if (live) {
#pragma unroll
            for (int st = 0; st < 4; st++)
                if (st < w.nst) {
                    float q0[4], q1[4];
                    mb_qrow(J[0], st, q0);
                    mb_qrow(J[1], st, q1);
                    uint2 hi0, lo0, hi1, lo1;
                    mb_q_halves(q0, inv_scale[st], hi0, lo0);
                    mb_q_halves(q1, inv_scale[st], hi1, lo1);
                    const uint4 H4 = make_uint4(hi0.x, hi0.y, hi1.x, hi1.y);
                    __half *qrow = w.Aq + ((long long)c * w.Mq + p * w.nst + st) * w.Kq;
                    *reinterpret_cast<uint4 *>(qrow + 4 * a0) = H4;
                    int k = w.KA;
                    if (w.int8) {
                        *reinterpret_cast<uint4 *>(qrow + k + 4 * a0) = H4;
                        k += w.KA;
                    }
                    if (w.planes == 2)
                        *reinterpret_cast<uint4 *>(qrow + k + 4 * a0) = make_uint4(lo0.x, lo0.y, lo1.x, lo1.y);
                }
        }
        __syncthreads(); // smax is reused by the next beam
    }
}

// ---------------------------------------------------------------------------
// Voltages: legacy [s][c][input] (4+4-bit bytes, high nibble real, or int8
// re, im) -> B operand V [c][s][4A] (bf16 or fp16, exact) and the integrated
// per-tile coherencies C [c][t][Kb] (fp16; exact hi/lo halves for 8-bit).
// ---------------------------------------------------------------------------
struct MbConvArgs {
    const uint8_t *v;
    int int8, fp16;
    int ns, nfine, ni, A, nint, nint_p, Kb;
    const uint32_t *polQ, *polP;
    unsigned *status;     // kErrBadInput when polQ / polP name an input outside the row
    uint16_t *V;
    __half *C;
};

__device__ __forceinline__ int nib4(uint32_t x) { return ((int)(x << 28)) >> 28; }

// One block per (channel, integration), channels fastest so that neighbouring
// blocks read neighbouring bytes of each sample: the 10 voltage rows (2A
// inputs each) are staged in shared memory with 16-byte loads, then each
// thread gathers its tiles' (Q, P) inputs through polQ/polP.
__global__ void __launch_bounds__(128) mb_convert_kernel(const MbConvArgs g)
{
    extern __shared__ uint4 conv_smem[];
    uint8_t *rows = reinterpret_cast<uint8_t *>(conv_smem);
    const int c = blockIdx.x, t = blockIdx.y;
    const bool h16 = g.fp16 != 0;
    const int rowbytes = g.ni * (g.int8 ? 2 : 1); // a multiple of 32 (nant % 16 == 0)
    const int per_row = rowbytes / 16;
    // all of the block's row loads in flight at once (asynchronous copies), one wait
    for (int e = threadIdx.x; e < kMbInt * per_row; e += blockDim.x) {
        const int k = e / per_row, i = e - k * per_row;
        const uint4 *src = reinterpret_cast<const uint4 *>(g.v + ((long long)(t * kMbInt + k) * g.nfine + c) * rowbytes) + i;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(&conv_smem[e])), "l"(src) : "memory");
    }
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
    __syncthreads();
    for (int a = threadIdx.x; a < g.A; a += blockDim.x) {
        const uint32_t iq = g.polQ[a], ip = g.polP[a];
        if (iq >= (uint32_t)g.ni || ip >= (uint32_t)g.ni) {
            atomicOr(g.status, kErrBadInput);
            continue;
        }
        int cqq = 0, cpp = 0, cr = 0, ci = 0;
        for (int k = 0; k < kMbInt; k++) {
            const int s = t * kMbInt + k;
            const uint8_t *r = rows + k * rowbytes;
            int qr, qi, pr, pi;
            if (g.int8) {
                const char2 vq = reinterpret_cast<const char2 *>(r)[iq];
                const char2 vp = reinterpret_cast<const char2 *>(r)[ip];
                qr = vq.x; qi = vq.y; pr = vp.x; pi = vp.y;
            } else {
                const uint32_t bq = r[iq], bp = r[ip];
                qr = nib4(bq >> 4); qi = nib4(bq); pr = nib4(bp >> 4); pi = nib4(bp);
            }
            cqq += qr * qr + qi * qi;
            cpp += pr * pr + pi * pi;
            cr += qr * pr + qi * pi; // Re(vQ vP*)
            ci += qi * pr - qr * pi; // Im(vQ vP*)
            const uint2 o = make_uint2(to_bits((float)qr, h16) | ((uint32_t)to_bits((float)qi, h16) << 16),
                                       to_bits((float)pr, h16) | ((uint32_t)to_bits((float)pi, h16) << 16));
            *reinterpret_cast<uint2 *>(g.V + ((long long)c * g.ns + s) * (4 * g.A) + 4 * a) = o;
        }
        const int cv[4] = {cqq, cpp, cr, ci};
        uint16_t hi[4], lo[4];
        for (int j = 0; j < 4; j++) {
            const __half h = __float2half_rn((float)cv[j]);
            hi[j] = __half_as_ushort(h);
            lo[j] = __half_as_ushort(__float2half_rn((float)(cv[j] - (int)__half2float(h))));
        }
        __half *row = g.C + ((long long)c * g.nint_p + t) * g.Kb;
        *reinterpret_cast<uint2 *>(row + 4 * a) =
            make_uint2(hi[0] | ((uint32_t)hi[1] << 16), hi[2] | ((uint32_t)hi[3] << 16));
        if (g.int8)
            *reinterpret_cast<uint2 *>(row + 4 * g.A + 4 * a) =
                make_uint2(lo[0] | ((uint32_t)lo[1] << 16), lo[2] | ((uint32_t)lo[3] << 16));
    }
}

// ---------------------------------------------------------------------------
// The beam GEMM (persistent, one CTA per SM)
// ---------------------------------------------------------------------------
// One ring stage: kPlanes weight tiles (128 rows x 64 K, bf16/fp16) and the
// voltage tile (256 samples x 64 K); 192 KB of ring either way.
template <int kPlanes> struct MbRing {
    static constexpr int kTileA = 128 * 128;
    static constexpr int kTileB = kMbN * 128;
    static constexpr int kStage = kPlanes * kTileA + kTileB;
    static constexpr int kStages = kPlanes == 2 ? 3 : 4;
};

template <int kPlanes> struct MbSmem {
    uint8_t ring[MbRing<kPlanes>::kStages][MbRing<kPlanes>::kStage];
    uint64_t full[MbRing<kPlanes>::kStages], empty[MbRing<kPlanes>::kStages];
    uint64_t tfull[2], tempty[2], drain;
    uint32_t tmem;
};

struct MbBeamArgs {
    int nfine, ns, nint, B, Mrows, mtiles, ntn, nk;
    long long total;      // tiles: nfine * ntn * mtiles
    const float *R;       // [nfine][Mq][nint_p]
    const float *qscale;  // [nfine][Mq]
    int Mq, nint_p;
    float invw;
    float *S;             // [nfine][B][nst][nint]
    MbStats stats;
    unsigned *status;
};

// Epilogue of one accumulator tile (beam tile m, sample tile n, fine channel
// c) by one thread of an epilogue warp: TMEM lane `row` of the tile at `tacc`
// (lane quarter and buffer included), integrations [kI0, kI1) of the tile's
// 25 (columns 10 kI0 .. 10 kI1 - 1; the kMbEpq warps of a lane quarter take
// one range each, so every Stokes value is still formed by one thread from
// its 10 columns). Lanes 4b..4b+3 hold beam b's Xr, Xi, Yr, Yi; XX, YY, XY
// are formed across them, integrated over 10 samples, the autocorrelation
// term subtracted (form_beam.cpp:300-371) and Stokes written
// [chan][beam][stokes][t], with each row's extremes folded into
// order-preserving integer atomics for the 8-bit stage. `wait` blocks until
// the accumulator is complete (false: it gave up, nothing is written);
// `release` hands the TMEM buffer back once every load of it has finished.
template <int kNst, int kI0, int kI1, class Wait, class Release>
__device__ __forceinline__ bool mb_epilogue_tile(const MbBeamArgs &g, uint32_t tacc, int m, int n, int c, int row,
                                                 Wait &&wait, Release &&release)
{
    constexpr int kC0 = kMbInt * kI0, kC1 = kMbInt * kI1;   // columns of this range
    const int lane = threadIdx.x & 31;
    const int l = lane & 3;
    const int bl = row >> 2;
    const int p = m * kMbBeamsPerTile + bl;
    const int t0 = n * kMbNint;
    const int nv = min(kMbNint, g.nint - t0);
    const int st = kNst == 4 ? l : 0;
    const bool writer = p < g.B && (kNst == 4 || l == 0);
    const long long rrow = (long long)c * g.Mq + (long long)p * kNst + st;
    float rv[kI1 - kI0];
    float qs = 0.f;
    if (writer) qs = g.qscale[rrow];
#pragma unroll
    for (int i = kI0; i < kI1; i++) rv[i - kI0] = (writer && i < nv) ? g.R[rrow * g.nint_p + t0 + i] : 0.f;
    float *srow = g.S + (((long long)c * g.B + p) * kNst + st) * g.nint + t0;
    float smin = __int_as_float(0x7f800000), smax = -__int_as_float(0x7f800000);

    if (!wait()) {
        if (lane == 0) atomicOr(g.status, kErrWaitTimeout);
        return false;
    }
    tc_fence_after();
    float sq = 0.f, pb = 0.f, pc = 0.f;
#pragma unroll
    for (int j = kC0 / 32; j <= (kC1 - 1) / 32; j++) {
        float v[32];
        tmem_ld32(tacc + 32 * j, v);
#pragma unroll
        for (int col = 0; col < 32; col++) {
            const int gcol = 32 * j + col;
            if (gcol >= kC0 && gcol < kC1) {
                const float x = v[col];
                sq = fmaf(x, x, sq);
                if (kNst == 4) {
                    const float xb = __shfl_xor_sync(0xffffffffu, x, 2);
                    const float xc = __shfl_xor_sync(0xffffffffu, x, 3);
                    pb = fmaf(x, xb, pb);
                    pc = fmaf(x, xc, pc);
                }
                if (gcol % kMbInt == kMbInt - 1) {
                    const int ti = gcol / kMbInt;
                    float val;
                    if (kNst == 4) {
                        // lanes of a beam: 0 Xr, 1 Xi, 2 Yr, 3 Yi
                        const float t1 = sq + __shfl_xor_sync(0xffffffffu, sq, 1);
                        const float t1o = __shfl_xor_sync(0xffffffffu, t1, 2);
                        const float xx = l < 2 ? t1 : t1o, yy = l < 2 ? t1o : t1;
                        const float re = pb + __shfl_xor_sync(0xffffffffu, pb, 1);
                        const float d = __shfl_xor_sync(0xffffffffu, pc, 1) - pc;
                        const float im = (l == 0 || l == 3) ? d : -d;
                        val = l == 0 ? xx + yy : l == 1 ? xx - yy : l == 2 ? 2.f * re : -2.f * im;
                    } else {
                        float t1 = sq + __shfl_xor_sync(0xffffffffu, sq, 1);
                        t1 += __shfl_xor_sync(0xffffffffu, t1, 2);
                        val = t1;
                    }
                    if (writer && ti < nv) {
                        const float sv = g.invw * (val - qs * rv[ti - kI0]);
                        srow[ti] = sv;
                        smin = fminf(smin, sv);
                        smax = fmaxf(smax, sv);
                        if (kI0 == 0 && ti == 0 && t0 == 0)
                            g.stats.nan0[((long long)c * g.B + p) * kNst + st] = sv != sv;
                    }
                    sq = pb = pc = 0.f;
                }
            }
        }
    }
    tc_fence_before();
    __syncwarp();
    release();
    if (writer && kI0 < nv) {
        const long long r = ((long long)c * g.B + p) * kNst + st;
        atomicMin(&g.stats.mn[r], fkey(smin));
        atomicMax(&g.stats.mx[r], fkey(smax));
    }
    return true;
}

// Epilogue warp e (0 .. kMbEpiWarps - 1) of a CTA: lane quarter = its warp
// index % 4 (the TMEM lanes a warp may read), integrations part e / 4 of the
// tile's 25 split into kMbEpq ranges.
template <int kNst, class Wait, class Release>
__device__ __forceinline__ bool mb_epilogue_part(int part, const MbBeamArgs &g, uint32_t tacc, int m, int n, int c,
                                                 int row, Wait &&wait, Release &&release)
{
    static_assert(kMbEpq == 3, "three integration ranges");
    constexpr int a = kMbNint / 3, b = 2 * kMbNint / 3;   // 8, 16 of 25
    if (part == 0) return mb_epilogue_tile<kNst, 0, a>(g, tacc, m, n, c, row, wait, release);
    if (part == 1) return mb_epilogue_tile<kNst, a, b>(g, tacc, m, n, c, row, wait, release);
    return mb_epilogue_tile<kNst, b, kMbNint>(g, tacc, m, n, c, row, wait, release);
}

template <int kPlanes, bool kF16, int kNst>
__global__ void __launch_bounds__(kMbThreads, 1)
    mb_beam_kernel(const __grid_constant__ CUtensorMap tw, const __grid_constant__ CUtensorMap tv, const MbBeamArgs g)
{
    using Ring = MbRing<kPlanes>;
    constexpr int kStages = Ring::kStages;
    extern __shared__ uint8_t mb_raw[];
    MbSmem<kPlanes> &sm =
        *reinterpret_cast<MbSmem<kPlanes> *>((reinterpret_cast<uintptr_t>(mb_raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        prefetch_tmap(&tw);
        prefetch_tmap(&tv);
        for (int s = 0; s < kStages; s++) {
            mbar_init(&sm.full[s], 1);
            mbar_init(&sm.empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&sm.tfull[b], 1);
            mbar_init(&sm.tempty[b], kMbEpiWarps);
        }
        mbar_init(&sm.drain, 1);
        fence_mbar_init();
    }
    __syncwarp();
    if (warp == 0) {
        tmem_alloc(&sm.tmem, 512);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sm.tmem;
    const int per_tile = g.ntn * g.mtiles;

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer ----
            uint32_t it = 0;
            bool ok = true;
            for (long long tile = blockIdx.x; tile < g.total && ok; tile += gridDim.x) {
                const int m = (int)(tile % g.mtiles);
                const int n = (int)((tile / g.mtiles) % g.ntn);
                const int c = (int)(tile / per_tile);
                const int arow = c * g.Mrows + m * 128;
                const int brow = c * g.ns + n * kMbUsed;
                for (int kc = 0; kc < g.nk; kc++, it++) {
                    const int s = it % kStages;
                    const uint32_t r = it / kStages;
                    if (r > 0 && !mbar_wait_bounded(&sm.empty[s], (r - 1) & 1, kMbPolls)) {
                        atomicOr(g.status, kErrWaitTimeout);
                        ok = false;
                        break;
                    }
                    uint8_t *st = sm.ring[s];
                    mbar_arrive_expect_tx(&sm.full[s], Ring::kStage);
                    tma_load_2d(st, &tw, kc * 64, arow, &sm.full[s]);
                    if (kPlanes == 2) tma_load_2d(st + Ring::kTileA, &tw, kc * 64, arow + g.nfine * g.Mrows, &sm.full[s]);
                    tma_load_2d(st + kPlanes * Ring::kTileA, &tv, kc * 64, brow, &sm.full[s]);
                }
            }
            // every load issued must have landed before the CTA leaves
            for (uint32_t k = (it > kStages ? it - kStages : 0); k < it; k++)
                mbar_wait_bounded(&sm.full[k % kStages], (k / kStages) & 1, kMbPolls);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer ----
            const uint32_t idesc = idesc_bf16_f32(kMbN, false, kF16);
            uint32_t it = 0, tc = 0;
            bool ok = true;
            for (long long tile = blockIdx.x; tile < g.total && ok; tile += gridDim.x, tc++) {
                const int buf = tc & 1;
                const uint32_t u = tc >> 1;
                if (u > 0 && !mbar_wait_bounded(&sm.tempty[buf], (u - 1) & 1, kMbPolls)) {
                    atomicOr(g.status, kErrWaitTimeout);
                    break;
                }
                tc_fence_after();
                const uint32_t d = tmem + buf * kMbN;
                for (int kc = 0; kc < g.nk; kc++, it++) {
                    const int s = it % kStages;
                    if (!mbar_wait_bounded(&sm.full[s], (it / kStages) & 1, kMbPolls)) {
                        atomicOr(g.status, kErrWaitTimeout);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = smem_u32(sm.ring[s]);
                    const uint64_t a0 = sdesc_sw128(sa);
                    const uint64_t a1 = sdesc_sw128(sa + Ring::kTileA);
                    const uint64_t bd = sdesc_sw128(sa + kPlanes * Ring::kTileA);
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        tc_mma(d, sdesc_advance_k(a0, k), sdesc_advance_k(bd, k), idesc, (kc | k) != 0);
                        if (kPlanes == 2) tc_mma(d, sdesc_advance_k(a1, k), sdesc_advance_k(bd, k), idesc, 1);
                    }
                    tc_commit(&sm.empty[s]);
                }
                if (ok) tc_commit(&sm.tfull[buf]);
            }
            // all MMAs this thread issued have completed before teardown
            tc_commit(&sm.drain);
            mbar_wait_bounded(&sm.drain, 0, kMbPolls);
        }
    } else {
        // ---- epilogue: warps 2.., TMEM lane quarter = warp % 4, integration range (warp - 2) / 4 ----
        const int q4 = warp & 3, part = (warp - 2) >> 2;
        uint32_t tc = 0;
        for (long long tile = blockIdx.x; tile < g.total; tile += gridDim.x, tc++) {
            const int buf = tc & 1;
            const int m = (int)(tile % g.mtiles);
            const int n = (int)((tile / g.mtiles) % g.ntn);
            const int c = (int)(tile / per_tile);
            const bool ok = mb_epilogue_part<kNst>(
                part, g, tmem + ((uint32_t)(32 * q4) << 16) + buf * kMbN, m, n, c, 32 * q4 + lane,
                [&] { return mbar_wait_bounded(&sm.tfull[buf], (tc >> 1) & 1, kMbPolls); },
                [&] {
                    if (lane == 0) mbar_arrive(&sm.tempty[buf]);
                });
            if (!ok) break;
        }
    }
    __syncwarp();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, 512);
}

// ---------------------------------------------------------------------------
// The beam GEMM over CTA pairs (cta_group::2)
// ---------------------------------------------------------------------------
// mb_beam_kernel's 128 x 256 tile takes in 48 KB of operands per 64-wide K
// step from L2 for 2 M MACs (single plane), 64 KB in the split mode. Here the
// two CTAs of a cluster (the two SMs of a TPC) own beam tiles 2i and 2i + 1 of
// the same 256-sample tile: each stages its own 128 weight rows and HALF of
// the voltage tile (128 samples), and one thread of the even CTA issues
// 256 x 256 x 16 MMAs that read both CTAs' shared memory, so each SM takes in
// 32 KB per K step instead of 48 KB for the same MMA work. Each CTA's tensor
// memory holds its own 128 beam rows x 256 samples, and the epilogue is
// mb_beam_kernel's (identical arithmetic, same outputs).
//   warp 0 lane 0 (both CTAs): the TMA producer. Both CTAs' copies complete
//     on the even CTA's `full` barriers, whose expected byte count the even
//     CTA posts for the pair; each waits on its own `empty` barrier, which the
//     MMA commit reaches in both CTAs.
//   warp 1 lane 0 (even CTA): MMA issuer; each accumulator buffer is handed
//     to both CTAs' epilogues (`tfull`, multicast commit) and comes back when
//     every epilogue warp of the pair has arrived on the even CTA's `tempty`.
//   warps 2.. (both CTAs): epilogue of the CTA's own beam tile (mb_beam_kernel's
//     split: three warps per TMEM lane quarter, one integration range each).
// Every wait is bounded; the CTAs meet at a cluster barrier before either
// releases tensor memory or exits, so neither leaves while the other may
// still signal its barriers.
template <int kPlanes> struct Mb2Ring {
    static constexpr int kTileA = 128 * 128;         // 128 weight rows x 64 K, 16-bit
    static constexpr int kTileB = 128 * 128;         // half the voltage tile: 128 samples x 64 K
    static constexpr int kStage = kPlanes * kTileA + kTileB;
    static constexpr int kStages = kPlanes == 2 ? 4 : 6;
};

template <int kPlanes> struct Mb2Smem {
    uint8_t ring[Mb2Ring<kPlanes>::kStages][Mb2Ring<kPlanes>::kStage];
    uint64_t full[Mb2Ring<kPlanes>::kStages], empty[Mb2Ring<kPlanes>::kStages];
    uint64_t tfull[2], tempty[2], drain;
    uint32_t tmem;
};

template <int kPlanes, bool kF16, int kNst>
__global__ void __launch_bounds__(kMbThreads, 1)
    mb_beam_pair_kernel(const __grid_constant__ CUtensorMap tw, const __grid_constant__ CUtensorMap tv2,
                        const MbBeamArgs g)
{
    using Ring = Mb2Ring<kPlanes>;
    constexpr int kStages = Ring::kStages;
    extern __shared__ uint8_t mb_raw[];
    Mb2Smem<kPlanes> &sm =
        *reinterpret_cast<Mb2Smem<kPlanes> *>((reinterpret_cast<uintptr_t>(mb_raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = cluster_rank();
    const long long pair = blockIdx.x >> 1, npairs = gridDim.x >> 1;
    const int mtp = g.mtiles >> 1;                 // beam-tile pairs
    const long long per_c = (long long)g.ntn * mtp;
    const long long total = per_c * g.nfine;

    if (threadIdx.x == 0) {
        prefetch_tmap(&tw);
        prefetch_tmap(&tv2);
        for (int s = 0; s < kStages; s++) {
            mbar_init(&sm.full[s], 1);
            mbar_init(&sm.empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&sm.tfull[b], 1);
            mbar_init(&sm.tempty[b], 2 * kMbEpiWarps); // every epilogue warp of both CTAs
        }
        mbar_init(&sm.drain, 1);
        fence_mbar_init();
    }
    __syncwarp();
    if (warp == 0) {
        tmem_alloc_pair(&sm.tmem, 512);
        tmem_relinquish_pair();
    }
    tc_fence_before();
    // both CTAs' barriers are initialised before either signals the other's
    cluster_sync();
    tc_fence_after();
    const uint32_t tmem = sm.tmem;

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer (both CTAs) ----
            uint32_t it = 0;
            bool ok = true;
            for (long long pt = pair; pt < total && ok; pt += npairs) {
                const int mp = (int)(pt % mtp);
                const int n = (int)((pt / mtp) % g.ntn);
                const int c = (int)(pt / per_c);
                const int arow = c * g.Mrows + (2 * mp + (int)rank) * 128;
                const int brow = c * g.ns + n * kMbUsed + (int)rank * 128;
                for (int kc = 0; kc < g.nk; kc++, it++) {
                    const int s = it % kStages;
                    const uint32_t r = it / kStages;
                    if (r > 0 && !mbar_wait_bounded(&sm.empty[s], (r - 1) & 1, kMbPolls)) {
                        atomicOr(g.status, kErrWaitTimeout);
                        ok = false;
                        break;
                    }
                    uint8_t *st = sm.ring[s];
                    const uint32_t full0 = mapa_shared(smem_u32(&sm.full[s]), 0);
                    if (rank == 0) mbar_arrive_expect_tx(&sm.full[s], 2 * Ring::kStage);
                    tma_load_2d_pair(st, &tw, kc * 64, arow, full0);
                    if (kPlanes == 2)
                        tma_load_2d_pair(st + Ring::kTileA, &tw, kc * 64, arow + g.nfine * g.Mrows, full0);
                    tma_load_2d_pair(st + kPlanes * Ring::kTileA, &tv2, kc * 64, brow, full0);
                }
            }
            // the even CTA: every copy of the pair has landed before the
            // cluster barrier below lets either CTA leave
            if (rank == 0)
                for (uint32_t k = (it > kStages ? it - kStages : 0); k < it; k++)
                    mbar_wait_bounded(&sm.full[k % kStages], (k / kStages) & 1, kMbPolls);
        }
    } else if (warp == 1) {
        if (lane == 0 && rank == 0) {
            // ---- MMA issuer (even CTA) ----
            const uint32_t idesc = idesc_pair_f32(kMbN, kF16);
            uint32_t it = 0, tc = 0;
            bool ok = true;
            for (long long pt = pair; pt < total && ok; pt += npairs, tc++) {
                const int buf = tc & 1;
                const uint32_t u = tc >> 1;
                if (u > 0 && !mbar_wait_bounded(&sm.tempty[buf], (u - 1) & 1, kMbPolls)) {
                    atomicOr(g.status, kErrWaitTimeout);
                    break;
                }
                tc_fence_after();
                const uint32_t d = tmem + buf * kMbN;
                for (int kc = 0; kc < g.nk; kc++, it++) {
                    const int s = it % kStages;
                    if (!mbar_wait_bounded(&sm.full[s], (it / kStages) & 1, kMbPolls)) {
                        atomicOr(g.status, kErrWaitTimeout);
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t sa = smem_u32(sm.ring[s]);
                    const uint64_t a0 = sdesc_sw128(sa);
                    const uint64_t a1 = sdesc_sw128(sa + Ring::kTileA);
                    const uint64_t bd = sdesc_sw128(sa + kPlanes * Ring::kTileA);
#pragma unroll
                    for (int k = 0; k < 4; k++) {
                        tc_mma_pair(d, sdesc_advance_k(a0, k), sdesc_advance_k(bd, k), idesc, (kc | k) != 0);
                        if (kPlanes == 2) tc_mma_pair(d, sdesc_advance_k(a1, k), sdesc_advance_k(bd, k), idesc, 1);
                    }
                    tc_commit_pair_both(&sm.empty[s]);
                }
                if (ok) tc_commit_pair_both(&sm.tfull[buf]);
            }
            // all MMAs this thread issued have completed before teardown
            tc_commit_pair_own(&sm.drain);
            mbar_wait_bounded(&sm.drain, 0, kMbPolls);
        }
    } else {
        // ---- epilogue: warps 2.. of both CTAs, TMEM lane quarter = warp % 4, range (warp - 2) / 4 ----
        const int q4 = warp & 3, part = (warp - 2) >> 2;
        const uint32_t tempty0 = mapa_shared(smem_u32(&sm.tempty[0]), 0), tempty1 = mapa_shared(smem_u32(&sm.tempty[1]), 0);
        uint32_t tc = 0;
        for (long long pt = pair; pt < total; pt += npairs, tc++) {
            const int buf = tc & 1;
            const int mp = (int)(pt % mtp);
            const int n = (int)((pt / mtp) % g.ntn);
            const int c = (int)(pt / per_c);
            const bool ok = mb_epilogue_part<kNst>(
                part, g, tmem + ((uint32_t)(32 * q4) << 16) + buf * kMbN, 2 * mp + (int)rank, n, c, 32 * q4 + lane,
                [&] { return mbar_wait_bounded(&sm.tfull[buf], (tc >> 1) & 1, kMbPolls); },
                [&] {
                    if (lane == 0) mbar_arrive_cluster(buf ? tempty1 : tempty0);
                });
            if (!ok) break;
        }
    }
    __syncwarp();
    tc_fence_before();
    cluster_sync();
    tc_fence_after();
    if (warp == 0) tmem_dealloc_pair(tmem, 512);
}


// ---------------------------------------------------------------------------
// The plain FP32 CUDA-core beamformer: the same contraction, detection,
// integration and autocorrelation removal with FP32 weights and FP32 FMAs
// (no tensor cores). It is the baseline the tensor-core modes are measured
// and checked against.
// ---------------------------------------------------------------------------
constexpr int kSimtBeams = 32;   // beams per CTA
constexpr int kSimtSamp = 160;   // samples per CTA (16 integrations)
constexpr int kSimtK = 16;       // tiles per K chunk (32 complex inputs)
constexpr int kSimtRow = 33;     // padded smem row (float2)

struct MbSimtArgs {
    const float2 *W;      // [nfine][Bp][2][A][2]
    const uint16_t *V;    // [nfine][ns][4A] bf16 (exact voltages)
    const float *R;       // [nfine][Mq][nint_p]
    int A, Bp, B, ns, nint, nint_p, Mq;
    float invw;
    float *S;             // [nfine][B][nst][nint]
    MbStats stats;
};

// Thread: beams {bg, bg + 8} of its warp's 16 (x and y rows each) x one
// integration of 10 samples; a warp covers 16 beams x 4 integrations.
template <int kNst>
__global__ void __launch_bounds__(256, 1) mb_simt_beam_kernel(const MbSimtArgs g)
{
    extern __shared__ float2 simt_smem[];
    float2(*Ws)[kSimtRow] = reinterpret_cast<float2(*)[kSimtRow]>(simt_smem); // [2*beams][..]: row 2 * beam + x
    float2(*Vs)[kSimtRow] = reinterpret_cast<float2(*)[kSimtRow]>(simt_smem + 2 * kSimtBeams * kSimtRow); // [samples]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int bg = lane & 7, ig = lane >> 3;
    const int wb = warp & 1, ws = warp >> 1;
    const int c = blockIdx.z;
    const int p0 = blockIdx.y * kSimtBeams;
    const int s0 = blockIdx.x * kSimtSamp;
    const int lb[2] = {wb * 16 + bg, wb * 16 + bg + 8};   // local beams
    const int ls = ws * 40 + ig * 10;                    // local first sample

    float2 acc[2][2][10];
#pragma unroll
    for (int b = 0; b < 2; b++)
#pragma unroll
        for (int x = 0; x < 2; x++)
#pragma unroll
            for (int i = 0; i < 10; i++) acc[b][x][i] = make_float2(0.f, 0.f);

    for (int a0 = 0; a0 < g.A; a0 += kSimtK) {
        __syncthreads();
        // weights: 64 rows x 32 complex, rows contiguous in global memory
        for (int e = threadIdx.x; e < 2 * kSimtBeams * 2 * kSimtK; e += blockDim.x) {
            const int r = e / (2 * kSimtK), k = e % (2 * kSimtK);
            const int pb = r >> 1, x = r & 1;
            Ws[r][k] = g.W[((((long long)c * g.Bp + p0 + pb) * 2 + x) * g.A + a0) * 2 + k];
        }
        // voltages: 160 samples x 32 complex (bf16 re, im pairs)
        for (int e = threadIdx.x; e < kSimtSamp * 2 * kSimtK; e += blockDim.x) {
            const int sl = e / (2 * kSimtK), k = e % (2 * kSimtK);
            const int s = s0 + sl;
            float2 v = make_float2(0.f, 0.f);
            if (s < g.ns) {
                const uint32_t u =
                    *reinterpret_cast<const uint32_t *>(g.V + ((long long)c * g.ns + s) * (4 * g.A) + 4 * a0 + 2 * k);
                v = make_float2(__uint_as_float(u << 16), __uint_as_float(u & 0xFFFF0000u));
            }
            Vs[sl][k] = v;
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < 2 * kSimtK; k++) {
            float2 wv[2][2];
#pragma unroll
            for (int b = 0; b < 2; b++)
#pragma unroll
                for (int x = 0; x < 2; x++) wv[b][x] = Ws[2 * lb[b] + x][k];
#pragma unroll
            for (int i = 0; i < 10; i++) {
                const float2 v = Vs[ls + i][k];
#pragma unroll
                for (int b = 0; b < 2; b++)
#pragma unroll
                    for (int x = 0; x < 2; x++) {
                        acc[b][x][i].x = fmaf(wv[b][x].x, v.x, acc[b][x][i].x);
                        acc[b][x][i].x = fmaf(-wv[b][x].y, v.y, acc[b][x][i].x);
                        acc[b][x][i].y = fmaf(wv[b][x].x, v.y, acc[b][x][i].y);
                        acc[b][x][i].y = fmaf(wv[b][x].y, v.x, acc[b][x][i].y);
                    }
            }
        }
    }
    const int t = (s0 + ls) / kMbInt;
    const bool tval = t < g.nint;
#pragma unroll
    for (int b = 0; b < 2; b++) {
        const int p = p0 + lb[b];
        float xx = 0.f, yy = 0.f, re = 0.f, im = 0.f;
#pragma unroll
        for (int i = 0; i < 10; i++) {
            const float2 ex = acc[b][0][i], ey = acc[b][1][i];
            xx = fmaf(ex.x, ex.x, fmaf(ex.y, ex.y, xx));
            yy = fmaf(ey.x, ey.x, fmaf(ey.y, ey.y, yy));
            re = fmaf(ex.x, ey.x, fmaf(ex.y, ey.y, re));
            im = fmaf(ex.y, ey.x, fmaf(-ex.x, ey.y, im));
        }
        const float val[4] = {xx + yy, xx - yy, 2.f * re, -2.f * im};
#pragma unroll
        for (int st = 0; st < kNst; st++) {
            const long long row = ((long long)c * g.B + p) * kNst + st;
            float mn = __int_as_float(0x7f800000), mx = -__int_as_float(0x7f800000);
            if (p < g.B && tval) {
                const float r = g.R[((long long)c * g.Mq + p * kNst + st) * g.nint_p + t];
                const float sv = g.invw * (val[st] - r);
                g.S[row * g.nint + t] = sv;
                if (t == 0) g.stats.nan0[row] = sv != sv;
                mn = sv;
                mx = sv;
            }
            // the four lanes of a beam group (different integrations) share a row
            mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, 8));
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 8));
            mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, 16));
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, 16));
            if (ig == 0 && p < g.B) {
                atomicMin(&g.stats.mn[row], fkey(mn));
                atomicMax(&g.stats.mx[row], fkey(mx));
            }
        }
    }
}

// R[c][row][t] = sum_k Q[c][row][k] Cint[c][t][k] in FP32 (64 x 64 tiles,
// 4 x 4 per thread). The coherencies are read back from their exact FP16
// halves.
struct MbSimtAutoArgs {
    const float *Q;       // [nfine][Mq][4A]
    const __half *C;      // [nfine][nint_p][Kb]
    int KA, Kb, Mq, nint, nint_p, int8;
    float *R;             // [nfine][Mq][nint_p]
};

__global__ void __launch_bounds__(256) mb_simt_auto_kernel(const MbSimtAutoArgs g)
{
    __shared__ float Qs[16][65], Cs[16][65];
    const int c = blockIdx.z;
    const int r0 = blockIdx.y * 64, t0 = blockIdx.x * 64;
    const int tr = threadIdx.x >> 4, tt = threadIdx.x & 15;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < g.KA; k0 += 16) {
        __syncthreads();
        for (int e = threadIdx.x; e < 64 * 16; e += 256) {
            const int i = e >> 4, k = e & 15;
            Qs[k][i] = g.Q[((long long)c * g.Mq + r0 + i) * g.KA + k0 + k];
            const int t = t0 + i;
            float cv = 0.f;
            if (t < g.nint) {
                const __half *row = g.C + ((long long)c * g.nint_p + t) * g.Kb;
                cv = __half2float(row[k0 + k]);
                if (g.int8) cv += __half2float(row[g.KA + k0 + k]);
            }
            Cs[k][i] = cv;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < 16; k++) {
            float q[4], cv[4];
#pragma unroll
            for (int i = 0; i < 4; i++) {
                q[i] = Qs[k][tr + 16 * i];
                cv[i] = Cs[k][tt + 16 * i];
            }
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = fmaf(q[i], cv[j], acc[i][j]);
        }
    }
#pragma unroll
    for (int i = 0; i < 4; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int t = t0 + tt + 16 * j;
            if (t < g.nint_p) g.R[((long long)c * g.Mq + r0 + tr + 16 * i) * g.nint_p + t] = acc[i][j];
        }
}

// ---------------------------------------------------------------------------
// Scale-and-offset to 8 bits (form_beam.cpp:408-449 arithmetic, the same as
// renorm_kernel) from the beam-major Stokes [c][p][st][t], written in the
// PSRFITS order out[p][t][st][c] through a shared-memory transpose.
// ---------------------------------------------------------------------------
struct MbRenormArgs {
    const float *S;
    int nfine, B, nst, nint;
    uint8_t *out;
    long long out_p, out_s, out_st;
    float *offsets, *scales; // [(p * nst + st) * nfine + c]
    MbStats stats;
};

constexpr int kRnT = 128; // integrations per transpose chunk

// Block: (32 channels, one beam and Stokes parameter). The row extremes come
// from the beam epilogue (MbStats); one pass then quantises 128 integrations
// at a time, packs four channels' bytes into a word, transposes in shared
// memory and writes 16-byte runs of channels.
__global__ void __launch_bounds__(256, 4) mb_renorm_kernel(const MbRenormArgs a)
{
    __shared__ float s_off[32], s_scl[32];
    __shared__ uint32_t tile[kRnT][9];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int c0 = blockIdx.x * 32;
    const int st = blockIdx.y % a.nst, p = blockIdx.y / a.nst;
    if (threadIdx.x < 32) {
        const int c = c0 + threadIdx.x;
        float mn = 0.f, mx = 0.f;
        if (c < a.nfine) {
            const long long r = ((long long)c * a.B + p) * a.nst + st;
            if (a.stats.nan0[r]) {
                mn = mx = __int_as_float(0x7fffffff);
            } else {
                mn = fkey_inv(a.stats.mn[r]);
                mx = fkey_inv(a.stats.mx[r]);
            }
        }
        const float scale = (float)((double)(mx - mn) / 256.0);
        s_off[threadIdx.x] = mn;
        s_scl[threadIdx.x] = scale;
        if (c < a.nfine) {
            const long long si = ((long long)p * a.nst + st) * a.nfine + c;
            a.scales[si] = scale;
            a.offsets[si] = mn;
        }
    }
    __syncthreads();
    // warp w: channels 4w .. 4w+3 of the block
    const float *rows[4];
    float off[4], scl[4], rcp[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const int c = c0 + 4 * wid + k;
        rows[k] = a.S + (((long long)(c < a.nfine ? c : c0) * a.B + p) * a.nst + st) * a.nint;
        off[k] = s_off[4 * wid + k];
        scl[k] = s_scl[4 * wid + k];
        rcp[k] = 1.f / scl[k];
    }
    const bool wide = ((a.out_s | a.out_st | a.out_p) & 15) == 0 &&
                      (reinterpret_cast<uintptr_t>(a.out) & 15) == 0 && c0 + 32 <= a.nfine;
    for (int t0 = 0; t0 < a.nint; t0 += kRnT) {
        float e[4][4];
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const int t = t0 + lane + 32 * j;
#pragma unroll
            for (int k = 0; k < 4; k++) e[j][k] = t < a.nint ? rows[k][t] : 0.f;
        }
#pragma unroll
        for (int j = 0; j < 4; j++) {
            uint32_t w = 0;
#pragma unroll
            for (int k = 0; k < 4; k++) w |= (uint32_t)quant_u8(e[j][k], off[k], scl[k], rcp[k]) << (8 * k);
            tile[lane + 32 * j][wid] = w;
        }
        __syncthreads();
        const int tl = threadIdx.x >> 1, h = threadIdx.x & 1, t = t0 + tl;
        if (t < a.nint) {
            uint8_t *o = a.out + p * a.out_p + (long long)t * a.out_s + st * a.out_st + c0 + 16 * h;
            const uint4 v = make_uint4(tile[tl][4 * h], tile[tl][4 * h + 1], tile[tl][4 * h + 2], tile[tl][4 * h + 3]);
            if (wide) {
                *reinterpret_cast<uint4 *>(o) = v;
            } else {
                const uint32_t w4[4] = {v.x, v.y, v.z, v.w};
                for (int q = 0; q < 16; q++)
                    if (c0 + 16 * h + q < a.nfine) o[q] = (uint8_t)(w4[q >> 2] >> (8 * (q & 3)));
            }
        }
        __syncthreads();
    }
}

} // namespace vgb

using namespace vgb;

// ---------------------------------------------------------------------------
// Host object
// ---------------------------------------------------------------------------
struct vgb_multibeam {
    vgb_multibeam_config cfg;
    int nch, Bp, Mrows, Mq, KA, Kq, Kb, nint, nint_p, planes, ntn, mtiles, nk, fp16, int8;
    double *d_dt = nullptr;
    float4 *d_Binv = nullptr, *d_H = nullptr, *d_Dinv = nullptr, *d_G = nullptr;
    double *d_freq = nullptr;
    uint32_t *d_polQ = nullptr, *d_polP = nullptr;
    uint16_t *d_Aw = nullptr, *d_V = nullptr;
    __half *d_Aq = nullptr, *d_C = nullptr;
    float *d_qscale = nullptr, *d_R = nullptr, *d_S = nullptr;
    float2 *d_W32 = nullptr; // FP32 mode weights
    float *d_Q32 = nullptr;
    uint32_t *d_stats = nullptr; // min keys, max keys, first-is-NaN: 3 x [nfine][B][nst]
    bool simt = false;
    CUtensorMap tmW, tmV;
    CUtensorMap tmV2;            // voltages in 128-sample boxes: the pair kernel's half tiles
    int pair_clusters = -1;      // co-resident 2-CTA clusters of the pair kernel (-1: not yet asked)
    int beam_pick = 0;           // automatic choice: 0 undecided, 1 single-CTA kernel, 2 pair kernel
    int last_pair = 0;           // CTA pairs of the last beam GEMM (0: the single-CTA kernel ran)
    bool have_geometry = false, have_jones = false;
    int nsm = 0;
    int last_launches = 0; // kernels the last run launched
    cudaEvent_t *ev = nullptr; // timing: 6 events per coarse channel (stage boundaries)
    // host streaming (vgb_multibeam_run_host): two device slots of one
    // coarse channel-second each, upload and download streams
    uint8_t *d_vin[2] = {nullptr, nullptr}, *d_out[2] = {nullptr, nullptr};
    float *d_off[2] = {nullptr, nullptr}, *d_scl[2] = {nullptr, nullptr};
    cudaStream_t s_h2d = nullptr, s_d2h = nullptr;
    cudaEvent_t ev_h2d[2] = {}, ev_comp[2] = {}, ev_d2h[2] = {};
};

namespace {

template <typename T> int mb_alloc(T **p, size_t n, const char *what)
{
    if (cudaMalloc(reinterpret_cast<void **>(p), n * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return set_error(VGB_ERR_ALLOC, "multibeam: cannot allocate %s (%zu bytes)", what, n * sizeof(T));
    }
    return VGB_SUCCESS;
}

void mb_free(vgb_multibeam *mb)
{
    for (int b = 0; b < 2; b++) {
        for (void *p : {(void *)mb->d_vin[b], (void *)mb->d_out[b], (void *)mb->d_off[b], (void *)mb->d_scl[b]})
            if (p) cudaFree(p);
        for (cudaEvent_t e : {mb->ev_h2d[b], mb->ev_comp[b], mb->ev_d2h[b]})
            if (e) cudaEventDestroy(e);
    }
    if (mb->s_h2d) cudaStreamDestroy(mb->s_h2d);
    if (mb->s_d2h) cudaStreamDestroy(mb->s_d2h);
    if (mb->ev) {
        for (int i = 0; i < 6 * mb->cfg.ncc; i++)
            if (mb->ev[i]) cudaEventDestroy(mb->ev[i]);
        delete[] mb->ev;
        mb->ev = nullptr;
    }
    void *ptrs[] = {mb->d_dt, mb->d_Binv, mb->d_H, mb->d_Dinv, mb->d_G, mb->d_freq, mb->d_polQ, mb->d_polP,
                    mb->d_Aw, mb->d_V, mb->d_Aq, mb->d_C, mb->d_qscale, mb->d_R, mb->d_S, mb->d_W32, mb->d_Q32, mb->d_stats};
    for (void *p : ptrs)
        if (p) cudaFree(p);
}

// Beam GEMM kernel: 0 = the pair kernel where the beam tiles pair up and a
// 2-CTA cluster fits, else the single-CTA kernel; 1 = always the single-CTA
// kernel; 2 = the pair kernel wherever the beam tiles pair up.
std::atomic<int> g_mb_beam_variant{0};

// The pair kernel over as many co-resident 2-CTA clusters as the tiles need
// (at most the occupancy query's count). Returns 1 (nothing launched) when no
// cluster of that shape fits on the device.
template <int kPlanes, bool kF16, int kNst>
int mb_launch_beam_pair(vgb_multibeam *mb, const MbBeamArgs &a, cudaStream_t st)
{
    auto kern = mb_beam_pair_kernel<kPlanes, kF16, kNst>;
    const int smem = (int)sizeof(Mb2Smem<kPlanes>) + 1024;
    int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                        "cudaFuncSetAttribute(mb_beam_pair_kernel)");
    if (rc) return rc;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = 2;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kMbThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (mb->pair_clusters < 0) {
        int n = 0;
        cfg.gridDim = dim3(2 * (unsigned)mb->nsm);
        if (cudaOccupancyMaxActiveClusters(&n, kern, &cfg) != cudaSuccess) {
            cudaGetLastError();
            n = 0;
        }
        mb->pair_clusters = n;
    }
    if (mb->pair_clusters <= 0) return 1;
    const long long pairs = a.total / 2;
    const long long clusters = pairs < mb->pair_clusters ? pairs : mb->pair_clusters;
    cfg.gridDim = dim3(2 * (unsigned)clusters);
    rc = check_cuda(cudaLaunchKernelEx(&cfg, kern, mb->tmW, mb->tmV2, a), "cudaLaunchKernelEx(mb_beam_pair_kernel)");
    if (!rc) rc = check_launch("mb_beam_pair_kernel");
    if (!rc) mb->last_pair = (int)clusters;
    return rc;
}

template <int kPlanes, bool kF16, int kNst>
int mb_launch_beam_single(vgb_multibeam *mb, const MbBeamArgs &a, cudaStream_t st)
{
    auto kern = mb_beam_kernel<kPlanes, kF16, kNst>;
    const int smem = (int)sizeof(MbSmem<kPlanes>) + 1024;
    int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                        "cudaFuncSetAttribute(mb_beam_kernel)");
    if (rc) return rc;
    const long long grid = a.total < mb->nsm ? a.total : mb->nsm;
    kern<<<(unsigned)grid, kMbThreads, smem, st>>>(mb->tmW, mb->tmV, a);
    mb->last_pair = 0;
    return check_launch("mb_beam_kernel");
}

// The automatic choice for this object, made on its first beam GEMM outside
// stream capture: both kernels run twice on this coarse channel (each run
// writes the same Stokes and the same idempotent row extremes) and the faster
// is kept. The host waits for those four launches once.
template <int kPlanes, bool kF16, int kNst>
int mb_pick_beam(vgb_multibeam *mb, const MbBeamArgs &a, cudaStream_t st)
{
    cudaEvent_t ev[3] = {};
    int rc = VGB_SUCCESS;
    for (int i = 0; i < 3 && !rc; i++) rc = check_cuda(cudaEventCreate(&ev[i]), "cudaEventCreate");
    float t_single = 0.f, t_pair = 0.f;
    bool fits = true;
    if (!rc) rc = check_cuda(cudaEventRecord(ev[0], st), "cudaEventRecord");
    for (int i = 0; i < 2 && !rc; i++) rc = mb_launch_beam_single<kPlanes, kF16, kNst>(mb, a, st);
    if (!rc) rc = check_cuda(cudaEventRecord(ev[1], st), "cudaEventRecord");
    for (int i = 0; i < 2 && !rc && fits; i++) {
        const int r = mb_launch_beam_pair<kPlanes, kF16, kNst>(mb, a, st);
        if (r == 1) fits = false;
        else rc = r;
    }
    if (!rc) rc = check_cuda(cudaEventRecord(ev[2], st), "cudaEventRecord");
    if (!rc) rc = check_cuda(cudaEventSynchronize(ev[2]), "cudaEventSynchronize");
    if (!rc) rc = check_cuda(cudaEventElapsedTime(&t_single, ev[0], ev[1]), "cudaEventElapsedTime");
    if (!rc) rc = check_cuda(cudaEventElapsedTime(&t_pair, ev[1], ev[2]), "cudaEventElapsedTime");
    for (cudaEvent_t e : ev)
        if (e) cudaEventDestroy(e);
    if (!rc) mb->beam_pick = fits && t_pair < t_single ? 2 : 1;
    return rc;
}

template <int kPlanes, bool kF16, int kNst> int mb_launch_beam(vgb_multibeam *mb, const MbBeamArgs &a, cudaStream_t st)
{
    const int v = g_mb_beam_variant.load();
    const bool pairs_ok = mb->mtiles % 2 == 0;
    if (v == 2 && !pairs_ok)
        return set_error(VGB_ERR_UNSUPPORTED, "multibeam: the pair kernel needs an even number of beam tiles");
    if (v == 0 && pairs_ok && mb->beam_pick == 0) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cs) != cudaSuccess) {
            cudaGetLastError();
            cs = cudaStreamCaptureStatusActive;
        }
        if (cs == cudaStreamCaptureStatusNone) {
            const int rc = mb_pick_beam<kPlanes, kF16, kNst>(mb, a, st);
            if (rc) return rc;
        }
    }
    // undecided (first run inside a capture): the pair kernel
    if (v == 2 || (v == 0 && pairs_ok && mb->beam_pick != 1)) {
        const int r = mb_launch_beam_pair<kPlanes, kF16, kNst>(mb, a, st);
        if (r != 1) return r;
        if (v == 2) return set_error(VGB_ERR_UNSUPPORTED, "multibeam: no 2-CTA cluster of the pair kernel fits");
    }
    return mb_launch_beam_single<kPlanes, kF16, kNst>(mb, a, st);
}

} // namespace

extern "C" int vgb_multibeam_create(const vgb_multibeam_config *cfg, vgb_multibeam **out)
{
    if (!cfg || !out) return set_error(VGB_ERR_INVALID, "multibeam: NULL argument");
    *out = nullptr;
    const vgb_multibeam_config &c = *cfg;
    if (c.ncc <= 0 || c.nfine <= 0 || c.nfine > 4096)
        return set_error(VGB_ERR_INVALID, "multibeam: ncc and nfine must be positive (nfine <= 4096)");
    if (c.nant <= 0 || c.nant % 16 || c.nant > 2048)
        return set_error(VGB_ERR_INVALID, "multibeam: nant must be a positive multiple of 16, at most 2048 (got %d)",
                         c.nant);
    if (c.npointing <= 0) return set_error(VGB_ERR_INVALID, "multibeam: npointing must be positive");
    if (c.nsamples <= 0 || c.nsamples % kMbInt || c.nsamples / kMbInt > 65535)
        return set_error(VGB_ERR_INVALID, "multibeam: nsamples must be a positive multiple of %d, at most %d", kMbInt,
                         65535 * kMbInt);
    if (c.nstokes != 1 && c.nstokes != 4) return set_error(VGB_ERR_INVALID, "multibeam: nstokes must be 1 or 4");
    if (c.precision != VGB_MB_SPLIT_BF16 && c.precision != VGB_MB_BF16 && c.precision != VGB_MB_FP16 &&
        c.precision != VGB_MB_FP32)
        return set_error(VGB_ERR_UNSUPPORTED, "multibeam: unknown precision %d", c.precision);
    if (c.input != VGB_MB_INT4 && c.input != VGB_MB_INT8)
        return set_error(VGB_ERR_UNSUPPORTED, "multibeam: unknown input format %d", c.input);

    vgb_multibeam *mb = new vgb_multibeam();
    mb->cfg = c;
    mb->nch = c.nfine;
    mb->Bp = (c.npointing + kMbBeamsPerTile - 1) / kMbBeamsPerTile * kMbBeamsPerTile;
    mb->Mrows = 4 * mb->Bp;
    mb->mtiles = mb->Mrows / 128;
    mb->Mq = (c.nstokes * mb->Bp + 127) / 128 * 128;
    mb->KA = 4 * c.nant;
    mb->nk = mb->KA / 64;
    mb->int8 = c.input == VGB_MB_INT8;
    mb->planes = c.precision == VGB_MB_SPLIT_BF16 ? 2 : 1;
    // autocorrelation GEMM operands: [Q_hi (| Q_lo)] x [C] for 4-bit voltages,
    // [Q_hi | Q_hi (| Q_lo)] x [C_hi | C_lo] for 8-bit (Q_lo only in the split mode)
    mb->Kb = mb->int8 ? 8 * c.nant : 4 * c.nant;
    mb->Kq = (mb->int8 ? 8 * c.nant : 4 * c.nant) + (mb->planes == 2 ? 4 * c.nant : 0);
    mb->nint = c.nsamples / kMbInt;
    mb->nint_p = (mb->nint + 127) / 128 * 128;
    mb->fp16 = c.precision == VGB_MB_FP16;
    mb->simt = c.precision == VGB_MB_FP32;
    mb->ntn = (c.nsamples + kMbUsed - 1) / kMbUsed;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&mb->nsm, cudaDevAttrMultiProcessorCount, dev);
    if (mb->nsm <= 0) mb->nsm = 1;

    const size_t nf = c.nfine, A = c.nant;
    int rc = VGB_SUCCESS;
    if (!rc) rc = mb_alloc(&mb->d_dt, (size_t)mb->Bp * A, "delays");
    if (!rc) rc = mb_alloc(&mb->d_Binv, (size_t)c.ncc * mb->Bp * A * 2, "B^-1");
    if (!rc) rc = mb_alloc(&mb->d_H, (size_t)c.ncc * mb->Bp * A, "B B^H");
    if (!rc) rc = mb_alloc(&mb->d_Dinv, (size_t)c.ncc * nf * A * 2, "D^-1");
    if (!rc) rc = mb_alloc(&mb->d_G, (size_t)c.ncc * nf * A, "D^H D");
    if (!rc) rc = mb_alloc(&mb->d_freq, (size_t)c.ncc * nf, "frequencies");
    if (!rc) rc = mb_alloc(&mb->d_polQ, A, "polQ");
    if (!rc) rc = mb_alloc(&mb->d_polP, A, "polP");
    if (!rc && !mb->simt) rc = mb_alloc(&mb->d_Aw, (size_t)mb->planes * nf * mb->Mrows * mb->KA, "weights");
    if (!rc && mb->simt) rc = mb_alloc(&mb->d_W32, nf * mb->Bp * 2 * A * 2, "FP32 weights");
    if (!rc && mb->simt) rc = mb_alloc(&mb->d_Q32, nf * mb->Mq * mb->KA, "FP32 autocorrelation weights");
    if (!rc && mb->simt) rc = check_cuda(cudaMemset(mb->d_Q32, 0, nf * mb->Mq * mb->KA * sizeof(float)), "cudaMemset");
    if (!rc) rc = mb_alloc(&mb->d_V, nf * c.nsamples * mb->KA, "voltages");
    if (!rc) rc = mb_alloc(&mb->d_Aq, nf * mb->Mq * mb->Kq, "autocorrelation weights");
    if (!rc) rc = mb_alloc(&mb->d_C, nf * mb->nint_p * mb->Kb, "coherencies");
    if (!rc) rc = mb_alloc(&mb->d_qscale, nf * mb->Mq, "row scales");
    if (!rc) rc = mb_alloc(&mb->d_R, nf * mb->Mq * mb->nint_p, "autocorrelation terms");
    if (!rc) rc = mb_alloc(&mb->d_S, nf * c.npointing * c.nstokes * mb->nint, "Stokes");
    if (!rc) rc = mb_alloc(&mb->d_stats, 3 * nf * c.npointing * c.nstokes, "row statistics");
    if (!rc)
        rc = check_cuda(cudaMemset(mb->d_Aq, 0, nf * mb->Mq * mb->Kq * sizeof(__half)), "cudaMemset");
    if (!rc) rc = check_cuda(cudaMemset(mb->d_C, 0, nf * mb->nint_p * mb->Kb * sizeof(__half)), "cudaMemset");
    if (!rc && !mb->simt)
        rc = make_tmap_bf16(&mb->tmW, mb->d_Aw, (uint64_t)mb->planes * nf * mb->Mrows, mb->KA, (uint64_t)mb->KA * 2,
                            128, mb->fp16);
    if (!rc)
        rc = make_tmap_bf16(&mb->tmV, mb->d_V, (uint64_t)nf * c.nsamples, mb->KA, (uint64_t)mb->KA * 2, kMbN,
                            mb->fp16);
    if (!rc)
        rc = make_tmap_bf16(&mb->tmV2, mb->d_V, (uint64_t)nf * c.nsamples, mb->KA, (uint64_t)mb->KA * 2, kMbN / 2,
                            mb->fp16);
    if (rc) {
        mb_free(mb);
        delete mb;
        return rc;
    }
    *out = mb;
    return VGB_SUCCESS;
}

extern "C" void vgb_multibeam_destroy(vgb_multibeam *mb)
{
    if (!mb) return;
    cudaDeviceSynchronize();
    mb_free(mb);
    delete mb;
}

extern "C" int vgb_multibeam_set_geometry(vgb_multibeam *mb, const double *unit, const double *east,
                                          const double *north, const double *height, const double *cable,
                                          double href, void *stream)
{
    if (!mb || !unit || !east || !north || !height || !cable)
        return set_error(VGB_ERR_INVALID, "multibeam_set_geometry: NULL argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int n = mb->Bp * mb->cfg.nant;
    mb_pa_kernel<<<(n + 255) / 256, 256, 0, st>>>(unit, east, north, height, cable, href, nullptr,
                                                   mb->cfg.npointing, mb->Bp, mb->cfg.nant, mb->d_dt, mb->d_Binv,
                                                   mb->d_H);
    int rc = check_launch("mb_pa_kernel");
    if (!rc) mb->have_geometry = true;
    return rc;
}

extern "C" int vgb_multibeam_set_jones(vgb_multibeam *mb, const double *D, const double *Bj, const double *freqs,
                                       const uint32_t *polQ, const uint32_t *polP, void *stream)
{
    if (!mb || !D || !Bj || !freqs || !polQ || !polP)
        return set_error(VGB_ERR_INVALID, "multibeam_set_jones: NULL argument");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const vgb_multibeam_config &c = mb->cfg;
    const int A = c.nant, nf = c.nfine;
    int rc = VGB_SUCCESS;
    for (int cc = 0; cc < c.ncc && !rc; cc++) {
        const int npa = mb->Bp * A;
        // B^-1 and B B^H: the delays pass is skipped (unit == NULL)
        mb_pa_kernel<<<(npa + 255) / 256, 256, 0, st>>>(
            nullptr, nullptr, nullptr, nullptr, nullptr, 0.0,
            reinterpret_cast<const double2 *>(Bj) + 4ll * cc * c.npointing * A, c.npointing, mb->Bp, A, mb->d_dt,
            mb->d_Binv + 2ll * cc * npa, mb->d_H + (long long)cc * npa);
        if ((rc = check_launch("mb_pa_kernel"))) break;
        mb_ca_kernel<<<(nf * A + 255) / 256, 256, 0, st>>>(reinterpret_cast<const double2 *>(D) + 4ll * cc * A * nf,
                                                           A, nf, mb->d_Dinv + 2ll * cc * nf * A,
                                                           mb->d_G + (long long)cc * nf * A);
        rc = check_launch("mb_ca_kernel");
    }
    if (!rc)
        rc = check_cuda(cudaMemcpyAsync(mb->d_freq, freqs, sizeof(double) * c.ncc * nf, cudaMemcpyDeviceToDevice, st),
                        "cudaMemcpyAsync(freqs)");
    if (!rc)
        rc = check_cuda(cudaMemcpyAsync(mb->d_polQ, polQ, sizeof(uint32_t) * A, cudaMemcpyDeviceToDevice, st),
                        "cudaMemcpyAsync(polQ)");
    if (!rc)
        rc = check_cuda(cudaMemcpyAsync(mb->d_polP, polP, sizeof(uint32_t) * A, cudaMemcpyDeviceToDevice, st),
                        "cudaMemcpyAsync(polP)");
    if (!rc) mb->have_jones = true;
    return rc;
}

namespace {

// One coarse channel-second: weights, voltage conversion, autocorrelation
// GEMM, beam GEMM and (when out_cc is set) the 8-bit stage, on stream st.
int mb_run_cc(vgb_multibeam *mb, int cc, const uint8_t *v_cc, float *S_cc, uint8_t *out_cc, float *off_cc,
              float *scl_cc, cudaStream_t st, unsigned *status)
{
    NvtxRange range("vgb: multibeam coarse channel");
    const vgb_multibeam_config &c = mb->cfg;
    const int A = c.nant, nf = c.nfine, ns = c.nsamples;
    const long long nrow = (long long)nf * c.npointing * c.nstokes;
    const MbStats stats{mb->d_stats, mb->d_stats + nrow, mb->d_stats + 2 * nrow};
    int rc = VGB_SUCCESS;
    auto mark = [&](int cc_, int i) {
        if (mb->ev && !rc) rc = check_cuda(cudaEventRecord(mb->ev[6 * cc_ + i], st), "cudaEventRecord");
    };
    mb->last_launches += out_cc ? 5 : 4;
    mark(cc, 0);
    MbWeightArgs w{};
    w.dt = mb->d_dt;
    w.Binv = mb->d_Binv + 2ll * cc * mb->Bp * A;
    w.H = mb->d_H + (long long)cc * mb->Bp * A;
    w.Dinv = mb->d_Dinv + 2ll * cc * nf * A;
    w.G = mb->d_G + (long long)cc * nf * A;
    w.freq = mb->d_freq + (long long)cc * nf;
    w.A = A;
    w.Bp = mb->Bp;
    w.nfine = nf;
    w.nst = c.nstokes;
    w.planes = mb->planes;
    w.fp16 = mb->fp16;
    w.int8 = mb->int8;
    w.Mrows = mb->Mrows;
    w.Mq = mb->Mq;
    w.KA = mb->KA;
    w.Kq = mb->Kq;
    w.Aw = mb->d_Aw;
    w.Aq = mb->d_Aq;
    w.qscale = mb->d_qscale;
    w.W32 = mb->d_W32;
    w.Q32 = mb->d_Q32;
    w.stats = stats;
    w.B = c.npointing;
    if (A <= kMbPairMaxTiles && !mb->d_W32) {
        const int threads = std::max(32, (A / 2 + 31) / 32 * 32);
        mb_weights_pair_kernel<<<dim3((mb->Bp + kMbWeightBeams - 1) / kMbWeightBeams, nf), threads, 0, st>>>(w);
    } else {
        mb_weights_kernel<<<dim3(mb->Bp, nf), kMbWeightThreads, 0, st>>>(w);
    }
    if ((rc = check_launch("mb_weights_kernel"))) return rc;
    mark(cc, 1);

    MbConvArgs g{};
    g.v = v_cc;
    g.int8 = mb->int8;
    g.fp16 = mb->fp16;
    g.ns = ns;
    g.nfine = nf;
    g.ni = 2 * A;
    g.A = A;
    g.nint = mb->nint;
    g.nint_p = mb->nint_p;
    g.Kb = mb->Kb;
    g.polQ = mb->d_polQ;
    g.polP = mb->d_polP;
    g.status = status;
    g.V = mb->d_V;
    g.C = mb->d_C;
    const int conv_smem = kMbInt * 2 * A * (mb->int8 ? 2 : 1);
    if ((rc = check_cuda(cudaFuncSetAttribute(mb_convert_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              conv_smem),
                         "cudaFuncSetAttribute(mb_convert_kernel)")))
        return rc;
    mb_convert_kernel<<<dim3(nf, mb->nint), 128, conv_smem, st>>>(g);
    if ((rc = check_launch("mb_convert_kernel"))) return rc;
    mark(cc, 2);

    if (mb->simt) {
        MbSimtAutoArgs q{};
        q.Q = mb->d_Q32;
        q.C = mb->d_C;
        q.KA = mb->KA;
        q.Kb = mb->Kb;
        q.Mq = mb->Mq;
        q.nint = mb->nint;
        q.nint_p = mb->nint_p;
        q.int8 = mb->int8;
        q.R = mb->d_R;
        mb_simt_auto_kernel<<<dim3(mb->nint_p / 64, mb->Mq / 64, nf), 256, 0, st>>>(q);
        if ((rc = check_launch("mb_simt_auto_kernel"))) return rc;
        mark(cc, 3);
        MbSimtArgs b{};
        b.W = mb->d_W32;
        b.V = mb->d_V;
        b.R = mb->d_R;
        b.A = A;
        b.Bp = mb->Bp;
        b.B = c.npointing;
        b.ns = ns;
        b.nint = mb->nint;
        b.nint_p = mb->nint_p;
        b.Mq = mb->Mq;
        b.invw = c.invw;
        b.S = S_cc ? S_cc : mb->d_S;
        b.stats = stats;
        const dim3 grid((ns + kSimtSamp - 1) / kSimtSamp, mb->Bp / kSimtBeams, nf);
        const int smem = (2 * kSimtBeams + kSimtSamp) * kSimtRow * (int)sizeof(float2);
        auto kern = c.nstokes == 4 ? mb_simt_beam_kernel<4> : mb_simt_beam_kernel<1>;
        if ((rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                             "cudaFuncSetAttribute(mb_simt_beam_kernel)")))
            return rc;
        kern<<<grid, 256, smem, st>>>(b);
        if ((rc = check_launch("mb_simt_beam_kernel"))) return rc;
    } else {
    // autocorrelation terms R = Q C^T per channel (FP16 tensor path)
    // 4-bit split: R = Q_hi C + Q_lo C with C read once per K step (two A planes)
    if (!mb->int8 && mb->planes == 2 && mb->nint_p % 256 == 0)
        rc = gemm_batched_planes(mb->d_Aq, mb->d_C, mb->d_R, mb->Mq, mb->nint_p, mb->Kb, nf, true, st);
    else
        rc = gemm_batched(mb->d_Aq, mb->d_C, mb->d_R, mb->Mq, mb->nint_p, mb->Kq, nf, true, st, mb->Kb);
    if (rc) return rc;
    mark(cc, 3);

    MbBeamArgs b{};
    b.nfine = nf;
    b.ns = ns;
    b.nint = mb->nint;
    b.B = c.npointing;
    b.Mrows = mb->Mrows;
    b.mtiles = mb->mtiles;
    b.ntn = mb->ntn;
    b.nk = mb->nk;
    b.total = (long long)nf * mb->ntn * mb->mtiles;
    b.R = mb->d_R;
    b.qscale = mb->d_qscale;
    b.Mq = mb->Mq;
    b.nint_p = mb->nint_p;
    b.invw = c.invw;
    b.S = S_cc ? S_cc : mb->d_S;
    b.stats = stats;
    b.status = status;
    if (mb->planes == 2)
        rc = c.nstokes == 4 ? mb_launch_beam<2, false, 4>(mb, b, st) : mb_launch_beam<2, false, 1>(mb, b, st);
    else if (mb->fp16)
        rc = c.nstokes == 4 ? mb_launch_beam<1, true, 4>(mb, b, st) : mb_launch_beam<1, true, 1>(mb, b, st);
    else
        rc = c.nstokes == 4 ? mb_launch_beam<1, false, 4>(mb, b, st) : mb_launch_beam<1, false, 1>(mb, b, st);
    if (rc) return rc;
    }

    mark(cc, 4);
    if (out_cc) {
        MbRenormArgs r{};
        r.S = S_cc ? S_cc : mb->d_S;
        r.stats = stats;
        r.nfine = nf;
        r.B = c.npointing;
        r.nst = c.nstokes;
        r.nint = mb->nint;
        const long long out_st = nf, out_s = (long long)c.nstokes * nf, out_p = out_s * mb->nint;
        r.out = out_cc;
        r.out_p = out_p;
        r.out_s = out_s;
        r.out_st = out_st;
        r.offsets = off_cc;
        r.scales = scl_cc;
        mb_renorm_kernel<<<dim3((nf + 31) / 32, c.npointing * c.nstokes), 256, 0, st>>>(r);
        rc = check_launch("mb_renorm_kernel");
    }
    mark(cc, 5);
    return rc;
}

} // namespace

extern "C" int vgb_multibeam_run(vgb_multibeam *mb, const void *v, float *S, uint8_t *out, float *offsets,
                                 float *scales, void *stream)
{
    if (!mb || !v) return set_error(VGB_ERR_INVALID, "multibeam_run: NULL argument");
    if (reinterpret_cast<uintptr_t>(v) & 15) return set_error(VGB_ERR_INVALID, "multibeam_run: v must be 16-byte aligned");
    if (!mb->have_geometry || !mb->have_jones)
        return set_error(VGB_ERR_STATE, "multibeam_run: set_geometry and set_jones must come first");
    if (out && (!offsets || !scales))
        return set_error(VGB_ERR_INVALID, "multibeam_run: PSRFITS output needs offsets and scales");
    unsigned *status = status_word();
    if (!status) return set_error(VGB_ERR_CUDA, "device status word unavailable");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const vgb_multibeam_config &c = mb->cfg;
    const long long vbytes_cc = (long long)c.nsamples * c.nfine * 2 * c.nant * (mb->int8 ? 2 : 1);
    const long long s_cc = (long long)c.nfine * c.npointing * c.nstokes * mb->nint;
    const long long out_cc = (long long)c.npointing * mb->nint * c.nstokes * c.nfine;
    const long long stat_cc = (long long)c.npointing * c.nstokes * c.nfine;
    int rc = VGB_SUCCESS;
    mb->last_launches = 0;
    for (int cc = 0; cc < c.ncc && !rc; cc++)
        rc = mb_run_cc(mb, cc, static_cast<const uint8_t *>(v) + cc * vbytes_cc, S ? S + cc * s_cc : nullptr,
                       out ? out + cc * out_cc : nullptr, out ? offsets + cc * stat_cc : nullptr,
                       out ? scales + cc * stat_cc : nullptr, st, status);
    return rc;
}

extern "C" int vgb_multibeam_run_host(vgb_multibeam *mb, const void *v_host, uint8_t *out_host, float *off_host,
                                      float *scl_host, void *stream)
{
    if (!mb || !v_host || !out_host || !off_host || !scl_host)
        return set_error(VGB_ERR_INVALID, "multibeam_run_host: NULL argument");
    if (!mb->have_geometry || !mb->have_jones)
        return set_error(VGB_ERR_STATE, "multibeam_run_host: set_geometry and set_jones must come first");
    unsigned *status = status_word();
    if (!status) return set_error(VGB_ERR_CUDA, "device status word unavailable");
    const vgb_multibeam_config &c = mb->cfg;
    const size_t vbytes = (size_t)c.nsamples * c.nfine * 2 * c.nant * (mb->int8 ? 2 : 1);
    const size_t obytes = (size_t)c.npointing * mb->nint * c.nstokes * c.nfine;
    const size_t sbytes = (size_t)c.npointing * c.nstokes * c.nfine * sizeof(float);
    int rc = VGB_SUCCESS;
    if (!mb->s_h2d) {
        for (int b = 0; b < 2 && !rc; b++) {
            rc = mb_alloc(&mb->d_vin[b], vbytes, "streamed voltages");
            if (!rc) rc = mb_alloc(&mb->d_out[b], obytes, "streamed PSRFITS bytes");
            if (!rc) rc = mb_alloc(&mb->d_off[b], sbytes / sizeof(float), "streamed offsets");
            if (!rc) rc = mb_alloc(&mb->d_scl[b], sbytes / sizeof(float), "streamed scales");
            for (cudaEvent_t *e : {&mb->ev_h2d[b], &mb->ev_comp[b], &mb->ev_d2h[b]})
                if (!rc) rc = check_cuda(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "cudaEventCreate");
        }
        if (!rc) rc = check_cuda(cudaStreamCreateWithFlags(&mb->s_h2d, cudaStreamNonBlocking), "cudaStreamCreate");
        if (!rc) rc = check_cuda(cudaStreamCreateWithFlags(&mb->s_d2h, cudaStreamNonBlocking), "cudaStreamCreate");
        if (rc) return rc;
    }
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const uint8_t *vin = static_cast<const uint8_t *>(v_host);
    // the first two channels in as soon as each slot's last reader (the
    // previous call's compute on it) is done, so consecutive calls overlap;
    // on the first call the slot events have not been recorded and do not wait
    for (int cc = 0; cc < 2 && cc < c.ncc && !rc; cc++) {
        rc = check_cuda(cudaStreamWaitEvent(mb->s_h2d, mb->ev_comp[cc], 0), "cudaStreamWaitEvent");
        if (!rc)
            rc = check_cuda(cudaMemcpyAsync(mb->d_vin[cc], vin + cc * vbytes, vbytes, cudaMemcpyHostToDevice,
                                            mb->s_h2d),
                            "cudaMemcpyAsync(H2D)");
        if (!rc) rc = check_cuda(cudaEventRecord(mb->ev_h2d[cc], mb->s_h2d), "cudaEventRecord");
    }
    mb->last_launches = 0;
    for (int cc = 0; cc < c.ncc && !rc; cc++) {
        const int b = cc & 1;
        rc = check_cuda(cudaStreamWaitEvent(st, mb->ev_h2d[b], 0), "cudaStreamWaitEvent");
        if (!rc && cc >= 2) rc = check_cuda(cudaStreamWaitEvent(st, mb->ev_d2h[b], 0), "cudaStreamWaitEvent");
        if (!rc) rc = mb_run_cc(mb, cc, mb->d_vin[b], nullptr, mb->d_out[b], mb->d_off[b], mb->d_scl[b], st, status);
        if (!rc) rc = check_cuda(cudaEventRecord(mb->ev_comp[b], st), "cudaEventRecord");
        // products of this channel out ...
        if (!rc) rc = check_cuda(cudaStreamWaitEvent(mb->s_d2h, mb->ev_comp[b], 0), "cudaStreamWaitEvent");
        if (!rc)
            rc = check_cuda(cudaMemcpyAsync(out_host + cc * obytes, mb->d_out[b], obytes, cudaMemcpyDeviceToHost,
                                            mb->s_d2h),
                            "cudaMemcpyAsync(D2H)");
        if (!rc)
            rc = check_cuda(cudaMemcpyAsync(off_host + cc * (sbytes / sizeof(float)), mb->d_off[b], sbytes,
                                            cudaMemcpyDeviceToHost, mb->s_d2h),
                            "cudaMemcpyAsync(D2H)");
        if (!rc)
            rc = check_cuda(cudaMemcpyAsync(scl_host + cc * (sbytes / sizeof(float)), mb->d_scl[b], sbytes,
                                            cudaMemcpyDeviceToHost, mb->s_d2h),
                            "cudaMemcpyAsync(D2H)");
        if (!rc) rc = check_cuda(cudaEventRecord(mb->ev_d2h[b], mb->s_d2h), "cudaEventRecord");
        // ... and the channel after next in, once this slot's voltages are consumed
        if (!rc && cc + 2 < c.ncc) {
            rc = check_cuda(cudaStreamWaitEvent(mb->s_h2d, mb->ev_comp[b], 0), "cudaStreamWaitEvent");
            if (!rc)
                rc = check_cuda(cudaMemcpyAsync(mb->d_vin[b], vin + (cc + 2) * vbytes, vbytes, cudaMemcpyHostToDevice,
                                                mb->s_h2d),
                                "cudaMemcpyAsync(H2D)");
            if (!rc) rc = check_cuda(cudaEventRecord(mb->ev_h2d[b], mb->s_h2d), "cudaEventRecord");
        }
    }
    // the caller's stream completes only after every product has landed on the host
    for (int b = 0; b < 2 && b < c.ncc && !rc; b++)
        rc = check_cuda(cudaStreamWaitEvent(st, mb->ev_d2h[b], 0), "cudaStreamWaitEvent");
    return rc;
}

extern "C" int vgb_multibeam_enable_timing(vgb_multibeam *mb, int on)
{
    if (!mb) return set_error(VGB_ERR_INVALID, "multibeam_enable_timing: NULL handle");
    if (on && !mb->ev) {
        mb->ev = new cudaEvent_t[6 * mb->cfg.ncc]();
        for (int i = 0; i < 6 * mb->cfg.ncc; i++)
            if (cudaEventCreate(&mb->ev[i]) != cudaSuccess) {
                cudaGetLastError();
                return set_error(VGB_ERR_CUDA, "multibeam_enable_timing: cudaEventCreate failed");
            }
    } else if (!on && mb->ev) {
        for (int i = 0; i < 6 * mb->cfg.ncc; i++)
            if (mb->ev[i]) cudaEventDestroy(mb->ev[i]);
        delete[] mb->ev;
        mb->ev = nullptr;
    }
    return VGB_SUCCESS;
}

extern "C" int vgb_multibeam_stage_ms(vgb_multibeam *mb, float *ms, int n)
{
    if (!mb || !ms || n < 5) return set_error(VGB_ERR_INVALID, "multibeam_stage_ms: need 5 slots");
    if (!mb->ev) return set_error(VGB_ERR_STATE, "multibeam_stage_ms: timing is off");
    for (int i = 0; i < 5; i++) ms[i] = 0.f;
    for (int cc = 0; cc < mb->cfg.ncc; cc++) {
        int rc = check_cuda(cudaEventSynchronize(mb->ev[6 * cc + 5]), "cudaEventSynchronize");
        if (rc) return rc;
        for (int i = 0; i < 5; i++) {
            float t = 0.f;
            if ((rc = check_cuda(cudaEventElapsedTime(&t, mb->ev[6 * cc + i], mb->ev[6 * cc + i + 1]),
                                 "cudaEventElapsedTime")))
                return rc;
            ms[i] += t;
        }
    }
    return VGB_SUCCESS;
}

extern "C" int vgb_multibeam_launches(const vgb_multibeam *mb)
{
    // per coarse channel: weights, convert, R GEMM, beam GEMM (+ renormalise)
    return mb ? mb->last_launches : 0;
}

extern "C" int vgb_multibeam_beam_variant(int v)
{
    if (v < 0 || v > 2) return set_error(VGB_ERR_INVALID, "multibeam_beam_variant: 0, 1 or 2"), -1;
    return g_mb_beam_variant.exchange(v);
}

extern "C" int vgb_multibeam_last_pair(const vgb_multibeam *mb) { return mb ? mb->last_pair : 0; }
