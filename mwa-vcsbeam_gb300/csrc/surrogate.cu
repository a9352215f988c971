// Learned primary-beam surrogate: an MLP that maps (az, za, frequency,
// delay set) to the tile Jones matrix, standing in for the beam-model
// evaluation of vmCalcB (primary_beam.c:79-191) when thousands of beams are
// re-pointed every second.
//
// Network: 6 inputs (sin az, cos az, za, frequency, a 2-d learned embedding of
// the delay set) -> 4 hidden layers of 256 (GELU) -> 8 outputs (re, im of the
// 2x2 Jones matrix). Weights are BF16 (FP32 master copies for Adam), every
// product accumulates in FP32 on the tcgen05 tensor cores (gemm_batched).
// Activations and gradients travel as BF16 hi + lo halves, concatenated along
// K so that one GEMM forms hi*W + lo*W (weights read modulo their K width),
// and for the weight gradients [dP_hi | dP_hi | dP_lo] x [X_hi | X_lo]
// (error ~2^-16 instead of BF16's 2^-8). Weight gradients are split over
// batch slices (one GEMM batch per 512 samples) and summed by the Adam kernel.
//
// Training data come from the plain model (beam_model.cuh) on the device.
// After training a validation map records, per delay set and sky cell (32
// azimuth x 16 zenith-angle bins), the largest Jones error seen; inference
// answers a query from the network only where that error is within the
// tolerance and otherwise evaluates the plain model (the fallback).
#include <cuda_bf16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "beam_model.cuh"
#include "vgb_launch.cuh"

namespace vgb {

constexpr int kSurH = 256;       // hidden width
constexpr int kSurK0 = 64;       // input features padded to one K chunk
constexpr int kSurOut = 128;     // 8 outputs padded to a GEMM tile
constexpr int kSurSlice = 512;   // samples per weight-gradient GEMM batch
constexpr int kSurNaz = 32, kSurNza = 16;
constexpr double kSurZaMax = 80.0 * kBmPi / 180.0;

// parameter vector layout (FP32 masters, Adam moments and gradients share it)
struct SurLayout {
    int nsets;
    long long W0, W1, W2, W3, W4, b0, b4, emb, total; // b1..b3 follow b0
    SurLayout(int ns = 0) : nsets(ns)
    {
        W0 = 0;                        // [256][6]
        W1 = W0 + kSurH * 6;           // [256][256]
        W2 = W1 + kSurH * kSurH;
        W3 = W2 + kSurH * kSurH;
        W4 = W3 + kSurH * kSurH;       // [8][256]
        b0 = W4 + 8 * kSurH;           // [4][256]
        b4 = b0 + 4 * kSurH;           // [8]
        emb = b4 + 8;                  // [nsets][2]
        total = emb + 2 * (long long)nsets;
    }
};

__device__ __forceinline__ uint64_t sur_hash(uint64_t x)
{
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
__device__ __forceinline__ double sur_unit(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

__device__ __forceinline__ uint16_t bfbits(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }
__device__ __forceinline__ float bfval(uint16_t b) { return __bfloat162float(__ushort_as_bfloat16(b)); }
__device__ __forceinline__ void split_store(uint16_t *hi, uint16_t *lo, float x)
{
    const uint16_t h = bfbits(x);
    *hi = h;
    *lo = bfbits(x - bfval(h));
}

__device__ __forceinline__ float gelu(float x) { return 0.5f * x * (1.f + erff(x * 0.70710678118654752f)); }
__device__ __forceinline__ float gelu_grad(float x)
{
    return 0.5f * (1.f + erff(x * 0.70710678118654752f)) + x * 0.3989422804014327f * expf(-0.5f * x * x);
}

// features of one query: sin az, cos az, za scaled to [-1, 1) over 0..80 deg,
// frequency scaled to [-1, 1] over 80..300 MHz, embedding of the delay set
__device__ __forceinline__ void sur_features(double az, double za, double f, const float *emb, float (&x)[6])
{
    x[0] = (float)sin(az);
    x[1] = (float)cos(az);
    x[2] = (float)(za / (0.5 * kSurZaMax) - 1.0);
    x[3] = (float)((f - 190e6) / 110e6);
    x[4] = emb[0];
    x[5] = emb[1];
}

__device__ __forceinline__ int sur_cell(double az, double za)
{
    double a = az * (0.5 / kBmPi);
    a -= floor(a);
    int ia = (int)(a * kSurNaz);
    int iz = (int)(za / kSurZaMax * kSurNza);
    ia = ia < 0 ? 0 : ia >= kSurNaz ? kSurNaz - 1 : ia;
    iz = iz < 0 ? 0 : iz >= kSurNza ? kSurNza - 1 : iz;
    return ia * kSurNza + iz;
}

// ---------------------------------------------------------------------------
// training data
// ---------------------------------------------------------------------------
__global__ void sur_dirs_kernel(int ndir, uint64_t seed, double *az, double *za)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ndir) return;
    // uniform on the sky above 10 degrees elevation
    const double u = sur_unit(sur_hash(seed * 0x100000001ull + 2 * (uint64_t)i));
    const double v = sur_unit(sur_hash(seed * 0x100000001ull + 2 * (uint64_t)i + 1));
    const double cmin = cos(kSurZaMax);
    za[i] = acos(cmin + (1.0 - cmin) * u);
    az[i] = 2.0 * kBmPi * v;
}

// plain-model Jones [nfreq][ndir][4] complex -> FP32 targets [set][nfreq][ndir][8]
__global__ void sur_targets_kernel(const double *az, const double *za, int ndir, const double *freq, int nfreq,
                                   const uint32_t *delays, float *Y)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= (long long)nfreq * ndir) return;
    const int d = i % ndir, fi = i / ndir;
    double2 J[4];
    bm_jones(az[d], za[d], freq[fi], delays, J);
    float *o = Y + 8 * i;
    for (int e = 0; e < 4; e++) {
        o[2 * e] = (float)J[e].x;
        o[2 * e + 1] = (float)J[e].y;
    }
}

struct SurBatch {
    // one of: sampled from the training table, or given features
    const double *az, *za, *freq;  // table directions / frequencies
    int ndir, nfreq, nsets;
    const float *Y;                // [set][freq][dir][8]
    uint64_t seed;
    const uint64_t *seed_dev;      // training: seed of step kdev[0] (graph replay), or NULL
    const int *kdev;
    const float *feat_in;          // [B][4] given raw features (sin, cos, za, f scaled) or NULL
    const int *set_in;             // [B]
    const float *y_in;             // [B][8]
    const float *params;
    SurLayout L;
    int B;
    uint16_t *X0;                  // [B][128]
    int *set_of;                   // [B]
    float *y;                      // [B][8]
};

__global__ void sur_batch_kernel(const SurBatch a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.B) return;
    float x[6];
    int s;
    if (a.feat_in) {
        s = a.set_in[i];
        for (int k = 0; k < 4; k++) x[k] = a.feat_in[4 * i + k];
        x[4] = a.params[a.L.emb + 2 * s];
        x[5] = a.params[a.L.emb + 2 * s + 1];
        for (int k = 0; k < 8; k++) a.y[8 * i + k] = a.y_in[8 * i + k];
    } else {
        const long long n = (long long)a.nsets * a.nfreq * a.ndir;
        const uint64_t seed = a.seed_dev ? a.seed_dev[*a.kdev] : a.seed;
        const long long idx = (long long)(sur_hash(seed * 0x9E3779B1ull + i) % (uint64_t)n);
        const int d = idx % a.ndir, fi = (idx / a.ndir) % a.nfreq;
        s = idx / ((long long)a.ndir * a.nfreq);
        sur_features(a.az[d], a.za[d], a.freq[fi], a.params + a.L.emb + 2 * s, x);
        for (int k = 0; k < 8; k++) a.y[8 * i + k] = a.Y[8 * idx + k];
    }
    a.set_of[i] = s;
    uint16_t *row = a.X0 + (long long)i * 2 * kSurK0;
    for (int k = 0; k < kSurK0; k++) {
        const float v = k < 6 ? x[k] : 0.f;
        split_store(row + k, row + kSurK0 + k, v);
    }
}

// pre = C + b; H = GELU(pre) as hi | lo. One thread per column, 32 rows per block.
__global__ void sur_act_kernel(const float *C, const float *b, int B, float *pre, uint16_t *H)
{
    const int c = threadIdx.x, r0 = blockIdx.x * 32;
    for (int r = r0; r < r0 + 32 && r < B; r++) {
        const float p = C[(long long)r * kSurH + c] + b[c];
        pre[(long long)r * kSurH + c] = p;
        uint16_t *row = H + (long long)r * 2 * kSurH;
        split_store(row + c, row + kSurH + c, gelu(p));
    }
}

// outputs, loss and dL/dout = 2 (pred - y) / (8 B) as hi | lo (128 columns each)
__global__ void sur_out_kernel(const float *C4, const float *b4, const float *y, int B, float *pred, uint16_t *dY,
                               float *loss, float *db4, const int *kslot = nullptr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.f;
    if (i < B) {
        uint16_t *row = dY + (long long)i * 2 * kSurOut;
        for (int k = 0; k < kSurOut; k++) {
            float g = 0.f;
            if (k < 8) {
                const float p = C4[(long long)i * kSurOut + k] + b4[k];
                if (pred) pred[8 * i + k] = p;
                const float d = p - (y ? y[8 * i + k] : 0.f);
                l += d * d;
                g = 2.f * d / (8.f * B);
                if (db4) atomicAdd(&db4[k], g);
            }
            split_store(row + k, row + kSurOut + k, g);
        }
    }
    if (loss) {
        for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
        if ((threadIdx.x & 31) == 0) atomicAdd(kslot ? loss + *kslot : loss, l / (8.f * B));
    }
}

// dP = dH * GELU'(pre) as hi | lo, and the column sums into db
__global__ void sur_gbwd_kernel(const float *dH, const float *pre, int B, uint16_t *dP, float *db)
{
    const int c = threadIdx.x, r0 = blockIdx.x * 32;
    float acc = 0.f;
    for (int r = r0; r < r0 + 32 && r < B; r++) {
        const float g = dH[(long long)r * kSurH + c] * gelu_grad(pre[(long long)r * kSurH + c]);
        acc += g;
        uint16_t *row = dP + (long long)r * 2 * kSurH;
        split_store(row + c, row + kSurH + c, g);
    }
    atomicAdd(&db[c], acc);
}

// in [B][2K] (hi | lo) -> out [B/S][Kout][parts*S]: parts 2 = (hi, lo),
// parts 3 = (hi, hi, lo). Rows K .. Kout-1 of each slice are left alone.
__global__ void sur_transpose_kernel(const uint16_t *in, int B, int K, int Kout, int parts, uint16_t *out)
{
    __shared__ uint16_t t[32][33];
    const int k0 = blockIdx.x * 32, b0 = blockIdx.y * 32, part = blockIdx.z;
    const int src = (parts == 3 && part < 2) ? 0 : (parts == 3 ? 1 : part);
    for (int r = threadIdx.y; r < 32; r += 8) t[r][threadIdx.x] = in[(long long)(b0 + r) * 2 * K + src * K + k0 + threadIdx.x];
    __syncthreads();
    for (int r = threadIdx.y; r < 32; r += 8) {
        const int k = k0 + r, b = b0 + threadIdx.x;
        const int sl = b / kSurSlice, bs = b % kSurSlice;
        out[((long long)sl * Kout + k) * parts * kSurSlice + part * kSurSlice + bs] = t[threadIdx.x][r];
    }
}

__global__ void sur_emb_grad_kernel(const float *dX0, const int *set_of, int B, float *demb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B) return;
    atomicAdd(&demb[2 * set_of[i]], dX0[(long long)i * 128 + 4]);
    atomicAdd(&demb[2 * set_of[i] + 1], dX0[(long long)i * 128 + 5]);
}

struct SurAdamArgs {
    SurLayout L;
    float *p, *m, *v, *grad_out;      // grad_out (nullable): the summed gradient
    const float *dW0, *dW1, *dW2, *dW3, *dW4; // slice partials
    float *db, *demb;
    int nslice;
    float lr, b1, b2, eps, bc1, bc2;
    const float *sched;   // training: [step][3] (lr, bc1, bc2) of step kdev[0] (graph replay), or NULL
    const int *kdev;
    int update;
    uint16_t *W0p, *W1, *W2, *W3, *W4p, *W0t, *W1t, *W2t, *W3t, *W4t;
};

// Sum the gradient of one parameter, Adam-update it (when asked) and refresh
// its BF16 copies (and transposed copies) for the next step.
__global__ void sur_adam_kernel(const SurAdamArgs a)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= a.L.total) return;
    float g = 0.f;
    int kind = -1, r = 0, c = 0;
    if (i < a.L.W1) { // W0 [256][6]; partials [slice][256][128]
        kind = 0; r = (i - a.L.W0) / 6; c = (i - a.L.W0) % 6;
        for (int s = 0; s < a.nslice; s++) g += a.dW0[((long long)s * kSurH + r) * 128 + c];
    } else if (i < a.L.W4) { // W1..W3 [256][256]; partials [slice][256][256]
        kind = 1 + (int)((i - a.L.W1) / (kSurH * kSurH));
        const long long j = (i - a.L.W1) % (kSurH * kSurH);
        r = j / kSurH; c = j % kSurH;
        const float *d = kind == 1 ? a.dW1 : kind == 2 ? a.dW2 : a.dW3;
        for (int s = 0; s < a.nslice; s++) g += d[(long long)s * kSurH * kSurH + j];
    } else if (i < a.L.b0) { // W4 [8][256]; partials [slice][128][256]
        kind = 4; r = (i - a.L.W4) / kSurH; c = (i - a.L.W4) % kSurH;
        for (int s = 0; s < a.nslice; s++) g += a.dW4[((long long)s * kSurOut + r) * kSurH + c];
    } else if (i < a.L.emb) { // biases
        g = a.db[i - a.L.b0];
        a.db[i - a.L.b0] = 0.f;
    } else {
        g = a.demb[i - a.L.emb];
        a.demb[i - a.L.emb] = 0.f;
    }
    if (a.grad_out) a.grad_out[i] = g;
    float p = a.p[i];
    if (a.update) {
        float lr = a.lr, bc1 = a.bc1, bc2 = a.bc2;
        if (a.sched) {
            const float *sc = a.sched + 3 * (*a.kdev);
            lr = sc[0];
            bc1 = sc[1];
            bc2 = sc[2];
        }
        const float m = a.b1 * a.m[i] + (1.f - a.b1) * g;
        const float v = a.b2 * a.v[i] + (1.f - a.b2) * g * g;
        a.m[i] = m;
        a.v[i] = v;
        p -= lr * (m / bc1) / (sqrtf(v / bc2) + a.eps);
        a.p[i] = p;
    }
    const uint16_t w = bfbits(p);
    switch (kind) {
    case 0: a.W0p[r * kSurK0 + c] = w; a.W0t[c * kSurH + r] = w; break;
    case 1: a.W1[r * kSurH + c] = w; a.W1t[c * kSurH + r] = w; break;
    case 2: a.W2[r * kSurH + c] = w; a.W2t[c * kSurH + r] = w; break;
    case 3: a.W3[r * kSurH + c] = w; a.W3t[c * kSurH + r] = w; break;
    case 4: a.W4p[r * kSurH + c] = w; a.W4t[c * kSurOut + r] = w; break;
    default: break;
    }
}

// The training step index of a graph-replayed step, advanced once per step.
__global__ void sur_next_step_kernel(int *kdev) { *kdev += 1; }

// ---------------------------------------------------------------------------
// validation and inference
// ---------------------------------------------------------------------------
struct SurQueryArgs {
    const double *az, *za, *freq;
    int npointing, nfreq, nsets;
    const float *params;
    SurLayout L;
    long long row0, nrows;
    int B;
    uint16_t *X0;
    // validation: random queries, plain-model targets
    int validate;
    const uint32_t *delays; // [nsets][16]
    uint64_t seed;
    float *y;               // [B][8]
    int *cell_of;           // [B] set * cells + cell
    const int *set_list;    // queries: the delay sets evaluated (nsets of them), in row order
};

__global__ void sur_query_kernel(const SurQueryArgs a)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.B) return;
    const long long q = a.row0 + i;
    float x[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (q < a.nrows) {
        double az, za, f;
        int s;
        if (a.validate) {
            const uint64_t h = sur_hash(a.seed * 0x51ED27ull + (uint64_t)q);
            s = (int)(q % a.nsets);
            const double cmin = cos(kSurZaMax);
            za = acos(cmin + (1.0 - cmin) * sur_unit(sur_hash(h + 1)));
            az = 2.0 * kBmPi * sur_unit(sur_hash(h + 2));
            f = a.freq[sur_hash(h + 3) % (uint64_t)a.nfreq]; // the trained frequencies
            double2 J[4];
            bm_jones(az, za, f, a.delays + 16 * s, J);
            for (int e = 0; e < 4; e++) {
                a.y[8 * i + 2 * e] = (float)J[e].x;
                a.y[8 * i + 2 * e + 1] = (float)J[e].y;
            }
            a.cell_of[i] = s * kSurNaz * kSurNza + sur_cell(az, za);
        } else {
            s = a.set_list[q % a.nsets];
            const int p = (int)((q / a.nsets) % a.npointing);
            const int fi = (int)(q / ((long long)a.nsets * a.npointing));
            az = a.az[p];
            za = a.za[p];
            f = a.freq[fi];
        }
        sur_features(az, za, f, a.params + a.L.emb + 2 * s, x);
    } else if (a.validate) {
        a.cell_of[i] = -1;
    }
    uint16_t *row = a.X0 + (long long)i * 2 * kSurK0;
    for (int k = 0; k < kSurK0; k++) split_store(row + k, row + kSurK0 + k, k < 6 ? x[k] : 0.f);
}

__global__ void sur_val_err_kernel(const float *pred, const float *y, const int *cell_of, int B, unsigned *cell_err,
                                   unsigned *max_err)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= B || cell_of[i] < 0) return;
    float e = 0.f;
    for (int k = 0; k < 8; k++) e = fmaxf(e, fabsf(pred[8 * i + k] - y[8 * i + k]));
    atomicMax(&cell_err[cell_of[i]], __float_as_uint(e));
    atomicMax(max_err, __float_as_uint(e));
}

struct SurExpandArgs {
    const double *az, *za, *freq;
    int npointing, nfreq, nsets, ntile;
    const int *tile_set;      // [ntile] delay-set index, < 0: not covered
    const uint32_t *delays;   // [ntile][16]
    const float *Jsur;        // [nfreq][npointing][nslots][8]
    double2 *Bsur;            // [nfreq][npointing][nslots][4]: Jsur (x P)
    const int *slot_of;       // [nsets] row slot of each evaluated set, -1 if not evaluated
    int nslots;
    const unsigned *cell_err; // [nsets][cells]
    float tol;
    double lat;
    int pa;
    double2 *B;
    unsigned *nfallback;
};

// The network's Jones matrices per (frequency, pointing, evaluated set) in
// FP64, times the parallactic rotation when asked: B rows shared by every
// tile of the set (one rotation per pointing and set, not per tile).
__global__ void sur_rotate_kernel(const SurExpandArgs a, long long rows)
{
    const long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const int p = (int)((r / a.nslots) % a.npointing);
    const float *o = a.Jsur + 8 * r;
    double2 J[4];
    for (int e = 0; e < 4; e++) J[e] = make_double2(o[2 * e], o[2 * e + 1]);
    double2 *out = a.Bsur + 4 * r;
    if (!a.pa) {
        for (int e = 0; e < 4; e++) out[e] = J[e];
        return;
    }
    double P[4];
    bm_pa(a.lat, a.az[p], a.za[p], P);
    out[0] = make_double2(J[0].x * P[0] + J[1].x * P[2], J[0].y * P[0] + J[1].y * P[2]);
    out[1] = make_double2(J[0].x * P[1] + J[1].x * P[3], J[0].y * P[1] + J[1].y * P[3]);
    out[2] = make_double2(J[2].x * P[0] + J[3].x * P[2], J[2].y * P[0] + J[3].y * P[2]);
    out[3] = make_double2(J[2].x * P[1] + J[3].x * P[3], J[2].y * P[1] + J[3].y * P[3]);
}

// Per (frequency, pointing, tile): the network's B where its sky cell is
// within tolerance and the tile's set was trained; else the plain model's B,
// already in place (counted as fallback).
__global__ void sur_expand_kernel(const SurExpandArgs a)
{
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= (long long)a.nfreq * a.npointing * a.ntile) return;
    const int t = idx % a.ntile, p = (idx / a.ntile) % a.npointing, fi = idx / ((long long)a.ntile * a.npointing);
    const double az = a.az[p], za = a.za[p];
    const int s = a.tile_set[t];
    const int slot = s >= 0 && s < a.nsets ? a.slot_of[s] : -1;
    const bool use = slot >= 0 && za <= kSurZaMax &&
                     __uint_as_float(a.cell_err[s * kSurNaz * kSurNza + sur_cell(az, za)]) <= a.tol;
    if (!use) {
        atomicAdd(a.nfallback, 1u);
        return;
    }
    const uint4 *src = reinterpret_cast<const uint4 *>(a.Bsur + 4 * (((long long)fi * a.npointing + p) * a.nslots + slot));
    uint4 *dst = reinterpret_cast<uint4 *>(a.B + 4 * idx);
    dst[0] = src[0];
    dst[1] = src[1];
    dst[2] = src[2];
    dst[3] = src[3];
}

} // namespace vgb

using namespace vgb;

struct vgb_surrogate {
    int nsets = 0, B = 0, nslice = 0;
    SurLayout L;
    cudaStream_t st = nullptr;
    std::vector<void *> allocs;
    float *p = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr;
    uint16_t *W0p, *W1, *W2, *W3, *W4p, *W0t, *W1t, *W2t, *W3t, *W4t;
    uint16_t *X0, *H[5], *dY, *dP[4], *TA, *TB, *X0t;
    float *pre[4], *C, *C4, *dH, *dX0, *dW[5], *db, *demb, *y, *pred, *loss;
    int *set_of, *cell_of;
    // training table
    double *tab_az = nullptr, *tab_za = nullptr, *tab_f = nullptr;
    float *tab_Y = nullptr;
    uint32_t *tab_delays = nullptr;
    int ndir = 0, nfreq = 0;
    unsigned *cell_err = nullptr, *max_err = nullptr, *nfallback = nullptr;
    float tol = 1e-3f;
    bool validated = false;
    std::vector<int> cells_ok;           // per delay set: sky cells within the tolerance (host copy)
    long long step = 0;
    float *Jsur = nullptr;
    double2 *Bsur = nullptr;
    // training schedule for graph replay: [step][3] (lr, bc1, bc2), [step] seeds,
    // per-step losses, and the device step index
    float *sched = nullptr, *loss_dev = nullptr;
    uint64_t *seed_dev = nullptr;
    int *kdev = nullptr;
    long long sched_cap = 0;
    long long Jsur_cap = 0;
    int *set_map = nullptr; // queries: [nsets] evaluated sets in row order, then [nsets] slot of each set
};

namespace {

template <typename T> T *sur_alloc(vgb_surrogate *s, size_t n, int &rc)
{
    if (rc) return nullptr;
    void *p = nullptr;
    if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        rc = set_error(VGB_ERR_ALLOC, "surrogate: cannot allocate %zu bytes", n * sizeof(T));
        return nullptr;
    }
    s->allocs.push_back(p);
    if (cudaMemset(p, 0, n * sizeof(T)) != cudaSuccess) rc = set_error(VGB_ERR_CUDA, "surrogate: cudaMemset failed");
    return static_cast<T *>(p);
}

// forward through the five GEMMs; out: C4 [B][128] (pre-bias outputs)
int sur_forward(vgb_surrogate *s)
{
    const int B = s->B;
    int rc = gemm_batched(s->X0, s->W0p, s->C, B, kSurH, 2 * kSurK0, 1, false, s->st, kSurK0);
    if (rc) return rc;
    for (int l = 0; l < 4; l++) {
        if (l > 0) {
            const uint16_t *Wl = l == 1 ? s->W1 : l == 2 ? s->W2 : s->W3;
            if ((rc = gemm_batched(s->H[l], Wl, s->C, B, kSurH, 2 * kSurH, 1, false, s->st, kSurH))) return rc;
        }
        sur_act_kernel<<<(B + 31) / 32, kSurH, 0, s->st>>>(s->C, s->p + s->L.b0 + l * kSurH, B, s->pre[l],
                                                           s->H[l + 1]);
        if ((rc = check_launch("sur_act_kernel"))) return rc;
    }
    return gemm_batched(s->H[4], s->W4p, s->C4, B, kSurOut, 2 * kSurH, 1, false, s->st, kSurH);
}

int sur_transpose(vgb_surrogate *s, const uint16_t *in, int K, int parts, uint16_t *out, int Kout = 0)
{
    sur_transpose_kernel<<<dim3(K / 32, s->B / 32, parts), dim3(32, 8), 0, s->st>>>(in, s->B, K, Kout ? Kout : K,
                                                                                    parts, out);
    return check_launch("sur_transpose_kernel");
}

// backward after sur_out_kernel wrote dY; fills the gradient partials
int sur_backward(vgb_surrogate *s)
{
    const int B = s->B, ns = s->nslice, S = kSurSlice;
    int rc;
    // output layer
    if ((rc = sur_transpose(s, s->dY, kSurOut, 3, s->TA))) return rc;
    if ((rc = sur_transpose(s, s->H[4], kSurH, 2, s->TB))) return rc;
    if ((rc = gemm_batched(s->TA, s->TB, s->dW[4], kSurOut, kSurH, 3 * S, ns, false, s->st, 2 * S))) return rc;
    if ((rc = gemm_batched(s->dY, s->W4t, s->dH, B, kSurH, 2 * kSurOut, 1, false, s->st, kSurOut))) return rc;
    for (int l = 3; l >= 0; l--) {
        sur_gbwd_kernel<<<(B + 31) / 32, kSurH, 0, s->st>>>(s->dH, s->pre[l], B, s->dP[l], s->db + l * kSurH);
        if ((rc = check_launch("sur_gbwd_kernel"))) return rc;
        if ((rc = sur_transpose(s, s->dP[l], kSurH, 3, s->TA))) return rc;
        if (l > 0) {
            if ((rc = sur_transpose(s, s->H[l], kSurH, 2, s->TB))) return rc;
            if ((rc = gemm_batched(s->TA, s->TB, s->dW[l], kSurH, kSurH, 3 * S, ns, false, s->st, 2 * S))) return rc;
            const uint16_t *Wt = l == 1 ? s->W1t : l == 2 ? s->W2t : s->W3t;
            if ((rc = gemm_batched(s->dP[l], Wt, s->dH, B, kSurH, 2 * kSurH, 1, false, s->st, kSurH))) return rc;
        } else {
            if ((rc = sur_transpose(s, s->X0, kSurK0, 2, s->X0t, 128))) return rc;
            if ((rc = gemm_batched(s->TA, s->X0t, s->dW[0], kSurH, 128, 3 * S, ns, false, s->st, 2 * S))) return rc;
            if ((rc = gemm_batched(s->dP[0], s->W0t, s->dX0, B, 128, 2 * kSurH, 1, false, s->st, kSurH))) return rc;
            sur_emb_grad_kernel<<<(B + 255) / 256, 256, 0, s->st>>>(s->dX0, s->set_of, B, s->demb);
            if ((rc = check_launch("sur_emb_grad_kernel"))) return rc;
        }
    }
    return VGB_SUCCESS;
}

int sur_adam(vgb_surrogate *s, int update, float lr, float *grad_out, bool scheduled = false)
{
    SurAdamArgs a{};
    if (scheduled) {
        a.sched = s->sched;
        a.kdev = s->kdev;
    }
    a.L = s->L;
    a.p = s->p;
    a.m = s->m;
    a.v = s->v;
    a.grad_out = grad_out;
    a.dW0 = s->dW[0];
    a.dW1 = s->dW[1];
    a.dW2 = s->dW[2];
    a.dW3 = s->dW[3];
    a.dW4 = s->dW[4];
    a.db = s->db;
    a.demb = s->demb;
    a.nslice = s->nslice;
    a.lr = lr;
    a.b1 = 0.9f;
    a.b2 = 0.999f;
    a.eps = 1e-8f;
    const double t = (double)(s->step + 1);
    a.bc1 = (float)(1.0 - pow(0.9, t));
    a.bc2 = (float)(1.0 - pow(0.999, t));
    a.update = update;
    a.W0p = s->W0p; a.W1 = s->W1; a.W2 = s->W2; a.W3 = s->W3; a.W4p = s->W4p;
    a.W0t = s->W0t; a.W1t = s->W1t; a.W2t = s->W2t; a.W3t = s->W3t; a.W4t = s->W4t;
    sur_adam_kernel<<<(unsigned)((s->L.total + 255) / 256), 256, 0, s->st>>>(a);
    return check_launch("sur_adam_kernel");
}

} // namespace

extern "C" int vgb_surrogate_create(int nsets, int batch, unsigned long long seed, vgb_surrogate **out)
{
    if (!out) return set_error(VGB_ERR_INVALID, "surrogate_create: NULL handle");
    *out = nullptr;
    if (nsets <= 0 || nsets > 4096) return set_error(VGB_ERR_INVALID, "surrogate_create: nsets must be 1..4096");
    if (batch <= 0 || batch % kSurSlice)
        return set_error(VGB_ERR_INVALID, "surrogate_create: batch must be a positive multiple of %d", kSurSlice);
    vgb_surrogate *s = new vgb_surrogate();
    s->nsets = nsets;
    s->B = batch;
    s->nslice = batch / kSurSlice;
    s->L = SurLayout(nsets);
    int rc = VGB_SUCCESS;
    const size_t B = batch, P = s->L.total;
    s->p = sur_alloc<float>(s, P, rc);
    s->m = sur_alloc<float>(s, P, rc);
    s->v = sur_alloc<float>(s, P, rc);
    s->grad = sur_alloc<float>(s, P, rc);
    s->W0p = sur_alloc<uint16_t>(s, kSurH * kSurK0, rc);
    s->W1 = sur_alloc<uint16_t>(s, kSurH * kSurH, rc);
    s->W2 = sur_alloc<uint16_t>(s, kSurH * kSurH, rc);
    s->W3 = sur_alloc<uint16_t>(s, kSurH * kSurH, rc);
    s->W4p = sur_alloc<uint16_t>(s, kSurOut * kSurH, rc);
    s->W0t = sur_alloc<uint16_t>(s, 128 * kSurH, rc);
    s->W1t = sur_alloc<uint16_t>(s, kSurH * kSurH, rc);
    s->W2t = sur_alloc<uint16_t>(s, kSurH * kSurH, rc);
    s->W3t = sur_alloc<uint16_t>(s, kSurH * kSurH, rc);
    s->W4t = sur_alloc<uint16_t>(s, kSurH * kSurOut, rc);
    s->X0 = sur_alloc<uint16_t>(s, B * 2 * kSurK0, rc);
    s->H[0] = nullptr;
    for (int l = 1; l <= 4; l++) s->H[l] = sur_alloc<uint16_t>(s, B * 2 * kSurH, rc);
    s->dY = sur_alloc<uint16_t>(s, B * 2 * kSurOut, rc);
    for (int l = 0; l < 4; l++) s->dP[l] = sur_alloc<uint16_t>(s, B * 2 * kSurH, rc);
    s->TA = sur_alloc<uint16_t>(s, B * 3 * kSurH, rc);
    s->TB = sur_alloc<uint16_t>(s, B * 2 * kSurH, rc);
    s->X0t = sur_alloc<uint16_t>(s, B * 2 * 128, rc); // rows 64..127 stay zero
    for (int l = 0; l < 4; l++) s->pre[l] = sur_alloc<float>(s, B * kSurH, rc);
    s->C = sur_alloc<float>(s, B * kSurH, rc);
    s->C4 = sur_alloc<float>(s, B * kSurOut, rc);
    s->dH = sur_alloc<float>(s, B * kSurH, rc);
    s->dX0 = sur_alloc<float>(s, B * 128, rc);
    s->dW[0] = sur_alloc<float>(s, (size_t)s->nslice * kSurH * 128, rc);
    for (int l = 1; l <= 3; l++) s->dW[l] = sur_alloc<float>(s, (size_t)s->nslice * kSurH * kSurH, rc);
    s->dW[4] = sur_alloc<float>(s, (size_t)s->nslice * kSurOut * kSurH, rc);
    s->db = sur_alloc<float>(s, 4 * kSurH + 8, rc);
    s->demb = sur_alloc<float>(s, 2 * (size_t)nsets, rc);
    s->y = sur_alloc<float>(s, B * 8, rc);
    s->pred = sur_alloc<float>(s, B * 8, rc);
    s->loss = sur_alloc<float>(s, 1, rc);
    s->set_of = sur_alloc<int>(s, B, rc);
    s->cell_of = sur_alloc<int>(s, B, rc);
    s->cell_err = sur_alloc<unsigned>(s, (size_t)nsets * kSurNaz * kSurNza, rc);
    s->set_map = sur_alloc<int>(s, 2 * (size_t)nsets, rc);
    s->max_err = sur_alloc<unsigned>(s, 1, rc);
    s->nfallback = sur_alloc<unsigned>(s, 1, rc);
    if (!rc) rc = check_cuda(cudaStreamCreateWithFlags(&s->st, cudaStreamNonBlocking), "cudaStreamCreate");
    if (!rc) {
        // He-style initial weights (hash RNG on the host, uniform), zero biases,
        // embeddings spread in [-1, 1]
        std::vector<float> h(P, 0.f);
        uint64_t state = seed * 0x2545F4914F6CDD1Dull + 1;
        auto uni = [&]() {
            state ^= state << 13;
            state ^= state >> 7;
            state ^= state << 17;
            return (double)(state >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0;
        };
        auto fill = [&](long long off, long long n, int fan_in) {
            const double a = std::sqrt(6.0 / fan_in);
            for (long long i = 0; i < n; i++) h[off + i] = (float)(a * uni());
        };
        fill(s->L.W0, kSurH * 6, 6);
        fill(s->L.W1, kSurH * kSurH, kSurH);
        fill(s->L.W2, kSurH * kSurH, kSurH);
        fill(s->L.W3, kSurH * kSurH, kSurH);
        fill(s->L.W4, 8 * kSurH, kSurH);
        for (int k = 0; k < 2 * nsets; k++) h[s->L.emb + k] = (float)uni();
        rc = check_cuda(cudaMemcpy(s->p, h.data(), P * sizeof(float), cudaMemcpyHostToDevice), "cudaMemcpy(params)");
        if (!rc) rc = sur_adam(s, 0, 0.f, nullptr); // BF16 copies of the initial weights
        if (!rc) rc = check_cuda(cudaStreamSynchronize(s->st), "cudaStreamSynchronize");
    }
    if (rc) {
        for (void *p : s->allocs) cudaFree(p);
        if (s->st) cudaStreamDestroy(s->st);
        delete s;
        return rc;
    }
    *out = s;
    return VGB_SUCCESS;
}

extern "C" void vgb_surrogate_destroy(vgb_surrogate *s)
{
    if (!s) return;
    if (s->st) cudaStreamSynchronize(s->st);
    for (void *p : s->allocs) cudaFree(p);
    for (void *p : {(void *)s->tab_az, (void *)s->tab_za, (void *)s->tab_f, (void *)s->tab_Y, (void *)s->tab_delays,
                    (void *)s->Jsur, (void *)s->Bsur, (void *)s->sched, (void *)s->loss_dev, (void *)s->seed_dev,
                    (void *)s->kdev})
        if (p) cudaFree(p);
    if (s->st) cudaStreamDestroy(s->st);
    delete s;
}

extern "C" int vgb_surrogate_param_count(const vgb_surrogate *s) { return s ? (int)s->L.total : 0; }

extern "C" int vgb_surrogate_get_params(vgb_surrogate *s, float *host, int n)
{
    if (!s || !host || n < s->L.total) return set_error(VGB_ERR_INVALID, "surrogate_get_params: bad buffer");
    int rc = check_cuda(cudaStreamSynchronize(s->st), "cudaStreamSynchronize");
    if (!rc) rc = check_cuda(cudaMemcpy(host, s->p, s->L.total * sizeof(float), cudaMemcpyDeviceToHost), "cudaMemcpy");
    return rc;
}

extern "C" int vgb_surrogate_set_params(vgb_surrogate *s, const float *host, int n)
{
    if (!s || !host || n < s->L.total) return set_error(VGB_ERR_INVALID, "surrogate_set_params: bad buffer");
    int rc = check_cuda(cudaMemcpyAsync(s->p, host, s->L.total * sizeof(float), cudaMemcpyHostToDevice, s->st),
                        "cudaMemcpyAsync");
    if (!rc) rc = sur_adam(s, 0, 0.f, nullptr);
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s->st), "cudaStreamSynchronize");
    s->validated = false;
    return rc;
}

extern "C" int vgb_surrogate_set_training(vgb_surrogate *s, const uint32_t *delay_sets, const double *freqs_hz,
                                          int nfreq, int ndir, unsigned long long seed)
{
    if (!s || !delay_sets || !freqs_hz || nfreq <= 0 || ndir <= 0)
        return set_error(VGB_ERR_INVALID, "surrogate_set_training: bad arguments");
    for (void *p : {(void *)s->tab_az, (void *)s->tab_za, (void *)s->tab_f, (void *)s->tab_Y, (void *)s->tab_delays})
        if (p) cudaFree(p);
    s->tab_az = s->tab_za = s->tab_f = nullptr;
    s->tab_Y = nullptr;
    s->tab_delays = nullptr;
    s->ndir = ndir;
    s->nfreq = nfreq;
    int rc = VGB_SUCCESS;
    auto al = [&](void **p, size_t bytes) {
        if (!rc && cudaMalloc(p, bytes) != cudaSuccess) {
            cudaGetLastError();
            rc = set_error(VGB_ERR_ALLOC, "surrogate_set_training: cannot allocate %zu bytes", bytes);
        }
    };
    al((void **)&s->tab_az, ndir * sizeof(double));
    al((void **)&s->tab_za, ndir * sizeof(double));
    al((void **)&s->tab_f, nfreq * sizeof(double));
    al((void **)&s->tab_delays, (size_t)s->nsets * 16 * sizeof(uint32_t));
    al((void **)&s->tab_Y, (size_t)s->nsets * nfreq * ndir * 8 * sizeof(float));
    if (rc) return rc;
    rc = check_cuda(cudaMemcpyAsync(s->tab_f, freqs_hz, nfreq * sizeof(double), cudaMemcpyHostToDevice, s->st),
                    "cudaMemcpyAsync");
    if (!rc)
        rc = check_cuda(cudaMemcpyAsync(s->tab_delays, delay_sets, (size_t)s->nsets * 16 * sizeof(uint32_t),
                                        cudaMemcpyHostToDevice, s->st),
                        "cudaMemcpyAsync");
    if (rc) return rc;
    sur_dirs_kernel<<<(ndir + 255) / 256, 256, 0, s->st>>>(ndir, seed, s->tab_az, s->tab_za);
    if ((rc = check_launch("sur_dirs_kernel"))) return rc;
    const long long n = (long long)nfreq * ndir;
    for (int k = 0; k < s->nsets; k++) {
        sur_targets_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s->st>>>(
            s->tab_az, s->tab_za, ndir, s->tab_f, nfreq, s->tab_delays + 16 * k, s->tab_Y + (size_t)k * n * 8);
        if ((rc = check_launch("sur_targets_kernel"))) return rc;
    }
    s->validated = false;
    return check_cuda(cudaStreamSynchronize(s->st), "cudaStreamSynchronize");
}

// One training step on s->st with its schedule (seed, learning rate, Adam bias
// corrections) read on the device at index kdev[0], its loss accumulated into
// loss_dev[kdev[0]], and kdev advanced: the same launches every step, so the
// step is captured once and replayed.
static int sur_train_step(vgb_surrogate *s)
{
    SurBatch b{};
    b.az = s->tab_az;
    b.za = s->tab_za;
    b.freq = s->tab_f;
    b.ndir = s->ndir;
    b.nfreq = s->nfreq;
    b.nsets = s->nsets;
    b.Y = s->tab_Y;
    b.seed_dev = s->seed_dev;
    b.kdev = s->kdev;
    b.params = s->p;
    b.L = s->L;
    b.B = s->B;
    b.X0 = s->X0;
    b.set_of = s->set_of;
    b.y = s->y;
    sur_batch_kernel<<<(s->B + 255) / 256, 256, 0, s->st>>>(b);
    int rc = check_launch("sur_batch_kernel");
    if (!rc) rc = sur_forward(s);
    if (!rc) {
        sur_out_kernel<<<(s->B + 255) / 256, 256, 0, s->st>>>(s->C4, s->p + s->L.b4, s->y, s->B, nullptr, s->dY,
                                                              s->loss_dev, s->db + 4 * kSurH, s->kdev);
        rc = check_launch("sur_out_kernel");
    }
    if (!rc) rc = sur_backward(s);
    if (!rc) rc = sur_adam(s, 1, 0.f, nullptr, true);
    if (!rc) {
        sur_next_step_kernel<<<1, 1, 0, s->st>>>(s->kdev);
        rc = check_launch("sur_next_step_kernel");
    }
    return rc;
}

extern "C" int vgb_surrogate_train(vgb_surrogate *s, int steps, float lr_max, float lr_min, float *loss_host)
{
    if (!s || steps < 0) return set_error(VGB_ERR_INVALID, "surrogate_train: bad arguments");
    if (!s->tab_Y) return set_error(VGB_ERR_STATE, "surrogate_train: set_training first");
    if (steps == 0) return VGB_SUCCESS;
    int rc = VGB_SUCCESS;
    // the schedule on the host: cosine learning rate, Adam bias corrections, batch seeds
    if (steps > s->sched_cap) {
        for (void *p : {(void *)s->sched, (void *)s->loss_dev, (void *)s->seed_dev})
            if (p) cudaFree(p);
        s->sched = s->loss_dev = nullptr;
        s->seed_dev = nullptr;
        s->sched_cap = 0;
        rc = check_cuda(cudaMalloc(&s->sched, sizeof(float) * 3 * steps), "cudaMalloc(schedule)");
        if (!rc) rc = check_cuda(cudaMalloc(&s->loss_dev, sizeof(float) * steps), "cudaMalloc(losses)");
        if (!rc) rc = check_cuda(cudaMalloc(&s->seed_dev, sizeof(uint64_t) * steps), "cudaMalloc(seeds)");
        if (!rc && !s->kdev) rc = check_cuda(cudaMalloc(&s->kdev, sizeof(int)), "cudaMalloc(step index)");
        if (rc) return rc;
        s->sched_cap = steps;
    }
    std::vector<float> sched(3 * (size_t)steps);
    std::vector<uint64_t> seeds(steps);
    for (int k = 0; k < steps; k++) {
        const double t = (double)(s->step + k + 1);
        sched[3 * k] = lr_min + 0.5f * (lr_max - lr_min) * (1.f + cosf(3.14159265f * k / (float)steps));
        sched[3 * k + 1] = (float)(1.0 - pow(0.9, t));
        sched[3 * k + 2] = (float)(1.0 - pow(0.999, t));
        seeds[k] = (uint64_t)(s->step + k) * 0x632BE59BD9B4E019ull + 7;
    }
    rc = check_cuda(cudaMemcpyAsync(s->sched, sched.data(), sizeof(float) * sched.size(), cudaMemcpyHostToDevice,
                                    s->st),
                    "cudaMemcpyAsync(schedule)");
    if (!rc)
        rc = check_cuda(cudaMemcpyAsync(s->seed_dev, seeds.data(), sizeof(uint64_t) * steps, cudaMemcpyHostToDevice,
                                        s->st),
                        "cudaMemcpyAsync(seeds)");
    if (!rc) rc = check_cuda(cudaMemsetAsync(s->loss_dev, 0, sizeof(float) * steps, s->st), "cudaMemsetAsync");
    if (!rc) rc = check_cuda(cudaMemsetAsync(s->kdev, 0, sizeof(int), s->st), "cudaMemsetAsync");
    // the first step eagerly (the GEMM shapes get their tuned variants), then one
    // captured step replayed for the rest
    if (!rc) rc = sur_train_step(s);
    if (!rc && steps > 1) {
        cudaGraph_t graph = nullptr;
        cudaGraphExec_t exec = nullptr;
        rc = check_cuda(cudaStreamBeginCapture(s->st, cudaStreamCaptureModeRelaxed), "cudaStreamBeginCapture");
        if (!rc) {
            const int rs = sur_train_step(s);
            const int re = check_cuda(cudaStreamEndCapture(s->st, &graph), "cudaStreamEndCapture");
            rc = rs ? rs : re;
        }
        if (!rc) rc = check_cuda(cudaGraphInstantiate(&exec, graph, 0), "cudaGraphInstantiate");
        for (int k = 1; k < steps && !rc; k++) rc = check_cuda(cudaGraphLaunch(exec, s->st), "cudaGraphLaunch");
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
    if (!rc) s->step += steps;
    if (!rc && loss_host)
        rc = check_cuda(cudaMemcpyAsync(loss_host, s->loss_dev, sizeof(float) * steps, cudaMemcpyDeviceToHost, s->st),
                        "cudaMemcpyAsync(losses)");
    s->validated = false;
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s->st), "cudaStreamSynchronize");
    return rc;
}

extern "C" int vgb_surrogate_gradients(vgb_surrogate *s, const float *feat_host, const int *set_host,
                                       const float *y_host, float *grad_host, float *loss_host)
{
    if (!s || !feat_host || !set_host || !y_host || !grad_host)
        return set_error(VGB_ERR_INVALID, "surrogate_gradients: NULL argument");
    const size_t B = s->B;
    float *df = nullptr, *dy = nullptr;
    int *ds = nullptr;
    int rc = check_cuda(cudaMalloc(&df, B * 4 * sizeof(float)), "cudaMalloc");
    if (!rc) rc = check_cuda(cudaMalloc(&dy, B * 8 * sizeof(float)), "cudaMalloc");
    if (!rc) rc = check_cuda(cudaMalloc(&ds, B * sizeof(int)), "cudaMalloc");
    if (!rc) rc = check_cuda(cudaMemcpy(df, feat_host, B * 4 * sizeof(float), cudaMemcpyHostToDevice), "cudaMemcpy");
    if (!rc) rc = check_cuda(cudaMemcpy(dy, y_host, B * 8 * sizeof(float), cudaMemcpyHostToDevice), "cudaMemcpy");
    if (!rc) rc = check_cuda(cudaMemcpy(ds, set_host, B * sizeof(int), cudaMemcpyHostToDevice), "cudaMemcpy");
    if (!rc) {
        SurBatch b{};
        b.feat_in = df;
        b.set_in = ds;
        b.y_in = dy;
        b.params = s->p;
        b.L = s->L;
        b.B = s->B;
        b.X0 = s->X0;
        b.set_of = s->set_of;
        b.y = s->y;
        sur_batch_kernel<<<(s->B + 255) / 256, 256, 0, s->st>>>(b);
        rc = check_launch("sur_batch_kernel");
    }
    if (!rc) rc = check_cuda(cudaMemsetAsync(s->loss, 0, sizeof(float), s->st), "cudaMemsetAsync");
    if (!rc) rc = sur_forward(s);
    if (!rc) {
        sur_out_kernel<<<(s->B + 255) / 256, 256, 0, s->st>>>(s->C4, s->p + s->L.b4, s->y, s->B, s->pred, s->dY,
                                                              s->loss, s->db + 4 * kSurH);
        rc = check_launch("sur_out_kernel");
    }
    if (!rc) rc = sur_backward(s);
    if (!rc) rc = sur_adam(s, 0, 0.f, s->grad);
    if (!rc) rc = check_cuda(cudaStreamSynchronize(s->st), "cudaStreamSynchronize");
    if (!rc) rc = check_cuda(cudaMemcpy(grad_host, s->grad, s->L.total * sizeof(float), cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (!rc && loss_host) rc = check_cuda(cudaMemcpy(loss_host, s->loss, sizeof(float), cudaMemcpyDeviceToHost), "cudaMemcpy");
    cudaFree(df);
    cudaFree(dy);
    cudaFree(ds);
    return rc;
}

extern "C" int vgb_surrogate_validate(vgb_surrogate *s, long long nval, float tol, float *max_err, float *frac_cells_ok)
{
    if (!s || nval <= 0) return set_error(VGB_ERR_INVALID, "surrogate_validate: bad arguments");
    if (!s->tab_delays) return set_error(VGB_ERR_STATE, "surrogate_validate: set_training first");
    const size_t ncell = (size_t)s->nsets * kSurNaz * kSurNza;
    int rc = check_cuda(cudaMemsetAsync(s->cell_err, 0, ncell * sizeof(unsigned), s->st), "cudaMemsetAsync");
    if (!rc) rc = check_cuda(cudaMemsetAsync(s->max_err, 0, sizeof(unsigned), s->st), "cudaMemsetAsync");
    for (long long r0 = 0; r0 < nval && !rc; r0 += s->B) {
        SurQueryArgs q{};
        q.params = s->p;
        q.L = s->L;
        q.nsets = s->nsets;
        q.row0 = r0;
        q.nrows = nval;
        q.B = s->B;
        q.X0 = s->X0;
        q.validate = 1;
        q.freq = s->tab_f;
        q.nfreq = s->nfreq;
        q.delays = s->tab_delays;
        q.seed = 0xA5A5ull + (uint64_t)s->step;
        q.y = s->y;
        q.cell_of = s->cell_of;
        sur_query_kernel<<<(s->B + 255) / 256, 256, 0, s->st>>>(q);
        if ((rc = check_launch("sur_query_kernel"))) break;
        if ((rc = sur_forward(s))) break;
        sur_out_kernel<<<(s->B + 255) / 256, 256, 0, s->st>>>(s->C4, s->p + s->L.b4, nullptr, s->B, s->pred, s->dY,
                                                              nullptr, nullptr);
        if ((rc = check_launch("sur_out_kernel"))) break;
        sur_val_err_kernel<<<(s->B + 255) / 256, 256, 0, s->st>>>(s->pred, s->y, s->cell_of, s->B, s->cell_err,
                                                                  s->max_err);
        if ((rc = check_launch("sur_val_err_kernel"))) break;
    }
    if (rc) return rc;
    std::vector<unsigned> h(ncell);
    unsigned mx = 0;
    rc = check_cuda(cudaStreamSynchronize(s->st), "cudaStreamSynchronize");
    if (!rc) rc = check_cuda(cudaMemcpy(h.data(), s->cell_err, ncell * sizeof(unsigned), cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (!rc) rc = check_cuda(cudaMemcpy(&mx, s->max_err, sizeof(unsigned), cudaMemcpyDeviceToHost), "cudaMemcpy");
    if (rc) return rc;
    size_t ok = 0;
    for (unsigned e : h) {
        float f;
        std::memcpy(&f, &e, sizeof(f));
        ok += (e != 0u && f <= tol);
    }
    // a cell no validation sample reached stays unvalidated (error word 0 -> fallback)
    for (size_t i = 0; i < ncell; i++)
        if (h[i] == 0u) h[i] = 0x7f800000u;
    rc = check_cuda(cudaMemcpy(s->cell_err, h.data(), ncell * sizeof(unsigned), cudaMemcpyHostToDevice), "cudaMemcpy");
    s->cells_ok.assign(s->nsets, 0);
    for (size_t i = 0; i < ncell; i++) {
        float f;
        std::memcpy(&f, &h[i], sizeof(f));
        if (f <= tol) s->cells_ok[i / (kSurNaz * kSurNza)]++;
    }
    if (max_err) std::memcpy(max_err, &mx, sizeof(float));
    if (frac_cells_ok) *frac_cells_ok = (float)ok / (float)ncell;
    s->tol = tol;
    s->validated = !rc;
    return rc;
}

extern "C" int vgb_surrogate_beam(vgb_surrogate *s, const double *az, const double *za, int npointing,
                                  const double *freq_hz, int nfreq, const int *tile_set, const uint32_t *delays,
                                  int ntile, double latitude, int pa_correction, void *B, unsigned *nfallback,
                                  void *stream)
{
    if (!s || !az || !za || !freq_hz || !tile_set || !delays || !B)
        return set_error(VGB_ERR_INVALID, "surrogate_beam: NULL argument");
    if (npointing <= 0 || nfreq <= 0 || ntile <= 0) return set_error(VGB_ERR_INVALID, "surrogate_beam: empty shape");
    if (!s->validated) return set_error(VGB_ERR_STATE, "surrogate_beam: validate the network first");
    if ((reinterpret_cast<uintptr_t>(delays) | reinterpret_cast<uintptr_t>(B)) & 15)
        return set_error(VGB_ERR_INVALID, "surrogate_beam: delays and B must be 16-byte aligned");
    cudaStream_t caller = static_cast<cudaStream_t>(stream);
    // No sky cell of any trained set within the tolerance: every query falls
    // back, so the answer is the plain model's, on the caller's stream, with
    // no reads of the tile sets to the host.
    bool none_ok = true;
    for (int k : s->cells_ok) none_ok &= k == 0;
    if (none_ok) {
        PbArgs pb{az, za, npointing, freq_hz, nfreq, delays, ntile, latitude, pa_correction, static_cast<double2 *>(B)};
        const int rc0 = launch_beam_model(pb, caller);
        if (!rc0 && nfallback) *nfallback = (unsigned)((long long)nfreq * npointing * ntile);
        return rc0;
    }
    // the network runs only for the delay sets some tile uses (as vmCalcB
    // evaluates once per distinct configuration)
    std::vector<int> ts(ntile), list, slot(s->nsets, -1);
    std::vector<double> zah(npointing);
    int rc = check_cuda(cudaMemcpyAsync(ts.data(), tile_set, sizeof(int) * ntile, cudaMemcpyDeviceToHost, caller),
                        "cudaMemcpyAsync(tile_set)");
    if (!rc)
        rc = check_cuda(cudaMemcpyAsync(zah.data(), za, sizeof(double) * npointing, cudaMemcpyDeviceToHost, caller),
                        "cudaMemcpyAsync(za)");
    if (!rc) rc = check_cuda(cudaStreamSynchronize(caller), "cudaStreamSynchronize");
    if (rc) return rc;
    bool every_tile_trained = true;
    for (int t = 0; t < ntile; t++) {
        if (ts[t] >= 0 && ts[t] < s->nsets) {
            if (slot[ts[t]] < 0) {
                slot[ts[t]] = (int)list.size();
                list.push_back(ts[t]);
            }
        } else {
            every_tile_trained = false;
        }
    }
    // Work whose answers would all be discarded is skipped (the products are
    // the same): the network when no sky cell of the sets in use is within
    // the tolerance (every entry falls back), the plain model when every cell
    // is, every tile's set was trained and every pointing is within the
    // trained zenith angles (no entry falls back).
    bool any_cell_ok = false, all_cells_ok = every_tile_trained;
    for (int k : list) {
        any_cell_ok |= s->cells_ok[k] > 0;
        all_cells_ok &= s->cells_ok[k] == kSurNaz * kSurNza;
    }
    for (double z : zah) all_cells_ok &= z <= kSurZaMax;
    if (!any_cell_ok) {
        list.clear();
        for (int &k : slot) k = -1;
    }
    const int nslots = (int)list.size();
    const long long rows = (long long)nfreq * npointing * nslots;
    std::vector<int> map(2 * s->nsets, 0);
    for (int k = 0; k < nslots; k++) map[k] = list[k];
    for (int k = 0; k < s->nsets; k++) map[s->nsets + k] = slot[k];
    if (rows > s->Jsur_cap) {
        if (s->Jsur) cudaFree(s->Jsur);
        if (s->Bsur) cudaFree(s->Bsur);
        s->Jsur = nullptr;
        s->Bsur = nullptr;
        s->Jsur_cap = 0;
        if ((rc = check_cuda(cudaMalloc(&s->Bsur, rows * 4 * sizeof(double2)), "cudaMalloc(surrogate B rows)")))
            return rc;
        if ((rc = check_cuda(cudaMalloc(&s->Jsur, rows * 8 * sizeof(float)), "cudaMalloc(surrogate outputs)")))
            return rc;
        s->Jsur_cap = rows;
    }
    // order: the caller's stream -> the surrogate's stream -> the caller's stream
    cudaEvent_t ev;
    if ((rc = check_cuda(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "cudaEventCreate"))) return rc;
    rc = check_cuda(cudaEventRecord(ev, caller), "cudaEventRecord");
    if (!rc) rc = check_cuda(cudaStreamWaitEvent(s->st, ev, 0), "cudaStreamWaitEvent");
    if (!rc) rc = check_cuda(cudaMemsetAsync(s->nfallback, 0, sizeof(unsigned), s->st), "cudaMemsetAsync");
    if (!rc)
        rc = check_cuda(cudaMemcpyAsync(s->set_map, map.data(), sizeof(int) * map.size(), cudaMemcpyHostToDevice, s->st),
                        "cudaMemcpyAsync(set map)");
    for (long long r0 = 0; r0 < rows && !rc; r0 += s->B) {
        SurQueryArgs q{};
        q.az = az;
        q.za = za;
        q.freq = freq_hz;
        q.npointing = npointing;
        q.nfreq = nfreq;
        q.nsets = nslots;
        q.set_list = s->set_map;
        q.params = s->p;
        q.L = s->L;
        q.row0 = r0;
        q.nrows = rows;
        q.B = s->B;
        q.X0 = s->X0;
        sur_query_kernel<<<(s->B + 255) / 256, 256, 0, s->st>>>(q);
        if ((rc = check_launch("sur_query_kernel"))) break;
        if ((rc = sur_forward(s))) break;
        sur_out_kernel<<<(s->B + 255) / 256, 256, 0, s->st>>>(s->C4, s->p + s->L.b4, nullptr, s->B, s->pred, s->dY,
                                                              nullptr, nullptr);
        if ((rc = check_launch("sur_out_kernel"))) break;
        const long long n = rows - r0 < s->B ? rows - r0 : s->B;
        rc = check_cuda(cudaMemcpyAsync(s->Jsur + r0 * 8, s->pred, n * 8 * sizeof(float), cudaMemcpyDeviceToDevice,
                                        s->st),
                        "cudaMemcpyAsync");
    }
    // fallback answers: the plain model for every entry (once per distinct
    // delay set, copied to tiles), then the network's answers overwrite it
    if (!rc && !all_cells_ok) {
        PbArgs pb{az, za, npointing, freq_hz, nfreq, delays, ntile, latitude, pa_correction, static_cast<double2 *>(B)};
        rc = launch_beam_model(pb, s->st);
    }
    if (!rc) {
        SurExpandArgs e{az,      za,      freq_hz,    npointing,        nfreq,   s->nsets,   ntile,
                        tile_set, delays, s->Jsur,    s->Bsur,   s->set_map + s->nsets, nslots,
                        s->cell_err, s->tol, latitude, pa_correction, static_cast<double2 *>(B), s->nfallback};
        if (rows > 0) {
            sur_rotate_kernel<<<(unsigned)((rows + 127) / 128), 128, 0, s->st>>>(e, rows);
            rc = check_launch("sur_rotate_kernel");
        }
        const long long n = (long long)nfreq * npointing * ntile;
        if (!rc) {
            sur_expand_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s->st>>>(e);
            rc = check_launch("sur_expand_kernel");
        }
    }
    if (!rc && nfallback)
        rc = check_cuda(cudaMemcpyAsync(nfallback, s->nfallback, sizeof(unsigned), cudaMemcpyDeviceToHost, s->st),
                        "cudaMemcpyAsync");
    if (!rc) rc = check_cuda(cudaEventRecord(ev, s->st), "cudaEventRecord");
    if (!rc) rc = check_cuda(cudaStreamWaitEvent(caller, ev, 0), "cudaStreamWaitEvent");
    if (!rc && nfallback) rc = check_cuda(cudaStreamSynchronize(s->st), "cudaStreamSynchronize");
    cudaEventDestroy(ev);
    return rc;
}
