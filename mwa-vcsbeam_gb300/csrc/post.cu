// Table builders, detection post-processing and the legacy-input beamformer.
//
//  * tables: geometric phase (geometry.c:40-101), inverse Jones
//    (jones.c:97-157) and their product, the per-(tile, channel) weight
//    W = phi J^-1 the beam kernels apply. FP64 on the device, W rounded to FP32.
//  * renormalise: per-channel min/max scale-and-offset to 8 bits
//    (form_beam.cpp:408-449), writing the spliced multi-channel layout
//    directly when asked.
//  * incoherent beam of 4+4-bit legacy voltages (form_beam.cpp:60-87).
//  * beamformer for fine-channel voltages already in legacy layout
//    (v_IDX [s][c][i], 4+4-bit or complex FP64): vmApplyJ_kernel followed by
//    vmBeamform_kernel (form_beam.cpp:122-371) in one pass.
#include <cooperative_groups.h>

#include "vgb_launch.cuh"

namespace vgb {

// ---------------------------------------------------------------------------
// FP64 complex helpers with cuCmul's operation order.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double2 zmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ double2 zadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 zsub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }

// geometry.c:40-101 for one (pointing, tile, channel): phase terms use the
// reference's order of operations, 2*pi*dt*f. `u` is the pointing's (E, N, H)
// unit vector; the frequency is cast to whole Hz as the reference's is.
__device__ __forceinline__ double2 geometric_phase(const double *u, double east, double north, double height,
                                                   double cable, double href, double freq)
{
    const double L = cable - 0.0;
    const double w = (east - 0.0) * u[0] + (north - 0.0) * u[1] + (height - href) * u[2];
    const double dt = (w - L) / 299792458.0;
    const double f = (double)(uint32_t)freq;
    const double phase = 2.0 * 3.14159265358979323846 * dt * f;
    double s, co;
    sincos(phase, &s, &co);
    return make_double2(co, s);
}

__global__ void phase_kernel(const double *unit, const double *east, const double *north, const double *height,
                             const double *cable, const double *freqs, int npointing, int nant, int nchan,
                             double href, double2 *phi)
{
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long n = (long long)npointing * nant * nchan;
    if (idx >= n) return;
    const int c = idx % nchan;
    const int a = (idx / nchan) % nant;
    const int p = idx / ((long long)nchan * nant);
    phi[idx] = geometric_phase(unit + 3 * p, east[a], north[a], height[a], cable[a], href, freqs[c]);
}

// geometry.c:440-467 (calc_array_factor; Eq. A4 of Meyers et al. 2017): the
// tied-array response of the look direction's phases w at test direction
// psi, |sum_a conj(w_a) psi_a|^2 / nant^2. One block per test direction, the
// phases in FP64 with the geometric-delay kernel's operation order, the sum
// as the reference's sequential complex additions (thread 0 adds the tiles in
// order after each thread formed its products).
__global__ void array_factor_kernel(const double *look, const double *dirs, int npix, double freq,
                                    const double *east, const double *north, const double *height,
                                    const double *cable, double href, int nant, double *af)
{
    extern __shared__ double2 prod[];
    const int pix = blockIdx.x;
    if (pix >= npix) return;
    const double f = (double)(uint32_t)freq;
    for (int a = threadIdx.x; a < nant; a += blockDim.x) {
        double2 ph[2];
        for (int k = 0; k < 2; k++) {
            const double *u = k == 0 ? look : dirs + 3 * pix;
            const double L = cable[a] - 0.0;
            const double w = (east[a] - 0.0) * u[0] + (north[a] - 0.0) * u[1] + (height[a] - href) * u[2];
            const double dt = (w - L) / 299792458.0;
            const double phase = 2.0 * 3.14159265358979323846 * dt * f;
            double sn, cs;
            sincos(phase, &sn, &cs);
            ph[k] = make_double2(cs, sn);
        }
        // conj(w) * psi
        prod[a] = make_double2(ph[0].x * ph[1].x + ph[0].y * ph[1].y, ph[0].x * ph[1].y - ph[0].y * ph[1].x);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double2 s = make_double2(0.0, 0.0);
        for (int a = 0; a < nant; a++) s = make_double2(s.x + prod[a].x, s.y + prod[a].y);
        const double m = hypot(s.x, s.y) / nant;
        af[pix] = m * m;
    }
}

int launch_array_factor(const double *look, const double *dirs, int npix, double freq, const double *east,
                        const double *north, const double *height, const double *cable, double href, int nant,
                        double *af, cudaStream_t st)
{
    if (npix <= 0) return VGB_SUCCESS;
    array_factor_kernel<<<npix, 128, sizeof(double2) * nant, st>>>(look, dirs, npix, freq, east, north, height,
                                                                    cable, href, nant, af);
    return check_launch("array_factor_kernel");
}

// jones.c:97-157: J = inv2x2S(D[a][c] B[p][a] / ||D B||_F), zero if the norm is 0.
// jones.c:97-157 for one (pointing, tile, channel): J = D B normalised by
// its Frobenius norm, then inverted (zero when the norm is zero).
__device__ __forceinline__ void inverse_jones(const double2 *d, const double2 *b, double2 (&o)[4])
{
    double2 m[4];
    m[0] = zadd(zmul(d[0], b[0]), zmul(d[1], b[2]));
    m[1] = zadd(zmul(d[0], b[1]), zmul(d[1], b[3]));
    m[2] = zadd(zmul(d[2], b[0]), zmul(d[3], b[2]));
    m[3] = zadd(zmul(d[2], b[1]), zmul(d[3], b[3]));
    double F = 0.0;
    for (int i = 0; i < 4; i++) F += zmul(m[i], make_double2(m[i].x, -m[i].y)).x;
    F = sqrt(F);
    if (F == 0.0) {
        for (int i = 0; i < 4; i++) o[i] = make_double2(0.0, 0.0);
        return;
    }
    // one FP64 division instead of eight (FP64 is this GPU's slow pipe;
    // the products differ from the quotients by at most an ulp)
    const double rF = 1.0 / F;
    for (int i = 0; i < 4; i++) m[i] = make_double2(m[i].x * rF, m[i].y * rF);
    const double2 det = zsub(zmul(m[0], m[3]), zmul(m[1], m[2]));
    const double scale = 1.0 / (det.x * det.x + det.y * det.y);
    const double2 inv = make_double2(scale * det.x, -scale * det.y);
    const double2 ninv = make_double2(-inv.x, -inv.y);
    o[0] = zmul(inv, m[3]);
    o[1] = zmul(ninv, m[1]);
    o[2] = zmul(ninv, m[2]);
    o[3] = zmul(inv, m[0]);
}

// W = phi J in FP64, rounded to FP32 and stored as two float4:
// (w00, w01), (w10, w11).
__device__ __forceinline__ void store_weight(double2 ph, const double2 (&j)[4], float4 *W)
{
    double2 w[4];
    for (int i = 0; i < 4; i++) w[i] = zmul(ph, j[i]);
    W[0] = make_float4((float)w[0].x, (float)w[0].y, (float)w[1].x, (float)w[1].y);
    W[1] = make_float4((float)w[2].x, (float)w[2].y, (float)w[3].x, (float)w[3].y);
}

__global__ void jones_kernel(const double2 *D, const double2 *B, int npointing, int nant, int nchan, double2 *J)
{
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long n = (long long)npointing * nant * nchan;
    if (idx >= n) return;
    const int c = idx % nchan;
    const int a = (idx / nchan) % nant;
    const int p = idx / ((long long)nchan * nant);
    double2 o[4];
    inverse_jones(D + 4 * ((long long)a * nchan + c), B + 4 * ((long long)p * nant + a), o);
    for (int i = 0; i < 4; i++) J[4 * idx + i] = o[i];
}

// W[p][a][c] = phi[p][a][c] * J[p][a][c].
__global__ void weights_kernel(const double2 *J, const double2 *phi, long long n, float4 *W)
{
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (idx >= n) return;
    const double2 j[4] = {J[4 * idx], J[4 * idx + 1], J[4 * idx + 2], J[4 * idx + 3]};
    store_weight(phi[idx], j, W + 2 * idx);
}

// ---------------------------------------------------------------------------
// Per-second tracking (vmCalcJonesAndDelays, jones.c:170-188): the pointing
// of the current second, then B (primary-beam kernel), then J^-1, phi and
// W = phi J^-1 for every (coarse channel, tile, fine channel) in one pass.
// ---------------------------------------------------------------------------

// One thread: the second's pointing from the per-second table (the last entry
// holds past its end), its (E, N, H) unit vector as calc_beam_geom sets it
// (geometry.c:226-286, from az and el = pi/2 - za), and the counter stepped
// for the next second.
__global__ void track_select_kernel(const double *az_tab, const double *za_tab, int nseconds,
                                    long long *counter, double *cur)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const long long s = *counter;
    const int i = (int)(s < nseconds ? s : nseconds - 1);
    const double az = az_tab[i], za = za_tab[i];
    const double el = 0.5 * 3.14159265358979323846 - za;
    double saz, caz, sel, cel;
    sincos(az, &saz, &caz);
    sincos(el, &sel, &cel);
    cur[0] = az;
    cur[1] = za;
    cur[2] = cel * saz; // E
    cur[3] = cel * caz; // N
    cur[4] = sel;       // H
    *counter = s + 1;
}

// One thread per (cc, tile, fine channel): D [cc][a][c][2][2], B [cc][a][2][2]
// (one pointing, the coarse channel's beam frequency), freqs [cc][c].
__global__ void track_weights_kernel(const double2 *D, const double2 *B, const double *unit, const double *east,
                                     const double *north, const double *height, const double *cable,
                                     const double *freqs, int ncc, int nant, int nchan, double href, float4 *W)
{
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long n = (long long)ncc * nant * nchan;
    if (idx >= n) return;
    const int c = idx % nchan;
    const int a = (idx / nchan) % nant;
    const int cc = idx / ((long long)nchan * nant);
    double2 j[4];
    inverse_jones(D + 4 * idx, B + 4 * ((long long)cc * nant + a), j);
    const double2 ph = geometric_phase(unit, east[a], north[a], height[a], cable[a], href,
                                       freqs[(long long)cc * nchan + c]);
    store_weight(ph, j, W + 2 * idx);
}

int launch_track_select(const double *az_tab, const double *za_tab, int nseconds, long long *counter, double *cur,
                        cudaStream_t st)
{
    track_select_kernel<<<1, 32, 0, st>>>(az_tab, za_tab, nseconds, counter, cur);
    return check_launch("track_select_kernel");
}

int launch_track_weights(const double2 *D, const double2 *B, const double *unit, const double *east,
                         const double *north, const double *height, const double *cable, const double *freqs,
                         int ncc, int nant, int nchan, double href, float4 *W, cudaStream_t st)
{
    const long long n = (long long)ncc * nant * nchan;
    if (n == 0) return VGB_SUCCESS;
    track_weights_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(D, B, unit, east, north, height, cable, freqs,
                                                                      ncc, nant, nchan, href, W);
    return check_launch("track_weights_kernel");
}

int launch_phase(const double *unit, const double *east, const double *north, const double *height,
                 const double *cable, const double *freqs, int npointing, int nant, int nchan, double href,
                 double2 *phi, cudaStream_t st)
{
    const long long n = (long long)npointing * nant * nchan;
    if (n == 0) return VGB_SUCCESS;
    phase_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(unit, east, north, height, cable, freqs, npointing,
                                                               nant, nchan, href, phi);
    return check_launch("phase_kernel");
}

int launch_jones(const double2 *D, const double2 *B, int npointing, int nant, int nchan, double2 *J,
                 cudaStream_t st)
{
    const long long n = (long long)npointing * nant * nchan;
    if (n == 0) return VGB_SUCCESS;
    jones_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(D, B, npointing, nant, nchan, J);
    return check_launch("jones_kernel");
}

int launch_weights(const double2 *J, const double2 *phi, long long n, float4 *W, cudaStream_t st)
{
    if (n == 0) return VGB_SUCCESS;
    weights_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(J, phi, n, W);
    return check_launch("weights_kernel");
}

// ---------------------------------------------------------------------------
// renormalise_channels (form_beam.cpp:408-449)
// ---------------------------------------------------------------------------

// The float -> uint8 conversion of form_beam.cpp:443, (uint8_t)(val + 0.5)
// with val + 0.5 in FP64, as the reference's GPU build performs it: truncate
// to an integer and keep the low 8 bits, so a channel's maximum sample
// (256.5) becomes 0; NaN becomes 0. val is never negative here.
// One warp lane per channel; the 8 warps of a block split the samples.
constexpr int kRenormSplit = 8; // CTAs (one thread-block cluster) per (cc, pointing, stokes, 32 channels)

// Cluster of kRenormSplit CTAs over one (cc, pointing, stokes, 32 channels):
// CTA r scans samples [r n / 8, (r + 1) n / 8). Sequential-scan semantics of
// the reference: every partial starts from sample 0 and uses the same
// comparisons, so combining them in any order gives the same extremes (a NaN
// first sample makes the result NaN; other NaNs are skipped). The partials
// meet through distributed shared memory; each CTA then quantises its samples.
__global__ void __launch_bounds__(256) renorm_kernel(const RenormArgs a)
{
    namespace cg = cooperative_groups;
    cg::cluster_group cluster = cg::this_cluster();
    __shared__ float smin[8][32], smax[8][32];
    __shared__ float cmin[32], cmax[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int part = (int)cluster.block_rank();
    const int c = (blockIdx.x / kRenormSplit) * 32 + lane;
    const int st = blockIdx.y % a.nstokes, p = blockIdx.y / a.nstokes;
    const int cc = blockIdx.z;
    const bool live = c < a.nchan;
    const long long sstride = (long long)a.nstokes * a.nchan;
    const float *S = a.S + cc * a.S_cc + ((long long)p * a.nstep * a.nstokes + st) * a.nchan + (live ? c : 0);
    const int sb = (int)((long long)a.nstep * part / kRenormSplit);
    const int se = (int)((long long)a.nstep * (part + 1) / kRenormSplit);

    float mn, mx;
    if (a.st_mn) {
        // extremes gathered by the beam kernel: one pass over the samples
        const long long si = cc * a.stat_cc + ((long long)p * a.nstokes + st) * a.nchan + (live ? c : 0);
        if (a.st_nan0[si]) {
            mn = mx = __int_as_float(0x7fffffff);
        } else {
            mn = fkey_inv(a.st_mn[si]);
            mx = fkey_inv(a.st_mx[si]);
        }
    } else {
        const float s0 = S[0];
        mn = s0;
        mx = s0;
        // four independent loads in flight per lane (the scan order does not
        // change the extremes: a NaN first value stays, later NaNs are skipped)
        int s = sb + wid;
        for (; s + 24 < se; s += 32) {
            float v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = S[(long long)(s + 8 * u) * sstride];
#pragma unroll
            for (int u = 0; u < 4; u++) {
                mn = (v[u] < mn ? v[u] : mn);
                mx = (v[u] > mx ? v[u] : mx);
            }
        }
        for (; s < se; s += 8) {
            const float v = S[(long long)s * sstride];
            mn = (v < mn ? v : mn);
            mx = (v > mx ? v : mx);
        }
        smin[wid][lane] = mn;
        smax[wid][lane] = mx;
        __syncthreads();
        if (wid == 0) {
            for (int w = 1; w < 8; w++) {
                const float v0 = smin[w][lane], v1 = smax[w][lane];
                mn = (v0 < mn ? v0 : mn);
                mx = (v1 > mx ? v1 : mx);
            }
            cmin[lane] = mn;
            cmax[lane] = mx;
        }
        cluster.sync(); // every CTA's partial is in its shared memory
        mn = s0;
        mx = s0;
        for (int r = 0; r < kRenormSplit; r++) {
            const float v0 = *cluster.map_shared_rank(&cmin[lane], r);
            const float v1 = *cluster.map_shared_rank(&cmax[lane], r);
            mn = (v0 < mn ? v0 : mn);
            mx = (v1 > mx ? v1 : mx);
        }
        cluster.sync(); // no CTA leaves while another still reads its partials
    }
    const float scale = (float)((double)(mx - mn) / 256.0);
    const float offset = mn;
    if (live) {
        uint8_t *o = a.out + cc * a.out_cc + p * a.out_p + st * a.out_st + c;
        const float rcp = 1.f / scale;
        int s = sb + wid;
        for (; s + 24 < se; s += 32) {
            float v[4];
#pragma unroll
            for (int u = 0; u < 4; u++) v[u] = S[(long long)(s + 8 * u) * sstride];
#pragma unroll
            for (int u = 0; u < 4; u++) o[(long long)(s + 8 * u) * a.out_s] = quant_u8(v[u], offset, scale, rcp);
        }
        for (; s < se; s += 8) o[(long long)s * a.out_s] = quant_u8(S[(long long)s * sstride], offset, scale, rcp);
        if (part == 0 && wid == 0) {
            const long long si = cc * a.stat_cc + ((long long)p * a.nstokes + st) * a.nchan + c;
            a.scales[si] = scale;
            a.offsets[si] = offset;
        }
    }
}

int launch_renorm(const RenormArgs &a, int ncc, cudaStream_t st)
{
    if (a.nstep <= 0 || ncc <= 0) return VGB_SUCCESS;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(kRenormSplit * ((a.nchan + 31) / 32), a.npointing * a.nstokes, ncc);
    cfg.blockDim = dim3(256);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = kRenormSplit;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const int rc = check_cuda(cudaLaunchKernelEx(&cfg, renorm_kernel, a), "cudaLaunchKernelEx(renorm_kernel)");
    return rc ? rc : check_launch("renorm_kernel");
}

// ---------------------------------------------------------------------------
// Incoherent beam of 4+4-bit voltages (form_beam.cpp:60-87): exact integer
// sums of |v|^2 over all inputs. Eight lanes per (s, c) row of ninput bytes.
// ---------------------------------------------------------------------------
__device__ __forceinline__ int nib(uint32_t x) { return ((int)(x << 28)) >> 28; }

__device__ __forceinline__ int power4(uint32_t w)
{
    int acc = 0;
#pragma unroll
    for (int b = 0; b < 4; b++) {
        const uint32_t byte = (w >> (8 * b)) & 0xFFu;
        const int re = nib(byte >> 4), im = nib(byte);
        acc += re * re + im * im;
    }
    return acc;
}

__global__ void incoh_kernel(const uint8_t *data, long long nrows, int ninput, float *incoh)
{
    const long long row = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 3;
    const int sub = threadIdx.x & 7;
    int acc = 0;
    if (row < nrows) {
        const uint8_t *r = data + row * ninput;
        if ((ninput & 31) == 0) {
            for (int off = sub * 4; off < ninput; off += 32)
                acc += power4(*reinterpret_cast<const uint32_t *>(r + off));
        } else {
            for (int off = sub; off < ninput; off += 8) acc += power4(r[off]);
        }
    }
    acc += __shfl_xor_sync(0xffffffffu, acc, 1);
    acc += __shfl_xor_sync(0xffffffffu, acc, 2);
    acc += __shfl_xor_sync(0xffffffffu, acc, 4);
    if (row < nrows && sub == 0) incoh[row] = (float)acc;
}

int launch_incoh(const uint8_t *data, long long nrows, int ninput, float *incoh, cudaStream_t st)
{
    if (nrows <= 0) return VGB_SUCCESS;
    const long long threads = nrows * 8;
    incoh_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(data, nrows, ninput, incoh);
    return check_launch("incoh_kernel");
}

// ---------------------------------------------------------------------------
// Beamformer for legacy-layout fine voltages v[s][c][i].
// A block covers 16 channels x 4 samples = 64 voltage rows, four threads per
// row splitting the tiles (tile = part, part + 4, ...) and combining their
// sums with two shuffles; the 4+4-bit rows are staged in shared memory with a
// 4-byte pad (33 KB for 256 tiles, so several blocks share an SM).
// ---------------------------------------------------------------------------

constexpr int kLS = 4, kLC = 16; // samples, channels per block
constexpr int kLParts = 4;       // threads per row

template <bool kInt4>
__global__ void __launch_bounds__(256) legacy_beam_kernel(const LegacyArgs a)
{
    extern __shared__ __align__(16) unsigned char lsm[];
    const int ni = 2 * a.nant;
    const int tid = threadIdx.x;
    const int r = tid / kLParts, part = tid % kLParts;
    const int c0 = blockIdx.x * kLC, s0 = blockIdx.y * kLS;
    const int c = c0 + r % kLC, s = s0 + r / kLC;
    const bool live = c < a.nchan && s < a.nsamples;
    const int wpr = ni / 4 + 1;

    // Stage the 4+4-bit rows (s, c) of this block. Complex FP64 voltages are
    // read straight from global memory.
    if (kInt4) {
        // 4-byte asynchronous copies, all in flight before one wait (rows
        // outside the block's samples or channels are zero-filled)
        uint32_t *rows = reinterpret_cast<uint32_t *>(lsm);
        const int nw = ni / 4;
        const uint32_t *v32 = static_cast<const uint32_t *>(a.v);
        for (int idx = tid; idx < kLS * kLC * nw; idx += blockDim.x) {
            const int rr = idx / nw, wdx = idx % nw;
            const int rs = s0 + rr / kLC, rc = c0 + rr % kLC;
            const bool in = rs < a.nsamples && rc < a.nchan;
            const uint32_t *src = in ? v32 + ((long long)rs * a.nchan + rc) * (ni / 4) + wdx : v32;
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(smem_u32(&rows[rr * wpr + wdx])),
                         "l"(src), "r"(in ? 4u : 0u)
                         : "memory");
        }
        asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
    }
    // the tiles' (Q, P) input pairs, checked against the row once per block
    uint32_t *pq = reinterpret_cast<uint32_t *>(lsm + (kInt4 ? (size_t)kLS * kLC * wpr * 4 : 0));
    for (int ant = tid; ant < a.nant; ant += blockDim.x) {
        uint32_t iq = __ldg(a.polQ + ant), ip = __ldg(a.polP + ant);
        if (iq >= (uint32_t)ni || ip >= (uint32_t)ni) {
            if (blockIdx.x == 0 && blockIdx.y == 0) atomicOr(a.status, kErrBadInput);
            iq = ip = 0;
        }
        pq[ant] = iq | (ip << 16);
    }
    __syncthreads();
    const uint8_t *row8 = lsm + 4 * (r * wpr);

    for (int p = 0; p < a.npointing; p++) {
        float acc[8];
#pragma unroll
        for (int q = 0; q < 8; q++) acc[q] = 0.f;
        const float4 *Wp = a.W + ((long long)p * a.nant * a.nchan + (live ? c : 0)) * 2;
        if (live) {
#pragma unroll 4
            for (int ant = part; ant < a.nant; ant += kLParts) {
                const uint32_t iqp = pq[ant], iq = iqp & 0xFFFFu, ip = iqp >> 16;
                float2 vq, vp;
                if (kInt4) {
                    const uint32_t bq = row8[iq], bp = row8[ip];
                    vq = make_float2((float)nib(bq >> 4), (float)nib(bq));
                    vp = make_float2((float)nib(bp >> 4), (float)nib(bp));
                } else {
                    const double2 *row = static_cast<const double2 *>(a.v) + ((long long)s * a.nchan + c) * ni;
                    const double2 dq = __ldg(row + iq), dp = __ldg(row + ip);
                    vq = make_float2((float)dq.x, (float)dq.y);
                    vp = make_float2((float)dp.x, (float)dp.y);
                }
                const float4 wa = __ldg(Wp + (long long)ant * a.nchan * 2);
                const float4 wb = __ldg(Wp + (long long)ant * a.nchan * 2 + 1);
                const float exr = wa.x * vq.x - wa.y * vq.y + wa.z * vp.x - wa.w * vp.y;
                const float exi = wa.x * vq.y + wa.y * vq.x + wa.z * vp.y + wa.w * vp.x;
                const float eyr = wb.x * vq.x - wb.y * vq.y + wb.z * vp.x - wb.w * vp.y;
                const float eyi = wb.x * vq.y + wb.y * vq.x + wb.z * vp.y + wb.w * vp.x;
                acc[0] += exr;
                acc[1] += exi;
                acc[2] += eyr;
                acc[3] += eyi;
                acc[4] = fmaf(exr, exr, fmaf(exi, exi, acc[4]));
                acc[5] = fmaf(eyr, eyr, fmaf(eyi, eyi, acc[5]));
                acc[6] = fmaf(exr, eyr, fmaf(exi, eyi, acc[6]));
                acc[7] = fmaf(exi, eyr, fmaf(-exr, eyi, acc[7]));
            }
        }
        // the row's four partial sums (lanes 4k .. 4k+3 of a warp)
#pragma unroll
        for (int q = 0; q < 8; q++) {
            acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], 1);
            acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], 2);
        }
        if (!live || part != 0) continue;
        const float bnXX = acc[0] * acc[0] + acc[1] * acc[1] - acc[4];
        const float bnYY = acc[2] * acc[2] + acc[3] * acc[3] - acc[5];
        const float bxr = acc[0] * acc[2] + acc[1] * acc[3] - acc[6];
        const float bxi = acc[1] * acc[2] - acc[0] * acc[3] - acc[7];
        float *S = a.S + (((long long)p * a.nsamples + s) * a.nstokes) * a.nchan + c;
        S[0] = a.invw * (bnXX + bnYY);
        if (a.nstokes == 4) {
            S[a.nchan] = a.invw * (bnXX - bnYY);
            S[2 * a.nchan] = 2.0f * a.invw * bxr;
            S[3 * a.nchan] = -2.0f * a.invw * bxi;
        }
        if (a.e) a.e[((long long)p * a.nsamples + s) * a.nchan + c] = make_float4(acc[0], acc[1], acc[2], acc[3]);
    }
    if (kInt4 && a.incoh && live && part == 0) {
        const uint32_t *row = reinterpret_cast<const uint32_t *>(lsm) + r * wpr;
        int accp = 0;
        for (int wdx = 0; wdx < ni / 4; wdx++) accp += power4(row[wdx]);
        a.incoh[(long long)s * a.nchan + c] = (float)accp;
    }
}

int launch_legacy_beam(const LegacyArgs &a, cudaStream_t st)
{
    if (a.nsamples <= 0) return VGB_SUCCESS;
    const int ni = 2 * a.nant;
    const bool int4 = a.datatype == VGB_INT4;
    if (int4 && (ni % 4) != 0) return set_error(VGB_ERR_INVALID, "legacy beamformer: 2*nant must be a multiple of 4");
    if (ni > 65535) return set_error(VGB_ERR_INVALID, "legacy beamformer: at most 65535 inputs");
    const size_t smem = (int4 ? (size_t)kLS * kLC * (ni / 4 + 1) * 4 : 0) + (size_t)a.nant * 4;
    if (smem > 227 * 1024)
        return set_error(VGB_ERR_INVALID, "legacy beamformer: %d inputs do not fit the shared-memory tile", ni);
    if ((a.nsamples + kLS - 1) / kLS > 65535)
        return set_error(VGB_ERR_INVALID, "legacy beamformer: at most %d samples per call", 65535 * kLS);
    dim3 grid((a.nchan + kLC - 1) / kLC, (a.nsamples + kLS - 1) / kLS);
    if (int4) {
        int rc = check_cuda(cudaFuncSetAttribute(legacy_beam_kernel<true>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                            "cudaFuncSetAttribute(legacy)");
        if (rc) return rc;
        legacy_beam_kernel<true><<<grid, 256, smem, st>>>(a);
    } else {
        int rc = check_cuda(cudaFuncSetAttribute(legacy_beam_kernel<false>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                            "cudaFuncSetAttribute(legacy)");
        if (rc) return rc;
        legacy_beam_kernel<false><<<grid, 256, smem, st>>>(a);
    }
    return check_launch("legacy_beam_kernel");
}

} // namespace vgb
