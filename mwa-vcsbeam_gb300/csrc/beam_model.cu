// Primary-beam matrices B [pointing][tile][2][2] (vmCalcB,
// primary_beam.c:79-191) on the device, FP64, evaluated once per distinct
// delay set (tiles sharing a dipole configuration share B, as vmCalcB's
// per-configuration cache) and copied to the other tiles.
//
// The reference evaluates the MWA FEE model (mwa_hyperbeam's calc_jones, a
// Rust crate reading an HDF5 table of spherical-wave coefficients) once per
// distinct dead-dipole configuration and pointing, then multiplies the
// parallactic-angle rotation on the right. The FEE model is not available to
// this build; the model evaluated here is an analytic MWA tile:
//
//   * 16 dipoles on a 4 x 4 grid of 1.1 m pitch (row 0 north, column 0 west),
//     each delayed by d_i x 435 ps by the tile beamformer (d_i = 0..31, 32 =
//     dead dipole, amplitude 0: create_delays_amps_from_metafits,
//     primary_beam.c:260-284);
//   * array factor AF = (1/16) sum_i a_i exp(2 pi i f (tau_i - d_i 435 ps)),
//     tau_i = (x_i sin(za) sin(az) + y_i sin(za) cos(az)) / c;
//   * a ground plane 0.278 m below the dipoles,
//     G = sin(2 pi f h cos(za) / c) / sin(2 pi f h / c);
//   * short-dipole projections onto the sky basis (theta, phi) for the E-W (X)
//     and N-S (Y) dipoles: [[cos za sin az, cos za cos az], [cos az, -sin az]].
//
//   J = AF G [[cos za sin az, cos za cos az], [cos az, -sin az]]   (zenith-normalised)
//
// Parallactic angle (primary_beam.c:436-456, the spherical-triangle identity
// of the reference's doc/Definitions.md): horizon (az, el) -> (ha, dec) at
// latitude lat, chi = atan2(cos lat sin ha, sin lat cos dec - cos lat sin dec
// cos ha), P = [[-cos chi, -sin chi], [sin chi, -cos chi]], B = J P.
#include "beam_model.cuh"
#include "vgb_launch.cuh"

namespace vgb {

// Distinct delay sets, as vmCalcB evaluates the beam once per distinct
// dipole configuration (primary_beam.c:119-160): rep[t] = the first tile with
// tile t's 16 delays, list[k] = the k-th such first tile, count = their number.
// One block; O(ntile^2) comparisons of 16 words, early exit on the first match.
__global__ void beam_configs_kernel(const uint32_t *delays, int ntile, int *rep, int *list, int *count)
{
    __shared__ int s_first[1024];
    __shared__ int s_base;
    if (threadIdx.x == 0) s_base = 0;
    __syncthreads();
    for (int t0 = 0; t0 < ntile; t0 += blockDim.x) {
        const int t = t0 + threadIdx.x;
        int r = t;
        if (t < ntile) {
            const uint4 *dt = reinterpret_cast<const uint4 *>(delays + 16 * (long long)t);
            const uint4 a0 = dt[0], a1 = dt[1], a2 = dt[2], a3 = dt[3];
            for (int u = 0; u < t; u++) {
                const uint4 *du = reinterpret_cast<const uint4 *>(delays + 16 * (long long)u);
                const uint4 b0 = du[0], b1 = du[1], b2 = du[2], b3 = du[3];
                if (a0.x == b0.x && a0.y == b0.y && a0.z == b0.z && a0.w == b0.w && a1.x == b1.x && a1.y == b1.y &&
                    a1.z == b1.z && a1.w == b1.w && a2.x == b2.x && a2.y == b2.y && a2.z == b2.z && a2.w == b2.w &&
                    a3.x == b3.x && a3.y == b3.y && a3.z == b3.z && a3.w == b3.w) {
                    r = u;
                    break;
                }
            }
            rep[t] = r;
        }
        s_first[threadIdx.x] = t < ntile && r == t;
        __syncthreads();
        if (threadIdx.x == 0) { // compact this chunk's first tiles in tile order
            int k = s_base;
            for (int i = 0; i < (int)blockDim.x && t0 + i < ntile; i++)
                if (s_first[i]) list[k++] = t0 + i;
            s_base = k;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *count = s_base;
}

// B for (frequency, pointing, the k-th distinct delay set), written at that
// set's first tile. Threads with k >= count leave at once.
__global__ void beam_model_kernel(const PbArgs a, const int *list, const int *count)
{
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long per_k = (long long)a.nfreq * a.npointing;
    const int k = (int)(idx / per_k);
    if (k >= *count || k >= a.ntile) return;
    const int p = (int)(idx % a.npointing);
    const int fi = (int)((idx / a.npointing) % a.nfreq);
    const int t = list[k];
    double2 J[4];
    bm_jones(a.az[p], a.za[p], a.freq[fi], a.delays + 16 * (long long)t, J);
    double2 *o = a.B + 4 * (((long long)fi * a.npointing + p) * a.ntile + t);
    if (!a.pa) {
        for (int e = 0; e < 4; e++) o[e] = J[e];
        return;
    }
    double P[4];
    bm_pa(a.lat, a.az[p], a.za[p], P);
    // B = J P (complex x real, as mult2x2d_CxR)
    o[0] = make_double2(J[0].x * P[0] + J[1].x * P[2], J[0].y * P[0] + J[1].y * P[2]);
    o[1] = make_double2(J[0].x * P[1] + J[1].x * P[3], J[0].y * P[1] + J[1].y * P[3]);
    o[2] = make_double2(J[2].x * P[0] + J[3].x * P[2], J[2].y * P[0] + J[3].y * P[2]);
    o[3] = make_double2(J[2].x * P[1] + J[3].x * P[3], J[2].y * P[1] + J[3].y * P[3]);
}

// Every other tile copies its set's matrix (32 bytes per thread, two uint4).
__global__ void beam_expand_kernel(const PbArgs a, const int *rep)
{
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long n = (long long)a.nfreq * a.npointing * a.ntile;
    if (idx >= n) return;
    const int t = (int)(idx % a.ntile);
    const int r = rep[t];
    if (r == t) return;
    const uint4 *src = reinterpret_cast<const uint4 *>(a.B + 4 * (idx - t + r));
    uint4 *dst = reinterpret_cast<uint4 *>(a.B + 4 * idx);
    dst[0] = src[0];
    dst[1] = src[1];
    dst[2] = src[2];
    dst[3] = src[3];
}

int launch_beam_model(const PbArgs &a, cudaStream_t st, int *given)
{
    const long long n = (long long)a.nfreq * a.npointing * a.ntile;
    if (n <= 0) return VGB_SUCCESS;
    int *scratch = given; // rep [ntile], list [ntile], count
    int rc = VGB_SUCCESS;
    if (!given)
        rc = check_cuda(cudaMallocAsync(reinterpret_cast<void **>(&scratch), (2 * (size_t)a.ntile + 1) * sizeof(int),
                                        st),
                        "cudaMallocAsync(beam configurations)");
    if (rc) return rc;
    int *rep = scratch, *list = scratch + a.ntile, *count = scratch + 2 * a.ntile;
    beam_configs_kernel<<<1, 1024, 0, st>>>(a.delays, a.ntile, rep, list, count);
    rc = check_launch("beam_configs_kernel");
    if (!rc) {
        beam_model_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(a, list, count);
        rc = check_launch("beam_model_kernel");
    }
    if (!rc) {
        beam_expand_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(a, rep);
        rc = check_launch("beam_expand_kernel");
    }
    if (given) return rc;
    const int rf = check_cuda(cudaFreeAsync(scratch, st), "cudaFreeAsync(beam configurations)");
    return rc ? rc : rf;
}

} // namespace vgb

using namespace vgb;

// primary_beam.c:355-414: index of a live/dead dipole pattern among the 138
// cached configurations (0 all live, 1-16 one dead, 17-136 two dead, 137 all
// dead), or -1 for more than two (but not all) dead.
extern "C" int vgb_hash_dipole_config(const double *amps)
{
    if (!amps) {
        set_error(VGB_ERR_INVALID, "hash_dipole_config: NULL amps");
        return -2;
    }
    int dead[16], ndead = 0;
    for (int i = 0; i < 16; i++)
        if (amps[i] == 0.0) dead[ndead++] = i;
    switch (ndead) {
    case 0: return 0;
    case 1: return dead[0] + 1;
    case 2: return 16 * dead[0] - ((dead[0] + 2) * (dead[0] + 1)) / 2 + dead[1] + 17;
    case 16: return 137;
    default: return -1;
    }
}

extern "C" int vgb_primary_beam(const double *az, const double *za, int npointing, const double *freq_hz, int nfreq,
                                const uint32_t *delays, int ntile, double latitude, int pa_correction, void *B,
                                void *stream)
{
    if (!az || !za || !freq_hz || !delays || !B) return set_error(VGB_ERR_INVALID, "primary_beam: NULL argument");
    if (npointing <= 0 || nfreq <= 0 || ntile <= 0) return set_error(VGB_ERR_INVALID, "primary_beam: empty shape");
    if ((reinterpret_cast<uintptr_t>(delays) | reinterpret_cast<uintptr_t>(B)) & 15)
        return set_error(VGB_ERR_INVALID, "primary_beam: delays and B must be 16-byte aligned");
    PbArgs a{az, za, npointing, freq_hz, nfreq, delays, ntile, latitude, pa_correction, static_cast<double2 *>(B)};
    return launch_beam_model(a, static_cast<cudaStream_t>(stream));
}
