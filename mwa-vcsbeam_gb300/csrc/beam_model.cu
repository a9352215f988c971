// Primary-beam matrices B [pointing][tile][2][2] (vmCalcB,
// primary_beam.c:79-191) on the device, FP64.
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

__global__ void beam_model_kernel(const PbArgs a)
{
    const long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long n = (long long)a.nfreq * a.npointing * a.ntile;
    if (idx >= n) return;
    const int t = idx % a.ntile;
    const int p = (idx / a.ntile) % a.npointing;
    const int fi = idx / ((long long)a.ntile * a.npointing);
    double2 J[4];
    bm_jones(a.az[p], a.za[p], a.freq[fi], a.delays + 16 * t, J);
    double2 *o = a.B + 4 * idx;
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

int launch_beam_model(const PbArgs &a, cudaStream_t st)
{
    const long long n = (long long)a.nfreq * a.npointing * a.ntile;
    if (n <= 0) return VGB_SUCCESS;
    beam_model_kernel<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(a);
    return check_launch("beam_model_kernel");
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
    PbArgs a{az, za, npointing, freq_hz, nfreq, delays, ntile, latitude, pa_correction, static_cast<double2 *>(B)};
    return launch_beam_model(a, static_cast<cudaStream_t>(stream));
}
