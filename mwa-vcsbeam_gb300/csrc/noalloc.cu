// An entry point that allocates no memory: MWAX voltages to 8-bit PSRFITS
// bytes (fused PFB + beamformer, then the per-channel renormalise), with the
// full-resolution Stokes that pass between the two kernels kept in a
// fixed-size array in the library's own device memory.
//
// It exists for callers that cannot allocate device memory while they run:
// a real-time observing pipeline that reserves all GPU memory when it starts
// and must not fail or stall on an allocation mid-observation, or code
// running where allocation calls are not permitted. Such callers still pass
// every input and output buffer; this call adds no allocation of its own.
#include "vgb_launch.cuh"

namespace vgb {

// The scratch holds npointing(=1) x ncc x nspectra x nstokes x 128 floats:
// 24 MiB, one full-Stokes second of one coarse channel (20.48 MB). Every GPU
// that loads the library holds this array until the process exits.
constexpr long long kNoAllocMaxFloats = (24ll << 20) / 4;
static __device__ __align__(256) float g_noalloc_stokes[kNoAllocMaxFloats];

// Device address of the array, looked up once per device with that device
// current (in host code the symbol is only a host-side stand-in).
static float *noalloc_scratch(int *rc)
{
    static float *ptrs[64] = {};
    int dev = 0;
    *rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (*rc) return nullptr;
    if (dev < 0 || dev >= 64) {
        *rc = set_error(VGB_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
        return nullptr;
    }
    if (!ptrs[dev]) {
        void *p = nullptr;
        *rc = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_stokes), "cudaGetSymbolAddress(scratch)");
        if (*rc) return nullptr;
        ptrs[dev] = static_cast<float *>(p);
    }
    return ptrs[dev];
}

} // namespace vgb

using namespace vgb;

extern "C" int vgb_beamform_mwax_psrfits_noalloc(const vgb_voltages *v, int ncc, int nspectra, const int32_t *filter,
                                                 int ntaps, int nchan, unsigned pfb_flags, const void *W, int nant,
                                                 float invw, int nstokes, uint8_t *out, float *offsets,
                                                 float *scales, void *stream)
{
    if (ncc <= 0 || nspectra < 0 || (nstokes != 1 && nstokes != 4) || nchan != kK)
        return set_error(VGB_ERR_INVALID, "noalloc: bad sizes (ncc %d, nspectra %d, nstokes %d, nchan %d)", ncc,
                         nspectra, nstokes, nchan);
    const long long need = (long long)ncc * nspectra * nstokes * kK;
    if (need > kNoAllocMaxFloats)
        return set_error(VGB_ERR_INVALID,
                         "noalloc: %lld Stokes values (ncc %d x nspectra %d x nstokes %d x 128) exceed the "
                         "static scratch of %lld (24 MiB)",
                         need, ncc, nspectra, nstokes, kNoAllocMaxFloats);
    if (!out || !offsets || !scales) return set_error(VGB_ERR_INVALID, "noalloc: NULL output");
    int rc = VGB_SUCCESS;
    float *S = noalloc_scratch(&rc);
    if (rc) return rc;
    // Every element the renormalise reads is written by the beamformer first,
    // so no part of the scratch needs clearing between calls.
    rc = vgb_beamform_mwax(v, ncc, nspectra, filter, ntaps, nchan, pfb_flags, W, nant, invw, nstokes, S, nullptr,
                           nullptr, stream);
    if (rc) return rc;
    const long long per_cc = (long long)nspectra * nstokes * kK;
    return vgb_renormalise(S, ncc, 1, nspectra, nstokes, kK, out, per_cc, 0, (long long)nstokes * kK, kK, offsets,
                           scales, stream);
}
