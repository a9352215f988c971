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
//
// When the array gets its memory: this file is its own CUDA module, and under
// the default lazy module loading a module is placed on a device the first
// time something in it is used there -- for this array, at the first address
// lookup, i.e. inside the first call on that device. A caller that reserves
// the GPU's memory at start-up must therefore make one call before reserving
// (a call with nspectra = 0 only looks the address up and launches nothing),
// or run with CUDA_MODULE_LOADING=EAGER.
#include <cuda.h>

#include <mutex>
#include <utility>
#include <vector>

#include "vgb_launch.cuh"

namespace vgb {

// The scratch holds npointing(=1) x ncc x nspectra x nstokes x 128 floats:
// 24 MiB, one full-Stokes second of one coarse channel (20.48 MB). Every GPU
// that loads the library holds this array until the process exits.
constexpr long long kNoAllocMaxFloats = (24ll << 20) / 4;
static __device__ __align__(256) float g_noalloc_stokes[kNoAllocMaxFloats];

// Device address of the array in the current context (in host code the
// symbol is only a host-side stand-in). Outside stream capture it is looked
// up on every call, with the caller's device current, so a reset device or a
// different context never sees a stale address; the lookup is a host-side
// call. While `st` is being captured the address recorded for this context by
// an earlier call is used, so the first call must come before any capture.
static CUcontext current_context()
{
    // Through the runtime's entry-point query, so the library needs no link
    // to the driver library at load time (as the tensor-map encoder does).
    using Fn = CUresult (*)(CUcontext *);
    static Fn fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 4000, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<Fn>(p);
    }();
    CUcontext ctx = nullptr;
    if (!fn || fn(&ctx) != CUDA_SUCCESS) ctx = nullptr;
    return ctx;
}

static float *noalloc_scratch(cudaStream_t st, int *rc)
{
    static std::mutex mu;
    static std::vector<std::pair<CUcontext, float *>> seen;
    CUcontext ctx = current_context();
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    *rc = check_cuda(cudaStreamIsCapturing(st, &cs), "cudaStreamIsCapturing");
    if (*rc) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    if (cs != cudaStreamCaptureStatusNone) {
        for (auto &e : seen)
            if (e.first == ctx && ctx) return e.second;
        *rc = set_error(VGB_ERR_INVALID, "noalloc: first call on this device made during stream capture; "
                                         "call once (nspectra = 0 will do) before capturing");
        return nullptr;
    }
    void *p = nullptr;
    *rc = check_cuda(cudaGetSymbolAddress(&p, g_noalloc_stokes), "cudaGetSymbolAddress(scratch)");
    if (*rc) return nullptr;
    for (auto &e : seen)
        if (e.first == ctx) {
            e.second = static_cast<float *>(p);
            return e.second;
        }
    seen.emplace_back(ctx, static_cast<float *>(p));
    return static_cast<float *>(p);
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
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    int rc = VGB_SUCCESS;
    float *S = noalloc_scratch(st, &rc);
    if (rc) return rc;
    if (nspectra == 0) return VGB_SUCCESS; // set-up call: the array is placed and its address known
    if (!out || !offsets || !scales) return set_error(VGB_ERR_INVALID, "noalloc: NULL output");
    // Every element the renormalise reads is written by the beamformer first,
    // so no part of the scratch needs clearing between calls.
    rc = vgb_beamform_mwax(v, ncc, nspectra, filter, ntaps, nchan, pfb_flags, W, nant, invw, nstokes, S, nullptr,
                           nullptr, stream);
    if (rc) return rc;
    const long long per_cc = (long long)nspectra * nstokes * kK;
    return vgb_renormalise(S, ncc, 1, nspectra, nstokes, kK, out, per_cc, 0, (long long)nstokes * kK, kK, offsets,
                           scales, stream);
}
