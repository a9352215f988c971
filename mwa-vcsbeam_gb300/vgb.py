"""ctypes binding of the GB300 library's C ABI (include/vcsbeam_gb300.h).

The compute lives in ``lib/libvcsbeam_gb300.so`` (CUDA, sm_103a); this module
only marshals arguments. Device buffers are torch tensors (or raw integer
addresses); torch supplies allocation and the current stream, nothing else.
There is no fallback: if the library is missing, every call raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libvcsbeam_gb300.so")

NCHAN = 128
NTAPS = 12
VSPVB = 64000
FRAMES_PER_BLOCK = VSPVB // NCHAN
HIST_FRAMES = NTAPS

PFB_COMPLEX_INT4 = 0x10
PFB_COMPLEX_FLOAT64 = 0x20
PFB_IMAG_PART_FIRST = 0x100
PFB_EMULATE_FPGA = 0x200
PFB_SMART = 0x21D
PFB_FULL_PRECISION = 0x2D
WOLA_FP32 = 0x10000
WOLA_FP32_SPLIT = 0x20000
WOLA_INT32 = 0x40000
INT4 = 0
DBL = 1


class VGBError(RuntimeError):
    pass


class Voltages(ctypes.Structure):
    _fields_ = [
        ("hist", ctypes.c_void_p),
        ("hist_input_stride", ctypes.c_longlong),
        ("hist_cc_stride", ctypes.c_longlong),
        ("cur", ctypes.c_void_p),
        ("cur_block_stride", ctypes.c_longlong),
        ("cur_cc_stride", ctypes.c_longlong),
        ("ninputs", ctypes.c_int),
        ("nblocks", ctypes.c_int),
    ]


class MultibeamConfig(ctypes.Structure):
    _fields_ = [
        ("ncc", ctypes.c_int),
        ("nfine", ctypes.c_int),
        ("nant", ctypes.c_int),
        ("npointing", ctypes.c_int),
        ("nsamples", ctypes.c_int),
        ("nstokes", ctypes.c_int),
        ("precision", ctypes.c_int),
        ("input", ctypes.c_int),
        ("invw", ctypes.c_float),
    ]


MB_SPLIT_BF16, MB_BF16, MB_FP16, MB_FP32 = 0, 1, 2, 3
MB_INT4, MB_INT8 = 0, 1
MB_INT = 10  # samples per integration


class SubfileInfo(ctypes.Structure):
    _fields_ = [("header_bytes", ctypes.c_longlong), ("block_bytes", ctypes.c_longlong),
                ("file_bytes", ctypes.c_longlong), ("obs_id", ctypes.c_longlong), ("subobs_id", ctypes.c_longlong),
                ("ninputs", ctypes.c_int), ("samples_per_block", ctypes.c_int), ("secs_per_subobs", ctypes.c_int),
                ("coarse_channel", ctypes.c_int), ("metadata_blocks", ctypes.c_int), ("complete", ctypes.c_int)]


class PipelineConfig(ctypes.Structure):
    _fields_ = [
        ("ncc", ctypes.c_int),
        ("nant", ctypes.c_int),
        ("nblocks", ctypes.c_int),
        ("nstokes", ctypes.c_int),
        ("pfb_flags", ctypes.c_uint),
        ("do_ipfb", ctypes.c_int),
        ("invw", ctypes.c_float),
    ]


class Tracking(ctypes.Structure):
    """vgb_tracking: device tables the pipeline rebuilds W from every second."""
    _fields_ = [
        ("D", ctypes.c_void_p),
        ("delays", ctypes.c_void_p),
        ("east", ctypes.c_void_p),
        ("north", ctypes.c_void_p),
        ("height", ctypes.c_void_p),
        ("cable", ctypes.c_void_p),
        ("chan_freqs_hz", ctypes.c_void_p),
        ("beam_freqs_hz", ctypes.c_void_p),
        ("az", ctypes.c_void_p),
        ("za", ctypes.c_void_p),
        ("nseconds", ctypes.c_int),
        ("pa_correction", ctypes.c_int),
        ("href", ctypes.c_double),
        ("latitude", ctypes.c_double),
    ]


_lib = None
V = ctypes.c_void_p
I = ctypes.c_int
LL = ctypes.c_longlong
U = ctypes.c_uint
Fl = ctypes.c_float
Db = ctypes.c_double

_SIGS = {
    "vgb_last_error": (ctypes.c_char_p, []),
    "vgb_version": (I, []),
    "vgb_filter_fp32_exact": (I, [V, I, I]),
    "vgb_filter_wola_flags": (U, [V, I, I]),
    "vgb_check_device_status": (I, [V, ctypes.POINTER(U)]),
    "vgb_beamform_mwax": (I, [ctypes.POINTER(Voltages), I, I, V, I, I, U, V, I, Fl, I, V, V, V, V]),
    "vgb_fpfb": (I, [ctypes.POINTER(Voltages), I, I, V, I, I, V, U, V, V]),
    "vgb_wola": (I, [ctypes.POINTER(Voltages), I, V, I, I, V, V]),
    "vgb_round": (I, [V, LL, I, V]),
    "vgb_fft128": (I, [V, LL, V]),
    "vgb_pack": (I, [V, I, I, V, U, V, V]),
    "vgb_phase": (I, [V, V, V, V, V, V, I, I, I, Db, V, V]),
    "vgb_jones": (I, [V, V, I, I, I, V, V]),
    "vgb_weights": (I, [V, V, LL, V, V]),
    "vgb_beamform_legacy": (I, [V, I, I, I, I, V, V, V, I, Fl, I, V, V, V, V]),
    "vgb_incoh_beam": (I, [V, LL, I, V, V]),
    "vgb_renormalise": (I, [V, I, I, I, I, I, V, LL, LL, LL, LL, V, V, V]),
    "vgb_ipfb": (I, [V, LL, V, LL, V, I, I, I, I, V, V, V, I, V]),
    "vgb_pfb_variant_last": (I, []),
    "vgb_vdif_header_create": (I, [V, I, I, I, I, I, ctypes.c_char_p]),
    "vgb_vdif_header_set_epoch_mjd": (I, [V, I]),
    "vgb_vdif_header_epoch_mjd": (I, [V, ctypes.POINTER(I)]),
    "vgb_vdif_header_set_mjdsec": (I, [V, LL]),
    "vgb_vdif_header_set_frame": (I, [V, I]),
    "vgb_vdif_header_next": (I, [V, I]),
    "vgb_vdif_populate_header": (I, [V, I, Db, I, ctypes.c_char_p]),
    "vgb_vdif_advance": (I, [V, I, I, V]),
    "vgb_subfile_info_read": (I, [ctypes.c_char_p, ctypes.POINTER(SubfileInfo)]),
    "vgb_subfile_read_second": (I, [ctypes.c_char_p, LL, V, LL, I]),
    "vgb_legacy_read_second": (I, [ctypes.c_char_p, V, LL, I]),
    "vgb_volt_filename": (I, [ctypes.c_char_p, I, LL, LL, I, I]),
    "vgb_beamform_mwax_psrfits_noalloc": (I, [ctypes.POINTER(Voltages), I, I, V, I, I, U, V, I, Fl, I, V, V, V,
                                              V]),
    "vgb_gemm_bf16": (I, [V, V, V, I, I, I, V]),
    "vgb_cal_load_offringa": (I, [ctypes.c_char_p, I, I, I, I, I, V, V]),
    "vgb_cal_load_rts": (I, [ctypes.c_char_p, ctypes.c_char_p, I, I, I, V, I, I, V]),
    "vgb_cal_apply_corrections": (I, [V, I, I, I, I, ctypes.c_double, ctypes.c_double, LL, I]),
    "vgb_cal_pq_correction": (I, [ctypes.c_char_p, ctypes.c_uint32, V, V, V, I, V]),
    "vgb_cal_flag_tiles": (I, [V, I, I, V, I]),
    "vgb_load_filter": (I, [ctypes.c_char_p, I, ctypes.c_double, V, I, V, V]),
    "vgb_primary_beam": (I, [V, V, I, V, I, V, I, ctypes.c_double, I, V, V]),
    "vgb_hash_dipole_config": (I, [V]),
    "vgb_surrogate_create": (I, [I, I, ctypes.c_ulonglong, V]),
    "vgb_surrogate_destroy": (None, [V]),
    "vgb_surrogate_param_count": (I, [V]),
    "vgb_surrogate_get_params": (I, [V, V, I]),
    "vgb_surrogate_set_params": (I, [V, V, I]),
    "vgb_surrogate_set_training": (I, [V, V, V, I, I, ctypes.c_ulonglong]),
    "vgb_surrogate_train": (I, [V, I, Fl, Fl, V]),
    "vgb_surrogate_gradients": (I, [V, V, V, V, V, V]),
    "vgb_surrogate_validate": (I, [V, LL, Fl, V, V]),
    "vgb_surrogate_beam": (I, [V, V, V, I, V, I, V, V, I, ctypes.c_double, I, V, V, V]),
    "vgb_array_factor": (I, [V, V, I, ctypes.c_double, V, V, V, V, ctypes.c_double, I, V, V]),
    "vgb_multibeam_create": (I, [V, V]),
    "vgb_multibeam_destroy": (None, [V]),
    "vgb_multibeam_set_geometry": (I, [V, V, V, V, V, V, ctypes.c_double, V]),
    "vgb_multibeam_set_jones": (I, [V, V, V, V, V, V, V]),
    "vgb_multibeam_run": (I, [V, V, V, V, V, V, V]),
    "vgb_multibeam_run_host": (I, [V, V, V, V, V, V]),
    "vgb_multibeam_launches": (I, [V]),
    "vgb_multibeam_beam_variant": (I, [I]),
    "vgb_multibeam_last_pair": (I, [V]),
    "vgb_multibeam_enable_timing": (I, [V, I]),
    "vgb_multibeam_stage_ms": (I, [V, V, I]),
    "vgb_gemm_batched": (I, [V, V, V, I, I, I, I, I, V]),
    "vgb_gemm_batched_planes": (I, [V, V, V, I, I, I, I, I, V]),
    "vgb_gemm_variant": (I, [I]),
    "vgb_pfb_variant": (I, [I]),
    "vgb_pipeline_create": (I, [ctypes.POINTER(PipelineConfig), ctypes.POINTER(V)]),
    "vgb_pipeline_destroy": (I, [V]),
    "vgb_pipeline_set_filters": (I, [V, V, V]),
    "vgb_pipeline_set_weights": (I, [V, V, I]),
    "vgb_pipeline_set_vdif_header": (I, [V, V]),
    "vgb_pipeline_set_tracking": (I, [V, ctypes.POINTER(Tracking)]),
    "vgb_splice_psrfits": (I, [V, I, I, I, I, I, I, V]),
    "vgb_fp32_peak": (I, [I, I, ctypes.POINTER(ctypes.c_double), V]),
    "vgb_pipeline_run_device": (I, [V, V, LL]),
    "vgb_pipeline_run_host": (I, [V, V, LL]),
    "vgb_pipeline_fetch": (I, [V, V, V, V, V]),
    "vgb_pipeline_fetch_raw": (I, [V, V, V, V]),
    "vgb_pipeline_fetch_incoh": (I, [V, V, V, V]),
    "vgb_pipeline_set_host_incoh": (I, [V, V, V, V]),
    "vgb_pipeline_device_products": (I, [V, ctypes.POINTER(V), ctypes.POINTER(V), ctypes.POINTER(V),
                                         ctypes.POINTER(V), ctypes.POINTER(V)]),
    "vgb_pipeline_launch_count": (I, [V]),
    "vgb_pipeline_stream": (V, [V]),
    "vgb_pipeline_set_host_outputs": (I, [V, V, V, V, V]),
    "vgb_pipeline_sync": (I, [V]),
    "vgb_pipeline_enable_timing": (I, [V, I]),
    "vgb_pipeline_enable_graphs": (I, [V, I]),
    "vgb_pipeline_state_bytes": (LL, [V]),
    "vgb_pipeline_save_state": (I, [V, V, LL]),
    "vgb_pipeline_load_state": (I, [V, V, LL]),
    "vgb_selftest_bounded_wait": (I, [I, V]),
    "vgb_pipeline_stage_ms": (I, [V, ctypes.POINTER(Fl), I]),
}


def exported_symbols():
    """Names the C ABI exports (the header's declarations)."""
    return list(_SIGS)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise VGBError(f"{LIB_PATH} is not built; run __graft_entry__.build()")
        l = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            fn = getattr(l, name)
            fn.restype = res
            fn.argtypes = args
        _lib = l
    return _lib


def check(rc: int):
    if rc != 0:
        raise VGBError(f"vgb error {rc}: {lib().vgb_last_error().decode()}")


def ptr(x):
    """Device (or host) address of a torch tensor / numpy array / int / None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        return x.ctypes.data
    return x.data_ptr()


def stream_ptr(stream=None):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return s.cuda_stream


# --------------------------------------------------------------------------
# voltage descriptors
# --------------------------------------------------------------------------

def reference_buffer_voltages(buf, ninputs: int, nblocks: int, ncc: int = 1, cc_stride: int = 0) -> Voltages:
    """The reference's read buffer: one margin block then `nblocks` blocks
    (buffer.c:52-77). `buf` is a device tensor or address."""
    base = ptr(buf)
    block = ninputs * VSPVB * 2
    return Voltages(hist=base + (FRAMES_PER_BLOCK - HIST_FRAMES) * NCHAN * 2, hist_input_stride=VSPVB * 2,
                    hist_cc_stride=cc_stride, cur=base + block, cur_block_stride=block, cur_cc_stride=cc_stride,
                    ninputs=ninputs, nblocks=nblocks)


# --------------------------------------------------------------------------
# thin wrappers (all asynchronous on the given / current stream)
# --------------------------------------------------------------------------

def beamform_mwax(v: Voltages, ncc, nspectra, filt, flags, W, nant, invw, nstokes, S, e=None, incoh=None,
                  stream=None):
    check(lib().vgb_beamform_mwax(ctypes.byref(v), ncc, nspectra, ptr(filt), NTAPS, NCHAN, flags, ptr(W), nant,
                                  float(invw), nstokes, ptr(S), ptr(e), ptr(incoh), stream_ptr(stream)))


def beamform_mwax_psrfits_noalloc(v: Voltages, ncc, nspectra, filt, flags, W, nant, invw, nstokes, out, offsets,
                                  scales, stream=None):
    """Voltages to PSRFITS bytes with no allocation (a fixed 24 MiB array in
    the library holds the intermediate Stokes; see the C header)."""
    check(lib().vgb_beamform_mwax_psrfits_noalloc(ctypes.byref(v), ncc, nspectra, ptr(filt), NTAPS, NCHAN, flags,
                                                  ptr(W), nant, float(invw), nstokes, ptr(out), ptr(offsets),
                                                  ptr(scales), stream_ptr(stream)))


def gemm_bf16(A, B, C, M, N, K, stream=None):
    """C[M][N] = A[M][K] @ B[N][K]^T on the tensor cores (bf16 in, FP32 out)."""
    check(lib().vgb_gemm_bf16(ptr(A), ptr(B), ptr(C), M, N, K, stream_ptr(stream)))


def multibeam_beam_variant(v: int) -> int:
    """Force the many-beam GEMM kernel (0 automatic, 1 single CTA, 2 CTA
    pairs); returns the previous setting."""
    prev = lib().vgb_multibeam_beam_variant(v)
    if prev < 0:
        raise VGBError(lib().vgb_last_error().decode())
    return prev


def gemm_variant(v: int) -> int:
    """Force a GEMM kernel variant (0 autotuned, 128, 256, 512 persistent)."""
    prev = lib().vgb_gemm_variant(v)
    if prev < 0:
        raise VGBError(lib().vgb_last_error().decode())
    return prev


def pfb_variant(g: int) -> int:
    """Force the fused front end's variant (4 or 8 inputs per step, 5 the
    4-input shape at three CTAs per SM, 3 the warp-specialised kernel; 0 =
    timed choice)."""
    prev = lib().vgb_pfb_variant(g)
    if prev < 0:
        raise VGBError(lib().vgb_last_error().decode())
    return prev


def pfb_variant_last() -> int:
    """Variant of the last fused front-end launch (4, 8, 5 or 3; 0 before any)."""
    return lib().vgb_pfb_variant_last()


def gemm_batched(A, B, C, M, N, K, batch, fp16=False, stream=None):
    """C[b] = A[b] @ B[b]^T for b < batch (bf16, or fp16 operands; FP32 out)."""
    check(lib().vgb_gemm_batched(ptr(A), ptr(B), ptr(C), M, N, K, batch, int(bool(fp16)), stream_ptr(stream)))


def gemm_batched_planes(A, B, C, M, N, K, batch, fp16=False, stream=None):
    """C[b] = (A[b][:, :K] + A[b][:, K:]) @ B[b]^T, A rows 2K wide (split operand)."""
    check(lib().vgb_gemm_batched_planes(ptr(A), ptr(B), ptr(C), M, N, K, batch, int(bool(fp16)),
                                        stream_ptr(stream)))


def fpfb(v: Voltages, ncc, nspectra, filt, i_idx, flags, out, stream=None):
    check(lib().vgb_fpfb(ctypes.byref(v), ncc, nspectra, ptr(filt), NTAPS, NCHAN, ptr(i_idx), flags, ptr(out),
                         stream_ptr(stream)))


def wola(v: Voltages, nspectra, filt, b, stream=None):
    check(lib().vgb_wola(ctypes.byref(v), nspectra, ptr(filt), NTAPS, NCHAN, ptr(b), stream_ptr(stream)))


def round_(b, nvalues, emulate_fpga, stream=None):
    check(lib().vgb_round(ptr(b), nvalues, int(emulate_fpga), stream_ptr(stream)))


def fft128(rows, nrows, stream=None):
    check(lib().vgb_fft128(ptr(rows), nrows, stream_ptr(stream)))


def pack(ffted, nspectra, ninputs, i_idx, flags, out, stream=None):
    check(lib().vgb_pack(ptr(ffted), nspectra, ninputs, ptr(i_idx), flags, ptr(out), stream_ptr(stream)))


def phase(unit, east, north, height, cable, freqs, npointing, nant, nchan, href, phi, stream=None):
    check(lib().vgb_phase(ptr(unit), ptr(east), ptr(north), ptr(height), ptr(cable), ptr(freqs), npointing, nant,
                          nchan, float(href), ptr(phi), stream_ptr(stream)))


def jones(D, B, npointing, nant, nchan, J, stream=None):
    check(lib().vgb_jones(ptr(D), ptr(B), npointing, nant, nchan, ptr(J), stream_ptr(stream)))


def weights(J, phi, n, W, stream=None):
    check(lib().vgb_weights(ptr(J), ptr(phi), n, ptr(W), stream_ptr(stream)))


def beamform_legacy(v, datatype, nsamples, nchan, nant, polQ, polP, W, npointing, invw, nstokes, S, e=None,
                    incoh=None, stream=None):
    check(lib().vgb_beamform_legacy(ptr(v), datatype, nsamples, nchan, nant, ptr(polQ), ptr(polP), ptr(W),
                                    npointing, float(invw), nstokes, ptr(S), ptr(e), ptr(incoh),
                                    stream_ptr(stream)))


def incoh_beam(data, nrows, ninput, out, stream=None):
    check(lib().vgb_incoh_beam(ptr(data), nrows, ninput, ptr(out), stream_ptr(stream)))


def renormalise(S, ncc, npointing, nstep, nstokes, nchan, out, out_cc, out_p, out_s, out_st, offsets, scales,
                stream=None):
    check(lib().vgb_renormalise(ptr(S), ncc, npointing, nstep, nstokes, nchan, ptr(out), out_cc, out_p, out_s,
                                out_st, ptr(offsets), ptr(scales), stream_ptr(stream)))


def ipfb(e, e_job_stride, hist, hist_job_stride, coeffs, nsamples, njobs, out_f=None, vdif=None, hdr=None,
         frame_offset=0, stream=None):
    check(lib().vgb_ipfb(ptr(e), e_job_stride, ptr(hist), hist_job_stride, ptr(coeffs), NTAPS, NCHAN, nsamples,
                         njobs, ptr(out_f), ptr(vdif), ptr(hdr), frame_offset, stream_ptr(stream)))


VDIF_FRAMES_PER_SECOND = 10000


def _hdr_buf(hdr):
    if hdr is None:
        hdr = np.zeros(8, np.uint32)
    if not (isinstance(hdr, np.ndarray) and hdr.dtype == np.uint32 and hdr.flags.c_contiguous and hdr.size == 8):
        raise VGBError("a VDIF header is a contiguous uint32 array of 8 words")
    return hdr


def vdif_header_create(dataarraylength=512, threadid=0, bits=8, nchan=2, iscomplex=True, stationid="mw"):
    """createVDIFHeader: a new 8-word header (see the C header)."""
    hdr = np.zeros(8, np.uint32)
    check(lib().vgb_vdif_header_create(hdr.ctypes.data, dataarraylength, threadid, bits, nchan, int(iscomplex),
                                       stationid.encode()))
    return hdr


def vdif_header_set_epoch_mjd(hdr, mjd):
    check(lib().vgb_vdif_header_set_epoch_mjd(_hdr_buf(hdr).ctypes.data, int(mjd)))


def vdif_header_epoch_mjd(hdr):
    out = I()
    check(lib().vgb_vdif_header_epoch_mjd(_hdr_buf(hdr).ctypes.data, ctypes.byref(out)))
    return out.value


def vdif_header_set_mjdsec(hdr, mjdsec):
    check(lib().vgb_vdif_header_set_mjdsec(_hdr_buf(hdr).ctypes.data, int(mjdsec)))


def vdif_header_set_frame(hdr, frame):
    check(lib().vgb_vdif_header_set_frame(_hdr_buf(hdr).ctypes.data, int(frame)))


def vdif_header_next(hdr, frames_per_second=VDIF_FRAMES_PER_SECOND):
    check(lib().vgb_vdif_header_next(_hdr_buf(hdr).ctypes.data, int(frames_per_second)))


def vdif_populate_header(intmjd, fracmjd, threadid=0, stationid="mw"):
    """The header vmPopulateVDIFHeader gives a beam's first frame."""
    hdr = np.zeros(8, np.uint32)
    check(lib().vgb_vdif_populate_header(hdr.ctypes.data, int(intmjd), float(fracmjd), threadid,
                                         None if stationid is None else stationid.encode()))
    return hdr


def vdif_advance(d_hdr, njobs, nframes, stream=None):
    """Advance device header templates [njobs][8] by nframes frames."""
    check(lib().vgb_vdif_advance(ptr(d_hdr), njobs, nframes, stream_ptr(stream)))


def _nbytes(buf):
    if isinstance(buf, np.ndarray):
        return buf.nbytes
    return buf.numel() * buf.element_size()


def subfile_info(path):
    """Header fields of an MWAX voltage subfile (see the C header)."""
    info = SubfileInfo()
    check(lib().vgb_subfile_info_read(os.fsencode(path), ctypes.byref(info)))
    return {name: getattr(info, name) for name, _ in SubfileInfo._fields_}


def subfile_read_second(path, gps_second, dst, nthreads=4):
    """One second ([20 blocks][inputs][64000] char2) of a subfile into dst (host)."""
    check(lib().vgb_subfile_read_second(os.fsencode(path), int(gps_second), ptr(dst), _nbytes(dst), nthreads))


def legacy_read_second(path, dst, nthreads=4):
    check(lib().vgb_legacy_read_second(os.fsencode(path), ptr(dst), _nbytes(dst), nthreads))


def volt_filename(obs_id, gps_second, rec_chan, mwax=True):
    buf = ctypes.create_string_buffer(256)
    check(lib().vgb_volt_filename(buf, 256, int(obs_id), int(gps_second), int(rec_chan), int(mwax)))
    return buf.value.decode()


def selftest_bounded_wait(polls=1000, stream=None):
    """Make one bounded mbarrier wait expire on purpose (see the C header)."""
    check(lib().vgb_selftest_bounded_wait(polls, stream_ptr(stream)))


def check_device_status(stream=None) -> int:
    flags = U(0)
    rc = lib().vgb_check_device_status(stream_ptr(stream), ctypes.byref(flags))
    check(rc)
    return flags.value


def filter_fp32_exact(h: np.ndarray) -> bool:
    h = np.ascontiguousarray(h, dtype=np.int32)
    return bool(lib().vgb_filter_fp32_exact(h.ctypes.data, NTAPS, NCHAN))


def filter_wola_flags(h: np.ndarray) -> int:
    """WOLA_FP32, WOLA_FP32_SPLIT or 0 (int32): the fastest exact weighted
    overlap-add arithmetic for analysis filter h."""
    h = np.ascontiguousarray(h, dtype=np.int32)
    return int(lib().vgb_filter_wola_flags(h.ctypes.data, NTAPS, NCHAN))


# --------------------------------------------------------------------------
# pipeline
# --------------------------------------------------------------------------

# --------------------------------------------------------------------------
# table inputs on the host (calibration solutions, filter files)
# --------------------------------------------------------------------------
def _enc(p):
    return None if p is None else os.fsencode(p)


def cal_load_offringa(path, coarse_chan_idx, ncc, nant, nchan_cal, nfine):
    """D complex128 [nant][nfine][2][2] and the header counts."""
    D = np.zeros((nant, nfine, 2, 2), dtype=np.complex128)
    counts = np.zeros(4, dtype=np.uint32)
    check(lib().vgb_cal_load_offringa(_enc(path), coarse_chan_idx, ncc, nant, nchan_cal, nfine, D.ctypes.data,
                                      counts.ctypes.data))
    return D, counts


def cal_load_rts(dijones_path, bandpass_path, nant_cal, nchan_cal, chan_width_hz, cal_ant, nfine):
    cal_ant = np.ascontiguousarray(cal_ant, dtype=np.int32)
    D = np.zeros((cal_ant.size, nfine, 2, 2), dtype=np.complex128)
    check(lib().vgb_cal_load_rts(_enc(dijones_path), _enc(bandpass_path), nant_cal, nchan_cal, chan_width_hz,
                                 cal_ant.ctypes.data, cal_ant.size, nfine, D.ctypes.data))
    return D


def cal_apply_corrections(D, ref_ant=-1, keep_cross_terms=False, phase_slope=0.0, phase_offset=0.0,
                          chan_start_hz=0, coarse_chan_width_hz=1280000):
    """In place on a C-contiguous complex128 [nant][nfine][2][2] array."""
    assert D.dtype == np.complex128 and D.flags.c_contiguous
    check(lib().vgb_cal_apply_corrections(D.ctypes.data, D.shape[0], D.shape[1], int(ref_ant),
                                          int(bool(keep_cross_terms)), float(phase_slope), float(phase_offset),
                                          int(chan_start_hz), int(coarse_chan_width_hz)))
    return D


def cal_pq_correction(path, gpstime):
    slope, offset = ctypes.c_double(0.0), ctypes.c_double(0.0)
    found = ctypes.c_int(0)
    name = ctypes.create_string_buffer(32)
    check(lib().vgb_cal_pq_correction(_enc(path), gpstime, ctypes.byref(slope), ctypes.byref(offset), name, 32,
                                      ctypes.byref(found)))
    return bool(found.value), slope.value, offset.value, name.value.decode()


def cal_flag_tiles(D, ants):
    ants = np.ascontiguousarray(ants, dtype=np.int32)
    assert D.dtype == np.complex128 and D.flags.c_contiguous
    check(lib().vgb_cal_flag_tiles(D.ctypes.data, D.shape[0], D.shape[1], ants.ctypes.data, ants.size))
    return D


def load_filter(path, nchans=NCHAN, scale=1.0):
    """(coefficients float64, ntaps) from an ASCII filter file."""
    n, t = ctypes.c_int(0), ctypes.c_int(0)
    check(lib().vgb_load_filter(_enc(path), nchans, float(scale), None, 0, ctypes.byref(n), ctypes.byref(t)))
    out = np.empty(n.value, dtype=np.float64)
    check(lib().vgb_load_filter(_enc(path), nchans, float(scale), out.ctypes.data, out.size, ctypes.byref(n),
                                ctypes.byref(t)))
    return out, t.value


MWA_LATITUDE_RADIANS = -0.4660608448386394


def primary_beam(az, za, freq_hz, delays, B, pa_correction=True, latitude=MWA_LATITUDE_RADIANS, stream=None):
    """B [nfreq][npointing][ntile][2][2] complex (float64 device tensor view)."""
    check(lib().vgb_primary_beam(ptr(az), ptr(za), int(az.numel()), ptr(freq_hz), int(freq_hz.numel()),
                                 ptr(delays), int(delays.numel() // 16), float(latitude), int(bool(pa_correction)),
                                 ptr(B), stream_ptr(stream)))


def array_factor(look, dirs, freq_hz, east, north, height, cable, out, href=377.827, stream=None):
    """Tied-array array factor of `look` at each of `dirs` (device tensors)."""
    check(lib().vgb_array_factor(ptr(look), ptr(dirs), int(dirs.numel() // 3), float(freq_hz), ptr(east), ptr(north),
                                 ptr(height), ptr(cable), float(href), int(east.numel()), ptr(out),
                                 stream_ptr(stream)))


def hash_dipole_config(amps) -> int:
    a = np.ascontiguousarray(amps, dtype=np.float64)
    return lib().vgb_hash_dipole_config(a.ctypes.data)


class Surrogate:
    """The learned primary-beam surrogate (vgb_surrogate_*)."""

    def __init__(self, nsets, batch=8192, seed=1):
        h = V()
        check(lib().vgb_surrogate_create(nsets, batch, seed, ctypes.byref(h)))
        self.h = h
        self.nsets = nsets
        self.batch = batch
        self.nparams = lib().vgb_surrogate_param_count(h)

    def close(self):
        if self.h:
            lib().vgb_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.empty(self.nparams, dtype=np.float32)
        check(lib().vgb_surrogate_get_params(self.h, out.ctypes.data, out.size))
        return out

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        check(lib().vgb_surrogate_set_params(self.h, p.ctypes.data, p.size))

    def set_training(self, delay_sets, freqs_hz, ndir, seed=7):
        d = np.ascontiguousarray(delay_sets, dtype=np.uint32)
        f = np.ascontiguousarray(freqs_hz, dtype=np.float64)
        check(lib().vgb_surrogate_set_training(self.h, d.ctypes.data, f.ctypes.data, f.size, ndir, seed))

    def train(self, steps, lr_max=1e-3, lr_min=1e-5, want_loss=True):
        loss = np.zeros(max(steps, 1), dtype=np.float32) if want_loss else None
        check(lib().vgb_surrogate_train(self.h, steps, lr_max, lr_min, None if loss is None else loss.ctypes.data))
        return loss

    def gradients(self, feat, sets, y):
        feat = np.ascontiguousarray(feat, dtype=np.float32)
        sets = np.ascontiguousarray(sets, dtype=np.int32)
        y = np.ascontiguousarray(y, dtype=np.float32)
        g = np.empty(self.nparams, dtype=np.float32)
        loss = ctypes.c_float(0.0)
        check(lib().vgb_surrogate_gradients(self.h, feat.ctypes.data, sets.ctypes.data, y.ctypes.data, g.ctypes.data,
                                            ctypes.byref(loss)))
        return g, loss.value

    def validate(self, nval, tol=1e-3):
        mx, frac = ctypes.c_float(0.0), ctypes.c_float(0.0)
        check(lib().vgb_surrogate_validate(self.h, nval, tol, ctypes.byref(mx), ctypes.byref(frac)))
        return mx.value, frac.value

    def beam(self, az, za, freq_hz, tile_set, delays, B, pa_correction=True, latitude=MWA_LATITUDE_RADIANS,
             stream=None):
        nfb = ctypes.c_uint(0)
        check(lib().vgb_surrogate_beam(self.h, ptr(az), ptr(za), int(az.numel()), ptr(freq_hz), int(freq_hz.numel()),
                                       ptr(tile_set), ptr(delays), int(tile_set.numel()), float(latitude),
                                       int(bool(pa_correction)), ptr(B), ctypes.byref(nfb), stream_ptr(stream)))
        return nfb.value


class Multibeam:
    """Many-beam beamformer on the tensor cores (vgb_multibeam_*): tables on
    the device, then voltages -> integrated Stokes (and 8-bit PSRFITS)."""

    def __init__(self, ncc, nfine, nant, npointing, nsamples, nstokes=4, precision=MB_SPLIT_BF16, input=MB_INT4,
                 invw=None):
        cfg = MultibeamConfig(ncc=ncc, nfine=nfine, nant=nant, npointing=npointing, nsamples=nsamples,
                              nstokes=nstokes, precision=precision, input=input,
                              invw=float(invw if invw is not None else 1.0 / (2 * nant)))
        h = V()
        check(lib().vgb_multibeam_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        self.cfg = cfg
        self.nint = nsamples // MB_INT

    def close(self):
        if self.h:
            lib().vgb_multibeam_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_geometry(self, unit, east, north, height, cable, href=0.0, stream=None):
        check(lib().vgb_multibeam_set_geometry(self.h, ptr(unit), ptr(east), ptr(north), ptr(height), ptr(cable),
                                               float(href), stream_ptr(stream)))

    def set_jones(self, D, B, freqs, polQ, polP, stream=None):
        check(lib().vgb_multibeam_set_jones(self.h, ptr(D), ptr(B), ptr(freqs), ptr(polQ), ptr(polP),
                                            stream_ptr(stream)))

    def run(self, v, S=None, out=None, offsets=None, scales=None, stream=None):
        check(lib().vgb_multibeam_run(self.h, ptr(v), ptr(S), ptr(out), ptr(offsets), ptr(scales),
                                      stream_ptr(stream)))

    def run_host(self, v_host, out_host, off_host, scl_host, stream=None):
        """Pinned host tensors in, pinned host tensors out (double-buffered)."""
        check(lib().vgb_multibeam_run_host(self.h, ptr(v_host), ptr(out_host), ptr(off_host), ptr(scl_host),
                                           stream_ptr(stream)))

    def launches(self) -> int:
        return lib().vgb_multibeam_launches(self.h)

    def last_pair(self) -> int:
        """CTA pairs the last run's beam GEMM ran on (0: the single-CTA kernel)."""
        return lib().vgb_multibeam_last_pair(self.h)

    def enable_timing(self, on=True):
        check(lib().vgb_multibeam_enable_timing(self.h, int(bool(on))))

    STAGES = ("weights", "convert", "autocorr_gemm", "beam_gemm", "renormalise")

    def stage_ms(self) -> dict:
        ms = (ctypes.c_float * 5)()
        check(lib().vgb_multibeam_stage_ms(self.h, ms, 5))
        return dict(zip(self.STAGES, [float(x) for x in ms]))


def fp32_peak(packed: bool, iters: int = 20000, stream=None) -> float:
    """This GPU's FP32 FMA throughput in TFLOP/s (FFMA2 when packed)."""
    t = ctypes.c_double()
    check(lib().vgb_fp32_peak(int(packed), iters, ctypes.byref(t), stream_ptr(stream)))
    return t.value


def splice_psrfits(part: np.ndarray, cc_offset: int, ncc_total: int, out: np.ndarray):
    """Place one process's spliced PSRFITS rows part [ns][nstokes][ncc_part*128]
    (uint8, host) at coarse channel cc_offset of out [ns][nstokes][ncc_total*128]."""
    part = np.ascontiguousarray(part, dtype=np.uint8)
    ns, nst, w = part.shape
    if out.shape != (ns, nst, ncc_total * NCHAN) or out.dtype != np.uint8 or not out.flags.c_contiguous:
        raise VGBError("splice_psrfits: out must be contiguous uint8 [ns][nstokes][ncc_total*128]")
    check(lib().vgb_splice_psrfits(part.ctypes.data, ns, nst, NCHAN, w // NCHAN, cc_offset, ncc_total,
                                   out.ctypes.data))


class Pipeline:
    """One second of all coarse channels per step (vgb_pipeline_*)."""

    def __init__(self, ncc, nant, nblocks=20, nstokes=4, pfb_flags=0, do_ipfb=True, invw=None):
        cfg = PipelineConfig(ncc=ncc, nant=nant, nblocks=nblocks, nstokes=nstokes, pfb_flags=pfb_flags,
                             do_ipfb=int(do_ipfb), invw=float(invw if invw is not None else 1.0 / (2 * nant)))
        h = V()
        check(lib().vgb_pipeline_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        self.cfg = cfg
        self.nspectra = nblocks * FRAMES_PER_BLOCK
        self.second_bytes = nblocks * 2 * nant * VSPVB * 2

    def close(self):
        if self.h:
            lib().vgb_pipeline_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_filters(self, analysis: np.ndarray, synthesis: np.ndarray | None):
        a = np.ascontiguousarray(analysis, dtype=np.int32)
        s = None if synthesis is None else np.ascontiguousarray(synthesis, dtype=np.float32)
        check(lib().vgb_pipeline_set_filters(self.h, a.ctypes.data, None if s is None else s.ctypes.data))

    def set_weights(self, W, on_device: bool):
        check(lib().vgb_pipeline_set_weights(self.h, ptr(W), int(on_device)))

    def set_tracking(self, D, delays, east, north, height, cable, chan_freqs_hz, beam_freqs_hz, az, za,
                     href=0.0, latitude=0.0, pa_correction=True):
        """Rebuild W on the device every second from these device tensors
        (vgb_pipeline_set_tracking); az/za hold one pointing per second."""
        self._tracking = (D, delays, east, north, height, cable, chan_freqs_hz, beam_freqs_hz, az, za)
        t = Tracking(D=ptr(D), delays=ptr(delays), east=ptr(east), north=ptr(north), height=ptr(height),
                     cable=ptr(cable), chan_freqs_hz=ptr(chan_freqs_hz), beam_freqs_hz=ptr(beam_freqs_hz),
                     az=ptr(az), za=ptr(za), nseconds=int(az.numel()), pa_correction=int(pa_correction),
                     href=float(href), latitude=float(latitude))
        check(lib().vgb_pipeline_set_tracking(self.h, ctypes.byref(t)))

    def clear_tracking(self):
        check(lib().vgb_pipeline_set_tracking(self.h, None))
        self._tracking = None

    def set_vdif_header(self, hdr: np.ndarray):
        hdr = np.ascontiguousarray(hdr, dtype=np.uint32)
        check(lib().vgb_pipeline_set_vdif_header(self.h, hdr.ctypes.data))

    def run_device(self, d_volt, cc_stride=None):
        check(lib().vgb_pipeline_run_device(self.h, ptr(d_volt), cc_stride or self.second_bytes))

    def run_host(self, h_volt, cc_stride=None):
        check(lib().vgb_pipeline_run_host(self.h, ptr(h_volt), cc_stride or self.second_bytes))

    def fetch(self, psrfits=None, offsets=None, scales=None, vdif=None):
        check(lib().vgb_pipeline_fetch(self.h, ptr(psrfits), ptr(offsets), ptr(scales), ptr(vdif)))

    def fetch_incoh(self, psrfits=None, offsets=None, scales=None):
        """The incoherent beam's 8-bit rows [ns][ncc*128], offsets and scales [ncc][128]."""
        check(lib().vgb_pipeline_fetch_incoh(self.h, ptr(psrfits), ptr(offsets), ptr(scales)))

    def set_host_incoh(self, psrfits=None, offsets=None, scales=None):
        self._host_incoh = (psrfits, offsets, scales)  # keep them alive
        check(lib().vgb_pipeline_set_host_incoh(self.h, ptr(psrfits), ptr(offsets), ptr(scales)))

    def fetch_raw(self, S=None, e=None, incoh=None):
        check(lib().vgb_pipeline_fetch_raw(self.h, ptr(S), ptr(e), ptr(incoh)))

    def device_products(self):
        S, e, inc, ps, vd = V(), V(), V(), V(), V()
        check(lib().vgb_pipeline_device_products(self.h, ctypes.byref(S), ctypes.byref(e), ctypes.byref(inc),
                                                 ctypes.byref(ps), ctypes.byref(vd)))
        return S.value, e.value, inc.value, ps.value, vd.value

    def launch_count(self) -> int:
        return int(lib().vgb_pipeline_launch_count(self.h))

    def stream(self):
        """The pipeline's compute stream as a torch ExternalStream."""
        import torch

        return torch.cuda.ExternalStream(lib().vgb_pipeline_stream(self.h))

    def set_host_outputs(self, psrfits=None, offsets=None, scales=None, vdif=None):
        self._host_outputs = (psrfits, offsets, scales, vdif)  # keep them alive
        check(lib().vgb_pipeline_set_host_outputs(self.h, ptr(psrfits), ptr(offsets), ptr(scales), ptr(vdif)))

    def sync(self):
        check(lib().vgb_pipeline_sync(self.h))

    def enable_timing(self, on: bool = True):
        check(lib().vgb_pipeline_enable_timing(self.h, int(on)))

    def enable_graphs(self, on: bool = True):
        check(lib().vgb_pipeline_enable_graphs(self.h, int(on)))

    def save_state(self) -> np.ndarray:
        """The carry-over state of the next second (for resume)."""
        buf = np.empty(lib().vgb_pipeline_state_bytes(self.h), dtype=np.uint8)
        check(lib().vgb_pipeline_save_state(self.h, buf.ctypes.data, buf.size))
        return buf

    def load_state(self, buf: np.ndarray):
        buf = np.ascontiguousarray(buf, dtype=np.uint8)
        check(lib().vgb_pipeline_load_state(self.h, buf.ctypes.data, buf.size))

    def stage_ms(self, n: int = 4):
        """[PFB + beam, renormalise, IPFB + VDIF, history carry(, tracking tables)] ms."""
        arr = (Fl * n)()
        check(lib().vgb_pipeline_stage_ms(self.h, arr, n))
        return list(arr)
