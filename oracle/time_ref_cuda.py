"""Time the reference's OWN CUDA kernels on one coarse-channel-second.

Test/measurement infrastructure beside the oracle: it drives the unmodified
VCSBeam kernels (oracle/_ref/*.cubin, compiled by oracle/build_ref.sh) through
oracle/ref_harness.cu with the reference's launch shapes, on the workload of
one coarse channel x 1 s x 128 tiles (the unit of the full-band benchmark):

  forward PFB   vmWOLAChunk..vmPackChunk (memset, WOLA, rounding, 8 x cuFFT, pack)
  beamformer    vmApplyJChunk + vmBeamformChunk (1 pointing, full Stokes)
  renormalise   the kernel of vmSendSToFits
  inverse PFB   the kernel of cu_invert_pfb

Only device time between CUDA events is counted (the reference's host-side
repacking loops and synchronous copies are left out, which favours it). Its
real-time factor for the 24-channel band, run one channel after another as
the reference's one-process-per-channel model does on a single GPU, is
1 / (24 x t). Prints one JSON line.

    python oracle/time_ref_cuda.py [--smart]
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "mwa-vcsbeam_gb300"))

import oracle as O  # noqa: E402
import synthetic as SY  # noqa: E402

NANT, K, P, NBLK = 128, 128, 12, 20
NI = 2 * NANT
NS = NBLK * 500


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--smart", action="store_true", help="PFB_SMART (4-bit) instead of PFB_FULL_PRECISION")
    args = ap.parse_args()
    h = ctypes.CDLL(os.path.join(HERE, "_ref", "libref_harness.so"))
    h.refh_last_error.restype = ctypes.c_char_p
    if h.refh_init(os.path.join(HERE, "_ref").encode()):
        raise RuntimeError(h.refh_last_error().decode())
    V = ctypes.c_void_p
    h.refh_fpfb.argtypes = [V, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, V, ctypes.c_int, ctypes.c_int, V,
                            ctypes.c_int, V, V, V]
    h.refh_beamform.argtypes = [V, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, V, V, V, V, ctypes.c_int,
                                ctypes.c_double, ctypes.c_int, V, V, V]
    h.refh_ipfb.argtypes = [V, V, V, V, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, V, V]
    p = lambda a: a.ctypes.data_as(V)

    def chk(rc):
        if rc:
            raise RuntimeError(h.refh_last_error().decode())

    t0 = time.time()
    htr = O.mwax_buffer(7, NBLK + 1, NI)
    filt = SY.analysis_filter_int16()
    i_idx = SY.legacy_input_order(NANT)
    flags = O.PFB_SMART if args.smart else O.PFB_FULL_PRECISION
    out = np.empty((NS, K, NI), dtype=np.uint8 if args.smart else np.complex128)
    ms = ctypes.c_float()
    times = {}
    # warm once (cuFFT plan creation, module load), then time
    for rep in range(2):
        chk(h.refh_fpfb(p(htr), htr.nbytes, NI, NS, p(filt), K, P, p(i_idx), flags, None, p(out), ctypes.byref(ms)))
    times["pfb"] = ms.value

    J = O.calc_j(SY.calibration_jones(NANT, K, seed=11), SY.identity_beam(1, NANT))
    e_, n_, h_, c_ = SY.tile_layout(NANT, seed=7)
    phi = O.calc_phi(SY.unit_vectors(45.0, 20.0), e_, n_, h_, c_, SY.fine_chan_freqs_hz(SY.coarse_chan_start_hz(0)))
    polQ = np.ascontiguousarray(i_idx[0::2].astype(np.uint32))
    polP = np.ascontiguousarray(i_idx[1::2].astype(np.uint32))
    S = np.empty((1, NS, 4, K), dtype=np.float32)
    e = np.empty((1, NS, K, 2), dtype=np.complex128)
    for rep in range(2):
        chk(h.refh_beamform(p(out), 0 if args.smart else 1, NS, K, NANT, p(J), p(phi), p(polQ), p(polP), 1,
                            1.0 / NI, 4, p(S), p(e), ctypes.byref(ms)))
    times["beamform"] = ms.value

    coeffs = SY.synthesis_filter(scale=SY.synthesis_scale(filt))
    ftr, fti = O.ipfb_table(coeffs, K)
    x = np.concatenate([np.zeros((P, K, 2), np.complex128), e[0]], axis=0)
    ir = np.ascontiguousarray(x.real.astype(np.float32))
    ii = np.ascontiguousarray(x.imag.astype(np.float32))
    vo = np.empty((NS * K, 2, 2), dtype=np.float32)
    for rep in range(2):
        chk(h.refh_ipfb(p(ir), p(ii), p(ftr), p(fti), P, NS, K, 2, p(vo), ctypes.byref(ms)))
    times["ipfb"] = ms.value

    # renormalise: time on the device with the harness call's own events is
    # not available; it runs 512 threads once, measured by wall clock around
    # a synchronous call (an upper bound).
    off = np.empty((1, 4, K), np.float32)
    sc = np.empty((1, 4, K), np.float32)
    u8 = np.empty(S.shape, np.uint8)
    h.refh_renormalise.argtypes = [V, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, V, V, V]
    t1 = time.perf_counter()
    chk(h.refh_renormalise(p(S), 1, NS, 4, K, p(off), p(sc), p(u8)))
    times["renormalise_wall_incl_copies"] = 1e3 * (time.perf_counter() - t1)

    t_cc = sum(v for k, v in times.items()) / 1e3
    line = {"what": "reference CUDA build (unmodified kernels), one coarse-channel-second, 128 tiles, 1 beam",
            "mode": "PFB_SMART" if args.smart else "PFB_FULL_PRECISION", "ms": times,
            "seconds_per_cc_second": t_cc, "rtf_full_band_24cc": 1.0 / (24 * t_cc),
            "setup_s": time.time() - t0}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
