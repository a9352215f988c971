"""Generate golden vectors by running the reference's OWN CUDA kernels.

Run on a GPU machine after ``__graft_entry__.build()`` has built
``oracle/_ref/libref_harness.so`` (it needs the cubins that
``oracle/build_ref.sh`` compiles from the unmodified VCSBeam sources):

    python tests/golden/make_golden.py [out_dir]

Inputs come from the oracle's integer-only generators (identical bytes on
every machine) and seeded tables, which are stored beside the outputs so the
fixture is self-contained. Outputs are what the reference kernels produced,
driven with the reference's launch shapes by oracle/ref_harness.cu.
The CPU tests (tests/test_oracle_golden.py) pin the oracle against this file.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "mwa-vcsbeam_gb300"))

import oracle as O  # noqa: E402
import synthetic as SY  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "libref_harness.so")

# Case sizes: small enough to store, large enough to cross a voltage block
# boundary (spectra m >= 12 read the second block) and to exercise every
# channel and both pols.
I_IN = 32          # RF inputs (16 tiles x 2 pols); the reference's cuFFT batching needs I % 32 == 0
NANT = I_IN // 2
K = 128
P = 12
NSPEC_INT4 = 64
NSPEC_F64 = 16
SEED_V = 20240601
NS_IPFB = 64


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def load_harness():
    h = ctypes.CDLL(HARNESS)
    h.refh_last_error.restype = ctypes.c_char_p
    if h.refh_init(os.path.join(ROOT, "oracle", "_ref").encode()) != 0:
        raise RuntimeError(h.refh_last_error().decode())
    return h


def check(h, rc):
    if rc != 0:
        raise RuntimeError(h.refh_last_error().decode())


def main(out_dir: str) -> str:
    h = load_harness()
    c_void = ctypes.c_void_p
    h.refh_fpfb.argtypes = [c_void, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, c_void, ctypes.c_int,
                            ctypes.c_int, c_void, ctypes.c_int, c_void, c_void, c_void]
    h.refh_beamform.argtypes = [c_void, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_void,
                                c_void, c_void, c_void, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                c_void, c_void, c_void]
    h.refh_renormalise.argtypes = [c_void, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                   c_void, c_void, c_void]
    h.refh_incoh.argtypes = [c_void, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_void]
    h.refh_ipfb.argtypes = [c_void, c_void, c_void, c_void, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                            ctypes.c_int, c_void, c_void]

    g = {}
    # ---- forward PFB ------------------------------------------------------
    htr = O.mwax_buffer(SEED_V, 2, I_IN)
    filt = SY.analysis_filter_int16()
    i_idx = SY.legacy_input_order(NANT)
    g.update(filter=filt, i_idx=i_idx)

    wola = np.empty((NSPEC_INT4, I_IN, K, 2), dtype=np.int32)
    out4 = np.empty((NSPEC_INT4, K, I_IN), dtype=np.uint8)
    check(h, h.refh_fpfb(_p(htr), htr.nbytes, I_IN, NSPEC_INT4, _p(filt), K, P, _p(i_idx),
                         O.PFB_SMART, _p(wola), _p(out4), None))
    g["fpfb_smart_out"] = out4
    g["fpfb_wola_sha256"] = np.frombuffer(__import__("hashlib").sha256(wola.tobytes()).digest(),
                                          dtype=np.uint8)
    g["fpfb_wola_m0"] = wola[0]

    outd = np.empty((NSPEC_F64, K, I_IN), dtype=np.complex128)
    check(h, h.refh_fpfb(_p(htr), htr.nbytes, I_IN, NSPEC_F64, _p(filt), K, P, _p(i_idx),
                         O.PFB_FULL_PRECISION, None, _p(outd), None))
    assert np.array_equal(outd.astype(np.complex64).astype(np.complex128), outd)
    g["fpfb_full_out"] = outd.astype(np.complex64)

    # ---- beamformer -------------------------------------------------------
    Dcal = SY.calibration_jones(NANT, K, seed=5)
    B = SY.identity_beam(1, NANT) + 0.05 * (1 + 1j) * O.gauss(77, NANT * 4).reshape(1, NANT, 2, 2)
    J = O.calc_j(Dcal, np.ascontiguousarray(B))
    east, north, height, cable = SY.tile_layout(NANT, seed=9)
    unit = SY.unit_vectors(45.0, 20.0)
    freqs = SY.fine_chan_freqs_hz(SY.coarse_chan_start_hz(0))
    phi = O.calc_phi(unit, east, north, height, cable, freqs)
    polQ = np.ascontiguousarray(i_idx[0::2].astype(np.uint32))
    polP = np.ascontiguousarray(i_idx[1::2].astype(np.uint32))
    g.update(J=J, phi=phi, polQ=polQ, polP=polP)
    for tag, v, invw in (("int4", out4, 1.0 / I_IN), ("f64", outd, 1.0 / (I_IN - 2))):
        ns = v.shape[0]
        S = np.empty((1, ns, 4, K), dtype=np.float32)
        e = np.empty((1, ns, K, 2), dtype=np.complex128)
        check(h, h.refh_beamform(_p(np.ascontiguousarray(v)), 0 if v.dtype == np.uint8 else 1, ns, K, NANT,
                                 _p(J), _p(phi), _p(polQ), _p(polP), 1, invw, 4, _p(S), _p(e), None))
        g[f"bf_{tag}_invw"] = np.array(invw)
        g[f"bf_{tag}_S"] = S
        g[f"bf_{tag}_e"] = e.astype(np.complex64)
        g[f"bf_{tag}_e_err"] = np.array(np.abs(e - e.astype(np.complex64)).max())
    # Stokes I only
    S1 = np.empty((1, NSPEC_INT4, 1, K), dtype=np.float32)
    check(h, h.refh_beamform(_p(out4), 0, NSPEC_INT4, K, NANT, _p(J), _p(phi), _p(polQ), _p(polP),
                             1, 1.0 / I_IN, 1, _p(S1), None, None))
    g["bf_int4_S1"] = S1

    # ---- renormalise ------------------------------------------------------
    S = g["bf_int4_S"]
    Sx = S.copy()
    Sx[0, :, 1, 5] = 3.25          # a constant channel: scale 0, 0/0 -> NaN
    Sx[0, 7, 2, 9] = -1e30         # extreme values
    Sx[0, 8, 2, 9] = 1e30
    g["rn_in"] = Sx
    off = np.empty((1, 4, K), dtype=np.float32)
    sc = np.empty((1, 4, K), dtype=np.float32)
    u8 = np.empty(Sx.shape, dtype=np.uint8)
    check(h, h.refh_renormalise(_p(Sx), 1, NSPEC_INT4, 4, K, _p(off), _p(sc), _p(u8)))
    g.update(rn_off=off, rn_scale=sc, rn_u8=u8)

    # ---- incoherent beam (legacy 4+4-bit [s][c][i]) -------------------------
    inc = np.empty((NSPEC_INT4, K), dtype=np.float32)
    check(h, h.refh_incoh(_p(out4), NSPEC_INT4, K, I_IN, _p(inc)))
    g["incoh"] = inc

    # ---- inverse PFB ------------------------------------------------------
    coeffs = SY.synthesis_filter(scale=SY.synthesis_scale(filt))
    ftr, fti = O.ipfb_table(coeffs, K)
    g["ipfb_coeffs"] = coeffs
    # two "seconds" of beamformed voltages [2][ns][K][2pol]
    ev = (O.gauss(31, 2 * NS_IPFB * K * 2) + 1j * O.gauss(32, 2 * NS_IPFB * K * 2)) * 40.0
    ev = ev.reshape(2, NS_IPFB, K, 2)
    g["ipfb_e"] = ev.astype(np.complex64)
    ev = g["ipfb_e"].astype(np.complex128)
    for sec in range(2):
        # pack as cu_invert_pfb does (pfb.cpp:950-984)
        hist = np.zeros((P, K, 2), dtype=np.complex128) if sec == 0 else ev[0, NS_IPFB - P:]
        x = np.concatenate([hist, ev[sec]], axis=0)
        ir = np.ascontiguousarray(x.real.astype(np.float32))
        ii = np.ascontiguousarray(x.imag.astype(np.float32))
        out = np.empty((NS_IPFB * K, 2, 2), dtype=np.float32)
        check(h, h.refh_ipfb(_p(ir), _p(ii), _p(ftr), _p(fti), P, NS_IPFB, K, 2, _p(out), None))
        g[f"ipfb_out{sec}"] = out

    os.makedirs(out_dir, exist_ok=True)
    path = os.path.join(out_dir, "ref_golden.npz")
    np.savez_compressed(path, **g)
    print("wrote", path, os.path.getsize(path), "bytes")
    return path


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden"))
