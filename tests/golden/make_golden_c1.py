"""Golden vectors of one full C1 second, produced by the reference's OWN CUDA
kernels with the reference's own filters.

Workload: 1 coarse channel x 128 tiles x 2 pols x 1 s of 8-bit MWAX voltages
(Gaussian sigma 16, clipped to +-127; the oracle's integer generator, so the
same bytes on every machine) in the reference's read-buffer layout (one
margin block + 20 blocks), FINEPFB analysis filter, PFB_FULL_PRECISION;
calibration D = I + 0.1 CN(0,1) per tile, tiles uniform in a 3 km disc, one
beam at az 45 / za 20 deg, full Stokes at 100 us; inverse PFB with LSQ12 x
15/7.2 (app/make_mwa_tied_array_beam.c:162-163), first second (no history).

Run on a GPU machine after __graft_entry__.build() has built
oracle/_ref/libref_harness.so:

    python tests/golden/make_golden_c1.py [out_dir]

The full outputs are GBs, so the fixture keeps: SHA-256 of the 8-bit PSRFITS
bytes and of the VDIF payload bytes of the whole second; the offsets and
scales; and every 100th spectrum of the Stokes and beam voltages, every 20th
spectrum of the PSRFITS bytes and every 20th VDIF frame (the reference's IPFB
output quantised by the oracle's restatement of beam_vdif.c's quantiser, as
the reference's host code does after cu_invert_pfb).
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "mwa-vcsbeam_gb300"))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

import oracle as O  # noqa: E402
import synthetic as SY  # noqa: E402
from make_golden import _p, check, load_harness  # noqa: E402

NANT, K, P, NBLK = 128, 128, 12, 20
NI = 2 * NANT
NS = NBLK * 500
SEED_V = 20261204
SUB_S = 100     # Stokes / beam-voltage subsample stride (spectra)
SUB_B = 20      # PSRFITS-byte and VDIF-frame subsample stride


def c1_inputs():
    """Voltages and tables of the C1 case (shared with the GPU test)."""
    htr = O.mwax_buffer(SEED_V, NBLK + 1, NI)
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_filters.npz"))
    D = SY.calibration_jones(NANT, K, seed=11)
    B = SY.identity_beam(1, NANT)
    J = O.calc_j(D, B)
    east, north, height, cable = SY.tile_layout(NANT, seed=7)
    phi = O.calc_phi(SY.unit_vectors(45.0, 20.0), east, north, height, cable,
                     SY.fine_chan_freqs_hz(SY.coarse_chan_start_hz(0)))
    return htr, g["finepfb"].astype(np.int32), g["lsq12_scaled"], J, phi


def main(out_dir: str) -> str:
    h = load_harness()
    cv = ctypes.c_void_p
    h.refh_fpfb.argtypes = [cv, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, cv, ctypes.c_int, ctypes.c_int, cv,
                            ctypes.c_int, cv, cv, cv]
    h.refh_beamform.argtypes = [cv, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, cv, cv, cv, cv,
                                ctypes.c_int, ctypes.c_double, ctypes.c_int, cv, cv, cv]
    h.refh_renormalise.argtypes = [cv, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, cv, cv, cv]
    h.refh_ipfb.argtypes = [cv, cv, cv, cv, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, cv, cv]

    htr, fine, lsq, J, phi = c1_inputs()
    i_idx = SY.legacy_input_order(NANT)
    polQ = np.ascontiguousarray(i_idx[0::2].astype(np.uint32))
    polP = np.ascontiguousarray(i_idx[1::2].astype(np.uint32))

    v = np.empty((NS, K, NI), dtype=np.complex128)
    check(h, h.refh_fpfb(_p(htr), htr.nbytes, NI, NS, _p(fine), K, P, _p(i_idx), O.PFB_FULL_PRECISION, None,
                         _p(v), None))
    S = np.empty((1, NS, 4, K), dtype=np.float32)
    e = np.empty((1, NS, K, 2), dtype=np.complex128)
    check(h, h.refh_beamform(_p(v), 1, NS, K, NANT, _p(J), _p(phi), _p(polQ), _p(polP), 1, 1.0 / NI, 4, _p(S),
                             _p(e), None))
    del v
    off = np.empty((1, 4, K), dtype=np.float32)
    sc = np.empty((1, 4, K), dtype=np.float32)
    u8 = np.empty(S.shape, dtype=np.uint8)
    check(h, h.refh_renormalise(_p(S), 1, NS, 4, K, _p(off), _p(sc), _p(u8)))

    ftr, fti = O.ipfb_table(lsq, K)
    x = np.concatenate([np.zeros((P, K, 2), np.complex128), e[0]], axis=0)
    ir = np.ascontiguousarray(x.real.astype(np.float32))
    ii = np.ascontiguousarray(x.imag.astype(np.float32))
    out = np.empty((NS * K, 2, 2), dtype=np.float32)
    check(h, h.refh_ipfb(_p(ir), _p(ii), _p(ftr), _p(fti), P, NS, K, 2, _p(out), None))
    vdif = O.vdif_quantise(out.reshape(NS, 512))         # frame f = output samples 128 f .. 128 f + 127

    sha = lambda a: np.frombuffer(hashlib.sha256(np.ascontiguousarray(a).tobytes()).digest(), dtype=np.uint8)
    g = {"seed": np.array(SEED_V), "i_idx": i_idx,
         "S_sub": S[0, ::SUB_S], "e_sub": e[0, ::SUB_S].astype(np.complex64), "S_absmax": np.abs(S[0]).max(axis=0),
         "e_absmax": np.array(np.abs(e[0]).max()),
         "u8_sub": u8[0, ::SUB_B], "u8_sha256": sha(u8[0]), "offsets": off[0], "scales": sc[0],
         "vdif_sub": vdif[::SUB_B], "vdif_sha256": sha(vdif)}
    os.makedirs(out_dir, exist_ok=True)
    path = os.path.join(out_dir, "ref_golden_c1.npz")
    np.savez_compressed(path, **g)
    print("wrote", path, os.path.getsize(path), "bytes")
    return path


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden"))
