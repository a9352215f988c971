"""Golden vectors for several pointings, from the reference's OWN beamformer
kernels (vmApplyJ_kernel + vmBeamform_kernel per pointing, form_beam.cpp:
122-371, driven by oracle/ref_harness.cu with the reference's launch shapes).

Run on a GPU machine after ``__graft_entry__.build()``:

    python tests/golden/make_golden_multibeam.py [out_dir]

Stored beside the outputs: the calibration Jones D, per-pointing primary
beams B, pointing directions, tile geometry, channel frequencies, input
order and 4+4-bit legacy voltages, so the fixture is self-contained. The CPU
test pins the oracle's multi-pointing beamformer to it bit for bit; the GPU
test checks the many-beam tensor-core path against it (integrated over 10
samples).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import make_golden as MG  # noqa: E402
from make_golden import K, NANT, O, SY, _p, check, load_harness  # noqa: E402

NPNT = 5
NS = 60
SEED = 20240917


def inputs():
    D = SY.calibration_jones(NANT, K, seed=13)
    D = D * (1.0 + 0.05 * np.exp(2j * np.pi * np.random.default_rng(SEED).uniform(size=(NANT, K, 1, 1))))
    B = SY.identity_beam(NPNT, NANT) + 0.05 * (1 + 1j) * O.gauss(SEED + 1, NPNT * NANT * 4).reshape(NPNT, NANT, 2, 2)
    az, za = SY.grid_pointings(3, 0.5)
    az, za = az[:NPNT], za[:NPNT]
    unit = SY.unit_vectors(az, za)
    east, north, height, cable = SY.tile_layout(NANT, seed=SEED % 1000)
    freqs = SY.fine_chan_freqs_hz(SY.coarse_chan_start_hz(5))
    i_idx = SY.legacy_input_order(NANT, seed=SEED % 97)
    polQ = np.ascontiguousarray(i_idx[0::2].astype(np.uint32))
    polP = np.ascontiguousarray(i_idx[1::2].astype(np.uint32))
    v = O.gen_int4_bytes(SEED + 2, NS * K * 2 * NANT).reshape(NS, K, 2 * NANT)
    return dict(D=np.ascontiguousarray(D), B=np.ascontiguousarray(B), unit=np.ascontiguousarray(unit),
                east=east, north=north, height=height, cable=cable, freqs=freqs, polQ=polQ, polP=polP, v=v)


def main(out_dir: str) -> str:
    h = load_harness()
    c_void = MG.ctypes.c_void_p
    ci = MG.ctypes.c_int
    h.refh_beamform.argtypes = [c_void, ci, ci, ci, ci, c_void, c_void, c_void, c_void, ci, MG.ctypes.c_double, ci,
                                c_void, c_void, c_void]
    g = inputs()
    J = O.calc_j(g["D"], g["B"])
    phi = O.calc_phi(g["unit"], g["east"], g["north"], g["height"], g["cable"], g["freqs"])
    invw = 1.0 / (2 * NANT)
    S = np.empty((NPNT, NS, 4, K), dtype=np.float32)
    check(h, h.refh_beamform(_p(g["v"]), 0, NS, K, NANT, _p(J), _p(phi), _p(g["polQ"]), _p(g["polP"]), NPNT, invw, 4,
                             _p(S), None, None))
    g.update(S=S, invw=np.array(invw))
    os.makedirs(out_dir, exist_ok=True)
    path = os.path.join(out_dir, "ref_golden_multibeam.npz")
    np.savez_compressed(path, **g)
    print("wrote", path, os.path.getsize(path), "bytes")
    return path


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
