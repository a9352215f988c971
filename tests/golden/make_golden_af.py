"""Golden array factors from the reference's own calc_array_factor
(geometry.c:440-467), compiled here by oracle/build_ref.sh into
oracle/_ref/libref_host.so. Runs on the CPU:

    python tests/golden/make_golden_af.py [out_dir]

A 41 x 41 grid of test directions (0.5 deg steps around the look direction)
and a wide random set, 128 tiles in a 3-km disc, one fine-channel frequency.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "mwa-vcsbeam_gb300"))
import synthetic as SY  # noqa: E402

LIB = os.path.join(ROOT, "oracle", "_ref", "libref_host.so")


def inputs():
    nant = 128
    east, north, height, cable = SY.tile_layout(nant, seed=21)
    look = SY.unit_vectors(60.0, 25.0)[0]
    az0, za0 = 60.0, 25.0
    off = np.arange(-20, 21) * 0.5
    dza, daz = np.meshgrid(off, off, indexing="ij")
    grid = SY.unit_vectors((az0 + daz / np.sin(np.radians(za0))).ravel(), (za0 + dza).ravel())
    rng = np.random.default_rng(22)
    wide = SY.unit_vectors(rng.uniform(0, 360, 400), np.degrees(np.arccos(rng.uniform(0.2, 1, 400))))
    dirs = np.ascontiguousarray(np.concatenate([grid, wide]))
    freq = float(SY.fine_chan_freqs_hz(SY.coarse_chan_start_hz(7))[37])
    return dict(east=east, north=north, height=height, cable=cable, look=np.ascontiguousarray(look), dirs=dirs,
                freq=np.array(freq))


def reference_af(g):
    lib = ctypes.CDLL(LIB)
    V = ctypes.c_void_p
    lib.refhost_array_factor.argtypes = [V, V, ctypes.c_int, ctypes.c_uint32, ctypes.c_int, V, V, V, V, V]
    p = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(V)
    af = np.empty(g["dirs"].shape[0])
    arrs = [np.ascontiguousarray(g[k], dtype=np.float64) for k in ("look", "dirs", "east", "north", "height", "cable")]
    lib.refhost_array_factor(arrs[0].ctypes.data, arrs[1].ctypes.data, af.size, int(g["freq"]), g["east"].size,
                             arrs[2].ctypes.data, arrs[3].ctypes.data, arrs[4].ctypes.data, arrs[5].ctypes.data,
                             af.ctypes.data)
    return af


def main(out_dir):
    g = inputs()
    g["af"] = reference_af(g)
    path = os.path.join(out_dir, "ref_golden_af.npz")
    np.savez_compressed(path, **g)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
