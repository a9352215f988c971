"""Store the reference's own PFB filters as a fixture, loaded by the
reference's own code.

Run where the VCSBeam sources are present and oracle/build_ref.sh has built
oracle/_ref/libref_host.so (its RUNTIME_DIR links to the reference's
pfb_filter/*.dat):

    python tests/golden/make_golden_filters.py [out_dir]

It calls the reference's vmLoadFilter (filter.c:62-122) and
vmScaleFilterCoeffs (filter.c:134-165) through the shim
(refhost_load_filter) exactly as app/make_mwa_tied_array_beam.c:162-163
uses them for real MWA data:
  * FINEPFB, the analysis filter (128 channels; the forward PFB casts it to
    int, pfb.cpp:459-460);
  * LSQ12 scaled by 15/7.2, the synthesis filter of the inverse PFB.
Written to ref_filters.npz (finepfb int32 [1536], lsq12_scaled float64
[1536], and the tap counts), so the GPU tests can run the full-size parity
cases with the reference's filters on a machine without the reference tree.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libref_host.so")


def load(lib, name: str, synthesis: bool, scale: float):
    out = np.zeros(8192)
    nt = ctypes.c_int()
    n = lib.refhost_load_filter(name.encode(), int(synthesis), 128, scale, out.ctypes.data, out.size,
                                ctypes.byref(nt))
    if n <= 0:
        raise RuntimeError(f"reference vmLoadFilter failed for {name}")
    return out[:n].copy(), nt.value


def main(out_dir: str) -> str:
    lib = ctypes.CDLL(REF_LIB)
    V, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.refhost_load_filter.argtypes = [ctypes.c_char_p, I, I, D, V, I, V]
    fine, nt_a = load(lib, "FINEPFB", False, 1.0)
    lsq, nt_s = load(lib, "LSQ12", True, 15.0 / 7.2)
    fine_i = fine.astype(np.int32)                      # the forward PFB's (int) cast, pfb.cpp:459-460
    assert np.array_equal(fine_i.astype(np.float64), fine)
    path = os.path.join(out_dir, "ref_filters.npz")
    np.savez_compressed(path, finepfb=fine_i, finepfb_ntaps=np.array(nt_a), lsq12_scaled=lsq,
                        lsq12_ntaps=np.array(nt_s))
    print("wrote", path, os.path.getsize(path), "bytes")
    return path


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden"))
