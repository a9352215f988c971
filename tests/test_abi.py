"""The C ABI without a GPU: the library loads, exports every entry point
include/vcsbeam_gb300.h declares, the Python binding covers them all, and
argument checks fail with status codes (never by exiting the process)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "vcsbeam_gb300.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vgb_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def vgb_mod():
    import build as B
    import vgb

    if not os.path.exists(vgb.LIB_PATH):
        B.build()
    vgb.lib()
    return vgb


def test_header_declares_entry_points():
    names = declared()
    assert len(names) >= 30
    assert "vgb_beamform_mwax" in names and "vgb_pipeline_run_host" in names


def test_library_exports_every_declared_symbol(vgb_mod):
    lib = ctypes.CDLL(vgb_mod.LIB_PATH)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_the_header(vgb_mod):
    assert sorted(vgb_mod.exported_symbols()) == declared()


def test_argument_errors_are_status_codes(vgb_mod):
    lib = vgb_mod.lib()
    v = vgb_mod.Voltages(hist=16, hist_input_stride=128000, cur=32, cur_block_stride=16, ninputs=32, nblocks=1)
    rc = lib.vgb_beamform_mwax(ctypes.byref(v), 1, 10, None, 12, 128, 0, None, 16, 1.0, 4, None, None, None, None)
    assert rc == 1  # VGB_ERR_INVALID: block stride smaller than a block
    assert b"cur_block_stride" in lib.vgb_last_error()
    rc = lib.vgb_beamform_mwax(ctypes.byref(v), 1, 10, None, 12, 64, 0, None, 16, 1.0, 4, None, None, None, None)
    assert rc == 4  # VGB_ERR_UNSUPPORTED: 64 channels
    rc = lib.vgb_renormalise(None, 1, 1, 10, 4, 128, None, 0, 0, 0, 0, None, None, None)
    assert rc == 1
    rc = lib.vgb_beamform_mwax_psrfits_noalloc(ctypes.byref(v), 2, 10000, None, 12, 128, 0, None, 16, 1.0, 4,
                                               None, None, None, None)
    assert rc == 1 and b"static scratch" in lib.vgb_last_error()
    # inverse PFB: a negative or overflowing frame offset (checked before any launch)
    rc = lib.vgb_ipfb(16, 16 * 128 * 16, None, 0, 16, 12, 128, 16, 1, 16, None, None, -1, None)
    assert rc == 1 and b"frame_offset" in lib.vgb_last_error()
    rc = lib.vgb_ipfb(16, 16 * 128 * 16, None, 0, 16, 12, 128, 16, 1, 16, None, None, (1 << 31) - 8, None)
    assert rc == 1 and b"frame_offset" in lib.vgb_last_error()
    assert lib.vgb_vdif_advance(None, 1, 10, None) == 1
    assert lib.vgb_vdif_advance(16, 1, -1, None) == 1
    # readers: a missing file is a status code, not an exit
    info = vgb_mod.SubfileInfo()
    assert lib.vgb_subfile_info_read(b"/nonexistent/x.sub", ctypes.byref(info)) == 1
    assert lib.vgb_legacy_read_second(b"/nonexistent/x.dat", 16, 0, 1) == 1
    assert lib.vgb_pfb_variant(6) == -1


def test_filter_exactness_rule(vgb_mod):
    import numpy as np

    import synthetic as SY

    h = SY.analysis_filter_int16()
    assert vgb_mod.filter_fp32_exact(h)
    assert not vgb_mod.filter_fp32_exact(h * 4)
    # the arithmetic the library picks per filter: one FP32 sum for the
    # prototype, the even/odd split for the reference's FINEPFB (its worst
    # half-sum 129,763 x 128 < 2^24), int32 beyond that
    finepfb = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_filters.npz"))["finepfb"]
    assert vgb_mod.filter_wola_flags(h) == vgb_mod.WOLA_FP32
    assert vgb_mod.filter_wola_flags(finepfb) == vgb_mod.WOLA_FP32_SPLIT
    assert not SY.wola_fp32_exact(finepfb) and SY.wola_split_exact(finepfb)
    assert vgb_mod.filter_wola_flags(finepfb * 2) == 0 and not SY.wola_split_exact(finepfb * 2)
    # the bound counts |x| = 128 (int8 -128): a filter exactly at the limit
    # passes, one tap more does not
    edge = np.zeros(12 * 128, np.int32)
    edge[0] = 1 << 17                                  # 2^17 x 128 = 2^24
    assert vgb_mod.filter_fp32_exact(edge) and SY.wola_fp32_exact(edge)
    edge[128] = 1                                      # same sample position, another tap
    assert not vgb_mod.filter_fp32_exact(edge) and not SY.wola_fp32_exact(edge)
    assert vgb_mod.filter_wola_flags(edge) == vgb_mod.WOLA_FP32_SPLIT
