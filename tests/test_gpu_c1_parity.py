"""One whole C1 second through the pipeline against the FP64 oracle chain and
against the reference's own kernels.

C1: 1 coarse channel x 128 tiles x 2 pols x 1 s (10,000 fine spectra) of
8-bit MWAX voltages, Gaussian sigma 16 clipped to +-127; D = I + 0.1 CN(0,1)
per tile; tiles uniform in a 3 km disc; one beam at az 45 / za 20 deg; full
Stokes at 100 us; FP32 on the device. Run with the seeded int16 prototype
filter and with the reference's FINEPFB (analysis, peak tap 117,964, so the
exact WOLA runs in int32) and LSQ12 x 15/7.2 (synthesis) filters.

The pipeline starts from a checkpoint whose voltage history is the read
buffer's margin block (vgb_pipeline_load_state), so its second sees exactly
the voltages the reference's read buffer holds; its inverse-PFB history is
zero, as in the reference's first second.

Tolerances (each as written in the asserts):
  * Stokes and beam voltages: norm-wise, max |dev - ref| / max |ref| over
    the whole second < 1e-5; and per (Stokes, channel) series, max over time
    of |dev - ref| / max over time of |ref| < 1e-4.
  * 8-bit PSRFITS bytes against the oracle's renormalise of the oracle's own
    Stokes: at most 1e-4 of the samples differ by more than one LSB.
  * VDIF payload bytes against the oracle's inverse PFB of the oracle's own
    beam voltages: every byte within one LSB, at most 1e-4 of them differ.
  * Against the reference kernels' golden output (FINEPFB / LSQ12 only;
    tests/golden/ref_golden_c1.npz, subsampled): the same bounds, the VDIF
    frames of the first 12 fine samples excluded (the reference's inverse-PFB
    tap range truncates toward zero there, pfb.cpp:863).
"""
import os
import sys

import numpy as np
import pytest

import synthetic as SY
from helpers import byte_diff_stats, oracle_chain_second, rel_err, torch_cuda, weights_on_device

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
import make_golden_c1 as G  # noqa: E402

pytestmark = pytest.mark.gpu

K, P = 128, 12
NANT, NI, NBLK = 128, 256, 20
NS = NBLK * 500
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_golden_c1.npz")


def per_series_err(x, ref):
    """max over (Stokes, channel) of max_t |x - ref| / max_t |ref|."""
    num = np.abs(x - ref).max(axis=0)
    den = np.maximum(np.abs(ref).max(axis=0), 1e-30)
    return float((num / den).max())


def run_pipeline(vgb, torch, htr, filt, syn, J, phi):
    p = vgb.Pipeline(1, NANT, NBLK, nstokes=4, pfb_flags=0, do_ipfb=True, invw=1.0 / NI)
    p.set_filters(filt, syn)
    p.set_weights(weights_on_device(J, phi), on_device=True)
    # checkpoint: second 1 (any second after the first reads the carried
    # history), voltage history = the margin block's last 12 frames, beam
    # history zero
    st = p.save_state()
    st[24:32] = np.array([1], np.int64).view(np.uint8)
    hist = np.ascontiguousarray(htr[0, :, (500 - P) * K:, :]).reshape(-1).view(np.uint8)
    st[32:32 + hist.size] = hist
    st[32 + hist.size:] = 0
    p.load_state(st)
    d = torch.from_numpy(np.ascontiguousarray(htr[1:]).reshape(-1).view(np.uint8).copy()).cuda()
    p.run_device(d)
    ps = np.empty((NS, 4, K), np.uint8)
    off = np.empty((4, K), np.float32)
    sc = np.empty((4, K), np.float32)
    vd = np.empty((NS, 544), np.uint8)
    p.fetch(ps, off, sc, vd)
    S = np.empty((NS, 4, K), np.float32)
    e = np.empty((NS, K, 2), np.complex64)
    p.fetch_raw(S, e)
    p.close()
    return S, e, (off, sc, ps), vd


@pytest.fixture(scope="module")
def c1():
    torch = torch_cuda()
    import vgb

    vgb.lib()
    htr, fine, lsq, J, phi = G.c1_inputs()
    proto = SY.analysis_filter_int16()
    return torch, vgb, htr, J, phi, {"prototype": (proto, SY.synthesis_filter(scale=SY.synthesis_scale(proto))),
                                     "reference": (fine, lsq)}


@pytest.mark.parametrize("filters", ["prototype", "reference"])
def test_c1_second_against_oracle_chain(c1, filters):
    torch, vgb, htr, J, phi, fl = c1
    filt, syn = fl[filters]
    S, e, (off, sc, ps), vd = run_pipeline(vgb, torch, htr, filt, syn, J, phi)
    Sr, er, (offr, scr, psr), vdr = oracle_chain_second(htr, NI, filt, syn, J, phi, 1.0 / NI)
    errs = {"S": rel_err(S, Sr), "S_series": per_series_err(S, Sr), "e": rel_err(e, er),
            "e_series": per_series_err(e.reshape(NS, -1), er.reshape(NS, -1))}
    psr_stats = byte_diff_stats(ps, psr)
    vdif_stats = byte_diff_stats(vd[:, 32:], vdr)
    print(filters, errs, "psrfits", psr_stats, "vdif", vdif_stats)
    assert errs["S"] < 1e-5 and errs["e"] < 1e-5, errs
    assert errs["S_series"] < 1e-4 and errs["e_series"] < 1e-4, errs
    assert psr_stats[1] <= 1e-4, psr_stats
    assert rel_err(off, offr) < 1e-5 and rel_err(sc, scr) < 1e-5
    assert vdif_stats[0] <= 1 and vdif_stats[2] <= 1e-4, vdif_stats


def test_c1_second_against_reference_kernels(c1):
    """The device path with FINEPFB / LSQ12 against the reference's own CUDA
    kernels on the same second (and the oracle against them, which pins the
    oracle at 128 tiles with the reference's filters)."""
    torch, vgb, htr, J, phi, fl = c1
    g = dict(np.load(GOLDEN))
    assert int(g["seed"]) == G.SEED_V
    filt, syn = fl["reference"]
    S, e, (off, sc, ps), vd = run_pipeline(vgb, torch, htr, filt, syn, J, phi)
    s_err = rel_err(S[::G.SUB_S], g["S_sub"])
    e_err = rel_err(e[::G.SUB_S], g["e_sub"])
    b_stats = byte_diff_stats(ps[::G.SUB_B], g["u8_sub"])
    frames = np.arange(0, NS, G.SUB_B)
    keep = frames >= P                         # outside the reference's inverse-PFB tap bug
    v_stats = byte_diff_stats(vd[::G.SUB_B, 32:][keep], g["vdif_sub"][keep])
    print("vs reference kernels: S", s_err, "e", e_err, "psrfits", b_stats, "vdif", v_stats)
    assert s_err < 1e-5 and e_err < 1e-5
    assert b_stats[1] <= 1e-4, b_stats
    assert rel_err(off, g["offsets"]) < 1e-5 and rel_err(sc, g["scales"]) < 1e-5
    assert v_stats[0] <= 1 and v_stats[2] <= 1e-4, v_stats
