"""Pin the CPU oracle against outputs of the reference's OWN CUDA kernels.

tests/golden/ref_golden.npz was produced by tests/golden/make_golden.py,
which ran the unmodified VCSBeam kernels (compiled from src/pfb.cpp and
src/form_beam.cpp) on a GB300 with the reference's launch shapes. The inputs
are regenerated here from the same integer-only generator.

Tolerances (written per test): integer, index and packing work is
bit-exact; the reference's cuFFT (FP32) against the oracle's FP64 DFT is
within 1e-5 of the spectrum's rms; 4-bit rounding of FFT output may differ
by one LSB where a value sits within FP32 error of a rounding boundary.
"""
import hashlib

import numpy as np
import pytest

import synthetic as SY

I_IN, K, P = 32, 128, 12


@pytest.fixture(scope="module")
def htr(oracle_mod):
    return oracle_mod.mwax_buffer(20240601, 2, I_IN)


def test_wola_bit_exact(oracle_mod, golden, htr):
    b = oracle_mod.wola(htr, I_IN, 64, golden["filter"], K, P)
    assert np.array_equal(b[0], golden["fpfb_wola_m0"])
    assert hashlib.sha256(b.tobytes()).digest() == golden["fpfb_wola_sha256"].tobytes()


def test_fpfb_smart_int4(oracle_mod, golden, htr):
    ours = oracle_mod.fpfb(htr, I_IN, 64, golden["filter"], K, P, golden["i_idx"], oracle_mod.PFB_SMART)
    ref = golden["fpfb_smart_out"]
    mism = ours != ref
    # nibble-wise differences are at most one LSB, and rare
    hi = lambda x: ((x.astype(np.int16) >> 4) ^ 8) - 8
    lo = lambda x: ((x.astype(np.int16) & 15) ^ 8) - 8
    assert np.abs(hi(ours) - hi(ref)).max() <= 1
    assert np.abs(lo(ours) - lo(ref)).max() <= 1
    assert mism.mean() <= 1e-4, mism.sum()


def test_fpfb_full_precision(oracle_mod, golden, htr):
    ours = oracle_mod.fpfb(htr, I_IN, 16, golden["filter"], K, P, golden["i_idx"],
                           oracle_mod.PFB_FULL_PRECISION)
    ref = golden["fpfb_full_out"].astype(np.complex128)
    rms = np.sqrt(np.mean(np.abs(ref) ** 2))
    assert np.abs(ours - ref).max() / rms < 1e-5


@pytest.mark.parametrize("tag", ["int4", "f64"])
def test_beamform(oracle_mod, golden, tag):
    v = golden["fpfb_smart_out"] if tag == "int4" else golden["fpfb_full_out"].astype(np.complex128)
    S, e = oracle_mod.beamform(v, golden["J"], golden["phi"], golden["polQ"], golden["polP"],
                               float(golden[f"bf_{tag}_invw"]))
    Sref = golden[f"bf_{tag}_S"]
    # both sides are FP64 sums in the same order with the same float casts
    scale = np.abs(Sref).max()
    assert np.abs(S - Sref).max() <= 1e-6 * scale
    eref = golden[f"bf_{tag}_e"].astype(np.complex128)
    assert np.abs(e - eref).max() <= float(golden[f"bf_{tag}_e_err"]) + 1e-9 * np.abs(eref).max()


def test_beamform_stokes_i_only(oracle_mod, golden):
    S, _ = oracle_mod.beamform(golden["fpfb_smart_out"], golden["J"], golden["phi"], golden["polQ"],
                               golden["polP"], float(golden["bf_int4_invw"]), nstokes=1, want_e=False)
    assert np.abs(S - golden["bf_int4_S1"]).max() <= 1e-6 * np.abs(golden["bf_int4_S1"]).max()


def test_renormalise_bit_exact(oracle_mod, golden):
    off, sc, u8 = oracle_mod.renormalise(golden["rn_in"])
    assert np.array_equal(off, golden["rn_off"])
    assert np.array_equal(sc, golden["rn_scale"], equal_nan=True)
    assert np.array_equal(u8, golden["rn_u8"])


def test_u8_cast_wraps_at_channel_maximum(oracle_mod, golden):
    # the reference kernel turns each channel's maximum (256.5) into 0
    assert oracle_mod.sat_u8(256.5) == 0
    assert oracle_mod.sat_u8(255.9) == 255
    assert oracle_mod.sat_u8(float("nan")) == 0
    S = golden["rn_in"][0]
    u8 = golden["rn_u8"][0]
    imax = S.argmax(axis=0)
    st, c = np.meshgrid(np.arange(4), np.arange(K), indexing="ij")
    ok = np.isfinite(golden["rn_scale"][0]) & (golden["rn_scale"][0] > 0)
    assert np.all(u8[imax[ok], st[ok], c[ok]] == 0)


def test_incoherent_bit_exact(oracle_mod, golden):
    inc = oracle_mod.incoh_beam(golden["fpfb_smart_out"])
    assert np.array_equal(inc, golden["incoh"])


@pytest.mark.parametrize("sec", [0, 1])
def test_ipfb(oracle_mod, golden, sec):
    ev = golden["ipfb_e"].astype(np.complex128)
    ns = ev.shape[1]
    hist = np.zeros((P, K, 2)) if sec == 0 else ev[0, ns - P:]
    x = np.concatenate([hist, ev[sec]], axis=0)
    ref = golden[f"ipfb_out{sec}"]
    ref_c = ref[..., 0] + 1j * ref[..., 1]
    rms = np.sqrt(np.mean(np.abs(ref_c) ** 2))
    # the reference's own tap range, with zeros before its table
    quirk = oracle_mod.ipfb(x, golden["ipfb_coeffs"], P, reference_taps=True)
    assert np.abs(quirk - ref_c).max() / rms < 1e-5
    # the floor-correct tap range agrees wherever the reference's is correct
    fixed = oracle_mod.ipfb(x, golden["ipfb_coeffs"], P, reference_taps=False)
    n = np.arange(ns * K)
    good = (n >= P * K) | (n % K == 0)
    assert np.abs(fixed[good] - ref_c[good]).max() / rms < 1e-5
    # and differs where it is not (the first 1536 samples, n % 128 != 0)
    assert np.abs(fixed[~good] - ref_c[~good]).max() / rms > 1e-3


def test_table_builders_match_reference_host(oracle_mod):
    """vmCalcJ / calc_geometric_delays compiled from the reference (when the
    reference sources are present, oracle/_ref/libref_host.so)."""
    import ctypes
    import os

    lib = os.path.join(os.path.dirname(oracle_mod.__file__), "_ref", "libref_host.so")
    if not os.path.exists(lib):
        pytest.skip("reference host library not built (no reference sources here)")
    try:
        ref = ctypes.CDLL(lib)
    except OSError as exc:
        pytest.skip(f"reference host library not loadable: {exc}")
    pp = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    A, C = 16, 128
    D = SY.calibration_jones(A, C, seed=3)
    B = SY.identity_beam(2, A) + 0.2 * oracle_mod.gauss(5, 2 * A * 4).reshape(2, A, 2, 2)
    B[1, 2] = 0.0  # a zero matrix -> zero inverse
    B = np.ascontiguousarray(B)
    J = oracle_mod.calc_j(D, B)
    Jr = np.zeros_like(J)
    ref.refhost_calc_j(2, A, C, pp(D), pp(B), pp(Jr))
    assert np.array_equal(J, Jr)
    east, north, height, cable = SY.tile_layout(A, seed=4)
    unit = SY.unit_vectors(45.0, 20.0)[0]
    freqs = SY.fine_chan_freqs_hz(SY.coarse_chan_start_hz(3))
    phi = oracle_mod.calc_phi(unit, east, north, height, cable, freqs)
    ref.refhost_calc_geometric_delays.argtypes = [ctypes.c_double] * 3 + [ctypes.c_uint32, ctypes.c_int] + \
        [ctypes.c_void_p] * 5
    pr = np.zeros(A, dtype=np.complex128)
    for c in range(C):
        ref.refhost_calc_geometric_delays(*unit, int(freqs[c]), A, pp(east), pp(north), pp(height),
                                          pp(cable), pp(pr))
        assert np.array_equal(pr, phi[0, :, c])


def test_oracle_chain_c1_against_reference_kernels():
    """The FP64 oracle chain over one whole C1 second (128 tiles, FINEPFB,
    LSQ12 x 15/7.2) against the reference's own CUDA kernels on the same
    voltages (tests/golden/ref_golden_c1.npz): Stokes and beam voltages within
    1e-5 norm-wise (cuFFT FP32 against FP64), PSRFITS bytes within one LSB on
    <= 1e-4 of samples, VDIF frames (outside the reference's inverse-PFB tap
    bug, the first 12 fine samples) within one LSB on <= 1e-4."""
    import os
    import sys

    path = os.path.join(os.path.dirname(__file__), "golden", "ref_golden_c1.npz")
    if not os.path.exists(path):
        pytest.skip("C1 golden vectors not generated")
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    import make_golden_c1 as G
    from helpers import byte_diff_stats, oracle_chain_second, rel_err

    g = dict(np.load(path))
    htr, fine, lsq, J, phi = G.c1_inputs()
    S, e, (off, sc, u8), vd = oracle_chain_second(htr, 256, fine, lsq, J, phi, 1.0 / 256)
    assert rel_err(S[::G.SUB_S], g["S_sub"]) < 1e-5
    assert rel_err(e[::G.SUB_S], g["e_sub"]) < 1e-5
    assert byte_diff_stats(u8[::G.SUB_B], g["u8_sub"])[1] <= 1e-4
    assert rel_err(off, g["offsets"]) < 1e-5 and rel_err(sc, g["scales"]) < 1e-5
    keep = np.arange(0, 10000, G.SUB_B) >= 12
    mx, _, frac = byte_diff_stats(vd[::G.SUB_B][keep], g["vdif_sub"][keep])
    assert mx <= 1 and frac <= 1e-4
