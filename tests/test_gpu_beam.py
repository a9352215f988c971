"""Fused PFB + beamformer, the legacy-input beamformer and the device-built
tables, against the oracle and the reference's own kernels.

Tolerances: Stokes and beam voltages within 1e-5 of the largest magnitude
(FP32 accumulation against the reference's FP64); the incoherent sum of
4-bit voltages bit-exact (integer sums); tables within 1e-12 (FP64).
"""
import os

import numpy as np
import pytest

import synthetic as SY
from helpers import dev, host, pol_lists, rel_err, tables, torch_cuda, weights_on_device

pytestmark = pytest.mark.gpu

K = 128


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


@pytest.fixture(scope="module")
def vgb_mod(torch):
    import vgb

    vgb.lib()
    return vgb


def run_beam(vgb, torch, htr, nant, nblocks, nspectra, filt, flags, W, invw, nstokes=4, ncc=1, cc_stride=0):
    d = dev(htr.reshape(-1).view(np.uint8))
    v = vgb.reference_buffer_voltages(d, 2 * nant, nblocks, ncc, cc_stride)
    S = torch.empty(ncc * nspectra * nstokes * K, dtype=torch.float32, device="cuda")
    e = torch.empty(ncc * nspectra * K * 4, dtype=torch.float32, device="cuda")
    inc = torch.empty(ncc * nspectra * K, dtype=torch.float32, device="cuda")
    vgb.beamform_mwax(v, ncc, nspectra, dev(filt), flags, W, nant, invw, nstokes, S, e, inc)
    torch.cuda.synchronize()
    assert vgb.check_device_status() == 0
    return (host(S).reshape(ncc, nspectra, nstokes, K), host(e).view(np.complex64).reshape(ncc, nspectra, K, 2),
            host(inc).reshape(ncc, nspectra, K))


def our_fpfb(vgb, torch, htr, ninputs, nblocks, nspectra, filt, i_idx, flags):
    """The library's own packed PFB output (legacy layout)."""
    d = dev(htr.reshape(-1).view(np.uint8))
    v = vgb.reference_buffer_voltages(d, ninputs, nblocks)
    out = torch.empty(nspectra * K * ninputs, dtype=torch.uint8, device="cuda")
    vgb.fpfb(v, 1, nspectra, dev(filt), dev(i_idx), flags, out)
    torch.cuda.synchronize()
    return host(out).reshape(nspectra, K, ninputs)


@pytest.mark.parametrize("mode", ["smart", "full"])
def test_fused_beam_matches_oracle(vgb_mod, torch, oracle_mod, mode):
    nant, ninputs, ns = 16, 32, 256
    htr = oracle_mod.mwax_buffer(5, 2, ninputs)
    filt = SY.analysis_filter_int16()
    i_idx = SY.legacy_input_order(nant)
    polQ, polP = pol_lists(i_idx)
    J, phi = tables(nant)
    W = weights_on_device(J, phi)
    invw = 1.0 / 30
    flags = (vgb_mod.PFB_SMART if mode == "smart" else vgb_mod.PFB_FULL_PRECISION) | vgb_mod.WOLA_FP32
    S, e, inc = run_beam(vgb_mod, torch, htr, nant, 1, ns, filt, flags, W, invw)
    # oracle chain: PFB packed to the legacy layout, then the beamformer. In
    # the 4-bit mode the beamformer input is the library's own packed PFB
    # output (checked against the oracle's separately): a value one FP32
    # rounding away from a 4-bit boundary would otherwise dominate the
    # Stokes comparison.
    v = oracle_mod.fpfb(htr, ninputs, ns, filt, K, 12, i_idx, flags & 0xFFFF)
    if mode == "smart":
        ours = our_fpfb(vgb_mod, torch, htr, ninputs, 1, ns, filt, i_idx, flags)
        assert (ours != v).mean() <= 1e-4
        v = ours
    Sref, eref = oracle_mod.beamform(v, J, phi, polQ, polP, invw)
    for st in range(4):
        assert rel_err(S[0, :, st], Sref[0, :, st]) < 1e-5, st
    assert rel_err(e[0], eref[0]) < 1e-5
    if mode == "smart":
        assert np.array_equal(inc[0], oracle_mod.incoh_beam(v))
    else:
        assert rel_err(inc[0], (np.abs(v) ** 2).sum(axis=-1)) < 1e-5


@pytest.mark.parametrize("flags_name", ["smart", "full"])
def test_fused_beam_inputs_per_step_identical(vgb_mod, torch, oracle_mod, flags_name):
    """The front end's four shapes (4 inputs per step in 256-thread CTAs, 8 in
    512-thread CTAs, 4 at three CTAs per SM with the sums in tensor memory
    (variant 5), and the warp-specialised 416-thread CTAs of variant 3) give
    identical Stokes, beam voltages and incoherent sums; an odd tile
    count leaves the last step partly filled, and 70 spectra leave the last
    CTA partly filled."""
    nant, ns = 18, 70
    ninputs = 2 * nant
    htr = oracle_mod.mwax_buffer(31, 2, ninputs)
    filt = SY.analysis_filter_int16()
    J, phi = tables(nant)
    W = weights_on_device(J, phi)
    flags = (vgb_mod.PFB_SMART if flags_name == "smart" else vgb_mod.PFB_FULL_PRECISION) | vgb_mod.WOLA_FP32
    out = {}
    for g in (4, 8, 5, 3):
        prev = vgb_mod.pfb_variant(g)
        try:
            out[g] = run_beam(vgb_mod, torch, htr, nant, 1, ns, filt, flags, W, 1 / 36)
        finally:
            vgb_mod.pfb_variant(prev)
        assert vgb_mod.check_device_status() == 0
    for x4, x8, x5, x3 in zip(out[4], out[8], out[5], out[3]):
        assert np.array_equal(x4, x8)
        assert np.array_equal(x4, x5)
        assert np.array_equal(x4, x3)
    with pytest.raises(vgb_mod.VGBError):
        vgb_mod.pfb_variant(6)


def finepfb():
    """The reference's FINEPFB analysis filter (tests/golden/ref_filters.npz)."""
    return np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_filters.npz"))["finepfb"]


def test_split_wola_equals_int32(vgb_mod, torch, oracle_mod):
    """With the reference's FINEPFB filter one FP32 sum is not exact but the
    even/odd split is: on full-range voltages (uniform int8, so sums pass
    2^24) the split path gives the int32 path's Stokes, beam voltages and
    incoherent sums bit for bit in every front-end shape, and the PFB-only
    kernel's complex-double output too. One forced FP32 sum differs (the
    comparison can see a rounding). With FPGA rounding a split request takes
    the int32 sums."""
    h = finepfb()
    assert vgb_mod.filter_wola_flags(h) == vgb_mod.WOLA_FP32_SPLIT
    nant, ns = 18, 70
    ninputs = 2 * nant
    rng = np.random.default_rng(77)
    htr = rng.integers(-128, 128, size=(2, ninputs, 64000, 2), dtype=np.int8)
    J, phi = tables(nant)
    W = weights_on_device(J, phi)
    full = vgb_mod.PFB_FULL_PRECISION
    ref = run_beam(vgb_mod, torch, htr, nant, 1, ns, h, full, W, 1 / 36)
    for g in (4, 8, 5, 3):
        prev = vgb_mod.pfb_variant(g)
        try:
            got = run_beam(vgb_mod, torch, htr, nant, 1, ns, h, full | vgb_mod.WOLA_FP32_SPLIT, W, 1 / 36)
        finally:
            vgb_mod.pfb_variant(prev)
        for x, y in zip(got, ref):
            assert np.array_equal(x, y), g
    one = run_beam(vgb_mod, torch, htr, nant, 1, ns, h, full | vgb_mod.WOLA_FP32, W, 1 / 36)
    assert not np.array_equal(one[1], ref[1])
    # PFB only, complex double: per-input fine channels
    i_idx = SY.legacy_input_order(nant)
    d = dev(htr.reshape(-1).view(np.uint8))
    v = vgb_mod.reference_buffer_voltages(d, ninputs, 1)
    outs = []
    for extra in (0, vgb_mod.WOLA_FP32_SPLIT):
        out = torch.empty(ns * K * ninputs * 16, dtype=torch.uint8, device="cuda")
        vgb_mod.fpfb(v, 1, ns, dev(h), dev(i_idx), full | extra, out)
        torch.cuda.synchronize()
        outs.append(host(out))
    assert np.array_equal(outs[0], outs[1])
    # FPGA rounding: the split request is served by the int32 sums
    smart = vgb_mod.PFB_SMART
    a = run_beam(vgb_mod, torch, htr, nant, 1, ns, h, smart, W, 1 / 36)
    b = run_beam(vgb_mod, torch, htr, nant, 1, ns, h, smart | vgb_mod.WOLA_FP32_SPLIT, W, 1 / 36)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert vgb_mod.check_device_status() == 0


def test_fused_beam_stokes_i_only_and_batched(vgb_mod, torch, oracle_mod):
    nant, ninputs, ns = 16, 32, 64
    a = oracle_mod.mwax_buffer(21, 2, ninputs)
    b = oracle_mod.mwax_buffer(22, 2, ninputs)
    filt = SY.analysis_filter_int16()
    Ja, pa = tables(nant, cc=0)
    Jb, pb = tables(nant, cc=1)
    W = torch.cat([weights_on_device(Ja, pa), weights_on_device(Jb, pb)])
    flags = vgb_mod.PFB_SMART | vgb_mod.WOLA_FP32
    both = np.concatenate([a.reshape(-1), b.reshape(-1)])
    S, e, inc = run_beam(vgb_mod, torch, both, nant, 1, ns, filt, flags, W, 1 / 32, nstokes=1, ncc=2,
                         cc_stride=a.nbytes)
    S4a, _, _ = run_beam(vgb_mod, torch, a, nant, 1, ns, filt, flags, W[: W.shape[0] // 2], 1 / 32)
    assert np.array_equal(S[0, :, 0], S4a[0, :, 0])
    i_idx = SY.legacy_input_order(nant)
    polQ, polP = pol_lists(i_idx)
    vb = our_fpfb(vgb_mod, torch, b, ninputs, 1, ns, filt, i_idx, flags)
    Sref, _ = oracle_mod.beamform(vb, Jb, pb, polQ, polP, 1 / 32, nstokes=1, want_e=False)
    assert rel_err(S[1, :, 0], Sref[0, :, 0]) < 1e-5


@pytest.mark.parametrize("nant", [1, 256])
def test_fused_beam_edge_sizes(vgb_mod, torch, oracle_mod, nant):
    """The smallest and the largest arrays: one tile (half of the one step
    empty) and 256 tiles (512 inputs, MWA Phase III). Every front-end shape
    gives the same bytes, and they match the oracle's PFB + beamformer within
    1e-5 (norm-wise)."""
    ninputs, ns = 2 * nant, 24
    htr = oracle_mod.mwax_buffer(61 + nant, 2, ninputs)
    filt = SY.analysis_filter_int16()
    J, phi = tables(nant)
    W = weights_on_device(J, phi)
    invw = 1.0 / ninputs
    flags = vgb_mod.PFB_FULL_PRECISION | vgb_mod.WOLA_FP32
    out = {}
    for g in (4, 8, 5, 3):
        prev = vgb_mod.pfb_variant(g)
        try:
            out[g] = run_beam(vgb_mod, torch, htr, nant, 1, ns, filt, flags, W, invw)
        finally:
            vgb_mod.pfb_variant(prev)
    for g in (8, 5, 3):
        for x, y in zip(out[g], out[4]):
            assert np.array_equal(x, y), g
    i_idx = SY.legacy_input_order(nant)
    polQ, polP = pol_lists(i_idx)
    v = oracle_mod.fpfb(htr, ninputs, ns, filt, K, 12, i_idx, flags & 0xFFFF)
    Sref, eref = oracle_mod.beamform(v, J, phi, polQ, polP, invw)
    S, e, _ = out[4]
    assert rel_err(e[0], eref[0]) < 1e-5
    if nant > 1:        # one tile's Stokes cancel to rounding (the test below)
        for st in range(4):
            assert rel_err(S[0, :, st], Sref[0, :, st]) < 1e-5, st


def test_fused_beam_empty_and_bad_shapes(vgb_mod, torch, oracle_mod):
    """No spectra: success, nothing written. No coarse channels, or an input
    count that is not two per tile: a status code, nothing launched."""
    nant = 4
    htr = oracle_mod.mwax_buffer(3, 2, 2 * nant)
    d = dev(htr.reshape(-1).view(np.uint8))
    v = vgb_mod.reference_buffer_voltages(d, 2 * nant, 1)
    J, phi = tables(nant)
    W = weights_on_device(J, phi)
    filt = dev(SY.analysis_filter_int16())
    S = torch.full((16 * 4 * K,), 7.0, dtype=torch.float32, device="cuda")
    vgb_mod.beamform_mwax(v, 1, 0, filt, vgb_mod.PFB_FULL_PRECISION, W, nant, 0.125, 4, S)
    torch.cuda.synchronize()
    assert vgb_mod.check_device_status() == 0
    assert bool((S == 7.0).all())
    with pytest.raises(vgb_mod.VGBError, match="ncc"):
        vgb_mod.beamform_mwax(v, 0, 16, filt, vgb_mod.PFB_FULL_PRECISION, W, nant, 0.125, 4, S)
    with pytest.raises(vgb_mod.VGBError, match="2\\*nant"):
        vgb_mod.beamform_mwax(v, 1, 16, filt, vgb_mod.PFB_FULL_PRECISION, W, nant + 1, 0.125, 4, S)
    assert bool((S == 7.0).all())


def test_single_tile_autocorrelation_cancels(vgb_mod, torch, oracle_mod):
    """With one tile, |sum e|^2 - sum |e|^2 = 0: all Stokes vanish (to FP32
    rounding) while the beam voltages do not."""
    nant = 1
    htr = oracle_mod.mwax_buffer(8, 2, 2)
    J, phi = tables(nant)
    W = weights_on_device(J, phi)
    S, e, _ = run_beam(vgb_mod, torch, htr, nant, 1, 32, SY.analysis_filter_int16(),
                       vgb_mod.PFB_FULL_PRECISION | vgb_mod.WOLA_FP32, W, 0.5)
    assert np.abs(S).max() <= 1e-5 * np.abs(e).max() ** 2
    assert np.abs(e).max() > 0


def test_legacy_beamformer_matches_reference_kernels(vgb_mod, torch, golden):
    nant = 16
    W = weights_on_device(golden["J"], golden["phi"])
    for tag in ("int4", "f64"):
        v = golden["fpfb_smart_out"] if tag == "int4" else golden["fpfb_full_out"].astype(np.complex128)
        ns = v.shape[0]
        S = torch.empty(ns * 4 * K, dtype=torch.float32, device="cuda")
        e = torch.empty(ns * K * 4, dtype=torch.float32, device="cuda")
        inc = torch.empty(ns * K, dtype=torch.float32, device="cuda")
        dt = vgb_mod.INT4 if tag == "int4" else vgb_mod.DBL
        vgb_mod.beamform_legacy(dev(v), dt, ns, K, nant, dev(golden["polQ"]), dev(golden["polP"]), W, 1,
                                float(golden[f"bf_{tag}_invw"]), 4, S, e, inc)
        torch.cuda.synchronize()
        Sg = host(S).reshape(1, ns, 4, K)
        for st in range(4):
            assert rel_err(Sg[0, :, st], golden[f"bf_{tag}_S"][0, :, st]) < 1e-5
        assert rel_err(host(e).view(np.complex64).reshape(1, ns, K, 2), golden[f"bf_{tag}_e"]) < 1e-5
        if tag == "int4":
            assert np.array_equal(host(inc).reshape(ns, K), golden["incoh"])


def test_legacy_beamformer_many_pointings(vgb_mod, torch, oracle_mod):
    nant, ns, npnt = 32, 32, 3
    v = oracle_mod.gen_int4_bytes(3, ns * K * 2 * nant).reshape(ns, K, 2 * nant)
    i_idx = SY.legacy_input_order(nant, seed=9)
    polQ, polP = pol_lists(i_idx)
    J, phi = tables(nant, npointing=npnt)
    W = weights_on_device(J, phi)
    S = torch.empty(npnt * ns * 4 * K, dtype=torch.float32, device="cuda")
    vgb_mod.beamform_legacy(dev(v), vgb_mod.INT4, ns, K, nant, dev(polQ), dev(polP), W, npnt, 1 / 64, 4, S)
    torch.cuda.synchronize()
    Sref, _ = oracle_mod.beamform(v, J, phi, polQ, polP, 1 / 64, want_e=False)
    Sg = host(S).reshape(npnt, ns, 4, K)
    for p in range(npnt):
        assert rel_err(Sg[p], Sref[p]) < 1e-5


def test_legacy_beamformer_bad_input_index(vgb_mod, torch, oracle_mod):
    """polQ naming an input outside the row (2 nant + 1) is reported through
    the device status word, not read."""
    nant, ns = 8, 16
    v = oracle_mod.gen_int4_bytes(4, ns * K * 2 * nant).reshape(ns, K, 2 * nant)
    polQ, polP = pol_lists(SY.legacy_input_order(nant, seed=2))
    polQ = polQ.copy()
    polQ[5] = 2 * nant + 1
    J, phi = tables(nant)
    W = weights_on_device(J, phi)
    S = torch.empty(ns * 4 * K, dtype=torch.float32, device="cuda")
    vgb_mod.beamform_legacy(dev(v), vgb_mod.INT4, ns, K, nant, dev(polQ), dev(polP), W, 1, 1 / 16, 4, S)
    torch.cuda.synchronize()
    with pytest.raises(vgb_mod.VGBError, match="input index"):
        vgb_mod.check_device_status()
    assert vgb_mod.check_device_status() == 0


def test_device_tables_match_oracle(vgb_mod, torch, oracle_mod):
    nant, npnt = 24, 2
    D = SY.calibration_jones(nant, K, seed=4)
    B = SY.identity_beam(npnt, nant) + 0.3 * oracle_mod.gauss(9, npnt * nant * 4).reshape(npnt, nant, 2, 2)
    B[1, 5] = 0
    B = np.ascontiguousarray(B)
    Jd = torch.empty(npnt * nant * K * 8, dtype=torch.float64, device="cuda")
    vgb_mod.jones(dev(D), dev(B), npnt, nant, K, Jd)
    east, north, height, cable = SY.tile_layout(nant, seed=2)
    unit = SY.unit_vectors([45.0, 50.0], [20.0, 25.0])
    freqs = SY.fine_chan_freqs_hz(SY.coarse_chan_start_hz(5))
    phid = torch.empty(npnt * nant * K * 2, dtype=torch.float64, device="cuda")
    vgb_mod.phase(dev(unit), dev(east), dev(north), dev(height), dev(cable), dev(freqs), npnt, nant, K,
                  SY.MWA_ALTITUDE_METRES, phid)
    torch.cuda.synchronize()
    J = oracle_mod.calc_j(D, B)
    phi = oracle_mod.calc_phi(unit, east, north, height, cable, freqs)
    assert rel_err(host(Jd).view(np.complex128).reshape(J.shape), J) < 1e-12
    assert np.abs(host(phid).view(np.complex128).reshape(phi.shape) - phi).max() < 1e-9
