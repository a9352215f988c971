"""The many-beam tensor-core beamformer (vgb_multibeam_*) against the FP64
oracle chain: the reference's tables (vmCalcJ, vmCalcPhi), its beamformer
per sample (vmApplyJ + vmBeamform, autocorrelations removed) and a sum over
each 10-sample integration.

Tolerances (largest |difference| over the largest |reference| of each Stokes
parameter): split-BF16 weights 1e-3; single FP16 weights 4e-3; single BF16
weights 3e-2 (reported, the mode exists to show what the split buys); FP32
weights on the CUDA cores 2e-5. The
8-bit PSRFITS bytes are checked bit-exact against the oracle's renormalise of
the library's own Stokes (the byte stage is integer-exact given its input).
"""
import numpy as np
import pytest

import synthetic as SY
from helpers import dev, host, pol_lists, torch_cuda

pytestmark = pytest.mark.gpu

NINT = 10


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


@pytest.fixture(scope="module")
def vgb_mod(torch):
    import vgb

    vgb.lib()
    return vgb


def make_case(O, nant, npointing, nfine, ns, seed=1, int8=False, flag_tile=None, cc=0, natural=False):
    D = SY.calibration_jones(nant, nfine, seed=seed)
    rng = np.random.default_rng(seed + 50)  # a per-channel ripple so D^-1 differs across channels
    D = D * (1.0 + 0.05 * np.exp(2j * np.pi * rng.uniform(size=(nant, nfine, 1, 1))))
    if flag_tile is not None:
        D[flag_tile] = 0.0
    B = SY.identity_beam(npointing, nant) + 0.05 * (1 + 1j) * O.gauss(seed + 100, npointing * nant * 4).reshape(
        npointing, nant, 2, 2)
    B = np.ascontiguousarray(B)
    east, north, height, cable = SY.tile_layout(nant, seed=seed + 7)
    side = int(np.ceil(np.sqrt(npointing)))
    az, za = SY.grid_pointings(side, 0.02)
    unit = np.ascontiguousarray(SY.unit_vectors(az[:npointing], za[:npointing]))
    freqs = SY.fine_chan_freqs_hz(SY.coarse_chan_start_hz(cc))[:nfine].astype(np.float64)
    # the legacy order is a permutation of the inputs; natural = tile a's pols at inputs 2a, 2a + 1 (MWAX)
    polQ, polP = pol_lists(np.arange(2 * nant) if natural else SY.legacy_input_order(nant))
    if int8:
        raw = O.gen_int8(seed + 5, ns * nfine * 2 * nant * 2, sigma_num=16).reshape(ns, nfine, 2 * nant, 2)
        v_oracle = raw[..., 0].astype(np.float64) + 1j * raw[..., 1].astype(np.float64)
        v_dev = raw.view(np.uint8)
    else:
        v_dev = O.gen_int4_bytes(seed + 5, ns * nfine * 2 * nant).reshape(ns, nfine, 2 * nant)
        v_oracle = v_dev
    return dict(D=D, B=B, east=east, north=north, height=height, cable=cable, unit=unit, freqs=freqs, polQ=polQ,
                polP=polP, v_dev=np.ascontiguousarray(v_dev), v_oracle=v_oracle)


def oracle_stokes(O, case, nstokes, invw):
    """[c][p][st][t] float64: the reference's per-sample Stokes summed over
    each integration."""
    J = O.calc_j(case["D"], case["B"])
    phi = O.calc_phi(case["unit"], case["east"], case["north"], case["height"], case["cable"], case["freqs"])
    S, _ = O.beamform(case["v_oracle"], J, phi, case["polQ"], case["polP"], invw, nstokes=nstokes, want_e=False)
    npnt, ns, nst, nc = S.shape
    Si = S.astype(np.float64).reshape(npnt, ns // NINT, NINT, nst, nc).sum(axis=2)
    return np.ascontiguousarray(Si.transpose(3, 0, 2, 1))


def run_mb(vgb, torch, case, nant, npointing, nfine, ns, nstokes, precision, int8=False, invw=None, psrfits=False):
    mb = vgb.Multibeam(1, nfine, nant, npointing, ns, nstokes=nstokes, precision=precision,
                       input=vgb.MB_INT8 if int8 else vgb.MB_INT4, invw=invw)
    mb.set_geometry(dev(case["unit"]), dev(case["east"]), dev(case["north"]), dev(case["height"]),
                    dev(case["cable"]))
    mb.set_jones(dev(case["D"]), dev(case["B"]), dev(case["freqs"]), dev(case["polQ"]), dev(case["polP"]))
    nint = ns // NINT
    S = torch.full((nfine * npointing * nstokes * nint,), float("nan"), dtype=torch.float32, device="cuda")
    out = off = scl = None
    if psrfits:
        out = torch.empty(npointing * nint * nstokes * nfine, dtype=torch.uint8, device="cuda")
        off = torch.empty(npointing * nstokes * nfine, dtype=torch.float32, device="cuda")
        scl = torch.empty_like(off)
    mb.run(dev(case["v_dev"]), S=S, out=out, offsets=off, scales=scl)
    torch.cuda.synchronize()
    assert vgb.check_device_status() == 0
    res = dict(S=host(S).reshape(nfine, npointing, nstokes, nint), launches=mb.launches())
    if psrfits:
        res["out"] = host(out).reshape(npointing, nint, nstokes, nfine)
        res["off"] = host(off).reshape(npointing, nstokes, nfine)
        res["scl"] = host(scl).reshape(npointing, nstokes, nfine)
    mb.close()
    return res


def stokes_err(S, ref):
    return [float(np.abs(S[:, :, st] - ref[:, :, st]).max() / np.abs(ref[:, :, st]).max())
            for st in range(ref.shape[2])]


@pytest.mark.parametrize("precision,tol", [(0, 1e-3), (2, 4e-3), (1, 3e-2), (3, 2e-5)])
def test_multibeam_full_stokes(vgb_mod, torch, oracle_mod, precision, tol):
    nant, npnt, nfine, ns = 32, 40, 4, 500
    case = make_case(oracle_mod, nant, npnt, nfine, ns)
    invw = 1.0 / (2 * nant)
    ref = oracle_stokes(oracle_mod, case, 4, invw)
    res = run_mb(vgb_mod, torch, case, nant, npnt, nfine, ns, 4, precision, invw=invw)
    errs = stokes_err(res["S"], ref)
    print("precision", precision, "Stokes errors", errs)
    assert max(errs) < tol, errs
    assert res["launches"] == 4


def test_multibeam_split_beats_single(vgb_mod, torch, oracle_mod):
    nant, npnt, nfine, ns = 32, 64, 2, 250
    case = make_case(oracle_mod, nant, npnt, nfine, ns, seed=3)
    ref = oracle_stokes(oracle_mod, case, 4, 1.0)
    e_split = max(stokes_err(run_mb(vgb_mod, torch, case, nant, npnt, nfine, ns, 4, 0, invw=1.0)["S"], ref))
    e_single = max(stokes_err(run_mb(vgb_mod, torch, case, nant, npnt, nfine, ns, 4, 1, invw=1.0)["S"], ref))
    assert e_split * 10 < e_single, (e_split, e_single)


def test_multibeam_stokes_i_int8_flagged(vgb_mod, torch, oracle_mod):
    """8-bit voltages (coherencies split into exact FP16 halves), Stokes I
    only, one tile flagged (D = 0 -> zero weight, jones.c:144-147), a sample
    count that leaves the last tile partly used."""
    nant, npnt, nfine, ns = 48, 33, 3, 370
    case = make_case(oracle_mod, nant, npnt, nfine, ns, seed=9, int8=True, flag_tile=5)
    invw = 1.0 / (2 * nant - 2)
    ref = oracle_stokes(oracle_mod, case, 1, invw)
    res = run_mb(vgb_mod, torch, case, nant, npnt, nfine, ns, 1, 0, int8=True, invw=invw)
    errs = stokes_err(res["S"], ref)
    assert max(errs) < 1e-3, errs


@pytest.mark.parametrize("precision,tol", [(0, 1e-3), (2, 4e-3), (1, 3e-2)])
def test_multibeam_int8_natural_order(vgb_mod, torch, oracle_mod, precision, tol):
    """8-bit voltages in every tensor precision (each expands the raw bytes
    to its own 16-bit type inside the beam GEMM), full Stokes, with the tiles'
    inputs in the MWAX order (consecutive weight columns)."""
    nant, npnt, nfine, ns = 32, 40, 3, 520
    case = make_case(oracle_mod, nant, npnt, nfine, ns, seed=21, int8=True, natural=True)
    invw = 1.0 / (2 * nant)
    ref = oracle_stokes(oracle_mod, case, 4, invw)
    res = run_mb(vgb_mod, torch, case, nant, npnt, nfine, ns, 4, precision, int8=True, invw=invw)
    errs = stokes_err(res["S"], ref)
    assert max(errs) < tol, errs


def test_multibeam_bad_input_index(vgb_mod, torch, oracle_mod):
    """An input index outside the voltage row (polQ of a tile = 2 nant + 5) is
    skipped by the kernels and reported through the device status word."""
    nant, npnt, nfine, ns = 16, 32, 2, 100
    case = make_case(oracle_mod, nant, npnt, nfine, ns, seed=23)
    case["polQ"] = case["polQ"].copy()
    case["polQ"][3] = 2 * nant + 5
    with pytest.raises(vgb_mod.VGBError, match="input index"):
        run_mb(vgb_mod, torch, case, nant, npnt, nfine, ns, 4, 0)
    assert vgb_mod.check_device_status() == 0


def test_multibeam_psrfits_bytes(vgb_mod, torch, oracle_mod):
    nant, npnt, nfine, ns = 32, 36, 40, 300
    case = make_case(oracle_mod, nant, npnt, nfine, ns, seed=4)
    res = run_mb(vgb_mod, torch, case, nant, npnt, nfine, ns, 4, 0, psrfits=True)
    # oracle renormalise of the library's own Stokes, in the PSRFITS order [p][t][st][c]
    S_pfits = np.ascontiguousarray(res["S"].transpose(1, 3, 2, 0))
    off, scl, u8 = oracle_mod.renormalise(S_pfits)
    assert np.array_equal(res["off"], off)
    assert np.array_equal(res["scl"], scl)
    assert np.array_equal(res["out"], u8)
    assert res["launches"] == 5


def test_multibeam_fp32_stokes_i_int8(vgb_mod, torch, oracle_mod):
    nant, npnt, nfine, ns = 32, 70, 2, 330
    case = make_case(oracle_mod, nant, npnt, nfine, ns, seed=12, int8=True, flag_tile=0)
    ref = oracle_stokes(oracle_mod, case, 1, 0.5)
    res = run_mb(vgb_mod, torch, case, nant, npnt, nfine, ns, 1, 3, int8=True, invw=0.5)
    assert max(stokes_err(res["S"], ref)) < 2e-5


def test_multibeam_psrfits_repeat_runs(vgb_mod, torch, oracle_mod):
    """Row statistics are reset every run: a second run on different voltages
    gives the bytes of those voltages alone."""
    nant, npnt, nfine, ns = 16, 32, 32, 200
    vgb = vgb_mod
    cases = [make_case(oracle_mod, nant, npnt, nfine, ns, seed=s) for s in (21, 22)]
    mb = vgb.Multibeam(1, nfine, nant, npnt, ns, nstokes=4)
    c0 = cases[0]
    mb.set_geometry(dev(c0["unit"]), dev(c0["east"]), dev(c0["north"]), dev(c0["height"]), dev(c0["cable"]))
    mb.set_jones(dev(c0["D"]), dev(c0["B"]), dev(c0["freqs"]), dev(c0["polQ"]), dev(c0["polP"]))
    nint = ns // NINT
    for case in cases:
        S = torch.empty(nfine * npnt * 4 * nint, dtype=torch.float32, device="cuda")
        out = torch.empty(npnt * nint * 4 * nfine, dtype=torch.uint8, device="cuda")
        off = torch.empty(npnt * 4 * nfine, dtype=torch.float32, device="cuda")
        scl = torch.empty_like(off)
        mb.run(dev(case["v_dev"]), S=S, out=out, offsets=off, scales=scl)
        torch.cuda.synchronize()
        Sh = host(S).reshape(nfine, npnt, 4, nint)
        o, s_, u = oracle_mod.renormalise(np.ascontiguousarray(Sh.transpose(1, 3, 2, 0)))
        assert np.array_equal(host(out).reshape(npnt, nint, 4, nfine), u)
        assert np.array_equal(host(off).reshape(npnt, 4, nfine), o)
    mb.close()


@pytest.mark.parametrize("npnt,variant", [(32, 0), (64, 2)])
def test_multibeam_run_host_streams(vgb_mod, torch, oracle_mod, npnt, variant):
    """Three coarse channels from pinned host memory through the two device
    slots: the bytes equal vgb_multibeam_run's on device-resident input (one
    beam tile, single-CTA GEMM; and two, over CTA pairs)."""
    nant, nfine, ns, ncc = 16, 32, 200, 3
    prev = vgb_mod.multibeam_beam_variant(variant)
    try:
        vgb = vgb_mod
        cases = [make_case(oracle_mod, nant, npnt, nfine, ns, seed=30 + k) for k in range(ncc)]
        c0 = cases[0]
        mb = vgb.Multibeam(ncc, nfine, nant, npnt, ns, nstokes=4)
        mb.set_geometry(dev(c0["unit"]), dev(c0["east"]), dev(c0["north"]), dev(c0["height"]), dev(c0["cable"]))
        D = np.ascontiguousarray(np.stack([c["D"] for c in cases]))
        B = np.ascontiguousarray(np.stack([c["B"] for c in cases]))
        F = np.ascontiguousarray(np.concatenate([c["freqs"] for c in cases]))
        mb.set_jones(dev(D), dev(B), dev(F), dev(c0["polQ"]), dev(c0["polP"]))
        v = np.ascontiguousarray(np.stack([c["v_dev"] for c in cases]))
        nint = ns // NINT
        nout, nstat = ncc * npnt * nint * 4 * nfine, ncc * npnt * 4 * nfine
        out_d = torch.empty(nout, dtype=torch.uint8, device="cuda")
        off_d = torch.empty(nstat, dtype=torch.float32, device="cuda")
        scl_d = torch.empty_like(off_d)
        mb.run(dev(v), out=out_d, offsets=off_d, scales=scl_d)
        v_h = torch.from_numpy(v.reshape(-1).copy()).pin_memory()
        out_h = torch.zeros(nout, dtype=torch.uint8).pin_memory()
        off_h = torch.zeros(nstat, dtype=torch.float32).pin_memory()
        scl_h = torch.zeros(nstat, dtype=torch.float32).pin_memory()
        st = torch.cuda.current_stream()
        mb.run_host(v_h, out_h, off_h, scl_h, stream=st)
        st.synchronize()
        assert vgb.check_device_status() == 0
        assert torch.equal(out_h, out_d.cpu())
        assert torch.equal(off_h, off_d.cpu()) and torch.equal(scl_h, scl_d.cpu())
        assert mb.launches() == 5 * ncc
        assert (mb.last_pair() > 0) == (variant == 2)
        mb.close()
    finally:
        vgb_mod.multibeam_beam_variant(prev)


def test_multibeam_all_tiles_flagged(vgb_mod, torch, oracle_mod):
    """Every tile flagged (D = 0, as calibration.c's NaN rows become): all
    weights vanish, Stokes are exactly 0 and the 8-bit stage gives the
    reference's bytes for a constant row (scale 0 -> NaN quotient -> 0)."""
    nant, npnt, nfine, ns = 16, 32, 32, 100
    case = make_case(oracle_mod, nant, npnt, nfine, ns, seed=41)
    case["D"][:] = 0.0
    res = run_mb(vgb_mod, torch, case, nant, npnt, nfine, ns, 4, 0, psrfits=True)
    assert np.all(res["S"] == 0)
    assert np.all(res["out"] == 0) and np.all(res["scl"] == 0) and np.all(res["off"] == 0)
    off, scl, u8 = oracle_mod.renormalise(np.ascontiguousarray(res["S"].transpose(1, 3, 2, 0)))
    assert np.array_equal(res["out"], u8)


def test_multibeam_against_reference_kernels(vgb_mod, torch):
    """Five pointings of the reference's own beamformer kernels
    (tests/golden/ref_golden_multibeam.npz), summed over each 10-sample
    integration, against the tensor-core path built from the same D, B,
    geometry and voltages (split BF16: within 1e-3)."""
    import os

    g = dict(np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                  "ref_golden_multibeam.npz")))
    npnt, ns, nst, nfine = g["S"].shape[0], g["S"].shape[1], 4, g["S"].shape[3]
    nant = g["D"].shape[0]
    case = dict(D=g["D"], B=g["B"], unit=g["unit"], east=g["east"], north=g["north"], height=g["height"],
                cable=g["cable"], freqs=g["freqs"], polQ=g["polQ"], polP=g["polP"], v_dev=np.ascontiguousarray(g["v"]))
    res = run_mb(vgb_mod, torch, case, nant, npnt, nfine, ns, nst, 0, invw=float(g["invw"]))
    ref = g["S"].astype(np.float64).reshape(npnt, ns // NINT, NINT, nst, nfine).sum(axis=2).transpose(3, 0, 2, 1)
    errs = stokes_err(res["S"], ref)
    assert max(errs) < 1e-3, errs


def test_multibeam_rejects_bad_config(vgb_mod):
    with pytest.raises(vgb_mod.VGBError, match="multiple of 16"):
        vgb_mod.Multibeam(1, 4, 20, 8, 100)
    with pytest.raises(vgb_mod.VGBError, match="multiple of 10"):
        vgb_mod.Multibeam(1, 4, 32, 8, 105)


def test_mwax_smart_pfb_into_multibeam(vgb_mod, torch, oracle_mod):
    """The --smart many-beam flow on one device: MWAX 8-bit voltages through
    the fine PFB to 4+4-bit bytes in the legacy input order (vgb_fpfb), then
    the many-beam GEMMs read those bytes where they are, with polQ/polP from
    the same input order. The PFB bytes match the oracle's PFB (one LSB on
    <= 1e-4 of nibbles, the FFT's rounding), the Stokes match the FP64
    beamformer chain on the PFB's own bytes (split BF16, 1e-3)."""
    from helpers import pol_lists

    O = oracle_mod
    nant, npnt, ns, K, P = 16, 40, 500, 128, 12
    ni = 2 * nant
    htr = O.mwax_buffer(77, 2, ni)                 # the margin block, then one block: 500 spectra
    filt = SY.analysis_filter_int16()
    i_idx = SY.legacy_input_order(nant)
    d = dev(htr.reshape(-1).view(np.uint8))
    v = vgb_mod.reference_buffer_voltages(d, ni, 1)
    fine = torch.empty(ns * K * ni, dtype=torch.uint8, device="cuda")
    vgb_mod.fpfb(v, 1, ns, dev(filt), dev(i_idx), vgb_mod.PFB_SMART, fine)
    torch.cuda.synchronize()
    assert vgb_mod.check_device_status() == 0
    got = host(fine).reshape(ns, K, ni)
    ref = O.fpfb(htr, ni, ns, filt, K, P, i_idx, O.PFB_SMART)
    nib = lambda b: np.stack([(b.astype(np.int16) >> 4), (b.astype(np.int16) & 15)])
    dn = np.abs(((nib(got) + 8) % 16) - ((nib(ref) + 8) % 16))
    assert dn.max() <= 1 and (dn > 0).mean() <= 1e-4

    case = make_case(O, nant, npnt, K, ns)
    polQ, polP = pol_lists(i_idx)
    case.update(polQ=polQ, polP=polP, v_oracle=got)
    invw = 1.0 / ni
    mb = vgb_mod.Multibeam(1, K, nant, npnt, ns, nstokes=4, precision=vgb_mod.MB_SPLIT_BF16, input=vgb_mod.MB_INT4,
                           invw=invw)
    mb.set_geometry(dev(case["unit"]), dev(case["east"]), dev(case["north"]), dev(case["height"]),
                    dev(case["cable"]))
    mb.set_jones(dev(case["D"]), dev(case["B"]), dev(case["freqs"]), dev(polQ), dev(polP))
    S = torch.full((K * npnt * 4 * (ns // NINT),), float("nan"), dtype=torch.float32, device="cuda")
    mb.run(fine, S=S)
    torch.cuda.synchronize()
    assert vgb_mod.check_device_status() == 0
    mb.close()
    errs = stokes_err(host(S).reshape(K, npnt, 4, ns // NINT), oracle_stokes(O, case, 4, invw))
    assert max(errs) < 1e-3, errs


def _run_variant(vgb, torch, case, nant, npnt, nfine, ns, nstokes, precision, variant, int8=False):
    prev = vgb.multibeam_beam_variant(variant)
    try:
        mb = vgb.Multibeam(1, nfine, nant, npnt, ns, nstokes=nstokes, precision=precision,
                           input=vgb.MB_INT8 if int8 else vgb.MB_INT4)
        mb.set_geometry(dev(case["unit"]), dev(case["east"]), dev(case["north"]), dev(case["height"]),
                        dev(case["cable"]))
        mb.set_jones(dev(case["D"]), dev(case["B"]), dev(case["freqs"]), dev(case["polQ"]), dev(case["polP"]))
        nint = ns // NINT
        S = torch.full((nfine * npnt * nstokes * nint,), float("nan"), dtype=torch.float32, device="cuda")
        out = torch.empty(npnt * nint * nstokes * nfine, dtype=torch.uint8, device="cuda")
        off = torch.empty(npnt * nstokes * nfine, dtype=torch.float32, device="cuda")
        scl = torch.empty_like(off)
        mb.run(dev(case["v_dev"]), S=S, out=out, offsets=off, scales=scl)
        torch.cuda.synchronize()
        assert vgb.check_device_status() == 0
        res = dict(S=host(S), out=host(out), off=host(off), scl=host(scl), pair=mb.last_pair())
        mb.close()
        return res
    finally:
        vgb.multibeam_beam_variant(prev)


@pytest.mark.parametrize("precision,nstokes,int8", [(0, 4, False), (2, 4, False), (1, 4, False), (0, 1, True),
                                                    (2, 1, True)])
def test_multibeam_pair_kernel_equals_single(vgb_mod, torch, oracle_mod, precision, nstokes, int8):
    """The beam GEMM over CTA pairs (cta_group::2: two SMs share each 256-row
    MMA, each staging half of the voltage tile) gives the single-CTA kernel's
    Stokes and PSRFITS bytes bit for bit: four beam tiles (two pairs), a
    sample count that leaves the last sample tile partly used, three fine
    channels; and, checked against the FP64 oracle, within the mode's
    tolerance."""
    nant, npnt, nfine, ns = 32, 128, 3, 770
    case = make_case(oracle_mod, nant, npnt, nfine, ns, seed=61, int8=int8)
    single = _run_variant(vgb_mod, torch, case, nant, npnt, nfine, ns, nstokes, precision, 1, int8)
    pair = _run_variant(vgb_mod, torch, case, nant, npnt, nfine, ns, nstokes, precision, 2, int8)
    assert not single["pair"] and pair["pair"]
    assert not np.isnan(pair["S"]).any()
    for k in ("S", "out", "off", "scl"):
        assert np.array_equal(single[k], pair[k]), k
    ref = oracle_stokes(oracle_mod, case, nstokes, 1.0 / (2 * nant))
    errs = stokes_err(pair["S"].reshape(nfine, npnt, nstokes, ns // NINT), ref)
    tol = {0: 1e-3, 2: 4e-3, 1: 3e-2}[precision]
    assert max(errs) < tol, errs


def test_multibeam_pair_kernel_selection(vgb_mod, torch, oracle_mod):
    """The automatic choice times both kernels where the 32-beam tiles pair up
    (whichever it keeps, the bytes are the single-CTA kernel's) and takes the
    single-CTA kernel otherwise (three tiles); forcing the pair kernel on three
    tiles is an error, not a different result."""
    nant, nfine, ns = 16, 2, 250
    even = make_case(oracle_mod, nant, 64, nfine, ns, seed=62)
    odd = make_case(oracle_mod, nant, 70, nfine, ns, seed=63)
    auto = _run_variant(vgb_mod, torch, even, nant, 64, nfine, ns, 4, 0, 0)
    single = _run_variant(vgb_mod, torch, even, nant, 64, nfine, ns, 4, 0, 1)
    for k in ("S", "out", "off", "scl"):
        assert np.array_equal(auto[k], single[k]), k
    assert not _run_variant(vgb_mod, torch, odd, nant, 70, nfine, ns, 4, 0, 0)["pair"]
    with pytest.raises(vgb_mod.VGBError, match="even number of beam tiles"):
        _run_variant(vgb_mod, torch, odd, nant, 70, nfine, ns, 4, 0, 2)
    with pytest.raises(vgb_mod.VGBError):
        vgb_mod.multibeam_beam_variant(3)


@pytest.mark.parametrize("nant,npnt,nfine,ns,nstokes,int8", [
    (16, 64, 1, 250, 4, False),     # one beam-tile pair, one sample tile, one 64-wide K step
    (16, 40, 3, 10, 4, False),      # one integration: a sample tile with 10 of 256 columns used
    (64, 256, 2, 2500, 1, True),    # 8-bit, Stokes I, 4 pairs x 10 sample tiles x 2 channels
    (32, 64, 96, 260, 4, False),    # 1 pair x 2 sample tiles x 96 channels = 192 pair tiles
    (32, 96, 4, 260, 4, False),     # three beam tiles: odd, so the automatic choice is one CTA
])
def test_multibeam_pair_kernel_edges(vgb_mod, torch, oracle_mod, nant, npnt, nfine, ns, nstokes, int8):
    """The CTA-pair beam GEMM at the edges of its tiling equals the single-CTA
    kernel bit for bit (where the beam tiles pair up), including runs with
    more beam-tile pairs than co-resident clusters (80 and 192 pair tiles on
    at most 76 clusters)."""
    case = make_case(oracle_mod, nant, npnt, nfine, ns, seed=71, int8=int8)
    single = _run_variant(vgb_mod, torch, case, nant, npnt, nfine, ns, nstokes, 0, 1, int8)
    bp = (npnt + 31) // 32
    if bp % 2:
        auto = _run_variant(vgb_mod, torch, case, nant, npnt, nfine, ns, nstokes, 0, 0, int8)
        assert not auto["pair"]
        other = auto
    else:
        other = _run_variant(vgb_mod, torch, case, nant, npnt, nfine, ns, nstokes, 0, 2, int8)
        assert other["pair"] > 0
    for k in ("S", "out", "off", "scl"):
        assert np.array_equal(single[k], other[k]), k
    assert not np.isnan(single["S"]).any()
