"""The 1024-beam case at its full size (256 tiles x 2 pols of 4-bit voltages,
1024 beams, 128 fine channels x 1 s, full Stokes at 1 ms, split BF16),
checked through properties that do not depend on size:

* the 8-bit PSRFITS bytes, offsets and scales equal the oracle's renormalise
  of the device's own Stokes, bit for bit;
* three beams x two channels x the first 20 integrations match the FP64
  oracle chain (reference tables, per-sample beamformer summed over each
  integration) within 1e-4 of each Stokes parameter's largest magnitude;
* beams are independent: permuting the pointings (and their primary-beam
  matrices) permutes every product, bit for bit;
* the beam GEMM over CTA pairs (cta_group::2) and the single-CTA kernel give
  the same products, bit for bit.
"""
import numpy as np
import pytest

import synthetic as SY
from helpers import dev, host, pol_lists, torch_cuda

pytestmark = pytest.mark.gpu

NANT, NF, NS, NB, NINT = 256, 128, 10000, 1024, 10
NT = NS // NINT


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


@pytest.fixture(scope="module")
def vgb_mod(torch):
    import vgb

    vgb.lib()
    return vgb


def test_multibeam_full_size(vgb_mod, torch, oracle_mod):
    O, vgb = oracle_mod, vgb_mod
    D = SY.calibration_jones(NANT, NF, seed=3)
    B = np.ascontiguousarray(SY.identity_beam(NB, NANT) +
                             0.05 * (1 + 1j) * O.gauss(7, NB * NANT * 4).reshape(NB, NANT, 2, 2))
    east, north, height, cable = SY.tile_layout(NANT, seed=5)
    az, za = SY.grid_pointings(32, 0.02)
    unit = np.ascontiguousarray(SY.unit_vectors(az, za))
    freqs = SY.fine_chan_freqs_hz(SY.coarse_chan_start_hz(0))[:NF].astype(np.float64)
    polQ, polP = pol_lists(SY.legacy_input_order(NANT))
    g = torch.Generator(device="cuda").manual_seed(11)
    nb = NS * NF * 2 * NANT
    re = torch.randn(nb, device="cuda", generator=g).mul_(2.5).round_().clamp_(-8, 7).to(torch.int32)
    im = torch.randn(nb, device="cuda", generator=g).mul_(2.5).round_().clamp_(-8, 7).to(torch.int32)
    v = (((re & 15) << 4) | (im & 15)).to(torch.uint8)
    del re, im
    invw = 1.0 / (2 * NANT)

    def run(unit_, B_):
        mb = vgb.Multibeam(1, NF, NANT, NB, NS, nstokes=4, precision=vgb.MB_SPLIT_BF16, input=vgb.MB_INT4,
                           invw=invw)
        mb.set_geometry(dev(unit_), dev(east), dev(north), dev(height), dev(cable))
        mb.set_jones(dev(D), dev(np.ascontiguousarray(B_)), dev(freqs), dev(polQ), dev(polP))
        S = torch.empty(NF * NB * 4 * NT, dtype=torch.float32, device="cuda")
        out = torch.empty(NB * NT * 4 * NF, dtype=torch.uint8, device="cuda")
        off = torch.empty(NB * 4 * NF, dtype=torch.float32, device="cuda")
        scl = torch.empty_like(off)
        mb.run(v, S=S, out=out, offsets=off, scales=scl)
        torch.cuda.synchronize()
        assert vgb.check_device_status() == 0
        mb.close()
        return (host(S).reshape(NF, NB, 4, NT), host(out).reshape(NB, NT, 4, NF), host(off).reshape(NB, 4, NF),
                host(scl).reshape(NB, 4, NF))

    prev = vgb.multibeam_beam_variant(1)
    try:
        S1, u1, off1, sc1 = run(unit, B)
        vgb.multibeam_beam_variant(2)
        Sp, up, offp, scp = run(unit, B)
    finally:
        vgb.multibeam_beam_variant(prev)
    assert np.array_equal(Sp, S1) and np.array_equal(up, u1)
    assert np.array_equal(offp, off1) and np.array_equal(scp, sc1)
    del Sp, up

    # PSRFITS bytes from the device's own Stokes, in [beam][t][stokes][chan]
    off, sc, u8 = O.renormalise(np.ascontiguousarray(S1.transpose(1, 3, 2, 0)))
    assert np.array_equal(u1, u8)
    assert np.array_equal(off1, off) and np.array_equal(sc1, sc)

    # spot check against the FP64 oracle chain
    beams, chans, nsamp = [0, 517, 1023], [0, 77], 20 * NINT
    vsub = np.ascontiguousarray(v[: nsamp * NF * 2 * NANT].cpu().numpy().reshape(nsamp, NF, 2 * NANT)[:, chans])
    J = O.calc_j(np.ascontiguousarray(D[:, chans]), np.ascontiguousarray(B[beams]))
    phi = O.calc_phi(unit[beams], east, north, height, cable, freqs[chans])
    Sref, _ = O.beamform(vsub, J, phi, polQ, polP, invw, nstokes=4, want_e=False)
    ref = Sref.astype(np.float64).reshape(len(beams), 20, NINT, 4, len(chans)).sum(axis=2)   # [p][t][st][c]
    got = S1[chans][:, beams][..., :20].transpose(1, 3, 2, 0)                               # [p][t][st][c]
    for st in range(4):
        err = np.abs(got[:, :, st] - ref[:, :, st]).max() / np.abs(ref[:, :, st]).max()
        assert err < 1e-4, (st, err)

    # permuting the pointings permutes the products
    perm = np.random.default_rng(13).permutation(NB)
    S2, u2, off2, sc2 = run(unit[perm], B[perm])
    assert np.array_equal(S2, S1[:, perm])
    assert np.array_equal(u2, u1[perm])
    assert np.array_equal(off2, off1[perm]) and np.array_equal(sc2, sc1[perm])
    torch.cuda.empty_cache()


def test_multibeam_c3_full_size(vgb_mod, torch, oracle_mod):
    """The 256-beam case at its full size (128 tiles x 2 pols of 8-bit
    voltages, 256 beams, 128 fine channels x 1 s, Stokes I at 1 ms): the
    CTA-pair and single-CTA beam GEMMs give the same split-BF16 products bit
    for bit; the PSRFITS bytes, offsets and scales are the oracle's
    renormalise of the device's Stokes; FP16 weights stay within 1e-3 and
    split BF16 within 1e-5 of FP32 weights on the CUDA cores, all on the same
    voltages and tables."""
    O, vgb = oracle_mod, vgb_mod
    nant, nb, nf, ns = 128, 256, 128, 10000
    nt = ns // NINT
    D = SY.calibration_jones(nant, nf, seed=13)
    B = np.ascontiguousarray(SY.identity_beam(nb, nant) +
                             0.05 * (1 + 1j) * O.gauss(17, nb * nant * 4).reshape(nb, nant, 2, 2))
    east, north, height, cable = SY.tile_layout(nant, seed=15)
    az, za = SY.grid_pointings(16, 0.02)
    unit = np.ascontiguousarray(SY.unit_vectors(az, za))
    freqs = SY.fine_chan_freqs_hz(SY.coarse_chan_start_hz(3))[:nf].astype(np.float64)
    polQ, polP = pol_lists(np.arange(2 * nant))
    g = torch.Generator(device="cuda").manual_seed(19)
    v = torch.randn(ns * nf * 2 * nant * 2, device="cuda", generator=g).mul_(16).round_().clamp_(-127, 127)
    v = v.to(torch.int8).view(torch.uint8)
    invw = 1.0 / (2 * nant)

    def run(precision, variant):
        prev = vgb.multibeam_beam_variant(variant)
        try:
            mb = vgb.Multibeam(1, nf, nant, nb, ns, nstokes=1, precision=precision, input=vgb.MB_INT8, invw=invw)
            mb.set_geometry(dev(unit), dev(east), dev(north), dev(height), dev(cable))
            mb.set_jones(dev(D), dev(B), dev(freqs), dev(polQ), dev(polP))
            S = torch.empty(nf * nb * nt, dtype=torch.float32, device="cuda")
            out = torch.empty(nb * nt * nf, dtype=torch.uint8, device="cuda")
            off = torch.empty(nb * nf, dtype=torch.float32, device="cuda")
            scl = torch.empty_like(off)
            mb.run(v, S=S, out=out, offsets=off, scales=scl)
            torch.cuda.synchronize()
            assert vgb.check_device_status() == 0
            pair = mb.last_pair()
            mb.close()
            return S, host(out).reshape(nb, nt, 1, nf), host(off).reshape(nb, 1, nf), host(scl).reshape(nb, 1, nf), pair
        finally:
            vgb.multibeam_beam_variant(prev)

    S1, u1, o1, c1, p1 = run(vgb.MB_SPLIT_BF16, 1)
    S2, u2, o2, c2, p2 = run(vgb.MB_SPLIT_BF16, 2)
    assert p1 == 0 and p2 > 0
    assert torch.equal(S1, S2) and np.array_equal(u1, u2) and np.array_equal(o1, o2) and np.array_equal(c1, c2)
    off, sc, u8 = O.renormalise(np.ascontiguousarray(host(S1).reshape(nf, nb, 1, nt).transpose(1, 3, 2, 0)))
    assert np.array_equal(u1, u8) and np.array_equal(o1, off) and np.array_equal(c1, sc)
    S32 = run(vgb.MB_FP32, 0)[0]
    S16 = run(vgb.MB_FP16, 0)[0]
    scale = S32.abs().max().item()
    assert (S1 - S32).abs().max().item() / scale < 1e-5
    assert (S16 - S32).abs().max().item() / scale < 1e-3
    torch.cuda.empty_cache()
