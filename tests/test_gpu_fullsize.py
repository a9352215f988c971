"""The full-band second at its full size (24 coarse channels x 128 tiles x 20
MWAX blocks = 15.7 GB of voltages, Gaussian sigma 16 clipped to +-127 as the
benchmark draws them), checked through properties that do not depend on
size:

* the 8-bit PSRFITS bytes, offsets and scales of all 24 channels equal the
  oracle's renormalise of the device's own Stokes (bit for bit, spliced
  layout);
* one channel's whole second matches the FP64 oracle chain (PFB,
  beamformer, renormalise of the oracle's Stokes, inverse PFB of the oracle's
  beam voltages): Stokes and beam voltages within 1e-5 norm-wise, PSRFITS
  bytes within one LSB on <= 1e-4 of samples, VDIF bytes within one LSB on
  <= 1e-4; another channel's first 200 fine spectra match the oracle's PFB +
  beamformer and its VDIF the oracle's inverse PFB of the device's beam
  voltages;
* channels are independent: rolling the input channels (voltages and
  weights) rolls every product, bit for bit.
"""
import numpy as np
import pytest

import synthetic as SY
from helpers import byte_diff_stats, oracle_chain_second, pol_lists, rel_err, tables, torch_cuda, weights_on_device

pytestmark = pytest.mark.gpu

K, P = 128, 12
NANT, NCC, NBLK = 128, 24, 20
NI = 2 * NANT
NS = NBLK * 500
SPOT = 200          # spectra of the oracle spot checks
ROLL = 5


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


@pytest.fixture(scope="module")
def vgb_mod(torch):
    import vgb

    vgb.lib()
    return vgb


def run_second(vgb, volt, W, filt, syn, invw):
    p = vgb.Pipeline(NCC, NANT, NBLK, nstokes=4, pfb_flags=0, do_ipfb=True, invw=invw)
    p.set_filters(filt, syn)
    p.set_weights(W, on_device=True)
    p.run_device(volt)
    out = dict(ps=np.empty((NS, 4, NCC * K), np.uint8), off=np.empty((NCC, 4, K), np.float32),
               sc=np.empty((NCC, 4, K), np.float32), vd=np.empty((NCC, NS, 544), np.uint8),
               S=np.empty((NCC, NS, 4, K), np.float32), e=np.empty((NCC, NS, K, 2), np.complex64))
    p.fetch(out["ps"], out["off"], out["sc"], out["vd"])
    p.fetch_raw(out["S"], out["e"])
    p.close()
    assert vgb.check_device_status() == 0
    return out


def test_full_band_second(vgb_mod, torch, oracle_mod):
    O = oracle_mod
    g = torch.Generator(device="cuda").manual_seed(2024)
    volt = torch.empty((NCC, NBLK, NI, 64000, 2), dtype=torch.int8, device="cuda")
    for cc in range(NCC):
        x = torch.randn((NBLK, NI, 64000, 2), generator=g, device="cuda", dtype=torch.float32)
        volt[cc] = x.mul_(16.0).round_().clamp_(-127, 127).to(torch.int8)
        del x
    filt = SY.analysis_filter_int16()
    syn = SY.synthesis_filter(scale=SY.synthesis_scale(filt))
    tabs = [tables(NANT, cc=cc, seed=cc + 1) for cc in range(NCC)]
    W = torch.cat([weights_on_device(J, phi) for J, phi in tabs])
    invw = 1.0 / NI
    out = run_second(vgb_mod, volt, W, filt, syn, invw)

    # PSRFITS bytes of every channel from the device's own Stokes
    for cc in range(NCC):
        off, sc, u8 = O.renormalise(out["S"][cc][None])
        assert np.array_equal(out["ps"][:, :, cc * K:(cc + 1) * K], u8[0]), cc
        assert np.array_equal(out["off"][cc], off[0]) and np.array_equal(out["sc"][cc], sc[0]), cc

    # one whole channel against the oracle chain
    cc = 17
    blocks = volt[cc].cpu().numpy()
    buf = np.ascontiguousarray(np.concatenate([np.zeros_like(blocks[:1]), blocks], axis=0))
    J, phi = tabs[cc]
    Sr, er, (offr, scr, psr), vdr = oracle_chain_second(buf, NI, filt, syn, J, phi, invw)
    assert rel_err(out["S"][cc], Sr) < 1e-5 and rel_err(out["e"][cc], er) < 1e-5
    assert byte_diff_stats(out["ps"][:, :, cc * K:(cc + 1) * K], psr)[1] <= 1e-4
    mx, _, frac = byte_diff_stats(out["vd"][cc, :, 32:], vdr)
    assert mx <= 1 and frac <= 1e-4
    del blocks, buf

    # spot checks against the oracle's chain: another channel, first spectra, and its VDIF
    i_idx = np.arange(NI, dtype=np.int32)
    polQ, polP = pol_lists(i_idx)
    for cc in (0,):
        blk0 = volt[cc, 0].cpu().numpy()
        buf = np.ascontiguousarray(np.concatenate([np.zeros_like(blk0)[None], blk0[None]], axis=0))
        v = O.fpfb(buf, NI, SPOT, filt, K, P, i_idx, 0)
        J, phi = tabs[cc]
        Sref, eref = O.beamform(v, J, phi, polQ, polP, invw)
        assert rel_err(out["S"][cc][:SPOT], Sref[0]) < 1e-5, cc
        assert rel_err(out["e"][cc][:SPOT], eref[0]) < 1e-5, cc
        x = np.concatenate([np.zeros((P, K, 2)), out["e"][cc].astype(np.complex128)], axis=0)
        truth = O.ipfb(x, syn, P)
        flt = np.stack([truth.real, truth.imag], axis=-1).astype(np.float32).reshape(NS, 512)
        q = O.vdif_quantise(flt)
        dq = np.abs(out["vd"][cc, :, 32:].astype(np.int16) - q.astype(np.int16))
        assert dq.max() <= 1 and (dq > 0).mean() <= 1e-4, cc

    # channel independence: roll the channels (voltages and weights)
    rolled = torch.roll(volt, ROLL, dims=0)
    del volt
    Wr = torch.roll(W.view(NCC, -1, 8), ROLL, dims=0).reshape(W.shape).contiguous()
    out2 = run_second(vgb_mod, rolled, Wr, filt, syn, invw)
    del rolled
    assert np.array_equal(out2["S"], np.roll(out["S"], ROLL, axis=0))
    assert np.array_equal(out2["e"], np.roll(out["e"], ROLL, axis=0))
    assert np.array_equal(out2["vd"], np.roll(out["vd"], ROLL, axis=0))
    assert np.array_equal(out2["ps"].reshape(NS, 4, NCC, K), np.roll(out["ps"].reshape(NS, 4, NCC, K), ROLL, axis=2))
    torch.cuda.empty_cache()
