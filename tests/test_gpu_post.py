"""Renormalise / quantise, the incoherent beam and the inverse PFB + VDIF
against the reference's own kernels and the oracle.

Tolerances: renormalise and the incoherent beam are bit-exact (same FP32
operations as the reference kernel on the same inputs); the inverse PFB is
within 1e-5 of the output rms outside the 1,524 samples per second where the
reference's tap range is wrong; VDIF bytes within one LSB on <= 1e-4 of them.
"""
import numpy as np
import pytest

from helpers import dev, host, torch_cuda

pytestmark = pytest.mark.gpu

K, P = 128, 12


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


@pytest.fixture(scope="module")
def vgb_mod(torch):
    import vgb

    vgb.lib()
    return vgb


def renorm(vgb, torch, S, ncc=1):
    ncc_, npnt, nstep, nst, nc = S.shape
    out = torch.empty(S.size, dtype=torch.uint8, device="cuda")
    off = torch.empty(ncc_ * npnt * nst * nc, dtype=torch.float32, device="cuda")
    sc = torch.empty_like(off)
    vgb.renormalise(dev(S), ncc_, npnt, nstep, nst, nc, out, npnt * nstep * nst * nc, nstep * nst * nc,
                    nst * nc, nc, off, sc)
    torch.cuda.synchronize()
    return host(off).reshape(ncc_, npnt, nst, nc), host(sc).reshape(ncc_, npnt, nst, nc), host(out).reshape(S.shape)


def test_renormalise_matches_reference_kernel(vgb_mod, torch, golden):
    off, sc, u8 = renorm(vgb_mod, torch, golden["rn_in"][None])
    assert np.array_equal(off[0], golden["rn_off"])
    assert np.array_equal(sc[0], golden["rn_scale"], equal_nan=True)
    assert np.array_equal(u8[0], golden["rn_u8"])


def test_renormalise_rounding_boundaries(vgb_mod, torch, oracle_mod):
    """Values whose scaled quotient lies within a few ulps of every
    half-integer (where the byte changes), plus the wrap at the maximum: the
    division-free fast path must agree with the reference's divide bit for
    bit."""
    rng = np.random.default_rng(17)
    nstep, nc = 4000, K
    scale = np.float32(10.0 ** rng.uniform(-3, 3, size=nc)).astype(np.float32)
    k = rng.integers(0, 257, size=(nstep, nc))
    target = ((k + 0.5) * scale.astype(np.float64)).astype(np.float32)
    bits = target.view(np.int32) + rng.integers(-4, 5, size=target.shape).astype(np.int32)
    S = bits.view(np.float32).copy()
    S[0] = 0.0                                          # row minimum
    S[1] = (256.0 * scale.astype(np.float64)).astype(np.float32)   # row maximum
    S = np.ascontiguousarray(S.reshape(1, 1, nstep, 1, nc))
    off, sc, u8 = renorm(vgb_mod, torch, S)
    o, s_, u = oracle_mod.renormalise(S[0])
    assert np.array_equal(off[0], o) and np.array_equal(sc[0], s_)
    assert np.array_equal(u8[0], u)


def test_renormalise_spliced_layout(vgb_mod, torch, oracle_mod):
    """Two coarse channels written straight into spliced PSRFITS rows
    [s][stokes][cc*128 + c] (no gather step)."""
    rng = np.random.default_rng(3)
    S = rng.standard_normal((2, 1, 100, 4, K)).astype(np.float32)
    out = torch.empty(100 * 4 * 2 * K, dtype=torch.uint8, device="cuda")
    off = torch.empty(2 * 4 * K, dtype=torch.float32, device="cuda")
    sc = torch.empty_like(off)
    vgb_mod.renormalise(dev(S), 2, 1, 100, 4, K, out, K, 0, 4 * 2 * K, 2 * K, off, sc)
    torch.cuda.synchronize()
    spliced = host(out).reshape(100, 4, 2, K)
    for cc in range(2):
        o, s, u = oracle_mod.renormalise(S[cc])
        assert np.array_equal(spliced[:, :, cc, :], u[0])
        assert np.array_equal(host(off).reshape(2, 4, K)[cc], o[0])
        assert np.array_equal(host(sc).reshape(2, 4, K)[cc], s[0])


def test_incoherent_matches_reference_kernel(vgb_mod, torch, golden):
    data = golden["fpfb_smart_out"]
    ns, nc, ni = data.shape
    out = torch.empty(ns * nc, dtype=torch.float32, device="cuda")
    vgb_mod.incoh_beam(dev(data), ns * nc, ni, out)
    torch.cuda.synchronize()
    assert np.array_equal(host(out).reshape(ns, nc), golden["incoh"])
    # an input count that is not a multiple of 32 takes the byte path
    sub = np.ascontiguousarray(data[:, :, :20])
    out2 = torch.empty(ns * nc, dtype=torch.float32, device="cuda")
    vgb_mod.incoh_beam(dev(sub), ns * nc, 20, out2)
    torch.cuda.synchronize()
    import oracle as O

    assert np.array_equal(host(out2).reshape(ns, nc), O.incoh_beam(sub))


def run_ipfb(vgb, torch, e, hist, coeffs, want_vdif=True, hdr=None):
    njobs, ns = e.shape[0], e.shape[1]
    outf = torch.empty(njobs * ns * K * 4, dtype=torch.float32, device="cuda")
    vd = torch.empty(njobs * ns * 544, dtype=torch.uint8, device="cuda") if want_vdif else None
    vgb.ipfb(dev(e.astype(np.complex64)), ns * K * 16, None if hist is None else dev(hist.astype(np.complex64)),
             P * K * 16, dev(coeffs.astype(np.float32)), ns, njobs, out_f=outf, vdif=vd,
             hdr=None if hdr is None else dev(hdr))
    torch.cuda.synchronize()
    f = host(outf).reshape(njobs, ns * K, 2, 2)
    return f[..., 0] + 1j * f[..., 1], (host(vd).reshape(njobs, ns, 544) if want_vdif else None)


@pytest.mark.parametrize("sec", [0, 1])
def test_ipfb_matches_reference_kernel(vgb_mod, torch, golden, sec):
    ev = golden["ipfb_e"]
    ns = ev.shape[1]
    hist = None if sec == 0 else ev[0, ns - P:][None]
    ours, _ = run_ipfb(vgb_mod, torch, ev[sec][None], hist, golden["ipfb_coeffs"], want_vdif=False)
    ref = golden[f"ipfb_out{sec}"]
    ref_c = ref[..., 0] + 1j * ref[..., 1]
    n = np.arange(ns * K)
    good = (n >= P * K) | (n % K == 0)
    rms = np.sqrt(np.mean(np.abs(ref_c) ** 2))
    assert np.abs(ours[0][good] - ref_c[good]).max() / rms < 1e-5


def test_ipfb_vdif_against_oracle(vgb_mod, torch, oracle_mod, golden):
    ev = golden["ipfb_e"].astype(np.complex128)
    ns = ev.shape[1]
    hdr = np.array([[0x1234567, 0x2A000000, 68, 0x8C000000 | 0x6D77, 5, 6, 7, 8]], dtype=np.uint32)
    ours, vd = run_ipfb(vgb_mod, torch, ev[1][None], ev[0, ns - P:][None], golden["ipfb_coeffs"], hdr=hdr)
    x = np.concatenate([ev[0, ns - P:], ev[1]], axis=0)
    truth = oracle_mod.ipfb(x, golden["ipfb_coeffs"], P)           # [n][pol] complex
    rms = np.sqrt(np.mean(np.abs(truth) ** 2))
    assert np.abs(ours[0] - truth).max() / rms < 1e-5
    flt = np.stack([truth.real, truth.imag], axis=-1).astype(np.float32).reshape(ns, 512)
    qref = oracle_mod.vdif_quantise(flt)
    payload = vd[0, :, 32:]
    diff = np.abs(payload.astype(np.int16) - qref.astype(np.int16))
    assert diff.max() <= 1 and (diff > 0).mean() <= 1e-4
    words = vd[0, :, :32].copy().view(np.uint32)
    assert np.array_equal(words[:, 0], np.full(ns, hdr[0, 0]))
    assert np.array_equal(words[:, 1] & 0xFFFFFF, np.arange(ns, dtype=np.uint32))
    assert np.all(words[:, 1] >> 24 == 0x2A)
    assert np.array_equal(words[:, 2:], np.broadcast_to(hdr[0, 2:], (ns, 6)))


def test_vdif_headers_roll_over(vgb_mod, torch, golden):
    """Frame f of a call carries the template advanced f frames at 10000
    frames per second (nextVDIFHeader); vgb_vdif_advance takes a template the
    same number of frames as the host's vgb_vdif_header_next."""
    ev = golden["ipfb_e"]
    ns = ev.shape[1]
    hdrs = []
    for j, frame in enumerate([9990, 0, 10000 - ns]):
        h = vgb_mod.vdif_populate_header(60123 + j, 0.25, threadid=j)
        vgb_mod.vdif_header_set_frame(h, frame)
        hdrs.append(h)
    hdr = np.stack(hdrs)
    e = np.broadcast_to(ev[1][None], (3,) + ev[1].shape)
    _, vd = run_ipfb(vgb_mod, torch, np.ascontiguousarray(e), None, golden["ipfb_coeffs"], hdr=hdr)
    for j in range(3):
        h = hdr[j].copy()
        words = vd[j, :, :32].copy().view(np.uint32)
        for f in range(ns):
            assert np.array_equal(words[f], h), (j, f)
            vgb_mod.vdif_header_next(h)
    d = dev(hdr)
    for n in (1, 9, 10000, 23457):
        vgb_mod.vdif_advance(d, 3, n)
        for j in range(3):
            for _ in range(n):
                vgb_mod.vdif_header_next(hdr[j])
        torch.cuda.synchronize()
        assert np.array_equal(host(d, dtype=np.uint32).reshape(3, 8), hdr), n
