"""The one-second streaming pipeline (vgb_pipeline_*) over two seconds and two
coarse channels, against the oracle chain on the same timeline: the voltage
and beam histories carried across the second boundary, spliced PSRFITS
bytes, and VDIF.

Tolerances as in the per-kernel tests: Stokes within 1e-5 of the largest
magnitude; 8-bit bytes within one LSB on <= 1e-4 of samples (the reference
maps each channel's maximum to 0; both sides do, at the same sample).
"""
import numpy as np
import pytest

import synthetic as SY
from helpers import dev, host, pol_lists, rel_err, tables, torch_cuda

pytestmark = pytest.mark.gpu

K, P = 128, 12
NANT, NCC, NBLK = 16, 2, 2
NI = 2 * NANT
NS = NBLK * 500


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


@pytest.fixture(scope="module")
def vgb_mod(torch):
    import vgb

    vgb.lib()
    return vgb


@pytest.fixture(scope="module")
def setup(oracle_mod):
    # voltages [second][cc][block][input][sample][2]
    volt = oracle_mod.gen_int8(77, 2 * NCC * NBLK * NI * 64000 * 2, 16).reshape(2, NCC, NBLK, NI, 64000, 2)
    filt = SY.analysis_filter_int16()
    syn = SY.synthesis_filter(scale=SY.synthesis_scale(filt))
    tabs = [tables(NANT, cc=cc, seed=cc + 1) for cc in range(NCC)]
    return volt, filt, syn, tabs


def oracle_second(O, volt, t, cc, filt, J, phi, invw):
    margin = np.zeros((1, NI, 64000, 2), np.int8) if t == 0 else volt[t - 1, cc, NBLK - 1:]
    buf = np.ascontiguousarray(np.concatenate([margin, volt[t, cc]], axis=0))
    i_idx = np.arange(NI, dtype=np.int32)  # identity VCS order
    v = O.fpfb(buf, NI, NS, filt, K, P, i_idx, 0)
    polQ, polP = pol_lists(i_idx)
    return O.beamform(v, J, phi, polQ, polP, invw)


def make_pipeline(vgb, torch, filt, syn, tabs, invw):
    from helpers import weights_on_device

    p = vgb.Pipeline(NCC, NANT, NBLK, nstokes=4, pfb_flags=0, do_ipfb=True, invw=invw)
    p.set_filters(filt, syn)
    W = torch.cat([weights_on_device(J, phi) for J, phi in tabs])
    p.set_weights(W, on_device=True)
    p.set_vdif_header(vdif_templates(vgb))
    return p


def vdif_templates(vgb):
    """Channel 0 starts 600 frames before a second boundary, channel 1 at one."""
    hdrs = []
    for cc, frame in enumerate([10000 - 600, 0][:NCC]):
        h = vgb.vdif_populate_header(60123, 0.25 + cc / 86400)
        vgb.vdif_header_set_frame(h, frame)
        hdrs.append(h)
    return np.stack(hdrs)


def test_pipeline_two_seconds(vgb_mod, torch, oracle_mod, setup):
    volt, filt, syn, tabs = setup
    invw = 1.0 / NI
    p = make_pipeline(vgb_mod, torch, filt, syn, tabs, invw)
    e_prev = [None] * NCC
    hdr_run = vdif_templates(vgb_mod)
    for t in range(2):
        d = dev(volt[t].reshape(-1).view(np.uint8))
        p.run_device(d)
        assert p.launch_count() >= 4
        ps = np.empty((NS, 4, NCC * K), np.uint8)
        off = np.empty((NCC, 4, K), np.float32)
        sc = np.empty((NCC, 4, K), np.float32)
        vd = np.empty((NCC, NS, 544), np.uint8)
        p.fetch(ps, off, sc, vd)
        S = np.empty((NCC, NS, 4, K), np.float32)
        e = np.empty((NCC, NS, K, 2), np.complex64)
        p.fetch_raw(S, e)
        for cc in range(NCC):
            J, phi = tabs[cc]
            Sref, eref = oracle_second(oracle_mod, volt, t, cc, filt, J, phi, invw)
            assert rel_err(S[cc], Sref[0]) < 1e-5
            assert rel_err(e[cc], eref[0]) < 1e-5
            o, s, u = oracle_mod.renormalise(S[cc][None])
            assert np.array_equal(ps[:, :, cc * K:(cc + 1) * K], u[0])
            _, _, uref = oracle_mod.renormalise(Sref)
            d8 = np.abs(ps[:, :, cc * K:(cc + 1) * K].astype(np.int16) - uref[0].astype(np.int16))
            assert ((d8 > 1).mean() <= 1e-4) and ((d8 > 0).mean() <= 1e-3)
            # VDIF against the oracle IPFB of the oracle's beam voltages
            hist = np.zeros((P, K, 2)) if t == 0 else e_prev[cc][NS - P:]
            x = np.concatenate([hist, eref[0]], axis=0)
            truth = oracle_mod.ipfb(x, syn, P)
            flt = np.stack([truth.real, truth.imag], axis=-1).astype(np.float32).reshape(NS, 512)
            q = oracle_mod.vdif_quantise(flt)
            dq = np.abs(vd[cc, :, 32:].astype(np.int16) - q.astype(np.int16))
            assert dq.max() <= 1 and (dq > 0).mean() <= 1e-4
            # headers run on from the template across the second boundary
            h = hdr_run[cc]
            words = vd[cc, :, :32].copy().view(np.uint32)
            for f in range(NS):
                assert np.array_equal(words[f], h), (t, cc, f)
                vgb_mod.vdif_header_next(h)
            e_prev[cc] = eref[0]
    p.close()


def test_pipeline_host_equals_device(vgb_mod, torch, setup):
    volt, filt, syn, tabs = setup
    invw = 1.0 / NI
    outs = []
    for mode in ("device", "host"):
        p = make_pipeline(vgb_mod, torch, filt, syn, tabs, invw)
        res = []
        for t in range(2):
            if mode == "device":
                p.run_device(dev(volt[t].reshape(-1).view(np.uint8)))
            else:
                hb = torch.from_numpy(volt[t].reshape(-1).view(np.uint8).copy()).pin_memory()
                p.run_host(hb)
            ps = np.empty((NS, 4, NCC * K), np.uint8)
            vd = np.empty((NCC, NS, 544), np.uint8)
            p.fetch(ps, None, None, vd)
            res.append((ps, vd))
        p.close()
        outs.append(res)
    for (a, b), (c, d) in zip(outs[0], outs[1]):
        assert np.array_equal(a, c) and np.array_equal(b, d)


def test_pipeline_graph_replay_equals_eager(vgb_mod, torch, setup):
    """Seconds replayed from captured CUDA graphs (two resident buffers,
    alternating; the first second captured separately) give the bytes of
    eager execution."""
    volt, filt, syn, tabs = setup
    invw = 1.0 / NI
    bufs = [dev(volt[t].reshape(-1).view(np.uint8)) for t in range(2)]
    outs = []
    for graphs in (False, True):
        p = make_pipeline(vgb_mod, torch, filt, syn, tabs, invw)
        p.enable_graphs(graphs)
        res = []
        for t in range(4):
            p.run_device(bufs[t % 2])
            ps = np.empty((NS, 4, NCC * K), np.uint8)
            vd = np.empty((NCC, NS, 544), np.uint8)
            p.fetch(ps, None, None, vd)
            res.append((ps, vd))
            assert p.launch_count() == 6      # beam, renormalise x2 (tied-array, incoherent), inverse PFB, VDIF headers, history
        p.close()
        outs.append(res)
    for (a, b), (c, d) in zip(outs[0], outs[1]):
        assert np.array_equal(a, c) and np.array_equal(b, d)


def test_pipeline_checkpoint_resume(vgb_mod, torch, setup):
    """Save the carry-over state after two seconds, load it into a new
    pipeline and continue: seconds 3 and 4 equal those of an uninterrupted
    run (voltage history, inverse-PFB history and the second counter)."""
    volt, filt, syn, tabs = setup
    invw = 1.0 / NI
    bufs = [dev(volt[t].reshape(-1).view(np.uint8)) for t in range(2)]

    def second(p, t):
        p.run_device(bufs[t % 2])
        ps = np.empty((NS, 4, NCC * K), np.uint8)
        vd = np.empty((NCC, NS, 544), np.uint8)
        p.fetch(ps, None, None, vd)
        return ps, vd

    a = make_pipeline(vgb_mod, torch, filt, syn, tabs, invw)
    straight = [second(a, t) for t in range(4)]
    a.close()
    b = make_pipeline(vgb_mod, torch, filt, syn, tabs, invw)
    for t in range(2):
        second(b, t)
    state = b.save_state()
    b.close()
    c = make_pipeline(vgb_mod, torch, filt, syn, tabs, invw)
    c.load_state(state)
    for t in (2, 3):
        ps, vd = second(c, t)
        assert np.array_equal(ps, straight[t][0]) and np.array_equal(vd, straight[t][1])
    bad = state.copy()
    bad[8:12] = 0                      # another ncc
    with pytest.raises(vgb_mod.VGBError, match="different pipeline configuration"):
        c.load_state(bad)
    c.close()


def test_pipeline_from_subfiles(vgb_mod, torch, setup, tmp_path):
    """Whole seconds (20 blocks) read from MWAX subfiles straight into the
    pinned host buffer (vgb_subfile_read_second, one call per coarse channel)
    and streamed through the pipeline give the bytes of the same voltages
    already on the device."""
    _, filt, syn, tabs = setup
    invw = 1.0 / NI
    nblk, secs, subobs = 20, 2, 1300000000
    ns = nblk * 500
    rng = np.random.default_rng(21)
    volt = rng.integers(-127, 128, (secs, NCC, nblk, NI, 64000, 2), dtype=np.int8)
    paths = []
    for cc in range(NCC):
        text = f"HDR_SIZE 4096\nOBS_ID {subobs}\nSUBOBS_ID {subobs}\nNBIT 8\nNINPUTS {NI}\nSECS_PER_SUBOBS {secs}\n"
        hdr = text.encode() + b"\0" * (4096 - len(text))
        meta = np.zeros(NI * 64000 * 2, np.uint8)
        path = tmp_path / vgb_mod.volt_filename(subobs, subobs, 109 + cc)
        path.write_bytes(hdr + meta.tobytes() + np.ascontiguousarray(volt[:, cc]).tobytes())
        paths.append(path)

    def make():
        p = vgb_mod.Pipeline(NCC, NANT, nblk, nstokes=4, pfb_flags=0, do_ipfb=True, invw=invw)
        p.set_filters(filt, syn)
        from helpers import weights_on_device

        p.set_weights(torch.cat([weights_on_device(J, phi) for J, phi in tabs]), on_device=True)
        return p

    outs = []
    for mode in ("device", "files"):
        p = make()
        res = []
        for t in range(secs):
            if mode == "device":
                p.run_device(dev(volt[t].reshape(-1).view(np.uint8)))
            else:
                hb = torch.empty(NCC * nblk * NI * 64000 * 2, dtype=torch.uint8).pin_memory()
                view = hb.numpy().reshape(NCC, -1)
                for cc in range(NCC):
                    vgb_mod.subfile_read_second(paths[cc], subobs + t, view[cc])
                p.run_host(hb)
            ps = np.empty((ns, 4, NCC * K), np.uint8)
            vd = np.empty((NCC, ns, 544), np.uint8)
            p.fetch(ps, None, None, vd)
            res.append((ps, vd))
        p.close()
        outs.append(res)
    for (a, b), (c, d) in zip(outs[0], outs[1]):
        assert np.array_equal(a, c) and np.array_equal(b, d)


def test_pipeline_nan_channel(vgb_mod, torch, oracle_mod, setup):
    """A NaN weight makes one channel's Stokes NaN at every sample: the
    extremes the beam kernel gathers then flag the channel's first value as
    NaN, and the PSRFITS bytes, offsets and scales equal the oracle's
    renormalise of the device's own Stokes (the reference's sequential scan:
    a NaN first value makes the extremes NaN)."""
    from helpers import weights_on_device

    volt, filt, syn, tabs = setup
    p = vgb_mod.Pipeline(NCC, NANT, NBLK, nstokes=4, pfb_flags=0, do_ipfb=True, invw=1.0 / NI)
    p.set_filters(filt, syn)
    W = torch.cat([weights_on_device(J, phi) for J, phi in tabs])
    W[(0 * NANT + 3) * K + 17] = float("nan")            # cc 0, tile 3, channel 17
    p.set_weights(W, on_device=True)
    for t in range(2):
        p.run_device(dev(volt[t].reshape(-1).view(np.uint8)))
        ps = np.empty((NS, 4, NCC * K), np.uint8)
        off = np.empty((NCC, 4, K), np.float32)
        sc = np.empty((NCC, 4, K), np.float32)
        p.fetch(ps, off, sc, None)
        S = np.empty((NCC, NS, 4, K), np.float32)
        e = np.empty((NCC, NS, K, 2), np.complex64)
        p.fetch_raw(S, e)
        assert np.isnan(S[0, :, :, 17]).all() and not np.isnan(S[0, :, :, 16]).any()
        for cc in range(NCC):
            o, s, u = oracle_mod.renormalise(S[cc][None])
            assert np.array_equal(ps[:, :, cc * K:(cc + 1) * K], u[0]), (t, cc)
            assert np.array_equal(off[cc], o[0], equal_nan=True) and np.array_equal(sc[cc], s[0], equal_nan=True)
        assert np.isnan(off[0, :, 17]).all()
    p.close()


def test_pipeline_stokes_i_only(vgb_mod, torch, oracle_mod, setup):
    """Stokes I only (nstokes = 1): the gathered extremes and the spliced
    PSRFITS rows use the one-parameter layout; bytes, offsets and scales equal
    the oracle's renormalise of the device's own Stokes, and the Stokes equal
    the full-Stokes pipeline's I."""
    from helpers import weights_on_device

    volt, filt, syn, tabs = setup
    W = torch.cat([weights_on_device(J, phi) for J, phi in tabs])
    S = {}
    for nst in (1, 4):
        p = vgb_mod.Pipeline(NCC, NANT, NBLK, nstokes=nst, pfb_flags=0, do_ipfb=False, invw=1.0 / NI)
        p.set_filters(filt, syn)
        p.set_weights(W, on_device=True)
        p.run_device(dev(volt[0].reshape(-1).view(np.uint8)))
        ps = np.empty((NS, nst, NCC * K), np.uint8)
        off = np.empty((NCC, nst, K), np.float32)
        sc = np.empty((NCC, nst, K), np.float32)
        p.fetch(ps, off, sc, None)
        S[nst] = np.empty((NCC, NS, nst, K), np.float32)
        p.fetch_raw(S[nst], None)
        p.close()
        for cc in range(NCC):
            o, s, u = oracle_mod.renormalise(S[nst][cc][None])
            assert np.array_equal(ps[:, :, cc * K:(cc + 1) * K], u[0]), (nst, cc)
            assert np.array_equal(off[cc], o[0]) and np.array_equal(sc[cc], s[0]), (nst, cc)
    assert np.array_equal(S[1][:, :, 0], S[4][:, :, 0])


def test_pipeline_tracking_rebuilds_weights_every_second(vgb_mod, torch, oracle_mod, setup):
    """Per-second tracking (vmCalcJonesAndDelays inside the captured second):
    over three seconds with a different pointing each second, the pipeline
    that rebuilds W itself equals, byte for byte, a pipeline given the W that
    vgb_primary_beam -> vgb_jones / vgb_phase -> vgb_weights build for that
    second; and its Stokes match the oracle chain (oracle primary beam, calc_j,
    calc_phi, PFB, beamformer) within 1e-5 of the largest magnitude."""
    import beam_model as BM

    volt, filt, syn, _ = setup
    nsec = 3
    vol3 = np.concatenate([volt, volt[:1]], axis=0)[:nsec]
    invw = 1.0 / NI
    az = np.radians([45.0, 47.5, 50.0])
    za = np.radians([20.0, 21.0, 22.5])
    D = np.stack([SY.calibration_jones(NANT, K, seed=cc + 1) for cc in range(NCC)])
    delays = np.zeros((NANT, 16), np.uint32)
    delays[NANT // 2:] = np.arange(16, dtype=np.uint32) % 4          # a second dipole-delay set
    delays[1, 3] = 32                                                # a dead dipole on one tile
    east, north, height, cable = SY.tile_layout(NANT, seed=9)
    href = 377.827  # the array reference height the oracle's calc_phi uses (MWA_ALTITUDE_METRES)
    chan_f = np.stack([SY.fine_chan_freqs_hz(SY.coarse_chan_start_hz(cc)) for cc in range(NCC)])
    beam_f = np.array([SY.coarse_chan_start_hz(cc) + 640000 for cc in range(NCC)], np.float64)
    lat = BM.MWA_LATITUDE

    d = {k: dev(v) for k, v in dict(D=D, delays=delays, east=east, north=north, height=height, cable=cable,
                                      chan_f=chan_f, beam_f=beam_f, az=az, za=za).items()}
    pt = vgb_mod.Pipeline(NCC, NANT, NBLK, nstokes=4, pfb_flags=0, do_ipfb=True, invw=invw)
    pt.set_filters(filt, syn)
    pt.set_tracking(d["D"], d["delays"], d["east"], d["north"], d["height"], d["cable"], d["chan_f"], d["beam_f"],
                    d["az"], d["za"], href=href, latitude=lat, pa_correction=True)
    pw = vgb_mod.Pipeline(NCC, NANT, NBLK, nstokes=4, pfb_flags=0, do_ipfb=True, invw=invw)
    pw.set_filters(filt, syn)
    for t in range(nsec):
        # the fixed-weights pipeline gets this second's W from the separate table kernels
        B = torch.empty((NCC, 1, NANT, 8), dtype=torch.float64, device="cuda")
        vgb_mod.primary_beam(d["az"][t:t + 1], d["za"][t:t + 1], d["beam_f"], d["delays"], B, pa_correction=True,
                             latitude=lat)
        unit = dev(SY.unit_vectors(np.degrees(az[t]), np.degrees(za[t])))
        Ws = []
        for cc in range(NCC):
            Jd = torch.empty((NANT * K, 8), dtype=torch.float64, device="cuda")
            vgb_mod.jones(d["D"][cc], B[cc], 1, NANT, K, Jd)
            ph = torch.empty((NANT * K, 2), dtype=torch.float64, device="cuda")
            vgb_mod.phase(unit, d["east"], d["north"], d["height"], d["cable"], d["chan_f"][cc], 1, NANT, K, href, ph)
            W = torch.empty((NANT * K, 8), dtype=torch.float32, device="cuda")
            vgb_mod.weights(Jd, ph, NANT * K, W)
            Ws.append(W)
        pw.set_weights(torch.cat(Ws), on_device=True)
        dv = dev(vol3[t].reshape(-1).view(np.uint8))
        pt.run_device(dv)
        pw.run_device(dv)
        assert pt.launch_count() == pw.launch_count() + 5
        outs = []
        for p in (pt, pw):
            ps = np.empty((NS, 4, NCC * K), np.uint8)
            vd = np.empty((NCC, NS, 544), np.uint8)
            S = np.empty((NCC, NS, 4, K), np.float32)
            p.fetch(ps, None, None, vd)
            p.fetch_raw(S)
            outs.append((ps, vd, S))
        for a, b in zip(*outs):
            assert np.array_equal(a, b), t
        # the oracle chain for this second
        Bo = BM.primary_beam(az[t:t + 1], za[t:t + 1], beam_f, delays, pa=True, lat=lat)
        unit_o = SY.unit_vectors(np.degrees(az[t]), np.degrees(za[t]))
        for cc in range(NCC):
            J = oracle_mod.calc_j(D[cc], np.ascontiguousarray(Bo[cc]))
            phi = oracle_mod.calc_phi(unit_o, east, north, height, cable, chan_f[cc])
            Sref, _ = oracle_second(oracle_mod, vol3, t, cc, filt, J, phi, invw)
            assert rel_err(outs[0][2][cc], Sref[0]) < 1e-5, (t, cc)
    pt.close()
    pw.close()


def test_pipeline_incoherent_beam_psrfits(vgb_mod, torch, oracle_mod, setup):
    """The incoherent beam's 8-bit rows (Stokes I, spliced across the two
    coarse channels) over two seconds: bit for bit the oracle's renormalise
    of the device's incoherent sums, and within one LSB on <= 1e-4 of samples
    of the oracle's renormalise of the oracle's own incoherent sums (the sum
    of |v|^2 over the RF inputs of the oracle's fine channels); the same rows
    land in host buffers given to vgb_pipeline_set_host_incoh."""
    volt, filt, syn, tabs = setup
    invw = 1.0 / NI
    p = make_pipeline(vgb_mod, torch, filt, syn, tabs, invw)
    hps = np.zeros((NS, NCC * K), np.uint8)
    hoff = np.zeros((NCC, K), np.float32)
    hsc = np.zeros((NCC, K), np.float32)
    p.set_host_incoh(hps, hoff, hsc)
    for t in range(2):
        p.run_device(dev(volt[t].reshape(-1).view(np.uint8)))
        ps = np.empty((NS, NCC * K), np.uint8)
        off = np.empty((NCC, K), np.float32)
        sc = np.empty((NCC, K), np.float32)
        p.fetch_incoh(ps, off, sc)
        p.sync()
        assert np.array_equal(hps, ps) and np.array_equal(hoff, off) and np.array_equal(hsc, sc)
        inc = np.empty((NCC, NS, K), np.float32)
        p.fetch_raw(incoh=inc)
        for cc in range(NCC):
            o, s_, u = oracle_mod.renormalise(inc[cc][None, :, None, :])
            assert np.array_equal(ps[:, cc * K:(cc + 1) * K], u[0][:, 0])
            assert np.array_equal(off[cc], o[0][0]) and np.array_equal(sc[cc], s_[0][0])
            margin = np.zeros((1, NI, 64000, 2), np.int8) if t == 0 else volt[t - 1, cc, NBLK - 1:]
            buf = np.ascontiguousarray(np.concatenate([margin, volt[t, cc]], axis=0))
            v = oracle_mod.fpfb(buf, NI, NS, filt, K, P, np.arange(NI, dtype=np.int32), 0)
            iref = (np.abs(v) ** 2).sum(axis=-1).astype(np.float32)
            _, _, uref = oracle_mod.renormalise(iref[None, :, None, :])
            d8 = np.abs(ps[:, cc * K:(cc + 1) * K].astype(np.int16) - uref[0][:, 0].astype(np.int16))
            assert (d8 > 1).mean() <= 1e-4 and (d8 > 0).mean() <= 1e-3, (t, cc)
    p.close()
