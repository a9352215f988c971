"""VCSBeam's own API on the GB300 kernels (libvcsbeam_compat.so).

tests/compat/app_loop.c is a VCSBeam program's per-second loop, compiled
against VCSBeam's configured vcsbeam.h (the reference's header as
oracle/build_ref.sh configures it, with stand-in dependency headers) and
linked to this library's vm* / cu_* entry points. It runs as a child process
(the library ends the process on an error, as the reference does).

  * two seconds of 16 tiles, two chunks per second, per-second J^-1 and phi,
    VCS-ordered inputs: every product equals the streaming pipeline's
    (vgb_pipeline) on the same voltages and tables, bit for bit: 8-bit
    PSRFITS bytes, offsets, scales, Stokes, beam voltages, and the VDIF bytes
    of the inverse PFB's output;
  * one whole C1 second (128 tiles, FINEPFB / LSQ12 x 15/7.2): against the
    reference's own kernels (tests/golden/ref_golden_c1.npz) with the bounds
    of the C1 parity test;
  * tests/compat/legacy_loop.c: legacy recombined 4+4-bit input, three
    pointings, two seconds in two chunks each (vmPushChunk, vmApplyJChunk,
    vmBeamformChunk): every pointing's Stokes, beam voltages and PSRFITS
    bytes, offsets and scales equal this library's vgb_beamform_legacy and
    vgb_renormalise on the same inputs bit for bit, and its Stokes match the
    oracle's beamformer within 1e-5 (norm-wise).
"""
import os
import subprocess
import sys

import numpy as np
import pytest

import synthetic as SY
from helpers import byte_diff_stats, dev, host, rel_err, tables, torch_cuda, weights_on_device

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "mwa-vcsbeam_gb300", "lib")
REF_INC = os.path.join(ROOT, "oracle", "_ref", "include")
STUBS = os.path.join(ROOT, "oracle", "ref_stubs")
K, P = 128, 12
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))


def build_program(tmp_path_factory, name):
    torch_cuda()
    if not os.path.exists(os.path.join(REF_INC, "vcsbeam.h")):
        pytest.skip("no configured vcsbeam.h")
    if not os.path.exists(os.path.join(LIBDIR, "libvcsbeam_compat.so")):
        pytest.fail("libvcsbeam_compat.so was not built although vcsbeam.h is configured")
    exe = str(tmp_path_factory.mktemp(name) / name)
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    subprocess.run(["gcc", "-O2", "-D__NVCC__", "-w", "-I", REF_INC, "-I", STUBS, "-I", os.path.join(cuda, "include"),
                    os.path.join(ROOT, "tests", "compat", f"{name}.c"), "-o", exe, "-L", LIBDIR, "-lvcsbeam_compat",
                    "-lvcsbeam_gb300", "-L", os.path.join(cuda, "lib64"), "-lcudart", f"-Wl,-rpath,{LIBDIR}"],
                   check=True)
    return exe


@pytest.fixture(scope="module")
def legacy_app(tmp_path_factory):
    return build_program(tmp_path_factory, "legacy_loop")


@pytest.fixture(scope="module")
def app(tmp_path_factory):
    return build_program(tmp_path_factory, "app_loop")


def run_app(exe, tmp, nant, nsec, nchunks, volt, ana, syn, i_idx, J, phi):
    ind, outd = tmp / "in", tmp / "out"
    ind.mkdir()
    outd.mkdir()
    volt.tofile(ind / "volt.bin")
    np.asarray(ana, np.float64).tofile(ind / "ana.bin")
    np.asarray(syn, np.float64).tofile(ind / "syn.bin")
    np.asarray(i_idx, np.int32).tofile(ind / "i_idx.bin")
    np.asarray(J, np.complex128).tofile(ind / "J.bin")
    np.asarray(phi, np.complex128).tofile(ind / "phi.bin")
    r = subprocess.run([exe, str(nant), str(nsec), str(nchunks), str(ind), str(outd)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    ns = 10000
    out = []
    for t in range(nsec):
        rd = lambda name, dt: np.fromfile(outd / f"{name}_{t}.bin", dtype=dt)
        out.append({"psrfits": rd("psrfits", np.uint8).reshape(ns, 4, K),
                    "offsets": rd("offsets", np.float32).reshape(4, K),
                    "scales": rd("scales", np.float32).reshape(4, K),
                    "vdif_f": rd("vdif", np.float32).reshape(ns, 512),
                    "S": rd("S", np.float32).reshape(ns, 4, K),
                    "e": rd("e", np.complex128).reshape(ns, K, 2)})
    return out


def test_compat_loop_equals_pipeline(app, tmp_path, oracle_mod):
    torch = torch_cuda()
    import vgb

    nant, nsec = 16, 2
    ni = 2 * nant
    volt = oracle_mod.mwax_buffer(5150, 1 + 20 * nsec, ni)
    filt = SY.analysis_filter_int16()
    syn = SY.synthesis_filter(scale=SY.synthesis_scale(filt))
    i_idx = SY.legacy_input_order(nant)
    tabs = [tables(nant, seed=1 + t) for t in range(nsec)]
    J = np.stack([tb[0][0] for tb in tabs])
    phi = np.stack([tb[1][0] for tb in tabs])
    got = run_app(app, tmp_path, nant, nsec, 2, volt, filt.astype(np.float64), syn, i_idx, J, phi)

    # the streaming pipeline on the same seconds: history = the margin block
    p = vgb.Pipeline(1, nant, 20, nstokes=4, pfb_flags=0, do_ipfb=True, invw=1.0 / ni)
    p.set_filters(filt, syn)
    st = p.save_state()
    st[24:32] = np.array([1], np.int64).view(np.uint8)
    hist = np.ascontiguousarray(volt[0, :, (500 - P) * K:, :]).reshape(-1).view(np.uint8)
    st[32:32 + hist.size] = hist
    st[32 + hist.size:] = 0
    p.load_state(st)
    for t in range(nsec):
        p.set_weights(weights_on_device(*tabs[t]), on_device=True)
        p.run_device(dev(np.ascontiguousarray(volt[1 + 20 * t:1 + 20 * (t + 1)]).reshape(-1).view(np.uint8)))
        ps = np.empty((10000, 4, K), np.uint8)
        off = np.empty((4, K), np.float32)
        sc = np.empty((4, K), np.float32)
        vd = np.empty((10000, 544), np.uint8)
        p.fetch(ps, off, sc, vd)
        S = np.empty((10000, 4, K), np.float32)
        e = np.empty((10000, K, 2), np.complex64)
        p.fetch_raw(S, e)
        g = got[t]
        assert np.array_equal(g["S"], S), t
        assert np.array_equal(g["e"].astype(np.complex64), e) and np.array_equal(g["e"], e.astype(np.complex128)), t
        assert np.array_equal(g["psrfits"], ps), t
        assert np.array_equal(g["offsets"], off[None][0]) and np.array_equal(g["scales"], sc), t
        assert np.array_equal(oracle_mod.vdif_quantise(g["vdif_f"]), vd[:, 32:]), t
    p.close()


def test_compat_loop_c1_against_reference_kernels(app, tmp_path):
    import make_golden_c1 as G

    g = dict(np.load(os.path.join(ROOT, "tests", "golden", "ref_golden_c1.npz")))
    htr, fine, lsq, J, phi = G.c1_inputs()
    got = run_app(app, tmp_path, 128, 1, 1, htr, fine.astype(np.float64), lsq, g["i_idx"], J, phi)[0]
    import oracle as O

    assert rel_err(got["S"][::G.SUB_S], g["S_sub"]) < 1e-5
    assert rel_err(got["e"][::G.SUB_S], g["e_sub"]) < 1e-5
    assert byte_diff_stats(got["psrfits"][::G.SUB_B], g["u8_sub"])[1] <= 1e-4
    assert rel_err(got["offsets"], g["offsets"]) < 1e-5 and rel_err(got["scales"], g["scales"]) < 1e-5
    vq = O.vdif_quantise(got["vdif_f"])[::G.SUB_B]
    keep = np.arange(0, 10000, G.SUB_B) >= P
    mx, _, frac = byte_diff_stats(vq[keep], g["vdif_sub"][keep])
    assert mx <= 1 and frac <= 1e-4


def test_compat_legacy_pointings_equal_library_calls(legacy_app, tmp_path, oracle_mod):
    torch = torch_cuda()
    import vgb

    nant, npnt, nsec, ns = 16, 3, 2, 10000
    ni = 2 * nant
    volt = oracle_mod.gen_int4_bytes(777, nsec * ns * K * ni).reshape(nsec, ns, K, ni)
    i_idx = SY.legacy_input_order(nant)
    polQ = np.ascontiguousarray(i_idx[0::2].astype(np.uint32))
    polP = np.ascontiguousarray(i_idx[1::2].astype(np.uint32))
    tabs = [tables(nant, seed=3 + t, npointing=npnt) for t in range(nsec)]
    ind, outd = tmp_path / "in", tmp_path / "out"
    ind.mkdir()
    outd.mkdir()
    volt.tofile(ind / "volt.bin")
    np.asarray(i_idx, np.int32).tofile(ind / "i_idx.bin")
    np.stack([tb[0] for tb in tabs]).astype(np.complex128).tofile(ind / "J.bin")
    np.stack([tb[1] for tb in tabs]).astype(np.complex128).tofile(ind / "phi.bin")
    r = subprocess.run([legacy_app, str(nant), str(npnt), str(nsec), "2", str(ind), str(outd)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    invw = 1.0 / ni
    for t in range(nsec):
        S_c = np.fromfile(outd / f"S_{t}.bin", np.float32).reshape(npnt, ns, 4, K)
        e_c = np.fromfile(outd / f"e_{t}.bin", np.complex128).reshape(npnt, ns, K, 2)
        J, phi = tabs[t]
        W = weights_on_device(J, phi)
        dv = dev(volt[t].reshape(-1))
        S = torch.empty(npnt * ns * 4 * K, dtype=torch.float32, device="cuda")
        e = torch.empty(npnt * ns * K * 4, dtype=torch.float32, device="cuda")
        vgb.beamform_legacy(dv, vgb.INT4, ns, K, nant, dev(polQ), dev(polP), W, npnt, invw, 4, S, e)
        out = torch.empty(npnt * ns * 4 * K, dtype=torch.uint8, device="cuda")
        off = torch.empty(npnt * 4 * K, dtype=torch.float32, device="cuda")
        sc = torch.empty_like(off)
        vgb.renormalise(S, 1, npnt, ns, 4, K, out, 0, ns * 4 * K, 4 * K, K, off, sc)
        torch.cuda.synchronize()
        S_l = host(S).reshape(npnt, ns, 4, K)
        e_l = host(e).view(np.complex64).reshape(npnt, ns, K, 2)
        assert np.array_equal(S_c, S_l), t
        assert np.array_equal(e_c, e_l.astype(np.complex128)), t
        out_l = host(out).reshape(npnt, ns, 4, K)
        off_l = host(off).reshape(npnt, 4, K)
        sc_l = host(sc).reshape(npnt, 4, K)
        for p in range(npnt):
            ps = np.fromfile(outd / f"psrfits_{p}_{t}.bin", np.uint8).reshape(ns, 4, K)
            assert np.array_equal(ps, out_l[p]), (t, p)
            assert np.array_equal(np.fromfile(outd / f"offsets_{p}_{t}.bin", np.float32).reshape(4, K), off_l[p])
            assert np.array_equal(np.fromfile(outd / f"scales_{p}_{t}.bin", np.float32).reshape(4, K), sc_l[p])
        if t == 0:
            Sref, _ = oracle_mod.beamform(volt[t], J, phi, polQ, polP, invw)
            for p in range(npnt):
                assert rel_err(S_c[p], Sref[p]) < 1e-5, p
