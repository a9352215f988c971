"""Host-side table inputs (no GPU): calibration solution readers, their
corrections, tile flags and filter files, against the expected arrays of the
synthetic files and, where the reference's own calibration.c / filter.c are
compiled here (oracle/_ref/libref_host.so), against those bit for bit."""
import ctypes
import os
import struct

import numpy as np
import pytest

ORACLE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle")
REF_LIB = os.path.join(ORACLE, "_ref", "libref_host.so")
RUNTIME = os.path.join(ORACLE, "_ref", "runtime")


@pytest.fixture(scope="module")
def vgb_mod():
    import build as B
    import vgb

    if not os.path.exists(vgb.LIB_PATH):
        B.build()
    vgb.lib()
    return vgb


@pytest.fixture(scope="module")
def ref():
    if not os.path.exists(REF_LIB):
        pytest.skip("reference host library not built (no reference sources here)")
    try:
        lib = ctypes.CDLL(REF_LIB)
    except OSError as exc:
        pytest.skip(f"reference host library not loadable: {exc}")
    V, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    lib.refhost_load_offringa.argtypes = [ctypes.c_char_p, I, I, I, I, I, V]
    lib.refhost_load_rts.argtypes = [ctypes.c_char_p, I, I, I, I, I, V, I, V]
    lib.refhost_apply_corrections.argtypes = [V, I, I, I, I, D, D, ctypes.c_uint]
    lib.refhost_pq_correction.argtypes = [ctypes.c_uint, V, V, V, I]
    lib.refhost_load_filter.argtypes = [ctypes.c_char_p, I, I, D, V, I, V]
    return lib


def write_offringa(path, J, nintervals=1):
    """J complex128 [nant][nchan][2][2] -> an Offringa binary solution (48-byte
    header: 16 bytes of identifier, four uint32 counts, two doubles)."""
    nant, nchan = J.shape[:2]
    with open(path, "wb") as f:
        f.write(b"MWAOCAL\0" + struct.pack("<ii", 0, 0))
        f.write(struct.pack("<IIII", nintervals, nant, nchan, 4))
        f.write(struct.pack("<dd", 0.0, 8.0))
        for _ in range(nintervals):
            f.write(np.ascontiguousarray(J, dtype=np.complex128).tobytes())


def test_offringa_reader(vgb_mod, ref, tmp_path):
    rng = np.random.default_rng(1)
    nant, nchan_cal, ncc, nfine = 8, 32, 3, 128
    J = rng.standard_normal((nant, nchan_cal * ncc, 2, 2)) + 1j * rng.standard_normal((nant, nchan_cal * ncc, 2, 2))
    J[2, 40] = np.nan          # a flagged matrix
    path = str(tmp_path / "sol.bin")
    write_offringa(path, J, nintervals=2)
    for cc in range(ncc):
        D, counts = vgb_mod.cal_load_offringa(path, cc, ncc, nant, nchan_cal, nfine)
        assert list(counts) == [2, nant, nchan_cal * ncc, 4]
        want = np.repeat(J[:, cc * nchan_cal:(cc + 1) * nchan_cal], nfine // nchan_cal, axis=1)
        want = np.where(np.isnan(want.real), 0, want)
        assert np.array_equal(D, want)
        Dr = np.zeros_like(D)
        ref.refhost_load_offringa(path.encode(), cc, ncc, nant, nchan_cal, nfine, Dr.ctypes.data)
        assert np.array_equal(D, Dr)
    # the solution's own channel count wins over the request
    D, _ = vgb_mod.cal_load_offringa(path, 1, ncc, nant, 16, nfine)
    Dr = np.zeros_like(D)
    ref.refhost_load_offringa(path.encode(), 1, ncc, nant, 16, nfine, Dr.ctypes.data)
    assert np.array_equal(D, Dr)
    with pytest.raises(vgb_mod.VGBError, match="antennas"):
        vgb_mod.cal_load_offringa(path, 0, ncc, nant + 1, nchan_cal, nfine)


def write_rts(caldir, node, nant, nchan, rng, flagged_chans=(), absent_ants=()):
    amp = 1.2345
    A = rng.standard_normal(8)
    Jd = rng.standard_normal((nant, 8))
    with open(os.path.join(caldir, f"DI_JonesMatrices_node{node:03d}.dat"), "w") as f:
        f.write(f"{amp:.10f}\n")
        f.write(", ".join(f"{x:.12f}" for x in A) + "\n")
        for a in range(nant):
            f.write(", ".join(f"{x:.12f}" for x in Jd[a]) + "\n")
    chans = [c for c in range(nchan) if c not in flagged_chans]
    width_mhz = 1.28 / nchan
    amp_ph = rng.uniform(0.5, 1.5, (nant, 8, nchan)), rng.uniform(-3, 3, (nant, 8, nchan))
    with open(os.path.join(caldir, f"BandpassCalibration_node{node:03d}.dat"), "w") as f:
        f.write(",".join(f"{c * width_mhz:.6f}" for c in chans) + "\n")
        for a in range(nant):
            if a in absent_ants:
                continue
            for row in range(8):
                vals = ",".join(f"{amp_ph[0][a, row, c]:.9f},{amp_ph[1][a, row, c]:.9f}" for c in chans)
                f.write(f"{a + 1},{vals}\n")
    return int(round(width_mhz * 1e6))


@pytest.mark.parametrize("use_bandpass", [True, False])
def test_rts_reader(vgb_mod, ref, tmp_path, use_bandpass):
    rng = np.random.default_rng(2)
    nant, nchan_cal, nfine, node = 8, 32, 128, 5
    width = write_rts(str(tmp_path), node, nant, nchan_cal, rng, flagged_chans=(3, 17), absent_ants=(6,))
    cal_ant = rng.permutation(nant).astype(np.int32)
    dij = str(tmp_path / f"DI_JonesMatrices_node{node:03d}.dat")
    bp = str(tmp_path / f"BandpassCalibration_node{node:03d}.dat") if use_bandpass else None
    D = vgb_mod.cal_load_rts(dij, bp, nant, nchan_cal, width, cal_ant, nfine)
    Dr = np.zeros_like(D)
    ref.refhost_load_rts(str(tmp_path).encode(), int(use_bandpass), node - 1, nant, nchan_cal, width,
                         cal_ant.ctypes.data, nfine, Dr.ctypes.data)
    assert np.array_equal(D, Dr)
    if use_bandpass:
        # flagged channels and the absent antenna come out zero
        interp = nfine // nchan_cal
        assert np.all(D[:, 3 * interp:4 * interp] == 0)
        assert np.all(D[list(cal_ant).index(6)] == 0)


def test_corrections(vgb_mod, ref):
    rng = np.random.default_rng(3)
    nant, nfine = 10, 128
    D0 = rng.standard_normal((nant, nfine, 2, 2)) + 1j * rng.standard_normal((nant, nfine, 2, 2))
    D0[4, :, 0, 1] = 0.0        # a zero reference element: that rotation is skipped
    for ref_ant, keep, slope, offset in [(4, False, 2.1e-8, 0.3), (-1, True, -1e-9, 0.0), (0, True, 0.0, 0.0),
                                         (-1, False, 0.0, 0.0)]:
        D = np.ascontiguousarray(D0.copy())
        vgb_mod.cal_apply_corrections(D, ref_ant, keep, slope, offset, chan_start_hz=168_960_000)
        Dr = np.ascontiguousarray(D0.copy())
        ref.refhost_apply_corrections(Dr.ctypes.data, nant, nfine, ref_ant, int(keep), slope, offset, 168_960_000)
        assert np.array_equal(D, Dr), (ref_ant, keep, slope, offset)


def test_pq_correction(vgb_mod, ref):
    path = os.path.join(RUNTIME, "pq_phase_correction.txt")
    if not os.path.exists(path):
        pytest.skip("reference pq_phase_correction.txt not linked")
    times = [0, 1_000_000_000, 1_100_000_000, 1_200_000_000, 1_300_000_000, 1_400_000_000, 4_000_000_000]
    for line in open(path):
        if line[:1].isdigit():
            a, b = line.split()[:2]
            times += [int(a), int(b), (int(a) + int(b)) // 2]
    s, o = ctypes.c_double(), ctypes.c_double()
    name = ctypes.create_string_buffer(32)
    for t in times:
        found, slope, offset, tile = vgb_mod.cal_pq_correction(path, t)
        rf = ref.refhost_pq_correction(t, ctypes.byref(s), ctypes.byref(o), name, 32)
        assert found == bool(rf) and tile == name.value.decode()
        if found:
            assert slope == s.value and offset == o.value


def test_flag_tiles(vgb_mod):
    D = np.ones((6, 8, 2, 2), dtype=np.complex128)
    vgb_mod.cal_flag_tiles(D, [1, 4])
    assert np.all(D[[1, 4]] == 0) and np.all(D[[0, 2, 3, 5]] == 1)
    with pytest.raises(vgb_mod.VGBError, match="out of range"):
        vgb_mod.cal_flag_tiles(D, [6])


@pytest.mark.parametrize("name,scale", [("FINEPFB", 1.0), ("LSQ12", 15.0 / 7.2), ("MIRROR", 1.0)])
def test_filter_files(vgb_mod, ref, name, scale):
    path = os.path.join(RUNTIME, f"{name}.dat")
    if not os.path.exists(path):
        pytest.skip("reference filter files not linked")
    h, ntaps = vgb_mod.load_filter(path, 128, scale)
    out = np.zeros(8192)
    nt = ctypes.c_int()
    n = ref.refhost_load_filter(name.encode(), int(name != "FINEPFB"), 128, scale, out.ctypes.data, out.size,
                                ctypes.byref(nt))
    assert n == h.size and nt.value == ntaps
    assert np.array_equal(h, out[:n])
    if name == "FINEPFB":
        assert int(h.sum()) == 15106424   # documented checksum of the analysis filter


def test_filter_fixture_is_the_reference_filters(vgb_mod):
    """tests/golden/ref_filters.npz holds FINEPFB (analysis, int cast) and
    LSQ12 x 15/7.2 (synthesis) as the reference's vmLoadFilter and
    vmScaleFilterCoeffs loaded them (tests/golden/make_golden_filters.py);
    the full-size GPU parity tests run on it. Where the filter files are
    linked, this library's reader gives the same values."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_filters.npz"))
    fine, lsq = g["finepfb"], g["lsq12_scaled"]
    assert fine.shape == (1536,) and lsq.shape == (1536,)
    assert int(fine.sum()) == 15106424 and int(fine.max()) == 117964   # documented checksum and peak tap
    assert int(g["finepfb_ntaps"]) == 12 and int(g["lsq12_ntaps"]) == 12
    for name, scale, want in (("FINEPFB", 1.0, fine.astype(np.float64)), ("LSQ12", 15.0 / 7.2, lsq)):
        path = os.path.join(RUNTIME, f"{name}.dat")
        if os.path.exists(path):
            h, _ = vgb_mod.load_filter(path, 128, scale)
            assert np.array_equal(h, want)
