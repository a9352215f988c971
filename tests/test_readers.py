"""Voltage file readers (vgb_subfile_*, vgb_legacy_read_second,
vgb_volt_filename) on synthetic files written here in the documented
layouts: an MWAX subfile is an ASCII "KEY value" header of HDR_SIZE bytes,
one metadata block, then 20 blocks per second of [input][64000] char2; a
legacy recombined file is one second of bytes. mwalib, which VCSBeam reads
them with, is not available, so the layouts are restated, not pinned."""
import numpy as np
import pytest

SPB = 64000


@pytest.fixture(scope="module")
def vgb_mod():
    import vgb

    vgb.lib()
    return vgb


def write_subfile(path, ninputs, secs, subobs, hdr_size=4096, extra=(), nbit=8, truncate=0, seed=0):
    keys = [("HDR_SIZE", hdr_size), ("POPULATED", 1), ("OBS_ID", 1234567888), ("SUBOBS_ID", subobs),
            ("NBIT", nbit), ("NINPUTS", ninputs), ("SECS_PER_SUBOBS", secs), ("COARSE_CHANNEL", 109)] + list(extra)
    text = "".join(f"{k} {v}\n" for k, v in keys).encode()
    header = text + b"\0" * (hdr_size - len(text))
    rng = np.random.default_rng(seed)
    block = ninputs * SPB * 2
    meta = rng.integers(0, 256, block, dtype=np.uint8)
    data = rng.integers(0, 256, (secs, 20, ninputs, SPB, 2), dtype=np.uint8)
    blob = header + meta.tobytes() + data.tobytes()
    if truncate:
        blob = blob[:-truncate]
    path.write_bytes(blob)
    return data


def test_subfile_seconds(vgb_mod, tmp_path):
    p = tmp_path / "1234567888_1234567896_109.sub"
    data = write_subfile(p, ninputs=4, secs=3, subobs=1234567896)
    info = vgb_mod.subfile_info(p)
    assert (info["ninputs"], info["secs_per_subobs"], info["subobs_id"], info["obs_id"]) == (4, 3, 1234567896,
                                                                                             1234567888)
    assert (info["header_bytes"], info["block_bytes"], info["coarse_channel"], info["complete"]) == (4096,
                                                                                                     4 * SPB * 2, 109, 1)
    for k in (0, 2, 1):
        for nthreads in (1, 3, 8):
            dst = np.zeros((20, 4, SPB, 2), np.uint8)
            vgb_mod.subfile_read_second(p, 1234567896 + k, dst, nthreads=nthreads)
            assert np.array_equal(dst, data[k]), (k, nthreads)
    dst = np.zeros((20, 4, SPB, 2), np.uint8)
    for bad in (1234567895, 1234567899):
        with pytest.raises(vgb_mod.VGBError, match="outside the file"):
            vgb_mod.subfile_read_second(p, bad, dst)
    with pytest.raises(vgb_mod.VGBError, match="destination"):
        vgb_mod.subfile_read_second(p, 1234567896, np.zeros(100, np.uint8))


def test_subfile_header_size_and_truncation(vgb_mod, tmp_path):
    p = tmp_path / "a.sub"
    data = write_subfile(p, ninputs=2, secs=2, subobs=100, hdr_size=8192, extra=[("UTC_START", "2021-01-01-00:00:00")])
    dst = np.zeros((20, 2, SPB, 2), np.uint8)
    vgb_mod.subfile_read_second(p, 101, dst)
    assert np.array_equal(dst, data[1])
    q = tmp_path / "b.sub"
    write_subfile(q, ninputs=2, secs=2, subobs=100, truncate=1000)
    assert vgb_mod.subfile_info(q)["complete"] == 0
    vgb_mod.subfile_read_second(q, 100, dst)            # the first second is whole
    with pytest.raises(vgb_mod.VGBError, match="ends 1000 bytes early"):
        vgb_mod.subfile_read_second(q, 101, dst)


def test_subfile_bad_headers(vgb_mod, tmp_path):
    p = tmp_path / "c.sub"
    p.write_bytes(b"HDR_SIZE 4096\nOBS_ID 5\n" + b"\0" * 5000)
    with pytest.raises(vgb_mod.VGBError, match="NINPUTS"):
        vgb_mod.subfile_info(p)
    q = tmp_path / "d.sub"
    write_subfile(q, ninputs=2, secs=1, subobs=0, nbit=4)
    with pytest.raises(vgb_mod.VGBError, match="NBIT"):
        vgb_mod.subfile_info(q)
    with pytest.raises(vgb_mod.VGBError, match="cannot open"):
        vgb_mod.subfile_info(tmp_path / "missing.sub")


def test_legacy_second(vgb_mod, tmp_path):
    p = tmp_path / "1096952256_1096952256_ch109.dat"
    sec = np.random.default_rng(3).integers(0, 256, (10000, 128, 16), dtype=np.uint8)
    p.write_bytes(sec.tobytes())
    dst = np.zeros_like(sec)
    vgb_mod.legacy_read_second(p, dst, nthreads=5)
    assert np.array_equal(dst, sec)
    with pytest.raises(vgb_mod.VGBError, match="early"):
        vgb_mod.legacy_read_second(p, np.zeros((10001, 128, 16), np.uint8))


def test_volt_filenames(vgb_mod):
    assert vgb_mod.volt_filename(1313388760, 1313388775, 57) == "1313388760_1313388768_057.sub"
    assert vgb_mod.volt_filename(1313388760, 1313388760, 109) == "1313388760_1313388760_109.sub"
    assert vgb_mod.volt_filename(1096952256, 1096952257, 133, mwax=False) == "1096952256_1096952257_ch133.dat"
