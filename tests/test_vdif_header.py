"""VDIF frame headers built on the host (vgb_vdif_header_*), against the
VDIF 1.0 field layout and calendar arithmetic restated here with Python's
datetime: the reference epoch is the number of half-years from 2000-01-01 to
the date, the seconds field counts from the epoch's first day, and
nextVDIFHeader steps the frame number, rolling over to the next second at the
frame rate (beam_vdif.c:80, 178-211)."""
import datetime as dt

import numpy as np
import pytest

MJD_2000 = 51544          # 2000-01-01


def mjd_date(mjd):
    return dt.date(2000, 1, 1) + dt.timedelta(days=mjd - MJD_2000)


def date_mjd(d):
    return MJD_2000 + (d - dt.date(2000, 1, 1)).days


def expected_epoch(mjd):
    d = mjd_date(mjd)
    return 2 * (d.year - 2000) + (1 if d.month >= 7 else 0)


def fields(h):
    return dict(seconds=int(h[0]) & 0x3FFFFFFF, invalid=int(h[0]) >> 31, legacy=(int(h[0]) >> 30) & 1,
                frame=int(h[1]) & 0xFFFFFF, epoch=(int(h[1]) >> 24) & 0x3F, length8=int(h[2]) & 0xFFFFFF,
                lognchan=(int(h[2]) >> 24) & 0x1F, version=int(h[2]) >> 29, station=int(h[3]) & 0xFFFF,
                thread=(int(h[3]) >> 16) & 0x3FF, nbits=((int(h[3]) >> 26) & 0x1F) + 1, complex=int(h[3]) >> 31)


@pytest.fixture(scope="module")
def vgb_mod():
    import vgb

    vgb.lib()
    return vgb


def test_create_mwa_beam_header(vgb_mod):
    h = vgb_mod.vdif_header_create(512, 0, 8, 2, True, "mw")
    f = fields(h)
    assert f == dict(seconds=0, invalid=0, legacy=0, frame=0, epoch=0, length8=68, lognchan=1, version=0,
                     station=(ord("m") << 8) | ord("w"), thread=0, nbits=8, complex=1)
    assert np.all(h[4:] == 0)
    h = vgb_mod.vdif_header_create(8000, 513, 2, 16, False, "Pa")
    f = fields(h)
    assert (f["length8"], f["lognchan"], f["thread"], f["nbits"], f["complex"]) == (1004, 4, 513, 2, 0)
    assert f["station"] == (ord("P") << 8) | ord("a")


@pytest.mark.parametrize("mjd", [51544, 51725, 51726, 55000, 58849, 60310, 60491, 60492, 60676, 63140])
def test_epoch_from_mjd(vgb_mod, mjd):
    h = vgb_mod.vdif_header_create()
    vgb_mod.vdif_header_set_epoch_mjd(h, mjd)
    e = fields(h)["epoch"]
    assert e == expected_epoch(mjd)
    start = date_mjd(dt.date(2000 + e // 2, 1 + 6 * (e % 2), 1))
    assert vgb_mod.vdif_header_epoch_mjd(h) == start
    assert start <= mjd < start + 184


def test_seconds_from_mjdsec(vgb_mod):
    h = vgb_mod.vdif_header_create()
    vgb_mod.vdif_header_set_epoch_mjd(h, 60500)
    vgb_mod.vdif_header_set_mjdsec(h, 60500 * 86400 + 21600)
    assert fields(h)["seconds"] == (60500 - date_mjd(dt.date(2024, 7, 1))) * 86400 + 21600
    with pytest.raises(vgb_mod.VGBError):
        vgb_mod.vdif_header_set_mjdsec(h, 60000 * 86400)     # before the epoch


def test_populate_header(vgb_mod):
    # vmPopulateVDIFHeader: seconds = intmjd * 86400 + roundf(fracmjd * 86400) from the epoch start
    for intmjd, frac in [(60123, 0.0), (60123, 0.3), (59000, 0.999999), (60123, 0.5 / 86400)]:
        h = vgb_mod.vdif_populate_header(intmjd, frac)
        f = fields(h)
        start = vgb_mod.vdif_header_epoch_mjd(h)
        sec = np.float32(np.float32(frac * 86400.0))
        rounded = int(np.floor(sec + np.float32(0.5))) if sec >= 0 else int(np.ceil(sec - np.float32(0.5)))
        assert f["seconds"] == (intmjd - start) * 86400 + rounded
        assert (f["frame"], f["length8"], f["nbits"], f["complex"], f["lognchan"]) == (0, 68, 8, 1, 1)
        assert f["epoch"] == expected_epoch(intmjd)


def test_next_rolls_over(vgb_mod):
    h = vgb_mod.vdif_populate_header(60123, 0.25)
    s0 = fields(h)["seconds"]
    vgb_mod.vdif_header_set_frame(h, 9998)
    vgb_mod.vdif_header_next(h)
    assert (fields(h)["frame"], fields(h)["seconds"]) == (9999, s0)
    vgb_mod.vdif_header_next(h)
    assert (fields(h)["frame"], fields(h)["seconds"]) == (0, s0 + 1)
    for _ in range(25):
        vgb_mod.vdif_header_next(h, 10)
    assert (fields(h)["frame"], fields(h)["seconds"]) == (5, s0 + 3)
    assert h[2] == 68 | (1 << 24)


def test_bad_arguments(vgb_mod):
    with pytest.raises(vgb_mod.VGBError):
        vgb_mod.vdif_header_create(512, 0, 0, 2)            # bits
    with pytest.raises(vgb_mod.VGBError):
        vgb_mod.vdif_header_create(512, 0, 8, 3)            # channels not a power of two
    with pytest.raises(vgb_mod.VGBError):
        vgb_mod.vdif_header_create(500, 0, 8, 2)            # length not a multiple of 8
    with pytest.raises(vgb_mod.VGBError):
        vgb_mod.vdif_header_create(512, 1024, 8, 2)         # thread id
    h = vgb_mod.vdif_header_create()
    with pytest.raises(vgb_mod.VGBError):
        vgb_mod.vdif_header_set_epoch_mjd(h, 40000)         # 1968
    with pytest.raises(vgb_mod.VGBError):
        vgb_mod.vdif_header_set_frame(h, 1 << 24)
