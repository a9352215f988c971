"""Seeded synthetic observations standing in for MWA data.

No MWA observation, metafits file, calibration solution or FEE beam model
ships with this project, so tests, the benchmark and ``smoke()`` build their
inputs here:

* an analysis filter: a 1536-tap (12 taps x 128 channels) sinc x Hann
  prototype quantised to int16, in place of the reference's integer
  ``pfb_filter/FINEPFB.dat``;
* a synthesis filter of the same shape in floating point (peak 1.0), in place
  of ``LSQ12.dat``/``MIRROR.dat``;
* tile positions uniform in a 3 km disc at the array's reference height,
  cable lengths, calibration Jones matrices D = I + 0.1 CN(0, 1) per tile
  (frequency flat) and an identity primary-beam model B (the reference's FEE
  model, mwa_hyperbeam, is not available here);
* pointing direction cosines for (az, za), in the convention of the
  reference's calc_beam_geom (geometry.c:268-270).

All arrays use the reference's layouts (include/vcsbeam.h.in index macros).
"""
from __future__ import annotations

import numpy as np

NTAPS = 12
NCHAN = 128
MWA_ALTITUDE_METRES = 377.827
COARSE_CHAN_WIDTH_HZ = 1_280_000


def analysis_filter_int16(ntaps: int = NTAPS, nchan: int = NCHAN) -> np.ndarray:
    """Sinc x Hann low-pass prototype, cutoff 1/nchan, peak scaled to 32767."""
    n = ntaps * nchan
    j = np.arange(n, dtype=np.float64)
    c = (n - 1) / 2.0
    proto = np.sinc((j - c) / nchan) * (0.5 + 0.5 * np.cos(2.0 * np.pi * (j - c) / n))
    return np.round(proto * (32767.0 / proto.max())).astype(np.int32)


def synthesis_filter(ntaps: int = NTAPS, nchan: int = NCHAN, scale: float = 1.0) -> np.ndarray:
    """The same prototype in FP64 with peak 1.0, times `scale`."""
    n = ntaps * nchan
    j = np.arange(n, dtype=np.float64)
    c = (n - 1) / 2.0
    proto = np.sinc((j - c) / nchan) * (0.5 + 0.5 * np.cos(2.0 * np.pi * (j - c) / n))
    return proto / proto.max() * scale


def synthesis_scale(analysis: np.ndarray) -> float:
    """Gain compensation in the spirit of the reference's 15/7.2
    (app/make_mwa_tied_array_beam.c:163, where 7.2 = peak(FINEPFB)/16384)."""
    return 15.0 / (float(np.max(analysis)) / 16384.0)


def wola_fp32_exact(h: np.ndarray, ntaps: int = NTAPS, nchan: int = NCHAN) -> bool:
    """True when every partial sum of the weighted overlap-add of int8
    voltages (|x| <= 128) with filter h stays within 2^24, so FP32
    accumulation reproduces the int32 result exactly."""
    hh = np.abs(np.asarray(h, dtype=np.int64)).reshape(ntaps, nchan)
    return int(hh.sum(axis=0).max()) * 128 <= (1 << 24)


def wola_split_exact(h: np.ndarray, ntaps: int = NTAPS, nchan: int = NCHAN) -> bool:
    """True when the even-tap and the odd-tap sums are each exact in FP32
    (the split weighted overlap-add)."""
    hh = np.abs(np.asarray(h, dtype=np.int64)).reshape(ntaps, nchan)
    return max(int(hh[0::2].sum(axis=0).max()), int(hh[1::2].sum(axis=0).max())) * 128 <= (1 << 24)


def tile_layout(nant: int, seed: int = 7, radius_m: float = 1500.0):
    """East, north, height (m) and electrical cable length (m) per tile."""
    rng = np.random.default_rng(seed)
    r = radius_m * np.sqrt(rng.uniform(0.0, 1.0, nant))
    th = rng.uniform(0.0, 2.0 * np.pi, nant)
    east = r * np.cos(th)
    north = r * np.sin(th)
    height = np.full(nant, MWA_ALTITUDE_METRES)
    cable = rng.uniform(50.0, 500.0, nant)
    return east, north, height, cable


def calibration_jones(nant: int, nchan: int = NCHAN, seed: int = 11) -> np.ndarray:
    """D [nant][nchan][2][2] complex: I + 0.1 CN(0,1) per tile, flat in frequency."""
    rng = np.random.default_rng(seed)
    g = 0.1 * (rng.standard_normal((nant, 2, 2)) + 1j * rng.standard_normal((nant, 2, 2))) / np.sqrt(2)
    D = np.eye(2)[None] + g
    return np.ascontiguousarray(np.broadcast_to(D[:, None], (nant, nchan, 2, 2)), dtype=np.complex128)


def identity_beam(npointing: int, nant: int) -> np.ndarray:
    """B [npointing][nant][2][2] = identity (stand-in for the FEE model)."""
    return np.ascontiguousarray(np.broadcast_to(np.eye(2, dtype=np.complex128), (npointing, nant, 2, 2)))


def unit_vectors(az_deg, za_deg) -> np.ndarray:
    """[npointing][3] direction cosines (E, N, H) as calc_beam_geom forms
    them (geometry.c:268-270): N = cos(el)cos(az), E = cos(el)sin(az),
    H = sin(el)."""
    az = np.radians(np.atleast_1d(np.asarray(az_deg, dtype=np.float64)))
    el = np.radians(90.0 - np.atleast_1d(np.asarray(za_deg, dtype=np.float64)))
    return np.stack([np.cos(el) * np.sin(az), np.cos(el) * np.cos(az), np.sin(el)], axis=-1)


def grid_pointings(n_side: int, spacing_deg: float, az0_deg: float = 45.0, za0_deg: float = 20.0):
    """An n_side x n_side grid of (az, za) around (az0, za0), offsets in za and
    in az scaled by 1/sin(za) so the grid is roughly square on the sky."""
    off = (np.arange(n_side) - (n_side - 1) / 2.0) * spacing_deg
    dza, daz = np.meshgrid(off, off, indexing="ij")
    za = za0_deg + dza
    az = az0_deg + daz / np.sin(np.radians(za0_deg))
    return az.ravel(), za.ravel()


def fine_chan_freqs_hz(chan_start_hz: int, nfine: int = NCHAN,
                       coarse_width_hz: int = COARSE_CHAN_WIDTH_HZ) -> np.ndarray:
    """Lower-edge fine-channel frequencies as vmCreateGeometricDelays forms
    them (geometry.c:154-163): start + c * (width // nfine), integer Hz."""
    w = coarse_width_hz // nfine
    return np.array([chan_start_hz + w * c for c in range(nfine)], dtype=np.float64)


def coarse_chan_start_hz(cc: int, first_rec_chan: int = 109) -> int:
    """Start frequency of the cc-th coarse channel above receiver channel
    `first_rec_chan` (1.28 MHz channels centred on rec_chan * 1.28 MHz)."""
    centre = (first_rec_chan + cc) * COARSE_CHAN_WIDTH_HZ
    return centre - COARSE_CHAN_WIDTH_HZ // 2


def tile_delays(az_deg: float, za_deg: float) -> np.ndarray:
    """[16] analogue beamformer delays (units of 435 ps, 0..31) that point a
    4 x 4 dipole tile (1.1 m pitch, row-major from the north-west corner, as
    the device beam model lays it out) at (az, za)."""
    i = np.arange(16)
    x = ((i & 3) - 1.5) * 1.1
    y = (1.5 - (i >> 2)) * 1.1
    az, za = np.radians(az_deg), np.radians(za_deg)
    tau = (x * np.sin(za) * np.sin(az) + y * np.sin(za) * np.cos(az)) / 299792458.0
    d = np.round(tau / 435e-12)
    return np.clip(d - d.min(), 0, 31).astype(np.uint32)


def legacy_input_order(nant: int, seed: int = 3) -> np.ndarray:
    """i_idx[2*ant + pol] = vcs_order: a seeded permutation standing in for the
    metafits VCSOrder column (pfb.cpp:410-419)."""
    rng = np.random.default_rng(seed)
    return rng.permutation(2 * nant).astype(np.int32)


def tile_delays_toward(az: float, za: float) -> np.ndarray:
    """[16] analogue beamformer delays (0..31 steps of 435 ps) pointing a tile
    at (az, za) in radians: each dipole's geometric delay, quantised, offset to
    start at 0 (dipole i at column i % 4 east, row i // 4 from north, 1.1 m
    pitch)."""
    i = np.arange(16)
    x = ((i % 4) - 1.5) * 1.1
    y = (1.5 - (i // 4)) * 1.1
    tau = (x * np.sin(za) * np.sin(az) + y * np.sin(za) * np.cos(az)) / 299792458.0
    d = np.round(tau / 435e-12)
    return np.clip(d - d.min(), 0, 31).astype(np.uint32)


def tile_delay_sets(n: int, seed: int = 5, max_za_deg: float = 45.0, return_dirs: bool = False):
    """[n][16] delay settings of tiles pointed at random directions within
    max_za_deg of zenith (and, with return_dirs, their [n] az, za in radians)."""
    rng = np.random.default_rng(seed)
    out = np.zeros((n, 16), dtype=np.uint32)
    dirs = np.zeros((n, 2))
    for k in range(n):
        az = rng.uniform(0, 2 * np.pi)
        za = np.radians(rng.uniform(0, max_za_deg))
        out[k] = tile_delays_toward(az, za)
        dirs[k] = az, za
    return (out, dirs[:, 0], dirs[:, 1]) if return_dirs else out
