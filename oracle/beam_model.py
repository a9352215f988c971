"""FP64 numpy restatement of the primary-beam pieces (test infrastructure: the
checker for vgb_primary_beam and the training / validation reference of the
beam surrogate; never part of the product path).

* dipole configuration hash: primary_beam.c:355-414 (checked against the
  reference's own hash_dipole_config compiled here);
* parallactic-angle rotation: primary_beam.c:436-456 with the spherical-
  triangle identity of doc/Definitions.md (the reference calls PAL's
  palDh2e / palPa, not available here);
* the analytic MWA tile model that stands in for the FEE model
  (mwa_hyperbeam calc_jones, not available here): 4 x 4 dipoles of 1.1 m
  pitch with the tile beamformer's 435 ps delay steps, a ground plane 0.278 m
  below, short-dipole projections onto (theta, phi); zenith-normalised.
"""
from __future__ import annotations

import numpy as np

C = 299792458.0
PITCH = 1.1
DELAY_UNIT = 435e-12
HEIGHT = 0.278
MWA_LATITUDE = -0.4660608448386394


def hash_dipole_config(amps) -> int:
    dead = [i for i in range(16) if amps[i] == 0.0]
    if len(dead) == 0:
        return 0
    if len(dead) == 1:
        return dead[0] + 1
    if len(dead) == 2:
        d1, d2 = dead
        return 16 * d1 - ((d1 + 2) * (d1 + 1)) // 2 + d2 + 17
    if len(dead) == 16:
        return 137
    return -1


def tile_jones(az, za, freq, delays):
    """az, za (radians), freq (Hz): broadcastable arrays; delays [16].
    Returns complex128 [..., 2, 2] (rows theta, phi; columns X, Y dipole)."""
    az, za, freq = np.broadcast_arrays(np.asarray(az, float), np.asarray(za, float), np.asarray(freq, float))
    d = np.asarray(delays)
    k = 2.0 * np.pi * freq
    saz, caz, sza, cza = np.sin(az), np.cos(az), np.sin(za), np.cos(za)
    af = np.zeros(az.shape, dtype=np.complex128)
    live = 0
    for i in range(16):
        if d[i] == 32:
            continue
        live += 1
        x = ((i & 3) - 1.5) * PITCH
        y = (1.5 - (i >> 2)) * PITCH
        tau = (x * sza * saz + y * sza * caz) / C - float(d[i]) * DELAY_UNIT
        af += np.exp(1j * k * tau)
    J = np.zeros(az.shape + (2, 2), dtype=np.complex128)
    if live == 0:
        return J
    g = np.sin(k * HEIGHT * cza / C) / np.sin(k * HEIGHT / C)
    a = af / 16.0 * g
    J[..., 0, 0] = a * cza * saz
    J[..., 0, 1] = a * cza * caz
    J[..., 1, 0] = a * caz
    J[..., 1, 1] = a * -saz
    return J


def parallactic_rotation(lat, az, za):
    """P [..., 2, 2] = [[-cos chi, -sin chi], [sin chi, -cos chi]]."""
    az, za = np.broadcast_arrays(np.asarray(az, float), np.asarray(za, float))
    el = 0.5 * np.pi - za
    x = -np.cos(az) * np.cos(el) * np.sin(lat) + np.sin(el) * np.cos(lat)
    y = -np.sin(az) * np.cos(el)
    z = np.cos(az) * np.cos(el) * np.cos(lat) + np.sin(el) * np.sin(lat)
    r = np.hypot(x, y)
    ha = np.where(r == 0.0, 0.0, np.arctan2(y, x))
    dec = np.arctan2(z, r)
    num = np.cos(lat) * np.sin(ha)
    den = np.sin(lat) * np.cos(dec) - np.cos(lat) * np.sin(dec) * np.cos(ha)
    chi = np.where((num != 0.0) | (den != 0.0), np.arctan2(num, den), 0.0)
    P = np.empty(az.shape + (2, 2))
    P[..., 0, 0] = -np.cos(chi)
    P[..., 0, 1] = -np.sin(chi)
    P[..., 1, 0] = np.sin(chi)
    P[..., 1, 1] = -np.cos(chi)
    return P


def primary_beam(az, za, freqs, delays, pa=True, lat=MWA_LATITUDE):
    """B [nfreq][npointing][ntile][2][2] = J P (vmCalcB order)."""
    az, za = np.asarray(az, float), np.asarray(za, float)
    freqs = np.atleast_1d(np.asarray(freqs, float))
    delays = np.asarray(delays).reshape(-1, 16)
    out = np.empty((freqs.size, az.size, delays.shape[0], 2, 2), dtype=np.complex128)
    P = parallactic_rotation(lat, az, za) if pa else None
    for fi, f in enumerate(freqs):
        for t in range(delays.shape[0]):
            J = tile_jones(az, za, f, delays[t])
            out[fi, :, t] = J @ P if pa else J
    return out
