"""Primary beam (vmCalcB pieces): the dead-dipole hash against the
reference's own hash_dipole_config (CPU), the parallactic-angle rotation at
known geometries (CPU), and the device model against the FP64 oracle (GPU,
within 1e-12 of the largest |B|)."""
import ctypes
import itertools
import os

import numpy as np
import pytest

import beam_model as BM
from helpers import dev, host, torch_cuda

REF_LIB = os.path.join(os.path.dirname(BM.__file__), "_ref", "libref_host.so")


def patterns():
    rng = np.random.default_rng(5)
    out = [np.ones(16)]
    out += [np.where(np.arange(16) == i, 0.0, 1.0) for i in range(16)]
    out += [np.where((np.arange(16) == i) | (np.arange(16) == j), 0.0, 1.0)
            for i, j in itertools.combinations(range(16), 2)]
    out += [np.zeros(16)]
    out += [(rng.random(16) > 0.4).astype(float) for _ in range(50)]
    return out


@pytest.fixture(scope="module")
def vgb_mod():
    import build as B
    import vgb

    if not os.path.exists(vgb.LIB_PATH):
        B.build()
    vgb.lib()
    return vgb


def test_hash_dipole_config(vgb_mod):
    idx = [vgb_mod.hash_dipole_config(a) for a in patterns()]
    assert idx[:138] == list(range(138))            # every cached configuration, in order
    assert all(i == BM.hash_dipole_config(a) for i, a in zip(idx, patterns()))
    if os.path.exists(REF_LIB):
        ref = ctypes.CDLL(REF_LIB)
        for a, i in zip(patterns(), idx):
            a = np.ascontiguousarray(a)
            assert ref.refhost_hash_dipole_config(a.ctypes.data_as(ctypes.c_void_p)) == i


def test_parallactic_angle_known_geometry():
    lat = BM.MWA_LATITUDE
    # on the meridian south of zenith (az = pi): ha = 0 -> chi = 0 -> P = [[-1, 0], [0, -1]]
    P = BM.parallactic_rotation(lat, np.pi, 0.3)
    assert np.allclose(P, [[-1, 0], [0, -1]], atol=1e-12)
    # north of zenith at a southern site, towards the pole-side: chi = pi
    P = BM.parallactic_rotation(lat, 0.0, 0.2)
    assert np.allclose(P, [[1, 0], [0, 1]], atol=1e-12)
    # east and west mirror each other: chi(az) = -chi(2 pi - az)
    Pe, Pw = BM.parallactic_rotation(lat, 1.0, 0.5), BM.parallactic_rotation(lat, 2 * np.pi - 1.0, 0.5)
    assert np.isclose(Pe[0, 1], -Pw[0, 1]) and np.isclose(Pe[0, 0], Pw[0, 0])
    # rotation matrix
    P = BM.parallactic_rotation(lat, 2.2, 0.7)
    assert np.allclose(P @ P.T, np.eye(2), atol=1e-12)


def test_tile_model_zenith_normalised():
    J = BM.tile_jones(0.3, 0.0, 150e6, np.zeros(16))
    assert np.isclose(abs(np.linalg.det(J)), 1.0)   # unit response at zenith, all delays 0
    dead = np.full(16, 32)
    assert np.all(BM.tile_jones(0.3, 0.2, 150e6, dead) == 0)


@pytest.mark.gpu
def test_primary_beam_matches_oracle(vgb_mod):
    torch = torch_cuda()
    rng = np.random.default_rng(8)
    npnt, ntile = 40, 6
    az = rng.uniform(0, 2 * np.pi, npnt)
    za = rng.uniform(0, np.radians(80), npnt)
    freqs = np.array([80e6, 154.88e6, 300e6])
    delays = rng.integers(0, 32, (ntile, 16)).astype(np.uint32)
    delays[2, 3] = 32                 # a dead dipole
    delays[4, :] = 32                 # a dead tile -> zero
    for pa in (True, False):
        B = torch.zeros(freqs.size * npnt * ntile * 8, dtype=torch.float64, device="cuda")
        vgb_mod.primary_beam(dev(az), dev(za), dev(freqs), dev(delays), B, pa_correction=pa)
        torch.cuda.synchronize()
        got = host(B).view(np.complex128).reshape(freqs.size, npnt, ntile, 2, 2)
        want = BM.primary_beam(az, za, freqs, delays, pa=pa)
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
        assert np.all(got[:, :, 4] == 0)


@pytest.mark.gpu
def test_primary_beam_shared_configurations(vgb_mod):
    """Tiles sharing a delay set share B (evaluated once per distinct set and
    copied): 1,100 tiles drawn from 5 sets (one with a dead dipole), spread
    over more than one 1,024-tile chunk of the configuration scan."""
    torch = torch_cuda()
    rng = np.random.default_rng(9)
    npnt, ntile = 12, 1100
    az = rng.uniform(0, 2 * np.pi, npnt)
    za = rng.uniform(0, np.radians(70), npnt)
    freqs = np.array([120e6, 210e6])
    sets = rng.integers(0, 32, (5, 16)).astype(np.uint32)
    sets[3, 7] = 32
    pick = rng.integers(0, 5, ntile)
    pick[1050:] = 4                   # a set first seen in the second chunk
    pick[:1050][pick[:1050] == 4] = 0
    delays = np.ascontiguousarray(sets[pick])
    B = torch.zeros(freqs.size * npnt * ntile * 8, dtype=torch.float64, device="cuda")
    vgb_mod.primary_beam(dev(az), dev(za), dev(freqs), dev(delays), B)
    torch.cuda.synchronize()
    got = host(B).view(np.complex128).reshape(freqs.size, npnt, ntile, 2, 2)
    want_sets = BM.primary_beam(az, za, freqs, sets)
    want = want_sets[:, :, pick]
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
