"""The oracle's multi-pointing beamformer against the reference's own
kernels run for five pointings (tests/golden/ref_golden_multibeam.npz, made
by make_golden_multibeam.py): bit for bit, as for one pointing."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_golden_multibeam.npz")


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def test_oracle_multipointing_matches_reference_kernels(oracle_mod, gold):
    g = gold
    J = oracle_mod.calc_j(g["D"], g["B"])
    phi = oracle_mod.calc_phi(g["unit"], g["east"], g["north"], g["height"], g["cable"], g["freqs"])
    S, _ = oracle_mod.beamform(g["v"], J, phi, g["polQ"], g["polP"], float(g["invw"]), nstokes=4, want_e=False)
    assert S.shape == g["S"].shape == (5, 60, 4, 128)
    assert np.array_equal(S, g["S"])
