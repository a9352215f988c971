"""Array factor (calc_array_factor, geometry.c:440-467): the committed
fixture is what the reference's own C gives (regenerated and compared when
oracle/_ref/libref_host.so is built here), and the device kernel matches it
within 1e-12 of the peak (FP64 phases; sin/cos differ from glibc by an ulp)."""
import os
import sys

import numpy as np
import pytest

from helpers import dev, host, torch_cuda

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden", "ref_golden_af.npz")


def test_fixture_is_the_reference(tmp_path):
    sys.path.insert(0, os.path.join(HERE, "golden"))
    import make_golden_af as M

    if not os.path.exists(M.LIB):
        pytest.skip("reference host library not built (no reference sources here)")
    g = dict(np.load(GOLD))
    assert np.array_equal(M.reference_af(g), g["af"])
    assert g["af"][840] == 1.0            # the look direction itself (grid centre)


@pytest.mark.gpu
def test_device_array_factor_matches_reference():
    torch = torch_cuda()
    import vgb

    g = dict(np.load(GOLD))
    out = torch.empty(g["dirs"].shape[0], dtype=torch.float64, device="cuda")
    vgb.array_factor(dev(g["look"]), dev(g["dirs"]), float(g["freq"]), dev(g["east"]), dev(g["north"]),
                     dev(g["height"]), dev(g["cable"]), out)
    torch.cuda.synchronize()
    af = host(out)
    assert np.abs(af - g["af"]).max() <= 1e-12
