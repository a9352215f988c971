"""The FP32 throughput diagnostic (vgb_fp32_peak) the bench uses as the
compute denominator of the fused PFB + beamformer: both issue forms return a
plausible rate for a 152-SM GPU (between 10 and 400 TFLOP/s)."""
import pytest

from helpers import torch_cuda

pytestmark = pytest.mark.gpu


def test_fp32_peak_is_plausible():
    torch_cuda()
    import vgb

    scalar = vgb.fp32_peak(False, iters=4000)
    packed = vgb.fp32_peak(True, iters=4000)
    print("FP32 TFLOP/s: FFMA", scalar, "FFMA2", packed)
    assert 10.0 < scalar < 400.0 and 10.0 < packed < 400.0
