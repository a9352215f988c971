"""Failure detection without a GPU fault: a bounded wait that nothing
satisfies gives up, flags the device status word (VGB_ERR_DEVICE, 'bounded
wait expired') and leaves the context usable; errors come back as status
codes, never by exiting the process."""
import numpy as np
import pytest

from helpers import torch_cuda

pytestmark = pytest.mark.gpu


def test_bounded_wait_expires_and_context_survives():
    torch = torch_cuda()
    import vgb

    vgb.lib()
    assert vgb.check_device_status() == 0
    vgb.selftest_bounded_wait(polls=2000)
    with pytest.raises(vgb.VGBError, match="bounded wait expired"):
        vgb.check_device_status()
    # the status word was cleared and the context still runs kernels
    assert vgb.check_device_status() == 0
    A = torch.randn(128, 64, device="cuda").to(torch.bfloat16)
    C = torch.empty(128, 128, device="cuda")
    vgb.gemm_bf16(A, A, C, 128, 128, 64)
    torch.cuda.synchronize()
    assert vgb.check_device_status() == 0
    ref = A.float() @ A.float().T
    assert (C - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()


def test_host_side_faults_are_status_codes():
    torch_cuda()
    import vgb

    with pytest.raises(vgb.VGBError, match="polls"):
        vgb.selftest_bounded_wait(polls=0)
    with pytest.raises(vgb.VGBError):
        vgb.gemm_bf16(None, None, None, 128, 128, 64)
