"""The tcgen05 BF16 GEMM (vgb_gemm_bf16) against a plain PyTorch FP32
matmul of the same bf16 inputs. Tolerance: 1e-5 of the largest |C| (each
bf16 x bf16 product is exact in FP32; only the summation order differs)."""
import pytest

from helpers import torch_cuda

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 128, 64), (256, 384, 512), (384, 256, 1024), (128, 512, 192)])
def test_gemm_bf16_matches_fp32_reference(M, N, K):
    torch = torch_cuda()
    import vgb

    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    C = torch.full((M, N), float("nan"), device="cuda")
    vgb.gemm_bf16(A, B, C, M, N, K)
    torch.cuda.synchronize()
    assert vgb.check_device_status() == 0
    ref = A.float() @ B.float().T
    err = (C - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-5, err


@pytest.mark.parametrize("fp16", [False, True])
def test_gemm_batched(fp16):
    torch = torch_cuda()
    import vgb

    M, N, K, nb = 256, 256, 128, 3
    dt = torch.float16 if fp16 else torch.bfloat16
    g = torch.Generator(device="cuda").manual_seed(11 + fp16)
    A = torch.randn(nb, M, K, device="cuda", generator=g).to(dt)
    B = torch.randn(nb, N, K, device="cuda", generator=g).to(dt)
    C = torch.full((nb, M, N), float("nan"), device="cuda")
    vgb.gemm_batched(A, B, C, M, N, K, nb, fp16)
    torch.cuda.synchronize()
    assert vgb.check_device_status() == 0
    ref = A.float() @ B.float().transpose(1, 2)
    err = (C - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-5, err


@pytest.mark.parametrize("fp16", [False, True])
def test_gemm_batched_planes(fp16):
    """Two A planes (hi | lo halves of each row) against one B: the same sum
    as the K-concatenated product with B read modulo K, against FP32."""
    torch = torch_cuda()
    import vgb

    M, N, K, nb = 384, 512, 192, 3
    dt = torch.float16 if fp16 else torch.bfloat16
    g = torch.Generator(device="cuda").manual_seed(21 + fp16)
    A = torch.randn(nb, M, 2 * K, device="cuda", generator=g).to(dt)
    B = torch.randn(nb, N, K, device="cuda", generator=g).to(dt)
    C = torch.full((nb, M, N), float("nan"), device="cuda")
    vgb.gemm_batched_planes(A, B, C, M, N, K, nb, fp16)
    torch.cuda.synchronize()
    assert vgb.check_device_status() == 0
    ref = (A[:, :, :K].float() + A[:, :, K:].float()) @ B.float().transpose(1, 2)
    err = (C - ref).abs().max().item() / ref.abs().max().item()
    assert err < 1e-5, err


@pytest.mark.parametrize("variant", [128, 256, 512])
def test_gemm_variants_identical(variant):
    """Every kernel variant the autotuner chooses between (plain 128- and
    256-wide tiles, persistent 256-wide) gives the same bits."""
    torch = torch_cuda()
    import vgb

    M, N, K, nb = 384, 512, 320, 3
    g = torch.Generator(device="cuda").manual_seed(5)
    A = torch.randn(nb, M, K, device="cuda", generator=g).to(torch.float16)
    B = torch.randn(nb, N, K, device="cuda", generator=g).to(torch.float16)
    C0 = torch.full((nb, M, N), float("nan"), device="cuda")
    C1 = torch.full((nb, M, N), float("nan"), device="cuda")
    prev = vgb.gemm_variant(128)
    try:
        vgb.gemm_batched(A, B, C0, M, N, K, nb, True)
        vgb.gemm_variant(variant)
        vgb.gemm_batched(A, B, C1, M, N, K, nb, True)
    finally:
        vgb.gemm_variant(prev)
    torch.cuda.synchronize()
    assert vgb.check_device_status() == 0
    assert torch.equal(C0, C1)
    ref = A.float() @ B.float().transpose(1, 2)
    assert (C1 - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()


def test_gemm_rejects_bad_shapes():
    torch = torch_cuda()
    import vgb

    A = torch.zeros(100, 64, dtype=torch.bfloat16, device="cuda")
    C = torch.zeros(100, 128, device="cuda")
    with pytest.raises(vgb.VGBError, match="multiples of 128"):
        vgb.gemm_bf16(A, A, C, 100, 128, 64)
