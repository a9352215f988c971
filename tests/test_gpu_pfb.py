"""Forward fine PFB on the GPU against the oracle and the reference's own
kernels (golden vectors).

Tolerances: WOLA int32 output bit-exact; the 4-bit (SMART) output bit-exact
except where an FFT value sits within FP32 error of a rounding boundary
(<= 1e-4 of bytes, each nibble within one LSB); full-precision output within
1e-5 of the spectrum rms (FP32 FFT against FP64).
"""
import numpy as np
import pytest

import synthetic as SY
from helpers import dev, host, nibble_diff, torch_cuda

pytestmark = pytest.mark.gpu

I_IN, K = 32, 128


@pytest.fixture(scope="module")
def torch():
    return torch_cuda()


@pytest.fixture(scope="module")
def vgb_mod(torch):
    import vgb

    vgb.lib()
    return vgb


@pytest.fixture(scope="module")
def golden_input(oracle_mod):
    return oracle_mod.mwax_buffer(20240601, 2, I_IN)


def run_fpfb(vgb, torch, htr, ninputs, nblocks, nspectra, filt, i_idx, flags, ncc=1, cc_stride=0):
    d = dev(htr.reshape(-1).view(np.uint8))
    v = vgb.reference_buffer_voltages(d, ninputs, nblocks, ncc, cc_stride)
    if flags & vgb.PFB_COMPLEX_INT4:
        out = torch.empty(ncc * nspectra * K * ninputs, dtype=torch.uint8, device="cuda")
    else:
        out = torch.empty(ncc * nspectra * K * ninputs * 2, dtype=torch.float64, device="cuda")
    vgb.fpfb(v, ncc, nspectra, dev(filt), dev(i_idx), flags, out)
    torch.cuda.synchronize()
    assert vgb.check_device_status() == 0
    a = host(out)
    if not flags & vgb.PFB_COMPLEX_INT4:
        a = a.view(np.complex128)
    return a.reshape(ncc, nspectra, K, ninputs)


@pytest.mark.parametrize("fp32", [False, True])
def test_smart_matches_reference_kernels(vgb_mod, torch, golden, golden_input, fp32):
    flags = vgb_mod.PFB_SMART | (vgb_mod.WOLA_FP32 if fp32 else 0)
    assert vgb_mod.filter_fp32_exact(golden["filter"])
    ours = run_fpfb(vgb_mod, torch, golden_input, I_IN, 1, 64, golden["filter"], golden["i_idx"], flags)[0]
    ref = golden["fpfb_smart_out"]
    assert nibble_diff(ours, ref) <= 1
    assert (ours != ref).mean() <= 1e-4


def test_full_precision_matches_reference_and_oracle(vgb_mod, torch, oracle_mod, golden, golden_input):
    ours = run_fpfb(vgb_mod, torch, golden_input, I_IN, 1, 16, golden["filter"], golden["i_idx"],
                    vgb_mod.PFB_FULL_PRECISION)[0]
    ref = golden["fpfb_full_out"].astype(np.complex128)
    rms = np.sqrt(np.mean(np.abs(ref) ** 2))
    assert np.abs(ours - ref).max() / rms < 1e-5
    orc = oracle_mod.fpfb(golden_input, I_IN, 16, golden["filter"], K, 12, golden["i_idx"],
                          oracle_mod.PFB_FULL_PRECISION)
    assert np.abs(ours - orc).max() / rms < 1e-5
    # the values are FP32 numbers divided by 128, stored as doubles
    assert np.array_equal(ours.astype(np.complex64).astype(np.complex128), ours)


def test_imag_part_first_and_fpga_float64(vgb_mod, torch, oracle_mod, golden, golden_input):
    for flags in (vgb_mod.PFB_COMPLEX_INT4 | vgb_mod.PFB_IMAG_PART_FIRST | vgb_mod.PFB_EMULATE_FPGA,
                  vgb_mod.PFB_COMPLEX_FLOAT64 | vgb_mod.PFB_EMULATE_FPGA | vgb_mod.PFB_IMAG_PART_FIRST):
        ours = run_fpfb(vgb_mod, torch, golden_input, I_IN, 1, 32, golden["filter"], golden["i_idx"], flags)[0]
        orc = oracle_mod.fpfb(golden_input, I_IN, 32, golden["filter"], K, 12, golden["i_idx"], flags)
        if flags & vgb_mod.PFB_COMPLEX_INT4:
            assert nibble_diff(ours, orc) <= 1 and (ours != orc).mean() <= 1e-4
        else:
            assert np.abs(ours - orc).max() / np.sqrt(np.mean(np.abs(orc) ** 2)) < 1e-5


def test_staged_chain_equals_fused(vgb_mod, torch, oracle_mod, golden, golden_input):
    """vgb_wola -> vgb_round -> vgb_fft128 -> vgb_pack (the reference's four
    stages) reproduces the fused kernel bit for bit; WOLA is bit-exact."""
    ns = 48
    d = dev(golden_input.reshape(-1).view(np.uint8))
    v = vgb_mod.reference_buffer_voltages(d, I_IN, 1)
    b = torch.empty(ns * I_IN * K * 2, dtype=torch.int32, device="cuda")
    vgb_mod.wola(v, ns, dev(golden["filter"]), b)
    torch.cuda.synchronize()
    assert np.array_equal(host(b).reshape(ns, I_IN, K, 2),
                          oracle_mod.wola(golden_input, I_IN, ns, golden["filter"], K, 12))
    for flags in (vgb_mod.PFB_SMART, vgb_mod.PFB_FULL_PRECISION):
        b2 = b.clone()
        vgb_mod.round_(b2, b2.numel(), bool(flags & vgb_mod.PFB_EMULATE_FPGA))
        vgb_mod.fft128(b2, ns * I_IN)
        if flags & vgb_mod.PFB_COMPLEX_INT4:
            out = torch.empty(ns * K * I_IN, dtype=torch.uint8, device="cuda")
        else:
            out = torch.empty(ns * K * I_IN * 2, dtype=torch.float64, device="cuda")
        vgb_mod.pack(b2, ns, I_IN, dev(golden["i_idx"]), flags, out)
        torch.cuda.synchronize()
        staged = host(out)
        if not flags & vgb_mod.PFB_COMPLEX_INT4:
            staged = staged.view(np.complex128)
        fused = run_fpfb(vgb_mod, torch, golden_input, I_IN, 1, ns, golden["filter"], golden["i_idx"], flags)
        assert np.array_equal(staged.reshape(fused.shape), fused)


def test_partial_tile_and_batched_channels(vgb_mod, torch, oracle_mod, golden):
    """nspectra not a multiple of the 16-spectrum tile, and two coarse
    channels in one launch equal two separate launches."""
    a = oracle_mod.mwax_buffer(11, 2, I_IN)
    b = oracle_mod.mwax_buffer(12, 2, I_IN)
    both = np.concatenate([a.reshape(-1), b.reshape(-1)])
    stride = a.nbytes
    flags = vgb_mod.PFB_SMART
    full = run_fpfb(vgb_mod, torch, both, I_IN, 1, 37, golden["filter"], golden["i_idx"], flags, ncc=2,
                    cc_stride=stride)
    one = run_fpfb(vgb_mod, torch, a, I_IN, 1, 37, golden["filter"], golden["i_idx"], flags)
    two = run_fpfb(vgb_mod, torch, b, I_IN, 1, 37, golden["filter"], golden["i_idx"], flags)
    assert np.array_equal(full[0], one[0]) and np.array_equal(full[1], two[0])
    orc = oracle_mod.fpfb(a, I_IN, 37, golden["filter"], K, 12, golden["i_idx"], flags)
    assert (one[0] != orc).mean() <= 1e-4


def test_full_array_block_boundary(vgb_mod, torch, oracle_mod):
    """128 tiles (256 inputs), spectra crossing a voltage-block boundary."""
    ninputs = 256
    htr = oracle_mod.mwax_buffer(99, 3, ninputs)
    filt = SY.analysis_filter_int16()
    i_idx = SY.legacy_input_order(ninputs // 2)
    ours = run_fpfb(vgb_mod, torch, htr, ninputs, 2, 1000, filt, i_idx, vgb_mod.PFB_SMART | vgb_mod.WOLA_FP32)[0]
    # the oracle on spectra 480..519 (a buffer view starting 480 frames later
    # is not block aligned, so compare the first 520 spectra)
    orc = oracle_mod.fpfb(htr, ninputs, 520, filt, K, 12, i_idx, oracle_mod.PFB_SMART)
    assert nibble_diff(ours[:520], orc) <= 1
    assert (ours[:520] != orc).mean() <= 1e-4
    # spectra of the second block: the oracle on the buffer that starts one block later
    orc2 = oracle_mod.fpfb(np.ascontiguousarray(htr[1:]), ninputs, 500, filt, K, 12, i_idx, oracle_mod.PFB_SMART)
    assert (ours[500:] != orc2).mean() <= 1e-4


def test_int32_wola_for_large_filters(vgb_mod, torch, oracle_mod, golden_input, golden):
    """A filter whose FP32 accumulation would not be exact (peak 117964, like
    the reference's FINEPFB) goes through the int32 path, bit-exactly."""
    h = (SY.analysis_filter_int16().astype(np.int64) * 117964 // 32767).astype(np.int32)
    assert not vgb_mod.filter_fp32_exact(h)
    ours = run_fpfb(vgb_mod, torch, golden_input, I_IN, 1, 32, h, golden["i_idx"], vgb_mod.PFB_SMART)[0]
    orc = oracle_mod.fpfb(golden_input, I_IN, 32, h, K, 12, golden["i_idx"], oracle_mod.PFB_SMART)
    assert nibble_diff(ours, orc) <= 1 and (ours != orc).mean() <= 1e-4


def test_rejects_bad_arguments(vgb_mod, torch, golden):
    d = torch.zeros(2 * I_IN * 64000 * 2 + 64, dtype=torch.uint8, device="cuda")
    out = torch.empty(64 * K * I_IN, dtype=torch.uint8, device="cuda")
    v = vgb_mod.reference_buffer_voltages(d.data_ptr() + 1, I_IN, 1)  # misaligned
    with pytest.raises(vgb_mod.VGBError, match="aligned"):
        vgb_mod.fpfb(v, 1, 64, dev(golden["filter"]), dev(golden["i_idx"]), vgb_mod.PFB_SMART, out)
    v = vgb_mod.reference_buffer_voltages(d, I_IN, 1)
    with pytest.raises(vgb_mod.VGBError, match="nspectra"):
        vgb_mod.fpfb(v, 1, 501, dev(golden["filter"]), dev(golden["i_idx"]), vgb_mod.PFB_SMART, out)
    # an input map that repeats a column is not a permutation: flagged, nothing written
    bad = np.array(golden["i_idx"], dtype=np.int32)
    bad[5] = bad[6]
    out.fill_(0x5A)
    vgb_mod.fpfb(v, 1, 64, dev(golden["filter"]), dev(bad), vgb_mod.PFB_SMART, out)
    torch.cuda.synchronize()
    with pytest.raises(vgb_mod.VGBError, match="permutation"):
        vgb_mod.check_device_status()
    assert (host(out) == 0x5A).all()
