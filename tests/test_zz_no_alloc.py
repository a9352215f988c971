"""The entry point that allocates nothing (vgb_beamform_mwax_psrfits_noalloc).

Callers that cannot allocate device memory while they run (a real-time
pipeline that reserves the GPU's memory up front) get voltages -> PSRFITS
bytes with the intermediate Stokes held in a fixed 24 MiB array inside the
library. Its output must equal the allocating path's (vgb_beamform_mwax into a
caller buffer, then vgb_renormalise) on calls in a row with different inputs
and shapes (one and two coarse channels, so the per-channel strides of the
bytes, offsets and scales are exercised), since every call shares that one
array. Tolerance: the same kernels run on the same inputs, so the bytes,
offsets and scales are identical.

This file is named to be collected last.
"""
import numpy as np
import pytest

import synthetic as SY
from helpers import dev, host, tables, torch_cuda, weights_on_device

pytestmark = pytest.mark.gpu

K = 128
NANT, NI = 16, 32


def allocating_path(vgb, torch, v, ncc, nspectra, filt, flags, W, invw, nstokes):
    S = torch.empty(ncc * nspectra * nstokes * K, dtype=torch.float32, device="cuda")
    vgb.beamform_mwax(v, ncc, nspectra, filt, flags, W, NANT, invw, nstokes, S)
    out = torch.empty(ncc * nspectra * nstokes * K, dtype=torch.uint8, device="cuda")
    off = torch.empty(ncc * nstokes * K, dtype=torch.float32, device="cuda")
    sc = torch.empty_like(off)
    vgb.renormalise(S, ncc, 1, nspectra, nstokes, K, out, nspectra * nstokes * K, 0, nstokes * K, K, off, sc)
    torch.cuda.synchronize()
    return host(out), host(off), host(sc)


def test_noalloc_matches_allocating_path_on_calls_in_a_row():
    torch = torch_cuda()
    import oracle as O
    import vgb

    # The set-up call: looks up the array's address, launches nothing.
    vgb.beamform_mwax_psrfits_noalloc(vgb.Voltages(), 1, 0, None, 0, None, NANT, 1.0, 4, None, None, None)
    filt = dev(SY.analysis_filter_int16())
    flags = vgb.PFB_FULL_PRECISION | vgb.WOLA_FP32
    for call, (seed, ncc, nspectra, nstokes) in enumerate([(41, 1, 500, 4), (42, 1, 320, 1), (43, 2, 500, 4)]):
        bufs = [O.mwax_buffer(seed + 10 * c, 2, NI).reshape(-1).view(np.uint8) for c in range(ncc)]
        d = dev(np.concatenate(bufs))
        v = vgb.reference_buffer_voltages(d, NI, 1, ncc=ncc, cc_stride=bufs[0].size)
        Ws = []
        for c in range(ncc):
            J, phi = tables(NANT, cc=c, seed=1 + c)
            Ws.append(weights_on_device(J, phi))
        W = torch.cat(Ws)
        out = torch.empty(ncc * nspectra * nstokes * K, dtype=torch.uint8, device="cuda")
        off = torch.empty(ncc * nstokes * K, dtype=torch.float32, device="cuda")
        sc = torch.empty_like(off)
        vgb.beamform_mwax_psrfits_noalloc(v, ncc, nspectra, filt, flags, W, NANT, 1.0 / NI, nstokes, out, off, sc)
        torch.cuda.synchronize()
        assert vgb.check_device_status() == 0
        ref_out, ref_off, ref_sc = allocating_path(vgb, torch, v, ncc, nspectra, filt, flags, W, 1.0 / NI, nstokes)
        assert np.array_equal(host(out), ref_out), call
        assert np.array_equal(host(off), ref_off), call
        assert np.array_equal(host(sc), ref_sc), call


def test_noalloc_rejects_requests_beyond_its_scratch():
    torch = torch_cuda()
    import vgb

    d = torch.zeros(1 << 20, dtype=torch.uint8, device="cuda")
    v = vgb.reference_buffer_voltages(d, NI, 20)
    out = torch.empty(16, dtype=torch.uint8, device="cuda")
    with pytest.raises(vgb.VGBError, match="static scratch"):
        # 2 coarse channels x 10000 spectra x 4 Stokes x 128 > 24 MiB of floats
        vgb.beamform_mwax_psrfits_noalloc(v, 2, 10000, d, vgb.PFB_FULL_PRECISION, d, NANT, 1.0, 4, out, out, out)
