"""Helpers shared by the GPU parity tests: device transfer, the synthetic
observation tables, and the oracle-side reference chain.

The oracle (oracle/oracle.py) is the checker only; the values under test
always come from the CUDA library through its C ABI (vgb.py)."""
from __future__ import annotations

import numpy as np
import pytest

import synthetic as SY


def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def dev(a: np.ndarray):
    torch = torch_cuda()
    a = np.ascontiguousarray(a)
    if a.dtype == np.complex128:
        a = a.view(np.float64)
    elif a.dtype == np.complex64:
        a = a.view(np.float32)
    elif a.dtype == np.uint32:
        a = a.view(np.int32)
    return torch.from_numpy(a.copy()).cuda()


def host(t, dtype=None, shape=None):
    a = t.cpu().numpy()
    if dtype is not None:
        a = a.view(dtype)
    if shape is not None:
        a = a.reshape(shape)
    return a


def tables(nant: int, cc: int = 0, seed: int = 1, npointing: int = 1):
    """J [p][a][c][2][2] and phi [p][a][c] (complex128) from the oracle's FP64
    table builders for a synthetic observation."""
    import oracle as O

    D = SY.calibration_jones(nant, SY.NCHAN, seed=seed)
    B = SY.identity_beam(npointing, nant) + 0.05 * (1 + 1j) * O.gauss(seed + 100, npointing * nant * 4).reshape(
        npointing, nant, 2, 2)
    J = O.calc_j(D, np.ascontiguousarray(B))
    east, north, height, cable = SY.tile_layout(nant, seed=seed + 7)
    az = 45.0 + 0.5 * np.arange(npointing)
    unit = SY.unit_vectors(az, np.full(npointing, 20.0))
    freqs = SY.fine_chan_freqs_hz(SY.coarse_chan_start_hz(cc))
    phi = O.calc_phi(unit, east, north, height, cable, freqs)
    return J, phi


def weights_on_device(J: np.ndarray, phi: np.ndarray):
    """W = phi * J via the library's FP64 kernel; returns a device tensor of
    complex float [n][2][2] stored as float32 [n][8]."""
    import vgb

    torch = torch_cuda()
    n = phi.size
    dJ, dphi = dev(J), dev(phi)
    W = torch.empty((n, 8), dtype=torch.float32, device="cuda")
    vgb.weights(dJ, dphi, n, W)
    return W


def pol_lists(i_idx: np.ndarray):
    """polQ/polP (jones.c:40-64) from the MWAX->legacy input map."""
    return (np.ascontiguousarray(i_idx[0::2].astype(np.uint32)),
            np.ascontiguousarray(i_idx[1::2].astype(np.uint32)))


def rel_err(x, ref) -> float:
    ref = np.asarray(ref)
    return float(np.abs(np.asarray(x) - ref).max() / max(np.abs(ref).max(), 1e-30))


def nibble_diff(a: np.ndarray, b: np.ndarray) -> int:
    hi = lambda x: ((x.astype(np.int16) >> 4) ^ 8) - 8
    lo = lambda x: ((x.astype(np.int16) & 15) ^ 8) - 8
    return int(max(np.abs(hi(a) - hi(b)).max(), np.abs(lo(a) - lo(b)).max()))


def oracle_chain_second(htr, ninputs, filt, syn, J, phi, invw, blocks_per_chunk=4):
    """The FP64 oracle chain over one whole second of MWAX voltages in the
    reference's read-buffer layout (htr = margin block + the second's blocks):
    forward PFB (identity VCS order, PFB_FULL_PRECISION), beamformer,
    renormalise of the oracle's own Stokes, inverse PFB of the oracle's own
    beam voltages (no history: a first second) and VDIF quantisation.
    Processed a few blocks at a time so the complex-double fine channels stay
    small. Returns S [ns][4][128], e [ns][128][2], (offsets, scales, bytes)
    and the VDIF payload bytes [ns][512]."""
    import oracle as O

    K, P = 128, 12
    nblk = htr.shape[0] - 1
    i_idx = np.arange(ninputs, dtype=np.int32)
    polQ, polP = pol_lists(i_idx)
    S_parts, e_parts = [], []
    for b in range(0, nblk, blocks_per_chunk):
        k = min(blocks_per_chunk, nblk - b)
        v = O.fpfb(np.ascontiguousarray(htr[b:b + k + 1]), ninputs, k * 500, filt, K, P, i_idx, 0)
        S, e = O.beamform(v, J, phi, polQ, polP, invw)
        S_parts.append(S[0])
        e_parts.append(e[0])
        del v
    S = np.concatenate(S_parts)
    e = np.concatenate(e_parts)
    off, sc, u8 = O.renormalise(S[None])
    x = np.concatenate([np.zeros((P, K, 2), np.complex128), e], axis=0)
    out = O.ipfb(x, syn, P)
    flt = np.stack([out.real, out.imag], axis=-1).astype(np.float32).reshape(S.shape[0], 512)
    return S, e, (off[0], sc[0], u8[0]), O.vdif_quantise(flt)


def byte_diff_stats(a, b):
    """(largest |a - b|, fraction of samples differing by more than one LSB,
    fraction differing at all) of two uint8 arrays."""
    d = np.abs(np.asarray(a).astype(np.int16) - np.asarray(b).astype(np.int16))
    return int(d.max()), float((d > 1).mean()), float((d > 0).mean())
