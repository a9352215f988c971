"""Python face of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE. Only tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline leg import this module, and only as the checker (bench: as the
timed CPU baseline). The shipped library never routes through it.

Every wrapper takes and returns numpy arrays in the reference's layouts
(VCSBeam ``include/vcsbeam.h.in:234-268`` index macros). Complex arrays are
numpy complex128 / complex64 unless stated.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

VSPVB = 64000  # include/vcsbeam.h.in:238
PFB_COMPLEX_INT4 = 0x10
PFB_COMPLEX_FLOAT64 = 0x20
PFB_IMAG_PART_FIRST = 0x100
PFB_EMULATE_FPGA = 0x200
PFB_SMART = 0x21D  # include/vcsbeam.h.in:476
PFB_FULL_PRECISION = 0x2D  # include/vcsbeam.h.in:478

_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle.so with the committed Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(LIB_PATH) or (
        os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, "oracle.c"))
    ):
        subprocess.run(["make", "-s", "-C", HERE, "-B" if force else "liboracle.so"],
                       check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


P = ctypes.c_void_p
I32 = ctypes.c_int
U32 = ctypes.c_uint32
U64 = ctypes.c_uint64
SZ = ctypes.c_size_t
D = ctypes.c_double
F = ctypes.c_float
L = ctypes.c_long


def _declare(l):
    sig = {
        "orc_hash64": (U64, [U64, U64]),
        "orc_gauss": (D, [U64, U64]),
        "orc_gen_int8": (None, [U64, P, SZ, I32, I32, I32, I32]),
        "orc_gen_int4_bytes": (None, [U64, P, SZ, I32, I32]),
        "orc_wola": (None, [P, I32, I32, P, I32, I32, P]),
        "orc_fpga_round": (None, [P, SZ, P]),
        "orc_int2float": (None, [P, SZ, P]),
        "orc_fft_forward": (None, [P, P, I32, SZ]),
        "orc_pack": (None, [P, I32, I32, I32, P, U32, P]),
        "orc_fpfb": (None, [P, I32, I32, P, I32, I32, P, U32, P]),
        "orc_unpack_int4": (None, [P, SZ, P]),
        "orc_beamform": (None, [P, I32, I32, I32, I32, P, P, P, P, I32, D, I32, P, P]),
        "orc_renormalise": (None, [P, I32, I32, I32, I32, P, P, P]),
        "orc_sat_u8": (ctypes.c_uint8, [D]),
        "orc_incoh_beam": (None, [P, I32, I32, I32, P]),
        "orc_ipfb": (None, [P, I32, I32, I32, P, I32, I32, P]),
        "orc_ipfb_table": (None, [P, I32, I32, P, P]),
        "orc_vdif_quantise": (None, [P, SZ, P]),
        "orc_calc_j": (None, [I32, I32, I32, P, P, P]),
        "orc_calc_phi": (None, [I32, I32, I32, P, P, P, P, P, P, P]),
        "orc_roots_of_unity": (None, [I32, P]),
        "orc_mult2x2d": (None, [P, P, P]),
        "orc_norm2x2": (D, [P, P]),
        "orc_inv2x2S": (None, [P, P]),
        "orc32_pfb_beam": (I32, [P, I32, I32, I32, P, I32, I32, I32, P, F, P, P, P]),
        "orc32_ipfb_vdif": (I32, [P, I32, I32, I32, P, P, I32, L, L, P]),
        "orc32_renormalise": (I32, [P, I32, I32, I32, P, P, P]),
        "orc32_max_threads": (I32, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(l, name)
        fn.restype = res
        fn.argtypes = args


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be C-contiguous"
    return a.ctypes.data_as(ctypes.c_void_p)


# --------------------------------------------------------------------------
# synthetic inputs
# --------------------------------------------------------------------------

def gen_int8(seed: int, n: int, sigma_num: int = 16, sigma_den: int = 1,
             lo: int = -127, hi: int = 127) -> np.ndarray:
    out = np.empty(n, dtype=np.int8)
    lib().orc_gen_int8(seed, _p(out), n, sigma_num, sigma_den, lo, hi)
    return out


def gen_int4_bytes(seed: int, n: int, sigma_num: int = 5, sigma_den: int = 2) -> np.ndarray:
    out = np.empty(n, dtype=np.uint8)
    lib().orc_gen_int4_bytes(seed, _p(out), n, sigma_num, sigma_den)
    return out


def gauss(seed: int, n: int) -> np.ndarray:
    l = lib()
    return np.array([l.orc_gauss(seed, i) for i in range(n)], dtype=np.float64)


def mwax_buffer(seed: int, nblocks: int, ninputs: int, sigma: int = 16) -> np.ndarray:
    """MWAX voltages [nblocks][ninputs][VSPVB][2] int8 (block 0 = margin)."""
    return gen_int8(seed, nblocks * ninputs * VSPVB * 2, sigma).reshape(
        nblocks, ninputs, VSPVB, 2)


# --------------------------------------------------------------------------
# forward PFB
# --------------------------------------------------------------------------

def wola(htr: np.ndarray, ninputs: int, nspectra: int, h: np.ndarray, K: int, P_: int):
    h = np.ascontiguousarray(h, dtype=np.int32)
    b = np.empty((nspectra, ninputs, K, 2), dtype=np.int32)
    lib().orc_wola(_p(htr), ninputs, nspectra, _p(h), K, P_, _p(b))
    return b


def fpga_round(b: np.ndarray) -> np.ndarray:
    out = np.empty(b.shape, dtype=np.float32)
    lib().orc_fpga_round(_p(b), b.size, _p(out))
    return out


def int2float(b: np.ndarray) -> np.ndarray:
    out = np.empty(b.shape, dtype=np.float32)
    lib().orc_int2float(_p(b), b.size, _p(out))
    return out


def fft_forward(x: np.ndarray) -> np.ndarray:
    """FP64 forward DFT along the last axis of a complex array."""
    x = np.ascontiguousarray(x, dtype=np.complex128)
    K = x.shape[-1]
    out = np.empty_like(x)
    lib().orc_fft_forward(_p(x), _p(out), K, x.size // K)
    return out


def fpfb(htr: np.ndarray, ninputs: int, nspectra: int, h: np.ndarray, K: int, P_: int,
         i_idx: np.ndarray, flags: int) -> np.ndarray:
    """Whole forward PFB: uint8 [m][K][I] (int4 flags) or complex128 [m][K][I]."""
    h = np.ascontiguousarray(h, dtype=np.int32)
    i_idx = np.ascontiguousarray(i_idx, dtype=np.int32)
    if flags & PFB_COMPLEX_INT4:
        out = np.empty((nspectra, K, ninputs), dtype=np.uint8)
    else:
        out = np.empty((nspectra, K, ninputs), dtype=np.complex128)
    lib().orc_fpfb(_p(htr), ninputs, nspectra, _p(h), K, P_, _p(i_idx), flags, _p(out))
    return out


def unpack_int4(b: np.ndarray) -> np.ndarray:
    b = np.ascontiguousarray(b, dtype=np.uint8)
    out = np.empty(b.shape, dtype=np.complex128)
    lib().orc_unpack_int4(_p(b), b.size, _p(out))
    return out


# --------------------------------------------------------------------------
# beamformer
# --------------------------------------------------------------------------

def beamform(v: np.ndarray, J: np.ndarray, phi: np.ndarray, polQ: np.ndarray,
             polP: np.ndarray, invw: float, nstokes: int = 4, want_e: bool = True):
    """v: uint8 [s][c][2A] (int4) or complex128 [s][c][2A].
    J: complex128 [p][A][c][2][2]; phi: complex128 [p][A][c].
    Returns S float32 [p][s][nstokes][c] and e complex128 [p][s][c][2]."""
    datatype = 0 if v.dtype == np.uint8 else 1
    v = np.ascontiguousarray(v)
    ns, nc, ni = v.shape
    npnt, nant = J.shape[0], J.shape[1]
    J = np.ascontiguousarray(J, dtype=np.complex128)
    phi = np.ascontiguousarray(phi, dtype=np.complex128)
    polQ = np.ascontiguousarray(polQ, dtype=np.uint32)
    polP = np.ascontiguousarray(polP, dtype=np.uint32)
    S = np.empty((npnt, ns, nstokes, nc), dtype=np.float32)
    e = np.empty((npnt, ns, nc, 2), dtype=np.complex128) if want_e else None
    lib().orc_beamform(_p(v), datatype, ns, nc, nant, _p(J), _p(phi), _p(polQ), _p(polP),
                       npnt, float(invw), nstokes, _p(S), _p(e) if want_e else None)
    return S, e


def renormalise(S: np.ndarray):
    """S float32 [p][nstep][nstokes][nchan] -> (offsets, scales, u8)."""
    S = np.ascontiguousarray(S, dtype=np.float32)
    npnt, nstep, nst, nc = S.shape
    off = np.empty((npnt, nst, nc), dtype=np.float32)
    sc = np.empty((npnt, nst, nc), dtype=np.float32)
    out = np.empty(S.shape, dtype=np.uint8)
    lib().orc_renormalise(_p(S), npnt, nstep, nst, nc, _p(off), _p(sc), _p(out))
    return off, sc, out


def sat_u8(x: float) -> int:
    return int(lib().orc_sat_u8(float(x)))


def incoh_beam(data: np.ndarray) -> np.ndarray:
    """data uint8 [s][c][i] -> float32 [s][c]."""
    data = np.ascontiguousarray(data, dtype=np.uint8)
    ns, nc, ni = data.shape
    out = np.empty((ns, nc), dtype=np.float32)
    lib().orc_incoh_beam(_p(data), ns, nc, ni, _p(out))
    return out


# --------------------------------------------------------------------------
# inverse PFB and VDIF
# --------------------------------------------------------------------------

def ipfb(x: np.ndarray, coeffs: np.ndarray, ntaps: int, reference_taps: bool = False):
    """x complex [(nsamples+ntaps)][nchan][npol] -> complex128 [nsamples*nchan][npol]."""
    x = np.ascontiguousarray(x, dtype=np.complex128)
    nrow, nchan, npol = x.shape
    nsamples = nrow - ntaps
    f = np.ascontiguousarray(coeffs, dtype=np.float64)
    out = np.empty((nsamples * nchan, npol), dtype=np.complex128)
    lib().orc_ipfb(_p(x), nsamples, nchan, npol, _p(f), ntaps, int(reference_taps), _p(out))
    return out


def ipfb_table(coeffs: np.ndarray, nchan: int):
    c = np.ascontiguousarray(coeffs, dtype=np.float64)
    ftr = np.empty(c.size * nchan, dtype=np.float32)
    fti = np.empty(c.size * nchan, dtype=np.float32)
    lib().orc_ipfb_table(_p(c), c.size, nchan, _p(ftr), _p(fti))
    return ftr, fti


def vdif_quantise(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float32)
    out = np.empty(x.shape, dtype=np.uint8)
    lib().orc_vdif_quantise(_p(x), x.size, _p(out))
    return out


# --------------------------------------------------------------------------
# tables
# --------------------------------------------------------------------------

def calc_j(D: np.ndarray, B: np.ndarray) -> np.ndarray:
    """D complex [A][c][2][2], B complex [p][A][2][2] -> J complex [p][A][c][2][2]."""
    D = np.ascontiguousarray(D, dtype=np.complex128)
    B = np.ascontiguousarray(B, dtype=np.complex128)
    npnt, nant = B.shape[0], B.shape[1]
    nchan = D.shape[1]
    J = np.empty((npnt, nant, nchan, 2, 2), dtype=np.complex128)
    lib().orc_calc_j(npnt, nant, nchan, _p(D), _p(B), _p(J))
    return J


def calc_phi(unit: np.ndarray, east, north, height, cable, chan_freqs_hz) -> np.ndarray:
    unit = np.ascontiguousarray(unit, dtype=np.float64).reshape(-1, 3)
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (east, north, height, cable)]
    f = np.ascontiguousarray(chan_freqs_hz, dtype=np.float64)
    npnt, nant, nchan = unit.shape[0], arrs[0].size, f.size
    phi = np.empty((npnt, nant, nchan), dtype=np.complex128)
    lib().orc_calc_phi(npnt, nant, nchan, _p(unit), *[_p(a) for a in arrs], _p(f), _p(phi))
    return phi


def roots_of_unity(N: int) -> np.ndarray:
    out = np.empty(N, dtype=np.complex128)
    lib().orc_roots_of_unity(N, _p(out))
    return out


def mult2x2d(M1, M2):
    a = np.ascontiguousarray(M1, dtype=np.complex128).reshape(4)
    b = np.ascontiguousarray(M2, dtype=np.complex128).reshape(4)
    o = np.empty(4, dtype=np.complex128)
    lib().orc_mult2x2d(_p(a), _p(b), _p(o))
    return o


def norm2x2(M):
    a = np.ascontiguousarray(M, dtype=np.complex128).reshape(4)
    o = np.empty(4, dtype=np.complex128)
    nrm = lib().orc_norm2x2(_p(a), _p(o))
    return nrm, o


def inv2x2S(M):
    a = np.ascontiguousarray(M, dtype=np.complex128).reshape(4)
    o = np.empty(4, dtype=np.complex128)
    lib().orc_inv2x2S(_p(a), _p(o))
    return o


# --------------------------------------------------------------------------
# FP32 transcription (CPU baseline)
# --------------------------------------------------------------------------

def pfb_beam32(htr, ninputs, m_begin, m_end, h, K, P_, emulate_fpga, W, invw):
    h = np.ascontiguousarray(h, dtype=np.int32)
    W = np.ascontiguousarray(W, dtype=np.complex64)
    n = m_end - m_begin
    S = np.empty((n, 4, K), dtype=np.float32)
    e = np.empty((n, K, 2), dtype=np.complex64)
    inc = np.empty((n, K), dtype=np.float32)
    nt = lib().orc32_pfb_beam(_p(htr), ninputs, m_begin, m_end, _p(h), K, P_,
                              int(emulate_fpga), _p(W), float(invw), _p(S), _p(e), _p(inc))
    return S, e, inc, nt


def ipfb_vdif32(x, ft_real, ft_imag, ntaps, n_begin, n_end):
    x = np.ascontiguousarray(x, dtype=np.complex64)
    nrow, nchan, npol = x.shape
    out = np.empty(((n_end - n_begin), npol, 2), dtype=np.uint8)
    nt = lib().orc32_ipfb_vdif(_p(x), nrow - ntaps, nchan, npol, _p(ft_real), _p(ft_imag),
                               ntaps, n_begin, n_end, _p(out))
    return out, nt


def renormalise32(S):
    S = np.ascontiguousarray(S, dtype=np.float32)
    nstep, nst, nc = S.shape
    off = np.empty((nst, nc), dtype=np.float32)
    sc = np.empty((nst, nc), dtype=np.float32)
    out = np.empty(S.shape, dtype=np.uint8)
    nt = lib().orc32_renormalise(_p(S), nstep, nst, nc, _p(off), _p(sc), _p(out))
    return off, sc, out, nt


def max_threads() -> int:
    return int(lib().orc32_max_threads())
