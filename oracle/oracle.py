"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, to check results and time the CPU baseline.  The product library never
imports it.

Arrays are numpy complex128 of shape (batch, n) (interleaved re/im doubles,
transforms back to back), matching the layout of the reference harness
(includes/testing.cuh:29-34, thrust::complex<double> per includes/config.hpp:6).
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

SIZES = (8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096)


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        L.orc_dft_naive_ld.argtypes = [ctypes.c_int, ctypes.c_longlong, dp, dp]
        L.orc_fft_ld.argtypes = [ctypes.c_int, ctypes.c_longlong, dp, dp]
        L.orc_fft_f64.argtypes = [ctypes.c_int, ctypes.c_longlong, dp, dp, ctypes.c_int]
        for f in (L.orc_ref_tensor, L.orc_ref_legacy8, L.orc_ref_legacy16):
            f.argtypes = [ctypes.c_int, ctypes.c_longlong, dp, dp, ctypes.c_int]
            f.restype = ctypes.c_int
        L.orc_twiddle.argtypes = [ctypes.c_longlong, ctypes.c_longlong, dp, dp]
        L.orc_gen_uniform.argtypes = [ctypes.c_uint64, ctypes.c_longlong, dp]
        L.orc_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _prep(x):
    x = np.ascontiguousarray(x, dtype=np.complex128)
    if x.ndim == 1:
        x = x[None, :]
    return x


def _ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def dft_naive(x):
    """O(N^2) long-double DFT (forward, unnormalised)."""
    x = _prep(x)
    y = np.empty_like(x)
    lib().orc_dft_naive_ld(x.shape[1], x.shape[0], _ptr(x), _ptr(y))
    return y


def fft_ld(x):
    """Radix-2 long-double FFT: ground truth."""
    x = _prep(x)
    y = np.empty_like(x)
    lib().orc_fft_ld(x.shape[1], x.shape[0], _ptr(x), _ptr(y))
    return y


def fft_f64(x, threads=0):
    """FP64 radix-8/4/2 Stockham on `threads` host threads (0: all)."""
    x = _prep(x)
    y = np.empty_like(x)
    lib().orc_fft_f64(x.shape[1], x.shape[0], _ptr(x), _ptr(y), int(threads))
    return y


def ref_tensor(x, exact=True):
    """Lane-exact restatement of the reference's tensor_fft_N executor."""
    x = _prep(x)
    y = np.empty_like(x)
    rc = lib().orc_ref_tensor(x.shape[1], x.shape[0], _ptr(x), _ptr(y), 0 if exact else 1)
    if rc != 0:
        raise ValueError("no tensor_fft executor for n=%d" % x.shape[1])
    return y


def ref_legacy8(x, exact=True):
    x = _prep(x)
    y = np.empty_like(x)
    if lib().orc_ref_legacy8(x.shape[1], x.shape[0], _ptr(x), _ptr(y), 0 if exact else 1) != 0:
        raise ValueError("legacy8 needs n a power of 8")
    return y


def ref_legacy16(x, exact=True):
    x = _prep(x)
    y = np.empty_like(x)
    if lib().orc_ref_legacy16(x.shape[1], x.shape[0], _ptr(x), _ptr(y), 0 if exact else 1) != 0:
        raise ValueError("legacy16 needs n a power of 16")
    return y


def twiddle(n, k):
    re, im = ctypes.c_double(), ctypes.c_double()
    lib().orc_twiddle(n, k, ctypes.byref(re), ctypes.byref(im))
    return complex(re.value, im.value)


def gen_uniform(seed, count):
    out = np.empty(count, dtype=np.float64)
    lib().orc_gen_uniform(ctypes.c_uint64(seed), count, _ptr(out))
    return out


def max_threads():
    return lib().orc_max_threads()


def rel_l2(a, b):
    """||a - b||_2 / ||b||_2 over the whole array."""
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))
