"""GPU test of fftoc_c2c_fwd_host_noalloc, the host-buffer transform that
allocates no device memory (for callers whose device memory belongs to
another allocator or a fixed pool, or that cannot take cudaMalloc's implicit
synchronisation).  Its output must match the allocating host-buffer entry
point, fftoc_c2c_fwd_host, on two calls in a row (the compiled-in staging
array is reused and keeps the previous call's contents), match the oracle on
a strided sample of rows, and leave the device error flags clear (read with
fftoc_device_error_check, which allocates nothing either).  Pinned and
pageable host buffers are both accepted.  Collected last so a failure here
cannot hide the rest of the suite; it also passes alone."""
import ctypes

import numpy as np
import pytest

from fft_onchip_gb300 import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-13
SCRATCH_BYTES = 32 << 20


def _call(L, fn, n, x, out, engine, stream):
    return getattr(L, fn)(n, x.data_ptr(), out.data_ptr(), x.shape[0], engine, stream)


@pytest.mark.parametrize("n,engine", [(64, 0), (512, 2), (4096, 0), (256, 1), (8, 0)])
def test_noalloc_matches_allocating_host_path(cuda, fftoc_lib, n, engine):
    torch = cuda
    L = fftoc_lib
    batch = min(SCRATCH_BYTES // (16 * n), 20000)
    s = torch.cuda.current_stream()
    for call in range(2):                     # two calls in a row on the shared array
        x = torch.from_numpy(inputs.normal(n, batch, seed=100 * n + call)).pin_memory()
        got = torch.empty_like(x).pin_memory()
        ref = torch.empty_like(x).pin_memory()
        assert _call(L, "fftoc_c2c_fwd_host_noalloc", n, x, got, engine, s.cuda_stream) == 0, \
            L.fftoc_last_error_string()
        assert _call(L, "fftoc_c2c_fwd_host", n, x, ref, engine, s.cuda_stream) == 0
        s.synchronize()
        assert L.fftoc_device_error_check() == 0, L.fftoc_last_error_string()
        assert O.rel_l2(got.numpy(), ref.numpy()) < TOL, (n, engine, call)
        k = np.r_[np.arange(0, batch, max(1, batch // 64)), batch - 1]
        assert O.rel_l2(got.numpy()[k], O.fft_f64(x.numpy()[k])) < TOL


def test_noalloc_pageable_buffers(cuda, fftoc_lib):
    torch = cuda
    L = fftoc_lib
    n, batch = 128, 3000
    s = torch.cuda.current_stream()
    x = torch.from_numpy(inputs.uniform(n, batch, seed=9))          # pageable host memory
    got = torch.full_like(x, float("nan"))
    assert _call(L, "fftoc_c2c_fwd_host_noalloc", n, x, got, 0, s.cuda_stream) == 0, L.fftoc_last_error_string()
    s.synchronize()
    assert L.fftoc_device_error_check() == 0
    assert O.rel_l2(got.numpy(), O.fft_f64(x.numpy())) < TOL


def test_noalloc_rejects_batches_beyond_its_scratch(cuda, fftoc_lib):
    L = fftoc_lib
    n = 1024
    limit = SCRATCH_BYTES // (16 * n)
    buf = (ctypes.c_double * 16)()            # never touched: rejected before any copy
    p = ctypes.addressof(buf)
    p += (-p) % 16
    assert L.fftoc_c2c_fwd_host_noalloc(n, p, p, limit + 1, 0, None) == 2
    msg = L.fftoc_last_error_string().decode()
    assert "32 MiB" in msg and str(limit) in msg
    assert L.fftoc_c2c_fwd_host_noalloc(48, p, p, 1, 0, None) == 1
    assert L.fftoc_c2c_fwd_host_noalloc(n, p, p, 0, 0, None) == 0
