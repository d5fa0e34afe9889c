"""GPU tests of fftoc_c2c_fwd_host: host buffers in and out, chunked through
the device (64 MiB chunks on three streams)."""
import numpy as np
import pytest

from fft_onchip_gb300 import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL = 1e-13


@pytest.mark.parametrize("n", [8, 64, 512, 4096])
def test_host_path_pinned_multi_chunk(cuda, fftoc_lib, n):
    import fft_onchip_gb300 as F
    torch = cuda
    batch = (3 * (64 << 20)) // (16 * n) + 7          # three full chunks and a ragged tail
    x = torch.from_numpy(inputs.normal(n, batch, seed=n)).pin_memory()
    out = torch.empty_like(x).pin_memory()
    F.fft_host(x, out=out)
    idx = np.r_[0:8, batch // 2:batch // 2 + 8, batch - 8:batch]
    ref = O.fft_f64(x.numpy()[idx])
    assert O.rel_l2(out.numpy()[idx], ref) < TOL
    # every transform written (energy check over the whole batch)
    xa, ya = x.numpy(), out.numpy()
    e_in = np.sum(np.abs(xa) ** 2, axis=1)
    e_out = np.sum(np.abs(ya) ** 2, axis=1) / n
    assert np.max(np.abs(e_out - e_in) / e_in) < 1e-12


def test_host_path_pageable_and_inplace(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    n, batch = 256, 1000
    x = inputs.uniform(n, batch, seed=4)
    ref = O.fft_f64(x)
    got = F.fft_host(x)                                   # pageable numpy buffers
    assert O.rel_l2(got, ref) < TOL
    buf = cuda.from_numpy(x.copy()).pin_memory()
    F.fft_host(buf, out=buf)                              # in place, pinned
    assert O.rel_l2(buf.numpy(), ref) < TOL


def test_host_path_engines_and_stream_order(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    torch = cuda
    n, batch = 64, 5000
    x = inputs.normal(n, batch, seed=6)
    ref = O.fft_f64(x)
    for engine in ("f64", "fx"):
        assert O.rel_l2(F.fft_host(x, engine=engine), ref) < TOL, engine
    # the call is ordered after earlier work on the caller's stream
    s = torch.cuda.Stream()
    h = torch.from_numpy(x.copy()).pin_memory()
    o = torch.empty_like(h).pin_memory()
    with torch.cuda.stream(s):
        torch.cuda._sleep(1000000)
        F.fft_host_ptr(n, h.data_ptr(), o.data_ptr(), batch, s.cuda_stream)
    s.synchronize()
    assert O.rel_l2(o.numpy(), ref) < TOL


def test_host_path_argument_errors(cuda, fftoc_lib):
    L = fftoc_lib
    assert L.fftoc_c2c_fwd_host(48, 16, 16, 4, 0, None) == 1
    assert L.fftoc_c2c_fwd_host(64, 16, 16, -1, 0, None) == 2
    assert L.fftoc_c2c_fwd_host(64, None, 16, 4, 0, None) == 2
    assert L.fftoc_c2c_fwd_host(64, 24, 24, 4, 0, None) == 3
    assert L.fftoc_c2c_fwd_host(64, 16, 16, 0, 0, None) == 0
