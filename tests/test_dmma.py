"""FFTOC_ENGINE_DMMA: 8-point transforms as the Karatsuba complex product on
the FP64 tensor cores (fft_onchip_gb300/csrc/fft_dmma.cuh; the reference's
scheme, includes/tensor_utils.cuh:25-36 and tensor_fft_8.cuh:37-65, with an
exact DFT matrix).  CPU: the engine exists for n = 8 only, and its plan
description.  GPU: results meet the FP64 gate against the oracle for batch
tails, in place, special values and through the host-buffer entry point."""
import ctypes

import numpy as np
import pytest

from fft_onchip_gb300 import _lib, inputs

TOL = 1e-13


def test_dmma_engine_sizes(fftoc_lib):
    L = fftoc_lib
    buf = (ctypes.c_double * 64)()
    p = ctypes.addressof(buf)
    p += (-p) % 16
    for n in _lib.SIZES:
        if n == 8:
            continue
        assert L.fftoc_c2c_fwd_ex(n, p, p, 1, _lib.ENGINE_DMMA, None) == 7, n   # unsupported, nothing launched
    q = _lib.plan_query(8, _lib.ENGINE_DMMA)
    assert q["engine"] == _lib.ENGINE_DMMA and q["radix"][0] == 8 and q["variants"] == 1
    assert q["transforms_per_block"] * q["threads_per_transform"] == q["threads_per_block"]
    _lib.plan_select(8, _lib.ENGINE_DMMA, 0)
    assert _lib.plan_query(8, _lib.ENGINE_F64)["variant"] == 0      # no other engine's choice touched


@pytest.mark.gpu
@pytest.mark.parametrize("batch", [1, 7, 8, 9, 63, 1000003])
def test_dmma_matches_oracle(cuda, fftoc_lib, batch):
    import fft_onchip_gb300 as F
    from oracle import oracle as O
    x = inputs.normal(8, batch, seed=batch)
    d = cuda.from_numpy(x).cuda()
    y = F.fft(d, engine="dmma").cpu().numpy()
    k = np.r_[0:min(batch, 4096)]
    assert O.rel_l2(y[k], O.fft_f64(x[k])) < TOL
    if batch > 4096:
        assert O.rel_l2(y[-4096:], O.fft_f64(x[-4096:])) < TOL


@pytest.mark.gpu
def test_dmma_in_place_and_special_values(cuda, fftoc_lib):
    from oracle import oracle as O
    L = fftoc_lib
    x = inputs.uniform(8, 40, seed=2)
    x[3] = 0.0
    x[5, 2] = np.nan
    x[6] = 1e300 * np.exp(2j * np.pi * np.arange(8) / 8)
    x[7] = 1e-300
    d = cuda.from_numpy(x).cuda()
    s = cuda.cuda.current_stream().cuda_stream
    assert L.fftoc_c2c_fwd_ex(8, d.data_ptr(), d.data_ptr(), 40, _lib.ENGINE_DMMA, s) == 0
    y = d.cpu().numpy()
    assert np.all(y[3] == 0)
    assert np.all(np.isnan(y[5].real) | np.isnan(y[5].imag))
    ok = [i for i in range(40) if i != 5]
    ref = O.fft_f64(x[ok])
    for r, i in enumerate(ok):
        scale = 1e-300 if i == 6 else 1.0   # keep the norm's squares finite
        assert O.rel_l2(y[i:i + 1] * scale, ref[r:r + 1] * scale) < TOL, i


@pytest.mark.gpu
def test_dmma_host_buffers(cuda, fftoc_lib):
    from oracle import oracle as O
    L = fftoc_lib
    x = cuda.from_numpy(inputs.normal(8, 5000, seed=4)).pin_memory()
    y = cuda.empty_like(x).pin_memory()
    s = cuda.cuda.current_stream()
    assert L.fftoc_c2c_fwd_host(8, x.data_ptr(), y.data_ptr(), 5000, _lib.ENGINE_DMMA, s.cuda_stream) == 0
    s.synchronize()
    assert O.rel_l2(y.numpy(), O.fft_f64(x.numpy())) < TOL
