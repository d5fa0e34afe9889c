"""GPU test of failure detection without a GPU fault: a bounded device wait
that nothing completes gives up, raises the library's device error flag, and
the host reads FFTOC_ERR_TIMEOUT; the context stays usable (a transform after
it is correct) and the flag is cleared by the check."""
import time

import numpy as np
import pytest

from fft_onchip_gb300 import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_reports(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    L = F._lib.load()
    L.fftoc_device_error_check()  # clear
    t0 = time.time()
    F.check(L.fftoc_selftest_bounded_wait(2.0, 0))
    cuda.cuda.synchronize()
    assert time.time() - t0 < 30
    assert F._lib.STATUS_NAMES[L.fftoc_device_error_check()] == "FFTOC_ERR_TIMEOUT"
    assert L.fftoc_device_error_check() == 0  # cleared
    # the context is still usable
    x = inputs.normal(256, 16, seed=1)
    y = F.fft(cuda.from_numpy(x).cuda()).cpu().numpy()
    assert O.rel_l2(y, O.fft_f64(x)) < 1e-13
    with pytest.raises(F.FftocError):
        F.check(L.fftoc_selftest_bounded_wait(0.0, 0))
