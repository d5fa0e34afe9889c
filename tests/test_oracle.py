"""CPU tests of the oracle: pinned to the golden vectors, to the naive DFT and
to numpy.fft; the restatements of the reference executors are checked to
compute the forward DFT of the reference's convention."""
import os

import numpy as np
import pytest

from fft_onchip_gb300 import inputs
from oracle import oracle as O

SIZES = O.SIZES
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def gold(n):
    d = np.load(os.path.join(GOLD, "kat_%d.npz" % n))
    return list(d["names"]), d["x"], d["y"]


def err(a, b):
    return O.rel_l2(a, b)


@pytest.mark.parametrize("n", SIZES)
def test_fft_ld_matches_golden(n):
    names, x, y = gold(n)
    got = O.fft_ld(x)
    for i, name in enumerate(names):
        scale = max(np.linalg.norm(y[i]), 1.0)
        assert np.linalg.norm(got[i] - y[i]) / scale < 1e-15, (n, name)


@pytest.mark.parametrize("n", SIZES)
def test_fft_f64_matches_golden(n):
    names, x, y = gold(n)
    got = O.fft_f64(x)
    for i, name in enumerate(names):
        scale = max(np.linalg.norm(y[i]), 1.0)
        assert np.linalg.norm(got[i] - y[i]) / scale < 1e-15, (n, name)


@pytest.mark.parametrize("n", [n for n in SIZES if n <= 512])
def test_naive_dft_matches_golden(n):
    names, x, y = gold(n)
    got = O.dft_naive(x)
    for i, name in enumerate(names):
        scale = max(np.linalg.norm(y[i]), 1.0)
        assert np.linalg.norm(got[i] - y[i]) / scale < 1e-15, (n, name)


@pytest.mark.parametrize("n", SIZES)
def test_oracle_vs_numpy(n):
    x = inputs.normal(n, 8, seed=n)
    assert err(O.fft_ld(x), np.fft.fft(x, axis=1)) < 1e-15
    assert err(O.fft_f64(x), O.fft_ld(x)) < 1e-15


@pytest.mark.parametrize("n", [8, 64, 256, 1024])
def test_naive_vs_fast(n):
    x = inputs.uniform(n, 3, seed=5)
    assert err(O.dft_naive(x), O.fft_ld(x)) < 1e-16


def test_linearity_and_parseval():
    n = 256
    x = inputs.normal(n, 4, seed=1)
    y = inputs.uniform(n, 4, seed=2)
    a, b = 0.75 - 0.5j, -1.25 + 2j
    lhs = O.fft_ld(a * x + b * y)
    rhs = a * O.fft_ld(x) + b * O.fft_ld(y)
    assert err(lhs, rhs) < 1e-15
    X = O.fft_ld(x)
    np.testing.assert_allclose(np.sum(np.abs(X) ** 2, axis=1), n * np.sum(np.abs(x) ** 2, axis=1), rtol=1e-14)


def test_cpu_baseline_thread_count_invariant():
    x = inputs.normal(128, 64, seed=3)
    a = O.fft_f64(x, threads=1)
    b = O.fft_f64(x, threads=0)
    assert np.array_equal(a, b)


# --- restatements of the reference executors --------------------------------

@pytest.mark.parametrize("n", [8, 64, 128, 256, 512])
def test_reference_tensor_executors_compute_the_dft(n):
    """tensor_fft_{8,64,128,256,512} (lane-exact, exact twiddles) == DFT."""
    x = inputs.normal(n, 16, seed=11)
    assert err(O.ref_tensor(x, exact=True), O.fft_ld(x)) < 1e-15


@pytest.mark.parametrize("n,lo,hi", [(8, 1e-10, 1e-7), (64, 1e-9, 1e-7), (128, 1e-9, 1e-7),
                                     (256, 1e-8, 2e-6), (512, 1e-9, 1e-7)])
def test_reference_tensor_executors_own_twiddle_error(n, lo, hi):
    """With the reference's own twiddles (FP32 sincospif; 6-digit table for
    N=256) the executors are accurate only to ~1e-8..1e-6 (rel-L2)."""
    x = inputs.normal(n, 16, seed=12)
    e = err(O.ref_tensor(x, exact=False), O.fft_ld(x))
    assert lo < e < hi, e


def test_reference_tensor_4096_fragment_mismatch():
    """tensor_fft_4096 splits K of its A fragments as {0..3},{4..7}
    (includes/tensor_fft_4096.cuh:31-32) while c64_fft64 reuses the C fragment
    as the next B fragment with an even/odd K split; the lane-exact
    restatement shows the output is not the DFT (the reference never runs this
    executor: scripts/generate_bench.py:103-106 filters it out)."""
    x = inputs.normal(4096, 2, seed=13)
    assert err(O.ref_tensor(x, exact=True), O.fft_ld(x)) > 0.5


@pytest.mark.parametrize("n", [8, 64, 512, 4096])
def test_reference_legacy8(n):
    x = inputs.normal(n, 4, seed=14)
    ref = O.fft_ld(x)
    assert err(O.ref_legacy8(x, exact=True), ref) < 1e-15
    assert err(O.ref_legacy8(x, exact=False), ref) < 1e-11  # 12-digit sqrt(1/2)


@pytest.mark.parametrize("n", [16, 256, 4096])
def test_reference_legacy16(n):
    x = inputs.normal(n, 4, seed=15)
    ref = O.fft_ld(x)
    assert err(O.ref_legacy16(x, exact=True), ref) < 1e-15
    assert err(O.ref_legacy16(x, exact=False), ref) < 1e-11  # 12-digit constants


def test_twiddle_octants():
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    for n in (8, 12, 64, 4096):
        for k in range(0, 3 * n, max(1, n // 16)):
            w = O.twiddle(n, k)
            a = -2 * mp.pi * (k % n) / n
            # within half an ulp of 1 per part (exact symmetries give exact 0, +-1)
            assert abs(w.real - mp.cos(a)) <= 2.0 ** -54 and abs(w.imag - mp.sin(a)) <= 2.0 ** -54, (n, k)
