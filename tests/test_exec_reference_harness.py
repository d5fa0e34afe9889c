"""The reference's own harness kernel, testing::fft_tester
(includes/testing.cuh:16-57), compiled unmodified and driven with this
library's executors under the reference's names (include/fftoc/compat.cuh),
launched with its host driver's geometry (oracle/harness_runner.py).  One
call equals the library's batched kernel of the same plan bit for bit, the
ordinary rows meet the 1e-13 gate against the oracle, and repeated calls
compose as the harness's repeat mode assumes.  Needs the harness cubin,
which is built where the reference checkout exists (oracle/build_ref.py)."""
import numpy as np
import pytest

from fft_onchip_gb300 import _lib, inputs
from oracle import harness_runner as HR

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def harness(cuda, fftoc_lib):
    if not HR.available():
        pytest.skip("reference harness cubin not built (needs the reference checkout at build time)")
    h = HR.Harness()
    h.bind(fftoc_lib)
    return h


def _bits(t):
    import torch
    return torch.view_as_real(t).view(torch.int64)


@pytest.mark.parametrize("key", HR.KEYS)
def test_reference_harness_equals_batched_kernel(cuda, harness, key):
    import fft_onchip_gb300 as F
    from oracle import oracle as O
    n = key[0]
    s = harness.shapes[key]
    blocks = max(2, -(-6 // s["tpb"]))
    x = inputs.normal(n, blocks * s["tpb"], seed=500 + n)
    x[0] = 0.0
    x[1, n // 2] = np.nan
    d = cuda.from_numpy(x).cuda()
    out = d.clone()
    harness.run(key, out.data_ptr(), blocks, repeats=1)
    eng = _lib.ENGINE_FX
    p = 16 if HR.RADICES[n][0] == 16 else 8
    cur = F.plan_query(n, eng)["variant"]
    match = [v for v in range(F.plan_query(n, eng)["variants"])
             if (lambda q: q["points_per_thread"] == p and [r for r in q["radix"] if r > 1] == HR.RADICES[n])(
                 F.plan_query(n, eng, variant=v))]
    assert match
    try:
        F.plan_select(n, eng, match[0])
        ref = F.fft(d, engine="fx")
    finally:
        F.plan_select(n, eng, cur)
    cuda.cuda.synchronize()
    assert cuda.equal(_bits(out), _bits(ref))
    assert O.rel_l2(out.cpu().numpy()[2:], O.fft_f64(x[2:])) < 1e-13


@pytest.mark.parametrize("key", [(8, 1), (64, 2), (512, 2), (4096, 1)])
def test_reference_harness_repeats_compose(cuda, harness, key):
    s = harness.shapes[key]
    blocks = 2
    d = cuda.from_numpy(inputs.uniform(key[0], blocks * s["tpb"], seed=3)).cuda()
    once, twice = d.clone(), d.clone()
    harness.run(key, once.data_ptr(), blocks, repeats=1)
    harness.run(key, once.data_ptr(), blocks, repeats=1)
    harness.run(key, twice.data_ptr(), blocks, repeats=2)
    cuda.cuda.synchronize()
    assert cuda.equal(_bits(once), _bits(twice))
