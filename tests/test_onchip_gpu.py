"""GPU tests of the on-chip repeat harness (the reference's timing mode):
one repeat equals the batched entry point bit for bit, two repeats equal two
transforms, and the timing difference is positive and finite."""
import numpy as np
import pytest

from fft_onchip_gb300 import inputs

pytestmark = pytest.mark.gpu

SIZES = (8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096)


def bits(t):
    import torch
    return torch.view_as_real(t).view(torch.int64)


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("engine", ["auto", "f64"])
def test_one_and_two_repeats_match_the_batched_path(cuda, fftoc_lib, n, engine):
    import fft_onchip_gb300 as F
    from fft_onchip_gb300 import onchip
    eng = F.ENGINES[engine]
    tpb, var = onchip.onchip_plan(n, eng)
    blocks = 5
    x = cuda.from_numpy(inputs.normal(n, blocks * tpb, seed=n)).cuda()
    sel = F.plan_query(n, eng)["variant"]
    try:
        F.plan_select(n, eng if eng else F.auto_engine(n), var)
        ref1 = F.fft(x, engine=engine)
        ref2 = F.fft(ref1.clone(), engine=engine)
    finally:
        F.plan_select(n, eng if eng else F.auto_engine(n), sel)
    d1 = x.clone()
    onchip.run(n, d1, blocks, 1, eng)
    d2 = x.clone()
    onchip.run(n, d2, blocks, 2, eng)
    cuda.cuda.synchronize()
    assert cuda.equal(bits(d1), bits(ref1))
    assert cuda.equal(bits(d2), bits(ref2))


def test_timing_mode(cuda, fftoc_lib):
    from fft_onchip_gb300 import onchip
    r = onchip.time_onchip(64)
    assert r["us_per_pass"] > 0 and np.isfinite(r["ffts_per_s"])
    assert r["blocks"] * r["transforms_per_block"] <= 32 * 152 * 2
    with pytest.raises(Exception):
        onchip.onchip_plan(64, 4)  # split engine: not covered by the harness
