"""GPU tests of uneven batches (mixed sizes in one buffer, int64 offset table,
one CUDA graph): parity with the oracle, bit-identity with the per-size
batched entry points on the same plans, the per-size comparison path, and
the edge cases (empty, gaps, shuffled order, in place, bad entries, plan
changes, plan growth)."""
from contextlib import contextmanager

import numpy as np
import pytest

from fft_onchip_gb300 import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-13
SIZES = inputs.SIZES


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@contextmanager
def uneven_plans(F, engine="auto"):
    """Select, for every size, the plan the uneven path uses (plan_query's
    uneven_variant), so that the batched entry point runs the same
    arithmetic; restore the choices afterwards."""
    saved = []
    for n in SIZES:
        e = F.ENGINES[engine] or F.auto_engine(n)
        q = F.plan_query(n, e)
        saved.append((n, e, q["variant"]))
        F.plan_select(n, e, q["uneven_variant"])
    try:
        yield
    finally:
        for n, e, v in saved:
            F.plan_select(n, e, v)


def batched_reference(torch, F, xf, off, ns, engine="auto"):
    """Each size's transforms gathered into a contiguous batch, run through
    the per-size entry point on the uneven path's plans, scattered back (host
    side)."""
    out = np.zeros_like(xf)
    with uneven_plans(F, engine):
        for n in np.unique(ns):
            idx = np.nonzero(ns == n)[0]
            rows = np.stack([xf[off[i]:off[i] + n] for i in idx])
            y = F.fft(dev(torch, rows), engine=engine).cpu().numpy()
            for k, i in enumerate(idx):
                out[off[i]:off[i] + n] = y[k]
    return out


def oracle_err(xf, yf, off, ns):
    worst = 0.0
    for n in np.unique(ns):
        idx = np.nonzero(ns == n)[0]
        rows = np.stack([xf[off[i]:off[i] + n] for i in idx])
        got = np.stack([yf[off[i]:off[i] + n] for i in idx])
        worst = max(worst, O.rel_l2(got, O.fft_f64(rows)))
    return worst


def bits(t):
    import torch
    return torch.view_as_real(t).view(torch.int64)


def workload(count, seed=3):
    ns = inputs.uneven_sizes(count, seed=seed)
    off, total = inputs.uneven_layout(ns)
    return inputs.uniform_flat(total, seed=seed), off, ns


@pytest.mark.parametrize("engine", ["auto", "f64"])
def test_mixed_batch_matches_oracle_and_per_size_path(cuda, fftoc_lib, engine):
    import fft_onchip_gb300 as F
    xf, off, ns = workload(3000)
    plan = F.UnevenPlan(4096, engine=engine)
    y = plan(dev(cuda, xf), dev(cuda, off), dev(cuda, ns)).cpu().numpy()
    assert oracle_err(xf, y, off, ns) < TOL
    ref = batched_reference(cuda, F, xf, off, ns, engine)
    assert np.array_equal(y.view(np.uint64), ref.view(np.uint64))
    counts = plan.counts()
    for n in SIZES:
        assert counts[n] == int(np.sum(ns == n))
    y2 = plan(dev(cuda, xf), dev(cuda, off), dev(cuda, ns), per_size=True).cpu().numpy()
    assert np.array_equal(y2.view(np.uint64), y.view(np.uint64))
    # the graph sizes its per-size kernels on the device (one CTA per tile)
    assert plan.device_sized()
    plan.close()
    assert F._lib.load().fftoc_device_error_check() == 0


def test_device_sized_grids_follow_each_batch(cuda, fftoc_lib):
    """Back-to-back executions of one plan on batches of different size mixes
    (so different per-size grids, set on the device by each launch), queued
    on one stream without synchronising: each output equals the per-size
    path's on the same batch."""
    import fft_onchip_gb300 as F
    plan = F.UnevenPlan(6000)
    assert plan.device_sized()
    batches = []
    for count, seed in ((6000, 31), (40, 32), (2500, 33), (1, 34)):
        xf, off, ns = workload(count, seed=seed)
        if count == 1:
            ns[:] = 4096
            off, total = inputs.uneven_layout(ns)
            xf = inputs.uniform_flat(total, seed=seed)
        batches.append((dev(cuda, xf), dev(cuda, off), dev(cuda, ns)))
    outs = [plan(x, o, n) for (x, o, n) in batches]  # no synchronisation in between
    cuda.cuda.synchronize()
    for (x, o, n), y in zip(batches, outs):
        ref = plan(x, o, n, per_size=True)
        assert cuda.equal(bits(y), bits(ref))
    plan.close()
    assert F._lib.load().fftoc_device_error_check() == 0


def test_gaps_shuffled_order_and_in_place(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    rng = np.random.default_rng(5)
    ns = inputs.uneven_sizes(700, seed=9)
    gaps = rng.integers(0, 5, size=len(ns)) * 8
    off = np.zeros(len(ns), dtype=np.int64)
    pos = 0
    for i, n in enumerate(ns):
        pos += int(gaps[i])
        off[i] = pos
        pos += int(n)
    total = pos + 16
    xf = inputs.uniform_flat(total, seed=11)
    perm = rng.permutation(len(ns))
    off_p, ns_p = off[perm].copy(), ns[perm].copy()
    sentinel = np.full(total, 7.0 + 3.0j)
    d_out = dev(cuda, sentinel)
    plan = F.UnevenPlan(len(ns))
    y = plan(dev(cuda, xf), dev(cuda, off_p), dev(cuda, ns_p), out=d_out).cpu().numpy()
    covered = np.zeros(total, dtype=bool)
    for o, n in zip(off, ns):
        covered[o:o + n] = True
    assert np.all(y[~covered] == 7.0 + 3.0j)  # gaps untouched
    assert oracle_err(xf, y, off, ns) < TOL
    d = dev(cuda, xf)
    plan(d, dev(cuda, off_p), dev(cuda, ns_p), out=d)
    yi = d.cpu().numpy()
    assert np.array_equal(yi[covered].view(np.uint64), y[covered].view(np.uint64))


def test_single_size_and_single_transform(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    for n in (8, 512, 4096):
        for count in (1, 37):
            ns = np.full(count, n, dtype=np.int32)
            off, total = inputs.uneven_layout(ns)
            xf = inputs.uniform_flat(total, seed=n + count)
            y = F.fft_uneven(dev(cuda, xf), dev(cuda, off), dev(cuda, ns)).cpu().numpy()
            with uneven_plans(F):
                ref = F.fft(dev(cuda, xf.reshape(count, n))).cpu().numpy().reshape(-1)
            assert np.array_equal(y.view(np.uint64), ref.view(np.uint64)), (n, count)


def test_empty_and_capacity(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    plan = F.UnevenPlan(16)
    x = cuda.zeros(64, dtype=cuda.complex128, device="cuda")
    e = cuda.zeros(0, dtype=cuda.int64, device="cuda")
    n0 = cuda.zeros(0, dtype=cuda.int32, device="cuda")
    plan(x, e, n0)  # count 0: no-op
    ns = cuda.full((17,), 8, dtype=cuda.int32, device="cuda")
    off = cuda.arange(17, dtype=cuda.int64, device="cuda") * 8
    x = cuda.zeros(17 * 8, dtype=cuda.complex128, device="cuda")
    with pytest.raises(F.FftocError) as ei:
        plan(x, off, ns)
    assert ei.value.status_name == "FFTOC_ERR_INVALID_VALUE"
    with pytest.raises(F.FftocError):
        F.UnevenPlan(0)


def test_bad_entries_are_skipped_and_flagged(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    L = F._lib.load()
    L.fftoc_device_error_check()  # clear
    ns = np.array([64, 100, 8, -8, 16, 64], dtype=np.int32)
    off = np.array([0, 64, 164, 172, 180, -16], dtype=np.int64)
    total = 260
    xf = inputs.uniform_flat(total, seed=4)
    sentinel = np.full(total, 1.5 - 2.0j)
    d_out = dev(cuda, sentinel)
    plan = F.UnevenPlan(8)
    y = plan(dev(cuda, xf), dev(cuda, off), dev(cuda, ns), out=d_out).cpu().numpy()
    assert F._lib.STATUS_NAMES[L.fftoc_device_error_check()] == "FFTOC_ERR_INVALID_VALUE"
    # the valid entries (0: n=64 @0, 2: n=8 @164, 4: n=16 @180) are transformed
    good = [0, 2, 4]
    assert oracle_err(xf, y, off[good], ns[good]) < TOL
    # the skipped ones (n=100 @64, n=-8 @172, negative offset) are untouched
    assert np.all(y[64:164] == 1.5 - 2.0j)
    assert np.all(y[172:180] == 1.5 - 2.0j)
    counts = plan.counts()
    assert counts[64] == 1 and counts[8] == 1 and counts[16] == 1


def test_bad_entries_raise_the_device_flag(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    L = F._lib.load()
    L.fftoc_device_error_check()
    ns = cuda.tensor([64, 12], dtype=cuda.int32, device="cuda")
    off = cuda.tensor([0, 64], dtype=cuda.int64, device="cuda")
    x = cuda.zeros(128, dtype=cuda.complex128, device="cuda")
    F.UnevenPlan(2)(x, off, ns)
    cuda.cuda.synchronize()
    assert F._lib.STATUS_NAMES[L.fftoc_device_error_check()] == "FFTOC_ERR_INVALID_VALUE"
    assert L.fftoc_device_error_check() == 0  # cleared


def test_plan_change_recaptures(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    xf, off, ns = workload(1500, seed=21)
    plan = F.UnevenPlan(1500)
    cur = F.plan_query(64, F.ENGINE_FX)
    alt = next(v for v in range(cur["variants"])
               if v != cur["variant"] and not F.plan_query(64, F.ENGINE_FX, variant=v)["persistent"])
    try:
        F.plan_select(64, F.ENGINE_FX, alt)
        y = plan(dev(cuda, xf), dev(cuda, off), dev(cuda, ns)).cpu().numpy()
        ref = batched_reference(cuda, F, xf, off, ns)
    finally:
        F.plan_select(64, F.ENGINE_FX, cur["variant"])
    assert np.array_equal(y.view(np.uint64), ref.view(np.uint64))
    assert oracle_err(xf, y, off, ns) < TOL


def test_one_shot_grows(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    for count in (10, 5000):
        xf, off, ns = workload(count, seed=count)
        y = F.fft_uneven(dev(cuda, xf), dev(cuda, off), dev(cuda, ns)).cpu().numpy()
        assert oracle_err(xf, y, off, ns) < TOL


def test_full_size_mixed_batch_matches_per_size_path(cuda, fftoc_lib):
    """200,000 transforms, N in 8..4096 with P ~ 1/log2 N, uniform [-1, 1):
    bit-identical to the per-size batched launches, and a sample of
    transforms against the oracle."""
    import fft_onchip_gb300 as F
    xf, off, ns = workload(200000, seed=0)
    d_x, d_off, d_ns = dev(cuda, xf), dev(cuda, off), dev(cuda, ns)
    plan = F.UnevenPlan(200000)
    y = plan(d_x, d_off, d_ns)
    per = plan(d_x, d_off, d_ns, per_size=True)
    assert cuda.equal(bits(y), bits(per))
    yh = y.cpu().numpy()
    sample = np.arange(0, 200000, 997)
    assert oracle_err(xf, yh, off[sample], ns[sample]) < TOL
    # per-size batched launches on device copies of each size's transforms
    with uneven_plans(F):
        for n in SIZES:
            idx = np.nonzero(ns == n)[0]
            gather = (cuda.from_numpy(off[idx]).cuda()[:, None] + cuda.arange(n, device="cuda")[None, :]).reshape(-1)
            rows = d_x[gather].reshape(len(idx), n)
            ref = F.fft(rows)
            assert cuda.equal(bits(y[gather].reshape(len(idx), n)), bits(ref)), n
