"""GPU tests of the serving loop (fftoc_server_*): every request's result
matches the oracle, a request's result is bit-identical alone and inside a
mix of concurrent requests (and equal to the per-size entry point), pool
admission bounds the bytes on the device, and bad requests are refused."""
import numpy as np
import pytest

from fft_onchip_gb300 import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 1e-13


def pinned(torch, a):
    t = torch.empty(a.shape, dtype=torch.complex128, pin_memory=True)
    t.copy_(torch.from_numpy(np.ascontiguousarray(a)))
    return t


def bits(a):
    return np.ascontiguousarray(a).view(np.uint64)


def test_alone_equals_in_mix_and_matches_oracle(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    from fft_onchip_gb300.serve import Server
    # one stream slot: requests that arrive while a batch runs queue up and
    # leave together in the next batch
    srv = Server(pool_bytes=1 << 30, slots=1, max_batch_bytes=64 << 20, max_wait_us=200.0)
    target = inputs.normal(256, 37, seed=77)
    alone = srv.submit(pinned(cuda, target))
    srv.wait(alone)
    y_alone = alone.out.numpy().copy()
    assert O.rel_l2(y_alone, O.fft_f64(target)) < TOL
    # the same request inside a stream of mixed requests, submitted back to
    # back behind a large one that keeps the slot busy
    rng = np.random.default_rng(1)
    xs = [inputs.normal(4096, 2048, seed=999)]
    for i in range(60):
        if i == 31:
            xs.append(target)
        else:
            n = int(rng.choice(inputs.SIZES))
            xs.append(inputs.normal(n, int(rng.integers(1, 300)), seed=1000 + i))
    hs = [pinned(cuda, x) for x in xs]
    reqs = [srv.submit(h) for h in hs]
    for r in reqs:
        srv.wait(r)
    st = srv.stats()
    assert st["requests_done"] == 62 and st["pool_bytes_in_use"] == 0 and st["pending"] == 0
    assert st["batches"] < 40  # requests were batched together
    y_mix = reqs[32].out.numpy()
    assert np.array_equal(bits(y_mix), bits(y_alone))
    # the batched entry point on the plan the serving loop's uneven graphs use
    eng = F.auto_engine(256)
    q = F.plan_query(256, eng)
    try:
        F.plan_select(256, eng, q["uneven_variant"])
        ref = F.fft(cuda.from_numpy(target).cuda()).cpu().numpy()
    finally:
        F.plan_select(256, eng, q["variant"])
    assert np.array_equal(bits(y_mix), bits(ref))
    for x, r in zip(xs, reqs):
        assert O.rel_l2(r.out.numpy(), O.fft_f64(x)) < TOL
    srv.close()


def test_pool_admission_bounds_device_bytes(cuda, fftoc_lib):
    from fft_onchip_gb300.serve import Server
    # pool of 3 MiB: two 1.5 MiB requests fit, a third waits for memory
    srv = Server(pool_bytes=3 << 20, slots=4, max_batch_bytes=1 << 20, max_wait_us=0.0)
    xs = [inputs.uniform(512, 192, seed=s) for s in range(8)]  # 1.5 MiB each
    reqs = [srv.submit(pinned(cuda, x)) for x in xs]
    for x, r in zip(xs, reqs):
        srv.wait(r)
        assert O.rel_l2(r.out.numpy(), O.fft_f64(x)) < TOL
    st = srv.stats()
    assert st["requests_done"] == 8 and st["max_inflight_batches"] <= 2
    srv.close()


def test_refused_requests(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    from fft_onchip_gb300.serve import Server
    srv = Server(pool_bytes=1 << 20, slots=1, max_batch_bytes=1 << 20)
    with pytest.raises(F.FftocError) as e:
        srv.submit(pinned(cuda, inputs.uniform(4096, 32, seed=1)))  # 2 MiB > pool
    assert e.value.status_name == "FFTOC_ERR_INVALID_VALUE"
    with pytest.raises(F.FftocError) as e:
        srv.submit(pinned(cuda, inputs.uniform(100, 2, seed=1)))
    assert e.value.status_name == "FFTOC_ERR_INVALID_SIZE"
    with pytest.raises(F.FftocError):
        Server(pool_bytes=1 << 20, slots=0)
    srv.close()


def test_poll_and_close_with_work_queued(cuda, fftoc_lib):
    from fft_onchip_gb300.serve import Server
    srv = Server(pool_bytes=64 << 20, slots=2, max_batch_bytes=8 << 20)
    x = inputs.normal(1024, 100, seed=5)
    r = srv.submit(pinned(cuda, x))
    import time
    t0 = time.time()
    while not srv.poll(r):
        assert time.time() - t0 < 60
        time.sleep(0.001)
    assert O.rel_l2(r.out.numpy(), O.fft_f64(x)) < TOL
    for s in range(20):
        srv.submit(pinned(cuda, inputs.normal(2048, 50, seed=s)))
    srv.close()  # finishes batches in flight, fails the rest, returns


def test_replay_reports_latencies(cuda, fftoc_lib):
    from fft_onchip_gb300.serve import Server, latency_summary, make_trace
    srv = Server(pool_bytes=1 << 30, slots=4)
    arena = 1 << 24  # 256 MiB of complex values
    h_in = cuda.empty(arena, dtype=cuda.complex128, pin_memory=True)
    h_in.copy_(cuda.from_numpy(inputs.uniform_flat(arena, seed=2)))
    h_out = cuda.empty(arena, dtype=cuda.complex128, pin_memory=True)
    items, transforms, nbytes = make_trace(2e4, 200, arena, seed=3)
    lat, wall = srv.replay(items, h_in, h_out)
    assert len(lat) == 200 and np.all(lat > 0) and wall > 0
    s = latency_summary(lat)
    assert s["p99_ms"] >= s["p50_ms"] > 0
    st = srv.stats()
    assert st["requests_done"] == 200 and st["transforms_done"] == transforms
    srv.close()


def test_split_tagged_requests_in_the_mix(cuda, fftoc_lib):
    """Requests tagged with the split-precision form run on it (error of the
    form, not binary64), the others on the plain form, in one stream."""
    import fft_onchip_gb300 as F
    from fft_onchip_gb300.serve import Server
    srv = Server(pool_bytes=256 << 20, slots=2, max_batch_bytes=8 << 20)
    xs, reqs, engs = [], [], []
    for i in range(24):
        n = (16, 256, 4096)[i % 3]
        eng = "split_bf16x3" if i % 2 else "auto"
        x = inputs.normal(n, 7 + i, seed=300 + i)
        xs.append(x)
        engs.append(eng)
        reqs.append(srv.submit(pinned(cuda, x), engine=eng))
    for x, r, eng in zip(xs, reqs, engs):
        srv.wait(r)
        err = O.rel_l2(r.out.numpy(), O.fft_f64(x))
        if eng == "auto":
            assert err < TOL
        else:
            assert 1e-12 < err < 1e-6
            ref = F.fft(cuda.from_numpy(x).cuda(), engine=eng).cpu().numpy()
            assert np.array_equal(bits(r.out.numpy()), bits(ref))
    with pytest.raises(F.FftocError) as e:
        srv.submit(pinned(cuda, inputs.normal(8, 4, seed=1)), engine="split_bf16x3")
    assert e.value.status_name == "FFTOC_ERR_UNSUPPORTED"
    srv.close()
