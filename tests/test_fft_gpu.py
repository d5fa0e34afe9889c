"""GPU parity tests: the CUDA path through the C ABI against the CPU oracle
(and the golden vectors), for every size and engine of the FP64 form.

Bar: relative L2 error <= 1e-13 against the oracle (the FP64-form gate),
per transform as well as over the batch."""
import os

import numpy as np
import pytest

from fft_onchip_gb300 import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SIZES = (8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096)
ENGINES = ("f64", "fx", "auto")
TOL = 1e-13
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def run(torch, x, engine="auto", inplace=False):
    import fft_onchip_gb300 as F
    d = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    if inplace:
        F.fft(d, out=d, engine=engine)
        out = d
    else:
        out = F.fft(d, engine=engine)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def per_transform_err(a, b):
    # rows rescaled exactly (by a power of two) so that 1e300-sized or
    # subnormal values neither overflow nor underflow in the norm
    s = np.max(np.abs(b), axis=1, keepdims=True)
    s[s == 0] = 1.0
    k = -np.frexp(s)[1]

    def sc(z):
        return np.ldexp(z.real, k) + 1j * np.ldexp(z.imag, k)

    num = np.linalg.norm(sc(a) - sc(b), axis=1)
    den = np.maximum(np.linalg.norm(sc(b), axis=1), 1e-300)
    return num / den


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("engine", ENGINES)
def test_golden_vectors(cuda, fftoc_lib, n, engine):
    d = np.load(os.path.join(GOLD, "kat_%d.npz" % n))
    got = run(cuda, d["x"], engine)
    for i, name in enumerate(d["names"]):
        scale = max(np.linalg.norm(d["y"][i]), 1.0)
        assert np.linalg.norm(got[i] - d["y"][i]) / scale < TOL, (n, engine, name)


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("engine", ENGINES)
@pytest.mark.parametrize("family", ["uniform", "normal", "loguniform"])
def test_parity_random(cuda, fftoc_lib, n, engine, family):
    batch = max(3, 4096 // n) + 5  # not a multiple of any CTA tile
    x = inputs.FAMILIES[family](n, batch, seed=n + 17)
    ref = O.fft_f64(x)
    got = run(cuda, x, engine)
    assert np.all(np.isfinite(got))
    assert O.rel_l2(got, ref) < TOL
    assert per_transform_err(got, ref).max() < TOL


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("engine", ["f64", "fx"])
def test_every_compiled_plan(cuda, fftoc_lib, n, engine):
    """Each plan variant (the autotuner's candidates) is parity-checked."""
    import fft_onchip_gb300 as F
    eid = F.ENGINES[engine]
    cur = F.plan_query(n, eid)
    x = inputs.normal(n, max(3, 2048 // n) + 3, seed=n + 5)
    ref = O.fft_f64(x)
    try:
        for v in range(cur["variants"]):
            F.plan_select(n, eid, v)
            got = run(cuda, x, engine)
            assert per_transform_err(got, ref).max() < TOL, (n, engine, v)
            got = run(cuda, x, engine, inplace=True)
            assert per_transform_err(got, ref).max() < TOL, (n, engine, v, "inplace")
    finally:
        F.plan_select(n, eid, cur["variant"])


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("engine", ["f64", "fx"])
def test_code_forms_compute_the_same_bits(cuda, fftoc_lib, n, engine):
    """Variants that share points per thread and radices differ only in how
    the kernel is laid out (transforms per CTA, resident CTAs, L2 prefetch,
    persistence, code forms): they must give the same bits, including for
    transforms that take the rare input and output paths."""
    import fft_onchip_gb300 as F
    eid = F.ENGINES[engine]
    cur = F.plan_query(n, eid)
    x = inputs.normal(n, max(8, 4096 // n), seed=n + 11)
    x[1] = 1e300 * x[1]                                      # outputs overflow: slow output path
    x[2] = x[2] * 2.0 ** -1060                               # subnormal inputs: slow input path
    x[3, ::2] *= 2.0 ** 40                                   # spread beyond 2^31 within a transform
    x[4, n // 2] = np.inf                                    # non-finite: all-NaN transform
    groups = {}
    for v in range(cur["variants"]):
        p = F.plan_query(n, eid, variant=v)
        groups.setdefault((p["points_per_thread"], tuple(p["radix"])), []).append(v)
    try:
        for key, vs in groups.items():
            outs = []
            for v in vs:
                F.plan_select(n, eid, v)
                outs.append(run(cuda, x, engine))
            for v, o in zip(vs[1:], outs[1:]):
                assert np.array_equal(o.view(np.int64), outs[0].view(np.int64)), (n, engine, key, vs[0], v)
    finally:
        F.plan_select(n, eid, cur["variant"])


def test_autotune_selects_a_valid_plan(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    cur = F.plan_query(256, F.ENGINE_FX)
    try:
        v, ms = F.autotune(256, F.ENGINE_FX, 4096)
        assert 0 <= v < cur["variants"] and ms > 0
        assert F.plan_query(256, F.ENGINE_FX)["variant"] == v
        x = inputs.normal(256, 33, seed=1)
        assert O.rel_l2(run(cuda, x, "fx"), O.fft_f64(x)) < TOL
    finally:
        F.plan_select(256, F.ENGINE_FX, cur["variant"])


def test_config1_n64_batch65536_uniform_seed0(cuda, fftoc_lib):
    """Plain method, small: N=64, batch 65536, re/im uniform[-1,1) from seed 0."""
    x = inputs.uniform(64, 65536, seed=0)
    ref = O.fft_f64(x)
    for engine in ENGINES:
        got = run(cuda, x, engine)
        assert O.rel_l2(got, ref) < TOL, engine
        assert per_transform_err(got, ref).max() < TOL, engine
    # cuFFT (through torch.fft) on the same device as an independent check
    ref_dev = cuda.fft.fft(cuda.from_numpy(x).cuda(), dim=1).cpu().numpy()
    assert O.rel_l2(ref_dev, ref) < TOL


@pytest.mark.parametrize("n", [8, 64, 512, 4096])
def test_ground_truth_long_double(cuda, fftoc_lib, n):
    x = inputs.normal(n, 4, seed=99)
    ref = O.fft_ld(x)
    for engine in ("f64", "fx"):
        assert O.rel_l2(run(cuda, x, engine), ref) < 1e-14, engine


@pytest.mark.parametrize("n", [8, 32, 64, 256, 1024, 4096])
@pytest.mark.parametrize("batch", [1, 2, 31, 33, 257])
def test_batch_edges(cuda, fftoc_lib, n, batch):
    x = inputs.uniform(n, batch, seed=batch)
    ref = O.fft_f64(x)
    for engine in ("f64", "fx"):
        assert O.rel_l2(run(cuda, x, engine), ref) < TOL, engine


@pytest.mark.parametrize("n", SIZES)
def test_inplace_equals_out_of_place(cuda, fftoc_lib, n):
    x = inputs.normal(n, 37, seed=3)
    for engine in ("f64", "fx"):
        a = run(cuda, x, engine, inplace=False)
        b = run(cuda, x, engine, inplace=True)
        assert np.array_equal(a, b), engine


@pytest.mark.parametrize("n", [8, 16, 64, 512, 4096])
def test_guard_bands_and_full_coverage(cuda, fftoc_lib, n):
    """Output is written exactly: NaN-prefilled output becomes finite, canaries
    around the output stay untouched."""
    import fft_onchip_gb300 as F
    torch = cuda
    batch = 41
    x = torch.from_numpy(inputs.uniform(n, batch, seed=5)).cuda()
    guard = 64
    buf = torch.full((batch * n + 2 * guard,), complex(float("nan"), 12345.0), dtype=torch.complex128, device="cuda")
    out = buf[guard:guard + batch * n].view(batch, n)
    for engine in ("f64", "fx"):
        F.fft(x, out=out, engine=engine)
        torch.cuda.synchronize()
        h = buf.cpu().numpy()
        assert np.all(np.isfinite(h[guard:guard + batch * n])), engine
        assert np.all(np.isnan(h[:guard].real)) and np.all(h[:guard].imag == 12345.0)
        assert np.all(np.isnan(h[-guard:].real)) and np.all(h[-guard:].imag == 12345.0)


@pytest.mark.parametrize("n", [16, 64, 1024])
def test_special_scales(cuda, fftoc_lib, n):
    """Zero transforms, tiny and huge magnitudes, denormals, mixed scales."""
    base = inputs.normal(n, 6, seed=8)
    x = base.copy()
    x[0] = 0
    x[1] *= 1e-300
    x[2] *= 1e300
    x[3] = base[3] * 1e-310          # denormal range
    x[4, : n // 2] *= 1e-200         # huge dynamic range inside one transform
    x[5] *= 2.0 ** 900
    ref = O.fft_ld(x)
    for engine in ("f64", "fx"):
        got = run(cuda, x, engine)
        assert np.all(got[0] == 0), engine
        for i in (1, 2, 4, 5):
            assert per_transform_err(got[i:i + 1], ref[i:i + 1])[0] < TOL, (engine, i)
        # all-subnormal transform: binary64 arithmetic itself loses bits there
        e3 = per_transform_err(got[3:4], ref[3:4])[0]
        assert e3 < 1e-6, (engine, e3, got[3][:4], ref[3][:4])


def test_nonfinite_inputs(cuda, fftoc_lib):
    n = 64
    x = inputs.normal(n, 3, seed=9)
    x[1, 5] = np.nan
    x[2, 7] = np.inf
    got = run(cuda, x, "fx")
    assert np.all(np.isfinite(got[0]))
    assert np.all(np.isnan(got[1])) and np.all(np.isnan(got[2]))
    gotf = run(cuda, x, "f64")
    assert np.all(np.isfinite(gotf[0])) and not np.all(np.isfinite(gotf[1]))


def test_stream_ordering(cuda, fftoc_lib):
    """Launches follow the caller's stream."""
    import fft_onchip_gb300 as F
    torch = cuda
    n, batch = 256, 2048
    x = torch.from_numpy(inputs.normal(n, batch, seed=10)).cuda()
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        y = torch.empty_like(x)
        F.fft(x, out=y)
        z = F.fft(y)
    s.synchronize()
    ref = O.fft_f64(O.fft_f64(x.cpu().numpy()))
    assert O.rel_l2(z.cpu().numpy(), ref) < TOL


@pytest.mark.parametrize("n", SIZES)
def test_full_size_properties(cuda, fftoc_lib, n):
    """Sweep configuration (1 GiB of complex128 input per size): Parseval per
    transform and an oracle spot check of 64 transforms."""
    import fft_onchip_gb300 as F
    torch = cuda
    batch = (1 << 30) // (16 * n)
    g = torch.Generator(device="cuda").manual_seed(n)
    x = torch.randn(batch, n, dtype=torch.complex128, device="cuda", generator=g)
    y = F.fft(x)
    e_in = (x.abs() ** 2).sum(dim=1)
    e_out = (y.abs() ** 2).sum(dim=1) / n
    assert ((e_out - e_in).abs() / e_in).max().item() < 1e-13
    idx = torch.randint(0, batch, (64,), device="cuda", generator=g)
    xs = x[idx].cpu().numpy()
    assert O.rel_l2(y[idx].cpu().numpy(), O.fft_f64(xs)) < TOL
    del x, y
    torch.cuda.empty_cache()


@pytest.mark.parametrize("n", SIZES)
def test_matches_cufft(cuda, fftoc_lib, n):
    """Device-library cross-check: cuFFT's batched Z2Z forward transform
    (through torch.fft.fft), the stand-in for the reference's cuFFTDx path
    (includes/reference.cuh:9-24), which is not available here."""
    import fft_onchip_gb300 as F
    x = inputs.normal(n, max(4, (1 << 16) // n), seed=n + 5)
    d = cuda.from_numpy(x).cuda()
    ours = F.fft(d).cpu().numpy()
    cufft = cuda.fft.fft(d, dim=-1).cpu().numpy()
    ref = O.fft_f64(x)
    assert O.rel_l2(ours, cufft) < TOL
    assert O.rel_l2(cufft, ref) < TOL
