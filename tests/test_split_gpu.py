"""GPU tests of the split-precision form (tcgen05 BF16x3 / TF32x2 GEMM
passes): accuracy against the binary64 oracle per size, input family and
split, the per-transform scaling of out-of-range magnitudes, batch edges,
in place, and refusal of unsupported sizes.

Tolerances (relative L2 error per batch, stated per split): BF16x3 carries
FP32 data between passes and accumulates six BF16 term products in FP32,
so its error is a few FP32 roundings per pass (measured 6e-7..9e-7); TF32x2
keeps two 11-bit terms (22 bits) per operand (measured 6e-7..1e-6); the
exact-slice form keeps 48-bit digits with products exact in FP32 and must
meet the split form's 1e-11 gate."""
import numpy as np
import pytest

from fft_onchip_gb300 import inputs
from oracle import oracle as O

pytestmark = pytest.mark.gpu

SIZES = (16, 32, 64, 128, 256, 512, 1024, 2048, 4096)
TOL = {"split_bf16x3": 1e-6, "split_tf32x2": 1e-5, "split_exact": 1e-11}
KINDS = tuple(TOL)


def run(torch, x, engine, inplace=False):
    import fft_onchip_gb300 as F
    d = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    out = d if inplace else torch.empty_like(d)
    F.fft(d, out=out, engine=engine)
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("engine", KINDS)
@pytest.mark.parametrize("family", ["normal", "uniform", "loguniform"])
def test_split_matches_oracle(cuda, fftoc_lib, n, engine, family):
    batch = max(3, (1 << 17) // n)
    x = inputs.FAMILIES[family](n, batch, seed=n + 17)
    y = run(cuda, x, engine)
    ref = O.fft_f64(x)
    err = O.rel_l2(y, ref)
    assert err < TOL[engine], (n, engine, family, err)
    if engine != "split_exact":
        assert err > 1e-12  # really the reduced-precision path, not binary64


@pytest.mark.parametrize("engine", KINDS)
def test_split_scales_out_of_range_magnitudes(cuda, fftoc_lib, engine):
    n, batch = 256, 64
    x = inputs.normal(n, batch, seed=3)
    scales = np.array([1e300, 1e200, 1e40, 1e-40, 1e-200, 1e-300, 1e-310, 2.0 ** 70] * 8)[:batch, None]
    xs = x * scales
    y = run(cuda, xs, engine)
    ref = O.fft_f64(xs)
    # rows rescaled by exact powers of two so the norms neither overflow nor
    # underflow (complex division by a subnormal scale would)
    k = -np.frexp(np.max(np.abs(ref), axis=1, keepdims=True))[1]

    def sc(z):
        return np.ldexp(z.real, k) + 1j * np.ldexp(z.imag, k)

    err = np.linalg.norm(sc(y) - sc(ref), axis=1) / np.linalg.norm(sc(ref), axis=1)
    for b in range(batch):
        assert err[b] < TOL[engine], (b, scales[b], err[b])


@pytest.mark.parametrize("engine", KINDS)
def test_split_batch_edges_and_in_place(cuda, fftoc_lib, engine):
    import fft_onchip_gb300 as F
    for n in (16, 512, 4096):
        tpb = F.plan_query(n, F.ENGINES[engine])["transforms_per_block"]
        for batch in (1, tpb - 1 if tpb > 1 else 2, tpb + 1, 152 * 2 * tpb + 3):
            x = inputs.uniform(n, batch, seed=batch)
            y = run(cuda, x, engine)
            assert O.rel_l2(y, O.fft_f64(x)) < TOL[engine], (n, batch)
            yi = run(cuda, x, engine, inplace=True)
            assert np.array_equal(yi.view(np.uint64), y.view(np.uint64)), (n, batch)


@pytest.mark.parametrize("engine", KINDS)
def test_split_zero_and_nonfinite(cuda, fftoc_lib, engine):
    x = np.zeros((4, 256), dtype=np.complex128)
    x[2, 5] = np.nan
    x[3, 7] = np.inf
    y = run(cuda, x, engine)
    assert np.all(y[0] == 0) and np.all(y[1] == 0)
    assert not np.all(np.isfinite(y[2])) and not np.all(np.isfinite(y[3]))


def test_split_refuses_n8_and_reports_plan(cuda, fftoc_lib):
    import fft_onchip_gb300 as F
    d = cuda.zeros(4, 8, dtype=cuda.complex128, device="cuda")
    for eng in KINDS:
        with pytest.raises(F.FftocError) as e:
            F.fft(d, engine=eng)
        assert e.value.status_name == "FFTOC_ERR_UNSUPPORTED"
    p = F.plan_query(4096, F.ENGINE_SPLIT_BF16X3)
    assert p["radix"] == [16, 16, 16] and p["threads_per_block"] == 256
    assert F.plan_query(512, F.ENGINE_SPLIT_TF32X2)["radix"] == [16, 16, 2]
    L = F._lib.load()
    assert L.fftoc_device_error_check() == 0


def test_split_form_error_table(cuda, fftoc_lib):
    """The split form's error per N, family and split (printed for the
    record): rel-L2 and max-abs against the binary64 oracle."""
    rows = []
    for engine in KINDS:
        for n in (256, 512, 4096):
            for family in ("normal", "loguniform"):
                x = inputs.FAMILIES[family](n, max(4, (1 << 18) // n), seed=5)
                y = run(cuda, x, engine)
                ref = O.fft_f64(x)
                rel = O.rel_l2(y, ref)
                mabs = float(np.max(np.abs(y - ref)))
                rows.append((engine, n, family, rel, mabs))
                assert rel < TOL[engine]
    for r in rows:
        print("%-13s N=%-5d %-10s rel-L2 %.3e  max-abs %.3e" % r)
