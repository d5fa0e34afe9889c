"""CPU test of the engine arithmetic: tests/host/engine_check.cu compiles the
library's DFT kernels, twiddle products and binary64 <-> fixed-point
conversions as host code (nvcc, no GPU) and compares them with long double."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def engine_report():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "engine_check")
    src = os.path.join(ROOT, "tests", "host", "engine_check.cu")
    csrc = os.path.join(ROOT, "fft_onchip_gb300", "csrc")
    subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I" + csrc, "-I" + os.path.join(ROOT, "include"), "-o", exe, src], check=True)
    r = subprocess.run([exe], check=True, capture_output=True, text=True)
    return {k: float(v) for k, v in (line.split() for line in r.stdout.strip().splitlines())}


@pytest.mark.parametrize("name", ["f64_dft2", "f64_dft4", "f64_dft8", "f64_dft16"])
def test_f64_dft_kernels(engine_report, name):
    assert engine_report[name] < 5e-16


@pytest.mark.parametrize("name", ["fx_dft2", "fx_dft4", "fx_dft8", "fx_dft16"])
def test_fx_dft_kernels(engine_report, name):
    # fixed-point inputs of ~2^50: a few LSB of rounding in the constant products
    assert engine_report[name] < 2e-15


def test_fx_twiddle_product_error_in_lsb(engine_report):
    # four dropped low-limb products (< 1 LSB each) plus the rounding of the sum
    assert engine_report["fx_cmul_lsb"] < 6


def test_fx_constant_product_error_in_lsb(engine_report):
    assert engine_report["fx_mulc_lsb"] < 3


def test_fx_conversion_round_trip(engine_report):
    # relative to the transform's largest element; an all-subnormal transform
    # loses a few bits (its largest exponent field is 0)
    assert engine_report["fx_roundtrip"] < 1e-13


def _split_values():
    """Edge and random values of the fixed-point range |x| < 2^61."""
    import numpy as np
    rng = np.random.default_rng(7)
    lim = (1 << 61) - 1
    edges = [0, 1, -1, lim, -lim, 1 << 30, -(1 << 30), (1 << 30) - 1, -(1 << 30) + 1, (1 << 60), -(1 << 60)]
    edges += [k * (1 << 30) + d for k in (-3, -1, 0, 1, 5) for d in (-1, 0, 1)]
    rand = rng.integers(-lim, lim, size=200000, dtype=np.int64, endpoint=True)
    small = rng.integers(-(1 << 34), 1 << 34, size=50000, dtype=np.int64)
    return np.concatenate([np.array(edges, dtype=np.int64), rand, small])


def test_imad_split_low_limb_identity():
    """The multiply-add form of the limb split (ImadSplit plans) computes
    lo32(x) + xh * 0xC0000000 (mod 2^32) with xh = x >> 30; it must equal the
    mask form x & (2^30 - 1), and xh must fit 32 bits."""
    import numpy as np
    x = _split_values()
    xh = x >> 30                                            # arithmetic shift
    assert xh.min() >= -(1 << 31) and xh.max() < (1 << 31)
    lo32 = (x & 0xFFFFFFFF).astype(np.uint64)
    xh32 = (xh & 0xFFFFFFFF).astype(np.uint64)
    imad = (lo32 + xh32 * np.uint64(0xC0000000)) & np.uint64(0xFFFFFFFF)
    mask = (x & ((1 << 30) - 1)).astype(np.uint64)
    assert np.array_equal(imad, mask)
    # and the limbs put x back together
    assert np.array_equal(xh * (1 << 30) + mask.astype(np.int64), x)


def test_out_hi_zero_test_matches_the_integer_test():
    """OutHiZero plans test the high word of (double)x instead of x itself: a
    nonzero integer converts to a double of magnitude >= 1, whose high word
    is nonzero, and 0 converts to +0.0."""
    import numpy as np
    x = np.concatenate([_split_values(), np.array([np.iinfo(np.int64).min, np.iinfo(np.int64).max], dtype=np.int64)])
    hi = (x.astype(np.float64).view(np.uint64) >> np.uint64(32)).astype(np.uint32)
    assert np.array_equal(hi != 0, x != 0)


def test_fx_in_near_matches_fx_in_on_its_domain(engine_report):
    # two funnel shifts instead of the 64-bit shift: bit-identical where the
    # kernels take it (normal values within 2^31 of the transform maximum)
    assert engine_report["fx_in_near_mismatch"] == 0


def test_fx_out_matches_ldexp_in_the_normal_range(engine_report):
    # (double)x with K added to its exponent field, zero tested on the integer
    # or on the converted high word: the same bits as ldexp((double)x, K)
    assert engine_report["fx_out_mismatch"] == 0


def test_fx_constants_are_rounded_limbs(engine_report):
    # sqrt(1/2), cos(pi/8), sin(pi/8) and negatives as 30-bit limbs of v*2^60
    assert engine_report["fx_konst_ulp"] <= 0.5


@pytest.fixture(scope="module")
def exact_report():
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "exact_check")
    src = os.path.join(ROOT, "tests", "host", "exact_check.cu")
    csrc = os.path.join(ROOT, "fft_onchip_gb300", "csrc")
    subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I" + csrc, "-I" + os.path.join(ROOT, "include"), "-o", exe, src], check=True)
    r = subprocess.run([exe], check=True, capture_output=True, text=True)
    return {k: float(v) for k, v in (line.split() for line in r.stdout.strip().splitlines())}


def test_exact_digit_cut(exact_report):
    """The offset-binary byte cut gives balanced digits whose sum is the
    49-bit floor cut, and the byte-permute FP16 route (1024 + offset digit)
    minus 1024 + offset reproduces every digit exactly."""
    assert exact_report["exact_cut_bad"] == 0
    assert exact_report["exact_digit_bad"] == 0


def test_exact_operand_and_accumulators(exact_report):
    """The library's B operand holds integer digits |f| <= 128, and every
    emulated FP32 accumulator of a pass stays below 2^22 (exact, and in the
    range of the recombination's magic-number conversion)."""
    assert exact_report["exact_b_max"] <= 128
    assert exact_report["exact_acc_max"] < 2 ** 22
    # seeded with 1.5 * 2^23, every accumulator is an exact FP32 integer
    assert exact_report["exact_acc_inexact"] == 0


def test_exact_pass_matches_dft(exact_report):
    """A radix-16 pass emulated on the kernel's operand layout (twelve MMAs,
    integer recombination) matches the 16-point DFT in long double to the
    49-bit cut: error below 2^-46 of the pass's output bound, and outputs
    stay below the 2^58.5 bound the next pass relies on."""
    assert exact_report["exact_pass_err"] < 2.0 ** -46
    assert exact_report["exact_out_log2"] <= 58.5


def test_uneven_grid_rule():
    """The uneven graph's grid rule (uneven_grid, evaluated on the device from
    the bucket counts), compiled as host code: one CTA per tile for a size
    holding at least 40 % of the batch's bytes or fewer tiles than one wave, else one
    wave of persistent CTAs, never 0."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    out_dir = os.path.join(ROOT, "tests", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "uneven_grid_check")
    csrc = os.path.join(ROOT, "fft_onchip_gb300", "csrc")
    subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I" + csrc, "-I" + os.path.join(ROOT, "include"), "-o", exe,
                    os.path.join(ROOT, "tests", "host", "uneven_grid_check.cu")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout
