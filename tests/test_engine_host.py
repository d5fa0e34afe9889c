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
