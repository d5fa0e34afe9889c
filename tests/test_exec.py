"""Device-side executors of include/fftoc/exec.cuh (the reference's FFTExec
shape, includes/tensor_fft_64.cuh:12-45), driven by a harness with
testing::fft_tester semantics (tests/exec/exec_harness.cu).

CPU: the header compiles for sm_103a with the reference's element type
(thrust::complex<double>), every executor honours the concept's shape
contract, and fftoc_exec_twiddles rejects bad arguments.  GPU: one executor
call equals the library's batched kernel of the same plan bit for bit
(special transforms included), the results meet the 1e-13 gate against the
oracle, calls compose, and an unbound executor writes NaNs."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from fft_onchip_gb300 import _lib, inputs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "exec", "exec_harness.cu")
OUT = os.path.join(ROOT, "tests", "exec", "_build", "libexec_harness.so")
HDRS = [os.path.join(ROOT, "include", "fftoc.h"), os.path.join(ROOT, "include", "fftoc", "exec.cuh")]
SIZES = _lib.SIZES
ENGINES = {"fx": _lib.ENGINE_FX, "f64": _lib.ENGINE_F64}
# the executors' plans (include/fftoc/exec.cuh, plan_of): points per thread, radices
EXEC_PLANS = {8: (8, [8]), 16: (8, [8, 2]), 32: (8, [8, 4]), 64: (8, [8, 8]), 128: (16, [16, 8]),
              256: (16, [16, 16]), 512: (8, [8, 8, 8]), 1024: (16, [16, 16, 4]), 2048: (8, [8, 8, 8, 4]),
              4096: (16, [16, 16, 16])}


def _deps_mtime():
    csrc = os.path.join(ROOT, "fft_onchip_gb300", "csrc")
    files = HDRS + [SRC] + [os.path.join(csrc, f) for f in os.listdir(csrc) if f.endswith((".cuh", ".h"))]
    return max(os.path.getmtime(f) for f in files)


@pytest.fixture(scope="module")
def harness(fftoc_lib):
    """The harness library, compiled with nvcc if missing or stale (about 10 s)."""
    from fft_onchip_gb300 import build
    if not os.path.exists(OUT) or os.path.getmtime(OUT) < _deps_mtime():
        os.makedirs(os.path.dirname(OUT), exist_ok=True)
        # the flags a harness build needs (no --expt-relaxed-constexpr)
        cmd = [build.nvcc()] + build.ARCH + ["-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                                             "-I" + os.path.join(ROOT, "include"), "-shared", "-cudart", "shared",
                                             "-o", OUT + ".tmp", SRC, "-L" + build.LIBDIR, "-lfftoc",
                                             "-Xlinker", "-rpath," + build.LIBDIR]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-4000:]
        os.replace(OUT + ".tmp", OUT)
    H = ctypes.CDLL(OUT)
    pi = ctypes.POINTER(ctypes.c_int)
    H.exec_harness_shape.argtypes = [ctypes.c_int, ctypes.c_int, pi, pi, pi, pi]
    H.exec_harness_run.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_int,
                                   ctypes.c_void_p]
    for f in (H.exec_harness_shape, H.exec_harness_run, H.exec_harness_bind, H.exec_harness_unbind):
        f.restype = ctypes.c_int
    return H


def shape(H, n, engine):
    v = [ctypes.c_int() for _ in range(4)]
    assert H.exec_harness_shape(n, engine, *[ctypes.byref(x) for x in v]) == 0
    threads, upb, fpu, smem = (x.value for x in v)
    return {"threads": threads, "upb": upb, "fpu": fpu, "smem": smem, "tpb": upb * fpu}


# ---- CPU ---------------------------------------------------------------------

@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("engine", sorted(ENGINES))
def test_executor_shape_contract(harness, n, engine):
    s = shape(harness, n, ENGINES[engine])
    p, _ = EXEC_PLANS[n]
    t = n // p  # threads per transform
    assert s["threads"] % 32 == 0 and s["threads"] * s["upb"] <= 1024
    assert s["threads"] * s["upb"] == t * s["tpb"]           # every thread owns points of one transform
    assert s["smem"] == n * 16 * s["tpb"] <= 227 * 1024      # the tile is the only dynamic shared memory
    assert harness.exec_harness_shape(n + 1, ENGINES[engine], *[ctypes.byref(ctypes.c_int()) for _ in range(4)]) == -2


def test_compat_names_take_the_reference_parameter_lists(tmp_path):
    """include/fftoc/compat.cuh: the reference's executor names with their
    template parameter lists and defaults (includes/tensor_fft_64.cuh:12,
    tensor_fft_4096.cuh:12, tensor_fft_8.cuh:12, legacy8_fft.cuh:11,
    legacy16_fft.cuh:17) name this library's executors."""
    from fft_onchip_gb300 import build
    src = tmp_path / "compat_check.cu"
    src.write_text(r"""
#include <type_traits>
#include <thrust/complex.h>
#include <fftoc/compat.cuh>
namespace fft = fftoc::compat;
using CT = thrust::complex<double>;
static_assert(std::is_same<fft::tensor_fft_64<CT, 64>, fftoc::exec::fft<CT, 64, 2>>::value, "");
static_assert(std::is_same<fft::tensor_fft_64<CT, 64, 4, 1>, fftoc::exec::fft<CT, 64, 4>>::value, "");
static_assert(std::is_same<fft::tensor_fft_8<CT, 8>, fftoc::exec::fft<CT, 8, 1>>::value, "");
static_assert(std::is_same<fft::tensor_fft_4096<CT, 4096>, fftoc::exec::fft<CT, 4096, 1>>::value, "");
static_assert(std::is_same<fft::legacy_fft<CT, 512>, fftoc::exec::fft<CT, 512, 1>>::value, "");
static_assert(std::is_same<fft::legacy16_fft<CT, 256>, fftoc::exec::fft<CT, 256, 1>>::value, "");
static_assert(fft::tensor_fft_256<CT, 256, 2, 1>::units_per_block == 2, "");
template <class Exec>
__global__ void __launch_bounds__(Exec::max_threads_per_block) run(CT* d) {
  extern __shared__ __align__(16) char sh[];
  Exec f(reinterpret_cast<CT*>(sh));
  f();
}
template __global__ void run<fft::tensor_fft_64<CT, 64>>(CT*);
template __global__ void run<fft::legacy_fft<CT, 512>>(CT*);
""")
    r = subprocess.run([build.nvcc()] + build.ARCH + ["-std=c++17", "-I" + os.path.join(ROOT, "include"), "-c",
                                                      str(src), "-o", str(tmp_path / "compat_check.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


def test_exec_twiddles_argument_errors(fftoc_lib):
    L = fftoc_lib
    out = ctypes.c_void_p(1)
    r = (ctypes.c_int * 4)
    assert L.fftoc_exec_twiddles(60, 2, r(8, 8, 1, 1), ctypes.byref(out)) == 1       # size
    assert L.fftoc_exec_twiddles(64, 2, r(8, 4, 1, 1), ctypes.byref(out)) == 2       # product
    assert L.fftoc_exec_twiddles(64, 2, r(8, 1, 8, 1), ctypes.byref(out)) == 2       # gap
    assert L.fftoc_exec_twiddles(64, 2, r(32, 2, 1, 1), ctypes.byref(out)) == 2      # radix 32
    assert L.fftoc_exec_twiddles(64, 2, None, ctypes.byref(out)) == 2
    assert L.fftoc_exec_twiddles(64, 2, r(8, 8, 1, 1), None) == 2
    assert L.fftoc_exec_twiddles(64, 4, r(8, 8, 1, 1), ctypes.byref(out)) == 7       # split engine
    assert L.fftoc_exec_twiddles(64, 9, r(8, 8, 1, 1), ctypes.byref(out)) == 2
    out = ctypes.c_void_p(1)
    assert L.fftoc_exec_twiddles(8, 0, r(8, 1, 1, 1), ctypes.byref(out)) == 0        # one pass: no table
    assert out.value is None


# ---- GPU ---------------------------------------------------------------------

def _special_rows(n):
    """Transforms that leave the fast fixed-point paths: zeros, a non-finite
    value, subnormals, a huge range, values near the binary64 maximum."""
    rows = np.zeros((5, n), dtype=np.complex128)
    rows[1] = 1.0
    rows[1, n // 3] = np.nan
    rows[2] = 5e-324 * (np.arange(n) % 7 + 1)
    rows[3] = np.where(np.arange(n) % 2 == 0, 1e300, 1e-300)
    rows[4] = 1e306 * np.exp(2j * np.pi * np.arange(n) / n)
    return rows


def _bits(t):
    import torch
    return torch.view_as_real(t).view(torch.int64)


@pytest.mark.gpu
@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("engine", sorted(ENGINES))
def test_executor_equals_batched_kernel_of_the_same_plan(cuda, harness, n, engine):
    import fft_onchip_gb300 as F
    from oracle import oracle as O
    eng = ENGINES[engine]
    assert harness.exec_harness_bind() == 0
    s = shape(harness, n, eng)
    blocks = max(3, -(-8 // s["tpb"]))  # at least 8 transforms: 5 special, 3 ordinary
    x = inputs.normal(n, blocks * s["tpb"], seed=1000 + n)
    x[: 5] = _special_rows(n)
    d = cuda.from_numpy(x).cuda()
    out = d.clone()
    assert harness.exec_harness_run(n, eng, out.data_ptr(), blocks, 1, None) == 0
    # the library's batched kernel with the executor's plan
    p, radix = EXEC_PLANS[n]
    cur = F.plan_query(n, eng)["variant"]
    match = [v for v in range(F.plan_query(n, eng)["variants"])
             if (lambda q: q["points_per_thread"] == p and q["radix"] == radix)(F.plan_query(n, eng, variant=v))]
    assert match, "no compiled plan with the executor's radices"
    try:
        F.plan_select(n, eng, match[0])
        ref = F.fft(d, engine=engine)
    finally:
        F.plan_select(n, eng, cur)
    cuda.cuda.synchronize()
    assert cuda.equal(_bits(out), _bits(ref))
    # and the ordinary rows meet the FP64 gate against the oracle
    y = out.cpu().numpy()[5:]
    assert O.rel_l2(y, O.fft_f64(x[5:])) < 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("n", [8, 64, 512, 4096])
def test_executor_calls_compose(cuda, harness, n):
    eng = ENGINES["fx"]
    assert harness.exec_harness_bind() == 0
    s = shape(harness, n, eng)
    blocks = 2
    d = cuda.from_numpy(inputs.uniform(n, blocks * s["tpb"], seed=7)).cuda()
    once, twice, none = d.clone(), d.clone(), d.clone()
    assert harness.exec_harness_run(n, eng, once.data_ptr(), blocks, 1, None) == 0
    assert harness.exec_harness_run(n, eng, once.data_ptr(), blocks, 1, None) == 0
    assert harness.exec_harness_run(n, eng, twice.data_ptr(), blocks, 2, None) == 0
    assert harness.exec_harness_run(n, eng, none.data_ptr(), blocks, 0, None) == 0
    cuda.cuda.synchronize()
    assert cuda.equal(_bits(once), _bits(twice))
    assert cuda.equal(_bits(none), _bits(d))


@pytest.mark.gpu
def test_unbound_executor_writes_nan(cuda, harness):
    from oracle import oracle as O
    eng = ENGINES["fx"]
    try:
        assert harness.exec_harness_unbind() == 0
        for n in (8, 64):
            s = shape(harness, n, eng)
            x = inputs.uniform(n, s["tpb"], seed=3)
            d = cuda.from_numpy(x).cuda()
            assert harness.exec_harness_run(n, eng, d.data_ptr(), 1, 1, None) == 0
            y = d.cpu().numpy()
            if n == 8:   # one pass: needs no table
                assert O.rel_l2(y, O.fft_f64(x)) < 1e-13
            else:
                assert np.isnan(y.real).all() and np.isnan(y.imag).all()
    finally:
        assert harness.exec_harness_bind() == 0
