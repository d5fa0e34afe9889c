"""Build recipe for the reference's device code under oracle/_ref/ (test
infrastructure only).

* oracle/_ref/ref_kernels.cubin: oracle/ref_kernels.cu, which includes the
  reference's own executor headers (includes/);
* oracle/_ref/harness_kernels.cubin: oracle/harness_kernels.cu, the
  reference's harness kernel testing::fft_tester (includes/testing.cuh)
  instantiated with this library's executors under the reference's names
  (include/fftoc/compat.cuh); the entry-function names ptxas reports are
  written beside it (harness_kernels.json) for the driver-API runner.

Both are device-only cubins for sm_103a, so they travel with the repository
to the GPU machine, where oracle/ref_runner.py and oracle/harness_runner.py
load them.  The reference checkout is found through FFTOC_REFERENCE_INCLUDES
(its includes/ directory), FFTOC_REFERENCE (its root), or else a checkout
named `reference` beside this repository; without one nothing is built and
existing cubins are kept.  Nothing is copied from the reference into the
repository: oracle/_ref/ is git-ignored.
"""
import json
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_ref")
CUBIN = os.path.join(OUT_DIR, "ref_kernels.cubin")
SRC = os.path.join(HERE, "ref_kernels.cu")
HARNESS_CUBIN = os.path.join(OUT_DIR, "harness_kernels.cubin")
HARNESS_NAMES = os.path.join(OUT_DIR, "harness_kernels.json")
HARNESS_SRC = os.path.join(HERE, "harness_kernels.cu")


def ref_includes():
    if os.environ.get("FFTOC_REFERENCE_INCLUDES"):
        return os.environ["FFTOC_REFERENCE_INCLUDES"]
    root = os.environ.get("FFTOC_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
    return os.path.join(root, "includes")


def available():
    return os.path.isfile(os.path.join(ref_includes(), "testing.cuh"))


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _stale(out, srcs):
    return not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(s) for s in srcs)


def build(force=False):
    if not available():
        return CUBIN if os.path.exists(CUBIN) else None
    inc = ref_includes()
    os.makedirs(OUT_DIR, exist_ok=True)
    arch = ["-gencode", "arch=compute_103a,code=sm_103a"]
    if force or _stale(CUBIN, [SRC]):
        subprocess.run([_nvcc(), "-cubin", "-std=c++17"] + arch + ["-O3", "-I" + inc, "-o", CUBIN + ".tmp", SRC],
                       check=True)
        os.replace(CUBIN + ".tmp", CUBIN)
    hdrs = [HARNESS_SRC, os.path.join(ROOT, "include", "fftoc", "exec.cuh"),
            os.path.join(ROOT, "include", "fftoc", "compat.cuh"),
            os.path.join(ROOT, "fft_onchip_gb300", "csrc", "fft_kernel.cuh"),
            os.path.join(ROOT, "fft_onchip_gb300", "csrc", "fft_core.cuh")]
    if force or _stale(HARNESS_CUBIN, hdrs) or not os.path.exists(HARNESS_NAMES):
        r = subprocess.run([_nvcc(), "-cubin", "-std=c++17"] + arch +
                           ["-O3", "-I" + inc, "-I" + os.path.join(ROOT, "include"), "-Xptxas", "-v",
                            "-o", HARNESS_CUBIN + ".tmp", HARNESS_SRC], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("harness cubin build failed:\n" + r.stderr[-4000:])
        names = re.findall(r"Compiling entry function '([^']+)'", r.stderr)
        # key: size and the executor's UPB template argument (fftoc::exec::fft<CT, Size, UPB, Engine>)
        table = {}
        for nm in names:
            m = re.search(r"4exec3fftI\w+?_Li(\d+)ELi(\d+)ELi\d+EEE", nm)
            if m and "fft_tester" in nm:
                table["%s:%s" % (m.group(1), m.group(2))] = nm
        if len(table) != 12:
            raise RuntimeError("expected 12 harness instantiations, found %d" % len(table))
        with open(HARNESS_NAMES, "w") as f:
            json.dump(table, f, indent=1, sort_keys=True)
        os.replace(HARNESS_CUBIN + ".tmp", HARNESS_CUBIN)
    return CUBIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
