"""Build recipe for oracle/_ref/ref_kernels.cubin (test infrastructure only).

Compiles oracle/ref_kernels.cu, which includes the reference's own executor
headers from the reference checkout (includes/), with nvcc into a device-only
cubin for sm_103a.  Runs where the reference checkout exists (the build
container); the cubin then travels with the repository to the GPU machine,
where oracle/ref_runner.py loads it through the CUDA driver API.  Nothing is
copied from the reference into the repository: oracle/_ref/ is git-ignored.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_INCLUDES = os.environ.get("FFTOC_REFERENCE_INCLUDES", "/root/reference/includes")
OUT_DIR = os.path.join(HERE, "_ref")
CUBIN = os.path.join(OUT_DIR, "ref_kernels.cubin")
SRC = os.path.join(HERE, "ref_kernels.cu")


def available():
    return os.path.isdir(REF_INCLUDES)


def build(force=False):
    if not available():
        return CUBIN if os.path.exists(CUBIN) else None
    if not force and os.path.exists(CUBIN) and os.path.getmtime(CUBIN) >= os.path.getmtime(SRC):
        return CUBIN
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    subprocess.run([nvcc, "-cubin", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                    "-I" + REF_INCLUDES, "-o", CUBIN + ".tmp", SRC], check=True)
    os.replace(CUBIN + ".tmp", CUBIN)
    return CUBIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
