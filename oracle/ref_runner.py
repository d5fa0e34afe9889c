"""Run the reference's own executors on the GPU (test infrastructure only).

Loads oracle/_ref/ref_kernels.cubin (built by oracle/build_ref.py from the
reference's headers) with the CUDA driver API and launches its executors
with the reference harness's geometry (includes/testing.cuh:59-92):
block = (Exec::threads, UPB), one block per UPB*FPU transforms, dynamic
shared memory = 16 bytes per staged point.

    python -m oracle.ref_runner fixtures   # writes tests/golden/ref_out_*.npz
    python -m oracle.ref_runner timing     # on-chip us/pass like testing.cuh:94-127
    python -m oracle.ref_runner stream     # one pass over 1 GiB in HBM: GB/s

Fixtures record the reference's ACTUAL outputs on seeded inputs; the CPU
tests pin the oracle's restatements and conventions against them.
"""
import ctypes
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CUBIN = os.path.join(HERE, "_ref", "ref_kernels.cubin")
GOLD = os.path.join(ROOT, "tests", "golden")

# kernel: (N, threads per unit, points staged per block)
EXECUTORS = {
    "ref_tensor_fft_8": (8, 32, 64),
    "ref_tensor_fft_64": (64, 32, 64),
    "ref_tensor_fft_128": (128, 32, 128),
    "ref_tensor_fft_256": (256, 32, 256),
    "ref_tensor_fft_512": (512, 64, 512),
    "ref_tensor_fft_4096": (4096, 512, 4096),
    "ref_legacy8_fft_8": (8, 1, 8),
    "ref_legacy8_fft_64": (64, 8, 64),
    "ref_legacy8_fft_512": (512, 64, 512),
    "ref_legacy8_fft_4096": (4096, 512, 4096),
    "ref_legacy16_fft_16": (16, 1, 16),
    "ref_legacy16_fft_256": (256, 16, 256),
    "ref_legacy16_fft_4096": (4096, 256, 4096),
}


class Driver:
    def __init__(self):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.mod = ctypes.c_void_p()
        self._ok(self.cu.cuModuleLoad(ctypes.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        self.fns = {}

    def _ok(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s failed: CUresult %d" % (what, rc))

    def fn(self, name, smem):
        if name not in self.fns:
            f = ctypes.c_void_p()
            self._ok(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, name.encode()), "cuModuleGetFunction")
            # CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES = 8
            self._ok(self.cu.cuFuncSetAttribute(f, 8, ctypes.c_int(smem)), "cuFuncSetAttribute")
            self.fns[name] = f
        return self.fns[name]

    def launch(self, name, ptr, blocks, repeats=1, stream=0):
        n, threads, staged = EXECUTORS[name]
        smem = staged * 16
        f = self.fn(name, smem)
        p_data = ctypes.c_uint64(ptr)
        p_rep = ctypes.c_int(repeats)
        params = (ctypes.c_void_p * 2)(ctypes.cast(ctypes.byref(p_data), ctypes.c_void_p),
                                       ctypes.cast(ctypes.byref(p_rep), ctypes.c_void_p))
        self._ok(self.cu.cuLaunchKernel(f, blocks, 1, 1, threads, 1, 1, smem, ctypes.c_void_p(stream), params, None),
                 "cuLaunchKernel")


def run(drv, name, x):
    """Reference executor `name` on complex128 (batch, n) host array x."""
    import torch
    n, threads, staged = EXECUTORS[name]
    per_block = staged // n
    batch = x.shape[0]
    assert batch % per_block == 0
    d = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    drv.launch(name, d.data_ptr(), batch // per_block)
    torch.cuda.synchronize()
    return d.cpu().numpy()


def fixtures():
    sys.path.insert(0, ROOT)
    from fft_onchip_gb300 import inputs
    drv = Driver()
    for name, (n, threads, staged) in EXECUTORS.items():
        batch = 16 if n <= 64 else (4 if n <= 512 else 1)
        x = inputs.uniform(n, batch, seed=7)
        y = run(drv, name, x)
        np.savez_compressed(os.path.join(GOLD, "ref_out_%s.npz" % name[4:]), x=x, y=y)
        print(name, batch)


def _time_executor(drv, name, sm_multiplier):
    """us per on-chip pass of one executor: (t(1100) - t(100)) / 1000 with
    grid = sm_multiplier*SMs/(UPB*FPU) (includes/testing.cuh:68-69,115-124)."""
    import torch
    n, threads, staged = EXECUTORS[name]
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    per_block = staged // n
    blocks = max(1, (sm_multiplier * sms) // per_block)
    d = torch.randn(blocks * per_block, n, dtype=torch.complex128, device="cuda")
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    drv.launch(name, d.data_ptr(), blocks, 10)
    torch.cuda.synchronize()
    ev[0].record()
    drv.launch(name, d.data_ptr(), blocks, 100)
    ev[1].record()
    drv.launch(name, d.data_ptr(), blocks, 1100)
    ev[2].record()
    torch.cuda.synchronize()
    us = (ev[1].elapsed_time(ev[2]) - ev[0].elapsed_time(ev[1])) * 1e3 / 1000.0
    ffts = blocks * per_block
    return {"n": n, "sm_multiplier": sm_multiplier, "us_per_pass": us, "ffts_per_pass": ffts,
            "ffts_per_s": ffts / (us * 1e-6)}


def timing(sm_multiplier=32):
    """On-chip us per pass of every executor at the harness's default grid
    (data replicated per block)."""
    drv = Driver()
    out = {}
    for name in EXECUTORS:
        out[name] = _time_executor(drv, name, sm_multiplier)
        print(json.dumps({name: out[name]}))
    return out


def saturation(multipliers=(4, 8, 16, 32, 64, 128, 256)):
    """The reference's saturation sweep (src/saturation.cu:36-44): per-pass
    time of its tensor executors against blocks per SM."""
    drv = Driver()
    out = {}
    for name in ("ref_tensor_fft_8", "ref_tensor_fft_64", "ref_tensor_fft_128", "ref_tensor_fft_256",
                 "ref_tensor_fft_512"):
        out[name] = [_time_executor(drv, name, m) for m in multipliers]
        for r in out[name]:
            print(json.dumps({name: r}), flush=True)
    return out


def stream(gib=1.0, reps=5):
    """Each executor streamed over a 1 GiB batch once per launch (copy in,
    one transform, copy out: the harness with inner_repeats = 1), timed with
    CUDA events; GB/s counts one complex128 read and write per point."""
    import torch
    drv = Driver()
    out = {}
    for name, (n, threads, staged) in EXECUTORS.items():
        per_block = staged // n
        batch = int(gib * (1 << 30)) // (16 * n)
        batch -= batch % per_block
        blocks = batch // per_block
        d = torch.randn(batch, n, dtype=torch.complex128, device="cuda")
        drv.launch(name, d.data_ptr(), blocks, 1)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            drv.launch(name, d.data_ptr(), blocks, 1)
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / reps
        out[name] = {"n": n, "batch": batch, "ms": ms, "ffts_per_s": batch / (ms * 1e-3),
                     "hbm_gbs": 32.0 * n * batch / (ms * 1e-3) / 1e9}
        print(json.dumps({name: out[name]}), flush=True)
        del d
    return out


if __name__ == "__main__":
    what = sys.argv[1] if len(sys.argv) > 1 else "fixtures"
    if what == "fixtures":
        fixtures()
    elif what == "stream":
        stream()
    elif what == "saturation":
        saturation()
    else:
        timing()
