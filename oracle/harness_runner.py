"""Launch the reference's harness kernel on this library's executors (test
infrastructure only).

oracle/_ref/harness_kernels.cubin (oracle/build_ref.py) holds
testing::fft_tester, the kernel of the reference's own harness
(includes/testing.cuh:16-57), compiled unmodified and instantiated with this
library's executors under the reference's names (include/fftoc/compat.cuh).
This module loads it with the CUDA driver API, binds the executors to the
library's twiddle tables (fftoc_exec_twiddles, as fftoc::exec::bind() does)
and launches it with the geometry of the reference's host driver
run_fft_kernel (includes/testing.cuh:59-92): block (Exec::threads,
Exec::units_per_block), shared memory 16 * Size * units_per_block *
ffts_per_unit bytes, arguments (inner_repeats, data, with_transfers).
"""
import ctypes
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "harness_kernels.cubin")
NAMES = os.path.join(HERE, "_ref", "harness_kernels.json")

# instantiations in oracle/harness_kernels.cu, in order: (Size, UPB template argument)
KEYS = [(8, 1), (16, 2), (32, 0), (64, 2), (128, 2), (256, 2), (512, 2), (1024, 0), (2048, 0), (4096, 1),
        (512, 1), (256, 1)]
# the executors' radices (include/fftoc/exec.cuh, plan_of)
RADICES = {8: [8], 16: [8, 2], 32: [8, 4], 64: [8, 8], 128: [16, 8], 256: [16, 16], 512: [8, 8, 8],
           1024: [16, 16, 4], 2048: [8, 8, 8, 4], 4096: [16, 16, 16]}
SIZES = [8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096]


def available():
    return os.path.exists(CUBIN) and os.path.exists(NAMES)


class Harness:
    def __init__(self):
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # the primary context, current
        self.torch = torch
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.mod = ctypes.c_void_p()
        self._ok(self.cu.cuModuleLoad(ctypes.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        with open(NAMES) as f:
            self.names = json.load(f)
        self.fns = {}
        self.shapes = self._shapes()

    def _ok(self, rc, what):
        if rc != 0:
            raise RuntimeError("%s failed: CUresult %d" % (what, rc))

    def _fn(self, name):
        f = ctypes.c_void_p()
        self._ok(self.cu.cuModuleGetFunction(ctypes.byref(f), self.mod, name.encode()), "cuModuleGetFunction")
        return f

    def _launch(self, f, grid, block, smem, args):
        params = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.byref(a), ctypes.c_void_p) for a in args])
        self._ok(self.cu.cuLaunchKernel(f, grid, 1, 1, block[0], block[1], 1, smem, None, params, None),
                 "cuLaunchKernel")

    def _shapes(self):
        t = self.torch
        buf = t.zeros(len(KEYS) * 4, dtype=t.int32, device="cuda")
        self._launch(self._fn("fftoc_harness_shapes"), 1, (32, 1), 0, [ctypes.c_uint64(buf.data_ptr())])
        t.cuda.synchronize()
        v = buf.cpu().tolist()
        out = {}
        for i, key in enumerate(KEYS):
            n, threads, upb, fpu = v[4 * i: 4 * i + 4]
            assert n == key[0]
            out[key] = {"n": n, "threads": threads, "upb": upb, "fpu": fpu, "tpb": upb * fpu,
                        "smem": 16 * n * upb * fpu}
        return out

    def bind(self, lib, engine=None):
        """Store the twiddle tables of every executor (binary64 and fixed
        point; `engine` None binds both) in the module's table."""
        t = self.torch
        ptrs = [0] * 20
        for e, slot in ((0, 0), (2, 1)):
            if engine is not None and engine != e:
                continue
            for i, n in enumerate(SIZES):
                r = RADICES[n] + [1] * (4 - len(RADICES[n]))
                out = ctypes.c_void_p()
                st = lib.fftoc_exec_twiddles(n, e, (ctypes.c_int * 4)(*r), ctypes.byref(out))
                if st != 0:
                    raise RuntimeError("fftoc_exec_twiddles(%d) = %d" % (n, st))
                ptrs[slot * 10 + i] = out.value or 0
        d = t.tensor(ptrs, dtype=t.int64, device="cuda")
        self._launch(self._fn("fftoc_harness_bind"), 1, (32, 1), 0, [ctypes.c_uint64(d.data_ptr())])
        t.cuda.synchronize()

    def run(self, key, data_ptr, blocks, repeats=1, with_transfers=True):
        """fft_tester of executor `key` on `blocks` CTAs of data at data_ptr
        (blocks * tpb transforms of Size points), asynchronous."""
        s = self.shapes[key]
        if key not in self.fns:
            f = self._fn(self.names["%d:%d" % key])
            # CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES = 8
            self._ok(self.cu.cuFuncSetAttribute(f, 8, ctypes.c_int(s["smem"])), "cuFuncSetAttribute")
            self.fns[key] = f
        self._launch(self.fns[key], blocks, (s["threads"], s["upb"]), s["smem"],
                     [ctypes.c_int(repeats), ctypes.c_uint64(data_ptr), ctypes.c_bool(with_transfers)])
