"""fft_onchip_gb300 — batched forward complex FFTs (N = 8..4096) on GB300.

Host-side front end of libfftoc.so.  The compute path is the CUDA library;
PyTorch only provides device memory and streams.  There is no CPU fallback:
every call goes through the C ABI and raises FftocError if the library is
missing or a call fails.

Mirrors the per-size executor surface of gprabowski/fft_onchip
(includes/tensor_fft_N.cuh, includes/legacy8_fft.cuh, includes/legacy16_fft.cuh):
``tensor_fft_64(x)`` transforms every row of a (batch, 64) complex128 CUDA
tensor, forward (exp(-2*pi*i*n*k/N)), unnormalised, natural order, like
``fft::tensor_fft_64<CT,64>`` run by the reference harness
(includes/testing.cuh:16-57).
"""
from ._lib import (ENGINE_AUTO, ENGINE_DMMA, ENGINE_F64, ENGINE_FX, ENGINE_SPLIT_BF16X3, ENGINE_SPLIT_EXACT,
                   ENGINE_SPLIT_TF32X2, ENGINES, EXPORTS, SIZES, FftocError, autotune, check, load, plan_query,
                   plan_select)

__all__ = ["fft", "fft_ptr", "fft_host", "fft_host_ptr", "plan_query", "plan_select", "autotune", "FftocError", "SIZES",
           "ENGINES", "load", "auto_engine", "UnevenPlan", "fft_uneven"]


def _engine_id(engine):
    if isinstance(engine, str):
        if engine not in ENGINES:
            raise ValueError("unknown engine %r (one of %s)" % (engine, sorted(ENGINES)))
        return ENGINES[engine]
    return int(engine)


def auto_engine(n):
    return load().fftoc_auto_engine(int(n))


def fft_ptr(n, in_ptr, out_ptr, batch, stream_ptr=0, engine="auto"):
    """Raw C-ABI call: device pointers, batch count, cudaStream_t as int."""
    L = load()
    eng = _engine_id(engine)
    if eng == ENGINE_AUTO:
        fn = getattr(L, "fftoc_c2c_fwd_n%d" % n, None) if n in SIZES else None
        if fn is not None:
            return check(fn(in_ptr, out_ptr, int(batch), stream_ptr))
        return check(L.fftoc_c2c_fwd(int(n), in_ptr, out_ptr, int(batch), stream_ptr))
    return check(L.fftoc_c2c_fwd_ex(int(n), in_ptr, out_ptr, int(batch), eng, stream_ptr))


def fft(x, out=None, engine="auto", stream=None):
    """Forward FFT of every row of a (batch, n) complex128 CUDA tensor.

    ``out`` may be ``x`` (in place) or a separate tensor of the same shape.
    Runs asynchronously on ``stream`` (default: torch's current stream).
    """
    import torch

    if not isinstance(x, torch.Tensor) or x.dtype != torch.complex128 or not x.is_cuda:
        raise TypeError("x must be a complex128 CUDA tensor")
    if x.dim() == 1:
        x = x.unsqueeze(0)
    if x.dim() != 2 or not x.is_contiguous():
        raise ValueError("x must be a contiguous (batch, n) tensor")
    if out is None:
        out = torch.empty_like(x)
    elif out.shape != x.shape or out.dtype != x.dtype or not out.is_contiguous() or out.device != x.device:
        raise ValueError("out must match x")
    if stream is None:
        stream = torch.cuda.current_stream(x.device)
    with torch.cuda.device(x.device):
        fft_ptr(x.shape[1], x.data_ptr(), out.data_ptr(), x.shape[0], stream.cuda_stream, engine)
    return out


def fft_host_ptr(n, h_in_ptr, h_out_ptr, batch, stream_ptr=0, engine="auto"):
    """Raw C-ABI call on HOST pointers (fftoc_c2c_fwd_host)."""
    return check(load().fftoc_c2c_fwd_host(int(n), h_in_ptr, h_out_ptr, int(batch), _engine_id(engine), stream_ptr))


def fft_host(x_host, out=None, engine="auto", device=0):
    """End-to-end call with host memory: a numpy complex128 (batch, n) array
    (or a pinned CPU torch tensor) in, same out.  Blocks until done."""
    import numpy as np
    import torch

    if isinstance(x_host, torch.Tensor):
        src = x_host
    else:
        src = torch.from_numpy(np.ascontiguousarray(x_host, dtype=np.complex128))
    if src.dim() == 1:
        src = src.unsqueeze(0)
    if out is None:
        out = torch.empty_like(src)
    with torch.cuda.device(device):
        stream = torch.cuda.current_stream()
        fft_host_ptr(src.shape[-1], src.data_ptr(), out.data_ptr(), src.shape[0], stream.cuda_stream, engine)
        stream.synchronize()
    return out.numpy() if not isinstance(x_host, torch.Tensor) else out


def _uneven_check(x, offsets, ns, out):
    import torch

    if not isinstance(x, torch.Tensor) or x.dtype != torch.complex128 or not x.is_cuda or not x.is_contiguous():
        raise TypeError("x must be a contiguous complex128 CUDA tensor")
    if offsets.dtype != torch.int64 or ns.dtype != torch.int32 or offsets.device != x.device or ns.device != x.device:
        raise TypeError("offsets must be int64 and ns int32 tensors on x's device")
    if offsets.numel() != ns.numel() or not offsets.is_contiguous() or not ns.is_contiguous():
        raise ValueError("offsets and ns must be contiguous and of equal length")
    if out is None:
        out = torch.empty_like(x)
    elif out.dtype != x.dtype or out.numel() != x.numel() or not out.is_contiguous() or out.device != x.device:
        raise ValueError("out must match x")
    return out


class UnevenPlan:
    """Mixed-size batches in one CUDA graph (fftoc_uneven_plan_*).

    ``plan(x, offsets, ns)`` transforms, for every i, the ns[i] points of the
    packed complex128 CUDA tensor ``x`` starting at element offsets[i] (int64
    and int32 CUDA tensors).  ``per_size=True`` runs the comparison path (one
    launch per size after a synchronous read of the per-size counts).
    """

    def __init__(self, max_count, engine="auto"):
        import ctypes

        self._L = load()
        self._p = ctypes.c_void_p()
        check(self._L.fftoc_uneven_plan_create(ctypes.byref(self._p), int(max_count), _engine_id(engine)))
        self.max_count = int(max_count)

    def __call__(self, x, offsets, ns, out=None, stream=None, per_size=False):
        import torch

        out = _uneven_check(x, offsets, ns, out)
        if stream is None:
            stream = torch.cuda.current_stream(x.device)
        fn = self._L.fftoc_uneven_execute_per_size if per_size else self._L.fftoc_uneven_execute
        with torch.cuda.device(x.device):
            check(fn(self._p, x.data_ptr(), out.data_ptr(), offsets.data_ptr(), ns.data_ptr(), ns.numel(),
                     stream.cuda_stream))
        return out

    def device_sized(self):
        """True when the graph sizes its per-size kernels on the device (one CTA
        per tile), False when it runs persistent per-size kernels."""
        import ctypes

        v = ctypes.c_int(0)
        check(self._L.fftoc_uneven_plan_device_sized(self._p, ctypes.byref(v)))
        return bool(v.value)

    def counts(self):
        """Per-size transform counts of the last bucketing {n: count}."""
        import ctypes

        c = (ctypes.c_int64 * len(SIZES))()
        check(self._L.fftoc_uneven_counts(self._p, c))
        return {n: int(c[i]) for i, n in enumerate(SIZES)}

    def close(self):
        if self._p:
            check(self._L.fftoc_uneven_plan_destroy(self._p))
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fft_uneven(x, offsets, ns, out=None, stream=None):
    """One-shot uneven batch (fftoc_c2c_fwd_uneven, plan cached per device)."""
    import torch

    out = _uneven_check(x, offsets, ns, out)
    if stream is None:
        stream = torch.cuda.current_stream(x.device)
    with torch.cuda.device(x.device):
        check(load().fftoc_c2c_fwd_uneven(x.data_ptr(), out.data_ptr(), offsets.data_ptr(), ns.data_ptr(), ns.numel(),
                                          stream.cuda_stream))
    return out


def _make_size_entry(n):
    def entry(x, out=None, engine="auto", stream=None):
        if x.shape[-1] != n:
            raise ValueError("tensor_fft_%d expects rows of %d points" % (n, n))
        return fft(x, out=out, engine=engine, stream=stream)

    entry.__name__ = "tensor_fft_%d" % n
    entry.__doc__ = ("Forward %d-point FFT of every row (the reference's fft::tensor_fft_%d / legacy executor "
                     "surface)." % (n, n))
    return entry


for _n in SIZES:
    globals()["tensor_fft_%d" % _n] = _make_size_entry(_n)
    __all__.append("tensor_fft_%d" % _n)
del _n
