"""Serving loop front end (fftoc_server_*): continuous batching of FFT
requests of mixed sizes from host memory, admission against a fixed device
pool, latency per request.

    srv = Server(pool_bytes=8 << 30)
    req = srv.submit(x_pinned)          # (count, n) complex128 CPU tensor
    timing = srv.wait(req)              # req.out holds the transform
    lat_us, wall_s = srv.replay(items, h_in, h_out)   # load replay

``make_trace`` builds a Poisson-arrival request trace (1..4096 transforms
per request, log-uniform; N uniform over 8..4096) for ``Server.replay``.
"""
import ctypes

import numpy as np

from . import _lib
from ._lib import check, load

SIZES = _lib.SIZES


class Request:
    def __init__(self, rid, x, out):
        self.id = rid
        self.x = x  # kept alive until done
        self.out = out


class Server:
    def __init__(self, pool_bytes=8 << 30, slots=4, max_batch_bytes=256 << 20, max_wait_us=50.0):
        self._L = load()
        cfg = _lib.ServerConfig()
        self._L.fftoc_server_config_default(ctypes.byref(cfg))
        cfg.pool_bytes = int(pool_bytes)
        cfg.slots = int(slots)
        cfg.max_batch_bytes = int(max_batch_bytes)
        cfg.max_wait_us = float(max_wait_us)
        self._s = ctypes.c_void_p()
        check(self._L.fftoc_server_create(ctypes.byref(self._s), ctypes.byref(cfg)))

    def submit(self, x, out=None, engine="auto"):
        """Queue the transforms of every row of a (count, n) complex128 CPU
        tensor (pinned for full-speed copies).  Returns a Request."""
        import torch

        from . import _engine_id
        if not isinstance(x, torch.Tensor) or x.dtype != torch.complex128 or x.is_cuda or not x.is_contiguous():
            raise TypeError("x must be a contiguous complex128 CPU tensor")
        if x.dim() == 1:
            x = x.unsqueeze(0)
        if out is None:
            out = torch.empty(tuple(x.shape), dtype=x.dtype, pin_memory=x.is_pinned())
        rid = ctypes.c_int64()
        check(self._L.fftoc_server_submit(self._s, x.shape[1], x.shape[0], _engine_id(engine), x.data_ptr(),
                                          out.data_ptr(), ctypes.byref(rid)))
        return Request(rid.value, x, out)

    def wait(self, req, timeout=600.0):
        t = _lib.RequestTiming()
        check(self._L.fftoc_server_wait(self._s, req.id, float(timeout), ctypes.byref(t)))
        return {"submit_us": t.submit_us, "launch_us": t.launch_us, "done_us": t.done_us}

    def poll(self, req):
        done = ctypes.c_int()
        t = _lib.RequestTiming()
        check(self._L.fftoc_server_poll(self._s, req.id, ctypes.byref(done), ctypes.byref(t)))
        return bool(done.value)

    def stats(self):
        st = _lib.ServerStats()
        check(self._L.fftoc_server_stats(self._s, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in _lib.ServerStats._fields_}

    def replay(self, items, h_in, h_out):
        """Submit `items` (ReplayItem array) at their arrival times; returns
        (latency_us numpy array, wall seconds)."""
        m = len(items)
        lat = (ctypes.c_double * max(1, m))()
        wall = ctypes.c_double()
        check(self._L.fftoc_server_replay(self._s, items, m, h_in.data_ptr(), h_out.data_ptr(), lat,
                                          ctypes.byref(wall)))
        return np.frombuffer(lat, dtype=np.float64, count=m).copy(), wall.value

    def close(self):
        if self._s:
            check(self._L.fftoc_server_destroy(self._s))
            self._s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def make_trace(rate, m, arena_elems, seed=0, engines=(_lib.ENGINE_AUTO,)):
    """m requests with Poisson arrivals at `rate` per second: count log-uniform
    in 1..4096, N uniform over 8..4096, engine drawn uniformly from `engines`
    (a 50/50 tag with two entries; split-form tags on N = 8 run on the plain
    form, which the split form does not cover).  Inputs and outputs are ranges of arenas of
    `arena_elems` complex values (requests may share them).  Returns
    (ReplayItem array, total transforms, total bytes one way)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=m)
    arrival = np.cumsum(gaps) - gaps[0]
    count = np.floor(np.exp(rng.uniform(0.0, np.log(4097.0), size=m))).astype(np.int64)
    count = np.clip(count, 1, 4096)
    n = np.asarray(SIZES)[rng.integers(0, len(SIZES), size=m)]
    eng = np.asarray(engines)[rng.integers(0, len(engines), size=m)]
    # the split-precision form starts at N = 16: 8-point requests run on the plain form
    split = np.isin(eng, (_lib.ENGINE_SPLIT_BF16X3, _lib.ENGINE_SPLIT_TF32X2))
    eng = np.where(split & (n == 8), _lib.ENGINE_AUTO, eng)
    items = (_lib.ReplayItem * m)()
    transforms = 0
    nbytes = 0
    for i in range(m):
        elems = int(count[i] * n[i])
        if elems > arena_elems:
            raise ValueError("arena too small for a %d x %d request" % (count[i], n[i]))
        off = int(rng.integers(0, arena_elems - elems + 1)) & ~7
        items[i].arrival_us = float(arrival[i] * 1e6)
        items[i].n = int(n[i])
        items[i].engine = int(eng[i])
        items[i].count = int(count[i])
        items[i].in_offset = off
        items[i].out_offset = off
        transforms += int(count[i])
        nbytes += elems * 16
    return items, transforms, nbytes


def latency_summary(lat_us):
    lat = np.asarray(lat_us)
    return {"p50_ms": float(np.percentile(lat, 50)) / 1e3, "p99_ms": float(np.percentile(lat, 99)) / 1e3,
            "mean_ms": float(lat.mean()) / 1e3, "max_ms": float(lat.max()) / 1e3}
