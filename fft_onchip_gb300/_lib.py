"""ctypes binding of libfftoc.so (the C ABI declared in include/fftoc.h).

The library must have been built (``python -m fft_onchip_gb300.build`` or
``__graft_entry__.build()``); there is no fallback implementation.
"""
import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "lib", "libfftoc.so")

FFTOC_OK = 0
STATUS_NAMES = {
    0: "FFTOC_OK",
    1: "FFTOC_ERR_INVALID_SIZE",
    2: "FFTOC_ERR_INVALID_VALUE",
    3: "FFTOC_ERR_MISALIGNED",
    4: "FFTOC_ERR_NO_MEMORY",
    5: "FFTOC_ERR_CUDA",
    6: "FFTOC_ERR_TIMEOUT",
    7: "FFTOC_ERR_UNSUPPORTED",
}

ENGINE_AUTO, ENGINE_F64, ENGINE_FX, ENGINE_DMMA = 0, 1, 2, 3
ENGINE_SPLIT_BF16X3, ENGINE_SPLIT_TF32X2, ENGINE_SPLIT_EXACT = 4, 5, 6
ENGINES = {"auto": ENGINE_AUTO, "f64": ENGINE_F64, "fx": ENGINE_FX, "dmma": ENGINE_DMMA,
           "split_bf16x3": ENGINE_SPLIT_BF16X3, "split_tf32x2": ENGINE_SPLIT_TF32X2,
           "split_exact": ENGINE_SPLIT_EXACT}
SPLIT_BF16X3, SPLIT_TF32X2, SPLIT_EXACT = 1, 2, 3

SIZES = (8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096)

# Every symbol include/fftoc.h declares.
EXPORTS = tuple(["fftoc_c2c_fwd_n%d" % n for n in SIZES]) + (
    "fftoc_c2c_fwd",
    "fftoc_c2c_fwd_ex",
    "fftoc_c2c_fwd_host",
    "fftoc_c2c_fwd_host_noalloc",
    "fftoc_c2c_fwd_split",
    "fftoc_plan_query",
    "fftoc_plan_query_variant",
    "fftoc_plan_select",
    "fftoc_autotune",
    "fftoc_device_error_check",
    "fftoc_auto_engine",
    "fftoc_status_string",
    "fftoc_last_error_string",
    "fftoc_version",
    "fftoc_uneven_plan_create",
    "fftoc_uneven_execute",
    "fftoc_uneven_execute_per_size",
    "fftoc_uneven_counts",
    "fftoc_uneven_plan_device_sized",
    "fftoc_uneven_plan_destroy",
    "fftoc_c2c_fwd_uneven",
    "fftoc_server_config_default",
    "fftoc_server_create",
    "fftoc_server_submit",
    "fftoc_server_poll",
    "fftoc_server_wait",
    "fftoc_server_stats",
    "fftoc_server_replay",
    "fftoc_server_destroy",
    "fftoc_onchip_plan",
    "fftoc_onchip_run",
    "fftoc_selftest_bounded_wait",
    "fftoc_exec_twiddles",
)


class ServerConfig(ctypes.Structure):
    _fields_ = [("pool_bytes", ctypes.c_int64), ("slots", ctypes.c_int), ("max_batch_bytes", ctypes.c_int64),
                ("max_wait_us", ctypes.c_double)]


class RequestTiming(ctypes.Structure):
    _fields_ = [("submit_us", ctypes.c_double), ("launch_us", ctypes.c_double), ("done_us", ctypes.c_double),
                ("status", ctypes.c_int)]


class ServerStats(ctypes.Structure):
    _fields_ = [("batches", ctypes.c_int64), ("requests_done", ctypes.c_int64), ("transforms_done", ctypes.c_int64),
                ("bytes_done", ctypes.c_int64), ("pool_bytes_in_use", ctypes.c_int64), ("pending", ctypes.c_int64),
                ("max_inflight_batches", ctypes.c_int)]


class ReplayItem(ctypes.Structure):
    _fields_ = [("arrival_us", ctypes.c_double), ("n", ctypes.c_int), ("engine", ctypes.c_int),
                ("count", ctypes.c_int64), ("in_offset", ctypes.c_int64), ("out_offset", ctypes.c_int64)]


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int),
        ("engine", ctypes.c_int),
        ("threads_per_transform", ctypes.c_int),
        ("transforms_per_block", ctypes.c_int),
        ("threads_per_block", ctypes.c_int),
        ("smem_bytes", ctypes.c_int),
        ("passes", ctypes.c_int),
        ("radix", ctypes.c_int * 4),
        ("points_per_thread", ctypes.c_int),
        ("variant", ctypes.c_int),
        ("variants", ctypes.c_int),
        ("persistent", ctypes.c_int),
        ("stages", ctypes.c_int),
        ("prefetch", ctypes.c_int),
        ("code_flags", ctypes.c_int),
        ("uneven_variant", ctypes.c_int),
    ]


class FftocError(RuntimeError):
    def __init__(self, status, message):
        self.status = status
        self.status_name = STATUS_NAMES.get(status, str(status))
        super().__init__("%s: %s" % (self.status_name, message))


_lib = None


def load(path=None):
    """Load libfftoc.so (once) and declare the C signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise FftocError(-1, "libfftoc.so not built at %s (run fft_onchip_gb300/build.py)" % path)
    L = ctypes.CDLL(path)
    vp, i64, c_int = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    for n in SIZES:
        f = getattr(L, "fftoc_c2c_fwd_n%d" % n)
        f.argtypes = [vp, vp, i64, vp]
        f.restype = c_int
    L.fftoc_c2c_fwd.argtypes = [c_int, vp, vp, i64, vp]
    L.fftoc_c2c_fwd.restype = c_int
    L.fftoc_c2c_fwd_ex.argtypes = [c_int, vp, vp, i64, c_int, vp]
    L.fftoc_c2c_fwd_ex.restype = c_int
    L.fftoc_c2c_fwd_host.argtypes = [c_int, vp, vp, i64, c_int, vp]
    L.fftoc_c2c_fwd_host.restype = c_int
    L.fftoc_c2c_fwd_host_noalloc.argtypes = [c_int, vp, vp, i64, c_int, vp]
    L.fftoc_c2c_fwd_host_noalloc.restype = c_int
    L.fftoc_c2c_fwd_split.argtypes = [c_int, vp, vp, i64, c_int, vp]
    L.fftoc_c2c_fwd_split.restype = c_int
    L.fftoc_plan_query.argtypes = [c_int, c_int, ctypes.POINTER(PlanInfo)]
    L.fftoc_plan_query.restype = c_int
    L.fftoc_plan_query_variant.argtypes = [c_int, c_int, c_int, ctypes.POINTER(PlanInfo)]
    L.fftoc_plan_query_variant.restype = c_int
    L.fftoc_plan_select.argtypes = [c_int, c_int, c_int]
    L.fftoc_plan_select.restype = c_int
    L.fftoc_autotune.argtypes = [c_int, c_int, i64, vp, ctypes.POINTER(c_int), ctypes.POINTER(ctypes.c_float)]
    L.fftoc_autotune.restype = c_int
    L.fftoc_device_error_check.argtypes = []
    L.fftoc_device_error_check.restype = c_int
    L.fftoc_auto_engine.argtypes = [c_int]
    L.fftoc_auto_engine.restype = c_int
    L.fftoc_status_string.argtypes = [c_int]
    L.fftoc_status_string.restype = ctypes.c_char_p
    L.fftoc_last_error_string.argtypes = []
    L.fftoc_last_error_string.restype = ctypes.c_char_p
    L.fftoc_version.argtypes = []
    L.fftoc_version.restype = c_int
    L.fftoc_uneven_plan_create.argtypes = [ctypes.POINTER(vp), i64, c_int]
    L.fftoc_uneven_plan_create.restype = c_int
    for f in (L.fftoc_uneven_execute, L.fftoc_uneven_execute_per_size):
        f.argtypes = [vp, vp, vp, vp, vp, i64, vp]
        f.restype = c_int
    L.fftoc_uneven_counts.argtypes = [vp, ctypes.POINTER(i64)]
    L.fftoc_uneven_counts.restype = c_int
    L.fftoc_uneven_plan_device_sized.argtypes = [vp, ctypes.POINTER(c_int)]
    L.fftoc_uneven_plan_device_sized.restype = c_int
    L.fftoc_uneven_plan_destroy.argtypes = [vp]
    L.fftoc_uneven_plan_destroy.restype = c_int
    L.fftoc_c2c_fwd_uneven.argtypes = [vp, vp, vp, vp, i64, vp]
    L.fftoc_c2c_fwd_uneven.restype = c_int
    L.fftoc_server_config_default.argtypes = [ctypes.POINTER(ServerConfig)]
    L.fftoc_server_config_default.restype = None
    L.fftoc_server_create.argtypes = [ctypes.POINTER(vp), ctypes.POINTER(ServerConfig)]
    L.fftoc_server_create.restype = c_int
    L.fftoc_server_submit.argtypes = [vp, c_int, i64, c_int, vp, vp, ctypes.POINTER(i64)]
    L.fftoc_server_submit.restype = c_int
    L.fftoc_server_poll.argtypes = [vp, i64, ctypes.POINTER(c_int), ctypes.POINTER(RequestTiming)]
    L.fftoc_server_poll.restype = c_int
    L.fftoc_server_wait.argtypes = [vp, i64, ctypes.c_double, ctypes.POINTER(RequestTiming)]
    L.fftoc_server_wait.restype = c_int
    L.fftoc_server_stats.argtypes = [vp, ctypes.POINTER(ServerStats)]
    L.fftoc_server_stats.restype = c_int
    L.fftoc_server_replay.argtypes = [vp, ctypes.POINTER(ReplayItem), i64, vp, vp, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_double)]
    L.fftoc_server_replay.restype = c_int
    L.fftoc_server_destroy.argtypes = [vp]
    L.fftoc_server_destroy.restype = c_int
    L.fftoc_onchip_plan.argtypes = [c_int, c_int, ctypes.POINTER(c_int), ctypes.POINTER(c_int)]
    L.fftoc_onchip_plan.restype = c_int
    L.fftoc_onchip_run.argtypes = [c_int, c_int, vp, i64, c_int, vp]
    L.fftoc_onchip_run.restype = c_int
    L.fftoc_selftest_bounded_wait.argtypes = [ctypes.c_double, vp]
    L.fftoc_selftest_bounded_wait.restype = c_int
    L.fftoc_exec_twiddles.argtypes = [c_int, c_int, ctypes.POINTER(c_int), ctypes.POINTER(vp)]
    L.fftoc_exec_twiddles.restype = c_int
    _lib = L
    return L


def check(status):
    if status != FFTOC_OK:
        msg = load().fftoc_last_error_string()
        raise FftocError(status, msg.decode() if msg else "")
    return status


def _info_dict(info):
    return {
        "n": info.n,
        "engine": info.engine,
        "threads_per_transform": info.threads_per_transform,
        "transforms_per_block": info.transforms_per_block,
        "threads_per_block": info.threads_per_block,
        "smem_bytes": info.smem_bytes,
        "passes": info.passes,
        "radix": [info.radix[i] for i in range(info.passes)],
        "points_per_thread": info.points_per_thread,
        "variant": info.variant,
        "variants": info.variants,
        "persistent": info.persistent,
        "stages": info.stages,
        "prefetch": info.prefetch,
        "code_flags": info.code_flags,
        "uneven_variant": info.uneven_variant,
    }


def plan_query(n, engine=ENGINE_AUTO, variant=None):
    """Plan in use for (n, engine), or compiled plan `variant`."""
    info = PlanInfo()
    if variant is None:
        check(load().fftoc_plan_query(int(n), int(engine), ctypes.byref(info)))
    else:
        check(load().fftoc_plan_query_variant(int(n), int(engine), int(variant), ctypes.byref(info)))
    return _info_dict(info)


def plan_select(n, engine, variant):
    check(load().fftoc_plan_select(int(n), int(engine), int(variant)))


def autotune(n, engine, batch, stream_ptr=0):
    """Time every compiled plan; select and return (variant, ms per launch)."""
    best = ctypes.c_int()
    ms = ctypes.c_float()
    check(load().fftoc_autotune(int(n), int(engine), int(batch), stream_ptr, ctypes.byref(best), ctypes.byref(ms)))
    return best.value, ms.value
