"""CPU tests of the C ABI: the library loads, exports every symbol that
include/fftoc.h declares, and rejects bad arguments before touching a GPU."""
import ctypes
import os
import re

import pytest

from fft_onchip_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            text = open(os.path.join(ROOT, "include", name)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            syms |= set(re.findall(r"\b(fftoc_\w+)\s*\(", text))
    return syms


def test_header_declares_the_size_surface():
    syms = declared_symbols()
    for n in _lib.SIZES:
        assert "fftoc_c2c_fwd_n%d" % n in syms
    assert {"fftoc_c2c_fwd", "fftoc_c2c_fwd_ex", "fftoc_last_error_string"} <= syms


def test_library_exports_every_declared_symbol(fftoc_lib):
    missing = [s for s in sorted(declared_symbols()) if not hasattr(fftoc_lib, s)]
    assert not missing, missing
    assert set(_lib.EXPORTS) <= declared_symbols()


def test_version_and_status_strings(fftoc_lib):
    assert fftoc_lib.fftoc_version() >= 10000
    for st in range(8):
        assert fftoc_lib.fftoc_status_string(st)


@pytest.mark.parametrize("n", _lib.SIZES)
@pytest.mark.parametrize("engine", ["auto", "f64", "fx"])
def test_plan_query(fftoc_lib, n, engine):
    cur = _lib.plan_query(n, _lib.ENGINES[engine])
    assert cur["variants"] >= 1 and 0 <= cur["variant"] < cur["variants"]
    for v in range(cur["variants"]):
        p = _lib.plan_query(n, _lib.ENGINES[engine], variant=v)
        assert p["n"] == n and p["variant"] == v
        assert p["engine"] in (_lib.ENGINE_F64, _lib.ENGINE_FX)
        prod = 1
        for r in p["radix"]:
            prod *= r
            assert p["points_per_thread"] % r == 0
        assert prod == n
        assert p["threads_per_transform"] * p["points_per_thread"] == n
        assert p["threads_per_transform"] * p["transforms_per_block"] == p["threads_per_block"]
        assert p["threads_per_block"] <= 1024 and p["smem_bytes"] <= 227 * 1024


def test_plan_select(fftoc_lib):
    L = fftoc_lib
    cur = _lib.plan_query(64, _lib.ENGINE_FX)
    nv = cur["variants"]
    try:
        _lib.plan_select(64, _lib.ENGINE_FX, nv - 1)
        assert _lib.plan_query(64, _lib.ENGINE_FX)["variant"] == nv - 1
        assert L.fftoc_plan_select(64, _lib.ENGINE_FX, nv) == 2      # out of range
        assert L.fftoc_plan_select(64, _lib.ENGINE_FX, -1) == 2
        assert L.fftoc_plan_select(60, _lib.ENGINE_FX, 0) == 1
    finally:
        _lib.plan_select(64, _lib.ENGINE_FX, cur["variant"])


def _call(L, n, inp, out, batch, engine=0):
    return L.fftoc_c2c_fwd_ex(n, inp, out, batch, engine, None)


def test_argument_errors_without_gpu(fftoc_lib):
    L = fftoc_lib
    A = 1 << 20  # aligned fake device addresses: never dereferenced on these paths
    assert _call(L, 48, A, A, 4) == 1                     # FFTOC_ERR_INVALID_SIZE
    assert b"48" in L.fftoc_last_error_string()
    assert L.fftoc_c2c_fwd(100, A, A, 4, None) == 1
    assert _call(L, 64, A, A, -1) == 2                    # negative batch
    assert _call(L, 64, A, A, 0) == 0                     # empty batch: no-op
    assert _call(L, 64, None, A, 4) == 2                  # null
    assert _call(L, 64, A + 8, A + 8, 4) == 3             # misaligned
    assert _call(L, 64, A, A + 16, 4) == 2                # partial overlap
    assert _call(L, 64, A, A, 4, engine=9) == 2           # unknown engine
    assert _call(L, 64, A, A, 1 << 62) == 2               # batch*n overflows
    assert L.fftoc_auto_engine(64) in (_lib.ENGINE_F64, _lib.ENGINE_FX)
    assert L.fftoc_auto_engine(65) == -1


def test_python_front_end_raises(fftoc_lib):
    import fft_onchip_gb300 as F
    with pytest.raises(F.FftocError) as ei:
        F.fft_ptr(48, 1 << 20, 1 << 20, 4)
    assert ei.value.status == 1
    with pytest.raises(ValueError):
        F.fft_ptr(64, 1 << 20, 1 << 20, 4, engine="nope")


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(_lib.FftocError):
        saved = _lib._lib
        _lib._lib = None
        try:
            _lib.load(str(tmp_path / "libfftoc.so"))
        finally:
            _lib._lib = saved


@pytest.mark.parametrize("n", _lib.SIZES)
@pytest.mark.parametrize("engine", ["f64", "fx"])
def test_plan_code_flags_and_uneven_variant(fftoc_lib, n, engine):
    """code_flags carries only the documented bits; the uneven path uses its
    own default plan while the size's choice is variant 0, else the chosen
    plan (never a persistent one)."""
    from fft_onchip_gb300 import tune
    eid = _lib.ENGINES[engine]
    cur = _lib.plan_query(n, eid)
    nv = cur["variants"]
    for v in range(nv):
        p = _lib.plan_query(n, eid, variant=v)
        assert p["code_flags"] & ~15 == 0
        assert bool(p["code_flags"]) == bool(tune.code_str(p))
    uv = cur["uneven_variant"]
    assert 0 <= uv < nv and not _lib.plan_query(n, eid, variant=uv)["persistent"]
    try:
        for v in range(1, nv):
            _lib.plan_select(n, eid, v)
            got = _lib.plan_query(n, eid)["uneven_variant"]
            if _lib.plan_query(n, eid, variant=v)["persistent"]:
                assert got != v and not _lib.plan_query(n, eid, variant=got)["persistent"]
            else:
                assert got == v
    finally:
        _lib.plan_select(n, eid, cur["variant"])


@pytest.mark.parametrize("n", [128, 256, 512])
def test_small_cta_defaults_per_engine(fftoc_lib, n):
    """At N = 128, 256 and 512 the fixed-point default is the IEEE engine's
    default plan in 64-thread CTAs; the larger-CTA plan follows it and stays
    the plan of the uneven-batch kernels."""
    fx0, fx1 = (_lib.plan_query(n, _lib.ENGINE_FX, variant=v) for v in (0, 1))
    f0, f1 = (_lib.plan_query(n, _lib.ENGINE_F64, variant=v) for v in (0, 1))
    for a, b in ((fx0, f1), (fx1, f0)):
        assert (a["radix"], a["points_per_thread"], a["transforms_per_block"]) == \
               (b["radix"], b["points_per_thread"], b["transforms_per_block"])
    assert (fx0["radix"], fx0["points_per_thread"]) == (fx1["radix"], fx1["points_per_thread"])
    assert fx0["threads_per_transform"] * fx0["transforms_per_block"] == 64
    assert fx0["transforms_per_block"] < fx1["transforms_per_block"]
    assert _lib.plan_query(n, _lib.ENGINE_FX, variant=0)["uneven_variant"] == 1


def test_n1024_fixed_point_default(fftoc_lib):
    """At N = 1024 the fixed-point default runs one transform per 128-thread
    CTA; the 256-thread plan of the same radices follows it and stays the plan
    of the uneven-batch kernels.  The IEEE engine keeps its radix-16 default."""
    q0, q1 = (_lib.plan_query(1024, _lib.ENGINE_FX, variant=v) for v in (0, 1))
    assert q0["threads_per_block"] == 128 and q0["transforms_per_block"] == 1
    assert q1["threads_per_block"] == 256 and q1["transforms_per_block"] == 2
    assert (q0["radix"], q0["points_per_thread"]) == (q1["radix"], q1["points_per_thread"]) == ([8, 8, 8, 2], 8)
    assert q0["code_flags"] == q1["code_flags"]
    assert q0["uneven_variant"] == 1
    assert _lib.plan_query(1024, _lib.ENGINE_F64, variant=0)["radix"] == [16, 16, 4]


def test_onchip_plan_overrides(fftoc_lib):
    from fft_onchip_gb300 import onchip
    sizes = (128, 256, 512)
    before = {n: _lib.plan_query(n, _lib.ENGINE_FX)["variant"] for n in sizes}
    try:
        onchip.apply_plans("128:1,512:2", _lib.ENGINE_FX)
        assert _lib.plan_query(128, _lib.ENGINE_FX)["variant"] == 1
        assert _lib.plan_query(512, _lib.ENGINE_FX)["variant"] == 2
        onchip.apply_plans("256:1")  # engine chosen per size
        assert _lib.plan_query(256, fftoc_lib.fftoc_auto_engine(256))["variant"] == 1
    finally:
        for n, v in before.items():
            _lib.plan_select(n, _lib.ENGINE_FX, v)
