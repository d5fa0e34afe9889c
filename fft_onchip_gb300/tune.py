"""Plan autotuner front end (the runtime counterpart of the reference's
generated sweep, scripts/generate_bench.py:93-113, and its occupancy sweep,
src/saturation.cu:36-44).

For every size and engine it times each compiled plan through the C ABI
(fftoc_plan_select + fftoc_c2c_fwd_ex, CUDA events, inputs larger than L2),
selects the fastest, and can persist the choices as JSON keyed by GPU name:

    python -m fft_onchip_gb300.tune --engine fx --gib 0.5 --out tuning.json

``load(path)`` re-applies a saved choice table (fftoc_plan_select).
"""
import argparse
import json
import os

from . import _lib

SIZES = _lib.SIZES


def code_str(p):
    """The code-form flags of a plan, e.g. 'outlined-in,imad-split'."""
    names = ((1, "outlined-in"), (2, "imad-split"), (4, "out-hi-zero"), (8, "direct-io"))
    return ",".join(nm for bit, nm in names if p.get("code_flags", 0) & bit)


def time_variants(n, engine, gib=0.5, reps=20, warmup=5, device=0, rounds=2):
    """[(variant, ms per launch, plan dict)] for every compiled plan."""
    import torch
    torch.cuda.set_device(device)
    eid = _lib.ENGINES[engine] if isinstance(engine, str) else int(engine)
    batch = max(1, int(gib * (1 << 30)) // (16 * n))
    x = torch.randn(batch, n, dtype=torch.complex128, device="cuda")
    y = torch.empty_like(x)
    L = _lib.load()
    s = torch.cuda.current_stream()
    cur = _lib.plan_query(n, eid)
    out = []
    try:
        for v in range(cur["variants"]):
            _lib.plan_select(n, eid, v)
            for _ in range(warmup):
                _lib.check(L.fftoc_c2c_fwd_ex(n, x.data_ptr(), y.data_ptr(), batch, eid, s.cuda_stream))
            best = float("inf")
            for _ in range(rounds):
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(s)
                for _ in range(reps):
                    _lib.check(L.fftoc_c2c_fwd_ex(n, x.data_ptr(), y.data_ptr(), batch, eid, s.cuda_stream))
                b.record(s)
                b.synchronize()
                best = min(best, a.elapsed_time(b) / reps)
            out.append((v, best, _lib.plan_query(n, eid, variant=v)))
    finally:
        _lib.plan_select(n, eid, cur["variant"])
    return out


def tune(sizes=SIZES, engines=("fx", "f64"), gib=0.5, apply=True, verbose=True):
    import torch
    gpu = torch.cuda.get_device_name()
    table = {}
    for eng in engines:
        eid = _lib.ENGINES[eng]
        table[eng] = {}
        for n in sizes:
            res = time_variants(n, eng, gib)
            best = min(res, key=lambda r: r[1])
            table[eng][str(n)] = best[0]
            if apply:
                _lib.plan_select(n, eid, best[0])
            if verbose:
                for v, ms, p in res:
                    gbs = 32.0 * n * (int(gib * (1 << 30)) // (16 * n)) / (ms * 1e-3) / 1e9
                    print("%-4s N=%-5d variant %d radix=%-14s P=%-2d tpb=%-3d%s %8.4f ms %7.1f GB/s%s" % (
                        eng, n, v, "x".join(map(str, p["radix"])), p["points_per_thread"], p["transforms_per_block"],
                        " pf" if p.get("prefetch") else "   ", ms, gbs, "  <- best" if v == best[0] else "")
                      + (" [%s]" % code_str(p) if p.get("code_flags") else ""))
    return {"gpu": gpu, "choices": table}


def save(result, path):
    data = {}
    if os.path.exists(path):
        with open(path) as f:
            data = json.load(f)
    data[result["gpu"]] = result["choices"]
    with open(path, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)


def load(path, gpu=None):
    """Apply a saved choice table for this GPU; returns the table or None."""
    import torch
    with open(path) as f:
        data = json.load(f)
    gpu = gpu or torch.cuda.get_device_name()
    choices = data.get(gpu)
    if not choices:
        return None
    for eng, per_n in choices.items():
        for n, v in per_n.items():
            _lib.plan_select(int(n), _lib.ENGINES[eng], int(v))
    return choices


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--engine", default="fx,f64")
    ap.add_argument("--sizes", default=",".join(map(str, SIZES)))
    ap.add_argument("--gib", type=float, default=0.5)
    ap.add_argument("--out", default=None)
    a = ap.parse_args()
    res = tune([int(s) for s in a.sizes.split(",")], a.engine.split(","), a.gib)
    print(json.dumps(res))
    if a.out:
        save(res, a.out)


if __name__ == "__main__":
    main()
