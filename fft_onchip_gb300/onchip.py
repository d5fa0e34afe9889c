"""On-chip repeat harness: the reference's timing mode for this library's
plans, so its per-pass numbers (scripts/results/configs.csv,
saturation.csv) can be reproduced like for like.

The reference (includes/testing.cuh:59-127) launches
(sm_multiplier * SMs) / transforms_per_block blocks over a buffer holding
one copy of the input per block, times one launch with 100 and one with 1100
in-shared-memory repeats (CUDA events around each launch), and reports
(t(1100) - t(100)) / 1000 microseconds per pass; each pass transforms
sm_multiplier * SMs transforms.  ``time_onchip`` does the same through
fftoc_onchip_run.

    python -m fft_onchip_gb300.onchip --sizes 8,64,512 --engine auto
"""
import argparse
import ctypes
import json

from . import _lib
from ._lib import check, load


def onchip_plan(n, engine=_lib.ENGINE_AUTO):
    tpb, var = ctypes.c_int(), ctypes.c_int()
    check(load().fftoc_onchip_plan(int(n), int(engine), ctypes.byref(tpb), ctypes.byref(var)))
    return tpb.value, var.value


def run(n, data, blocks, repeats, engine=_lib.ENGINE_AUTO, stream_ptr=0):
    check(load().fftoc_onchip_run(int(n), int(engine), data.data_ptr(), int(blocks), int(repeats), stream_ptr))


def time_onchip(n, engine=_lib.ENGINE_AUTO, sm_multiplier=32, seed=0):
    """Microseconds per on-chip pass over sm_multiplier * SMs transforms,
    and the resulting transforms per second."""
    import torch

    from . import inputs
    tpb, var = onchip_plan(n, engine)
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    blocks = max(1, (sm_multiplier * sms) // tpb)
    x = torch.from_numpy(inputs.uniform(n, tpb, seed=seed)).cuda()
    data = x.repeat(blocks, 1).contiguous()  # one copy of the input per block
    s = torch.cuda.current_stream()
    run(n, data, blocks, 10, engine, s.cuda_stream)  # warm-up
    torch.cuda.synchronize()
    times = {}
    for reps in (100, 1100):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        run(n, data, blocks, reps, engine, s.cuda_stream)
        b.record(s)
        torch.cuda.synchronize()
        times[reps] = a.elapsed_time(b) * 1e3
    us = (times[1100] - times[100]) / 1000.0
    ffts = blocks * tpb
    return {"n": n, "us_per_pass": us, "ffts_per_pass": ffts, "ffts_per_s": ffts / (us * 1e-6),
            "transforms_per_block": tpb, "variant": var, "blocks": blocks, "sm_multiplier": sm_multiplier}


def saturation(n, multipliers=range(4, 257, 4), engine=_lib.ENGINE_AUTO):
    """Per-pass time against blocks per SM (the reference's
    src/saturation.cu:36-44 sweep)."""
    return [time_onchip(n, engine, m) for m in multipliers]


def apply_plans(spec, engine=_lib.ENGINE_AUTO):
    """Select plan variants from 'N:variant,...' (the engine's choice per N
    when engine is AUTO), as bench.py's --plan does."""
    for item in filter(None, spec.split(",")):
        pn, pv = item.split(":")
        n = int(pn)
        eng = engine if engine != _lib.ENGINE_AUTO else load().fftoc_auto_engine(n)
        _lib.plan_select(n, eng, int(pv))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--sizes", default="8,64,128,256,512,4096")
    ap.add_argument("--engine", default="auto")
    ap.add_argument("--sm-multiplier", type=int, default=32)
    ap.add_argument("--plan", default="", help="N:variant,... plan overrides (default: the library's choice)")
    ap.add_argument("--saturation", default="",
                    help="comma list of blocks-per-SM multipliers to sweep (the reference's saturation test)")
    a = ap.parse_args()
    eng = _lib.ENGINES[a.engine]
    mults = [int(v) for v in a.saturation.split(",") if v] or [a.sm_multiplier]
    apply_plans(a.plan, eng)
    for n in [int(v) for v in a.sizes.split(",")]:
        for m in mults:
            print(json.dumps(time_onchip(n, eng, m)), flush=True)


if __name__ == "__main__":
    main()
