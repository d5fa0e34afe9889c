"""Benchmark: batched forward complex-FP64 FFTs on GB300 through the C ABI.

Workload (one "step"): the plain-FP64 size sweep — N in {8, 16, 64, 128, 256,
512, 4096}, each a batch of 1 GiB of complex128 input (so 2 GiB of HBM
traffic per size), one call of the library's per-size entry point each.
Inputs are N(0,1) re/im from a seeded device generator, resident in HBM
before timing; every buffer is larger than L2 (129 MB), so no L2 flush is
needed between steps.

Prints ONE JSON line (rank 0).  `value` = FFTs/s over the whole sweep
(total transforms / total time, max over ranks); per-size FFT/s and % of the
measured HBM copy bandwidth are in `per_n`.  `e2e` repeats the sweep through
fftoc_c2c_fwd_host with pinned host buffers (host->device copy, transform,
device->host copy inside the timed region).

--impl reference times the CPU restatement of the path (the reference has no
CPU implementation; oracle/fftoc_oracle.c's FP64 Stockham port of its
radix-8 executor) on all host cores, one bounded sample per size per step.

Multi-GPU: torchrun --nproc-per-node N; each rank runs the full sweep on its
own GPU (independent transforms, no collective on the data path: weak
scaling); barrier + max over ranks around the timed region.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SWEEP = (8, 16, 64, 128, 256, 512, 4096)
GIB = 1 << 30
METRIC = "FFTs/s, %HBM peak: split vs FP64 at err<=1e-11; serve p50/p99"
WORKLOAD = "plain FP64 size sweep: N in {8,16,64,128,256,512,4096}, 1 GiB complex128 input per N"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--engine", default="auto")
    ap.add_argument("--sizes", default=",".join(str(n) for n in SWEEP))
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="CPU-baseline time of the all-threads leg")
    ap.add_argument("--gib", type=float, default=1.0, help="input GiB per size (1.0 = the sweep configuration)")
    ap.add_argument("--plan", default="", help="N:variant,... plan overrides (default: the library's choice)")
    ap.add_argument("--tuning", default="", help="tuning JSON written by fft_onchip_gb300.tune to apply")
    ap.add_argument("--forms", default="config1,split,uneven,serve,onchip,cufft",
                    help="extra workloads measured after the sweep (comma list of: config1, split, uneven, serve, "
                         "onchip, cufft; empty for none)")
    ap.add_argument("--serve-rates", default="1e3,1e4,1e5,1e6", help="offered request rates (req/s) of the serving loop")
    ap.add_argument("--uneven-count", type=int, default=200000)
    return ap.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_table():
    """Per-launch DRAM bytes from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if _cuda_ok() else "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def _cuda_ok():
    import torch
    return torch.cuda.is_available()


def allreduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], device="cuda" if _cuda_ok() else "cpu", dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ----------------------------------------------------------------------------
# CPU baseline: the oracle's FP64 Stockham port on all host cores
# ----------------------------------------------------------------------------
def _timed(fn, x, seconds):
    """(transforms, seconds) of repeated fn(x) for at least `seconds`."""
    t0 = time.perf_counter()
    reps = 0
    while True:
        fn(x)
        reps += 1
        el = time.perf_counter() - t0
        if el >= seconds:
            return reps * x.shape[0], el


CPU_FRACTION = 32  # CPU samples: 1/32 of each size's 1 GiB batch (the reference arm's and cpu_baseline's)


def cpu_samples(sizes):
    from fft_onchip_gb300 import inputs
    return {n: inputs.normal(n, max(1, (GIB // (16 * n)) // CPU_FRACTION), seed=n) for n in sizes}


def cpu_sweep(fn, samples, sizes, seconds):
    """Rounds of fn over every size's sample (each size once per round, so the
    per-size weighting is the GPU `value`'s: transforms in proportion to
    1 GiB / (16 N)) until `seconds` have run; (FFT/s, per-size FFT/s, rounds)."""
    ffts, el, per, rounds = 0, 0.0, {n: [0, 0.0] for n in sizes}, 0
    while rounds == 0 or el < seconds:
        for n in sizes:
            t0 = time.perf_counter()
            fn(samples[n])
            dt = time.perf_counter() - t0
            ffts += samples[n].shape[0]
            el += dt
            per[n][0] += samples[n].shape[0]
            per[n][1] += dt
        rounds += 1
    return ffts / el, {str(n): round(v[0] / v[1], 1) for n, v in per.items()}, rounds


def cpu_sample_rate(sizes, seconds):
    """The port on all host threads (the baseline, measured as the reference
    arm measures it), plus two secondary points on the same samples: the
    port on one thread and numpy.fft (pocketfft, one thread), each for a
    third of the time."""
    import numpy as np
    from oracle import oracle as O
    threads = O.max_threads()
    samples = cpu_samples(sizes)
    for n in sizes:  # warm the pool and caches
        O.fft_f64(samples[n][: max(1, samples[n].shape[0] // 16)], threads=0)
    v_all, per_all, rounds = cpu_sweep(lambda x: O.fft_f64(x, threads=0), samples, sizes, seconds)
    v_one, per_one, _ = cpu_sweep(lambda x: O.fft_f64(x, threads=1), samples, sizes, seconds / 3)
    v_np, per_np, _ = cpu_sweep(lambda x: np.fft.fft(x, axis=1), samples, sizes, seconds / 3)
    return v_all, threads, per_all, {
        "rounds": rounds,
        "nproc": os.cpu_count(),
        "one_core": {"value": v_one, "cores": 1, "per_n": per_one},
        "numpy_fft": {"value": v_np, "cores": 1, "what": "numpy.fft.fft (pocketfft) on the same samples",
                      "per_n": per_np}}


def run_reference(args, world, rank):
    if rank != 0:
        return
    sizes = [int(s) for s in args.sizes.split(",")]
    from oracle import oracle as O
    threads = O.max_threads()
    samples = cpu_samples(sizes)
    fn = lambda x: O.fft_f64(x, threads=0)
    for _ in range(args.warmup):
        for n in sizes:
            fn(samples[n])
    t0 = time.perf_counter()
    ffts = 0
    for _ in range(args.steps):
        for n in sizes:
            fn(samples[n])
            ffts += samples[n].shape[0]
    el = time.perf_counter() - t0
    value = ffts / el
    desc = "1/%d of each size's 1 GiB batch per step (%s transforms)" % (
        CPU_FRACTION, "+".join(str(samples[n].shape[0]) for n in sizes))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "FFT/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample": desc, "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": "FFT/s", "cores": threads, "kind": "port",
                         "sample": desc},
        "e2e": {"value": value, "unit": "FFT/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------
def _plan_str(p):
    from fft_onchip_gb300.tune import code_str
    return "%s%s P=%d tpb=%d%s%s" % ("persistent " if p.get("persistent") else "", "x".join(map(str, p["radix"])),
                                     p["points_per_thread"], p["transforms_per_block"],
                                     " L2-prefetch" if p.get("prefetch") else "",
                                     (" " + code_str(p)) if p.get("code_flags") else "")


def run_ours(args, world, rank, local):
    import torch
    import fft_onchip_gb300 as F
    from oracle import oracle as O

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = F.load()
    sizes = [int(s) for s in args.sizes.split(",")]
    eng = F._engine_id(args.engine)
    if args.tuning:
        from fft_onchip_gb300 import tune as T
        T.load(args.tuning)
    for item in filter(None, args.plan.split(",")):
        pn, pv = item.split(":")
        F.plan_select(int(pn), eng if eng != F.ENGINE_AUTO else F.auto_engine(int(pn)), int(pv))
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    bufs = {}
    for n in sizes:
        batch = int(args.gib * GIB) // (16 * n)
        g = torch.Generator(device=dev).manual_seed(1000 * rank + n)
        x = torch.randn(batch, n, dtype=torch.complex128, device=dev, generator=g)
        y = torch.empty_like(x)
        bufs[n] = (x, y, batch)
    torch.cuda.synchronize()

    def launch(n):
        x, y, batch = bufs[n]
        if eng == F.ENGINE_AUTO:
            F.check(getattr(L, "fftoc_c2c_fwd_n%d" % n)(x.data_ptr(), y.data_ptr(), batch, sptr))
        else:
            F.check(L.fftoc_c2c_fwd_ex(n, x.data_ptr(), y.data_ptr(), batch, eng, sptr))

    for _ in range(max(3, args.warmup)):
        for n in sizes:
            launch(n)
    torch.cuda.synchronize()

    K = args.steps
    ev = {n: [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(K)]
          for n in sizes}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    sampler = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    e0.record(stream)
    for k in range(K):
        for n in sizes:
            ev[n][k][0].record(stream)
            launch(n)
            ev[n][k][1].record(stream)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    clocks = sampler.stop()
    t_ms = allreduce_max(e0.elapsed_time(e1), world)

    total_ffts = world * K * sum(bufs[n][2] for n in sizes)
    value = total_ffts / (t_ms * 1e-3)
    hbm, peak_kind = peaks()
    per_n, launch_ms = {}, {}
    for n in sizes:
        ms = [a.elapsed_time(b) for a, b in ev[n]]
        avg = float(np.mean(ms))
        launch_ms[n] = avg
        batch = bufs[n][2]
        gbs = 32.0 * n * batch / (avg * 1e-3) / 1e9
        per_n[str(n)] = {"batch": batch, "ms": round(avg, 4), "fft_per_s": batch / (avg * 1e-3),
                         "hbm_gbs": round(gbs, 1), "frac_hbm": round(gbs / hbm, 4)}
    dom = max(sizes, key=lambda n: launch_ms[n])
    dom_gbs = 32.0 * dom * bufs[dom][2] / (launch_ms[dom] * 1e-3) / 1e9
    # per-launch DRAM bytes from the committed capture, used only when it was
    # taken on the plan that ran here
    tt = traffic_table().get(str(dom), {})
    dom_plan = F.plan_query(dom, eng)
    ename = {F.ENGINE_FX: "fx", F.ENGINE_F64: "f64", F.ENGINE_DMMA: "dmma", F.ENGINE_SPLIT_BF16X3: "split_bf16x3",
             F.ENGINE_SPLIT_TF32X2: "split_tf32x2", F.ENGINE_SPLIT_EXACT: "split_exact"}.get(dom_plan["engine"], "?")
    traffic = tt.get(ename) if ename in ("fx", "f64") else None
    if tt.get("plan") != _plan_str(dom_plan):
        traffic = None
    elif traffic is not None:  # the table holds a 1 GiB launch; scale to this launch's transforms
        traffic = int(round(traffic * bufs[dom][2] / (GIB // (16 * dom))))
    roofline = {"bound": "hbm", "achieved": round(dom_gbs, 1), "peak": hbm, "unit": "GB/s",
                "frac": round(dom_gbs / hbm, 4), "traffic": traffic,
                "kernel": "N=%d %s plan %s" % (dom, ename, _plan_str(dom_plan)),
                "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind if peak_kind == "measured" else "fallback 6800 GB/s",
                "algorithmic_bytes_per_launch": 32 * dom * bufs[dom][2],
                "per_n": {str(n): {"achieved": per_n[str(n)]["hbm_gbs"], "frac": per_n[str(n)]["frac_hbm"]}
                          for n in sizes}}

    # correctness guard on the timed outputs: 64 transforms per size vs the oracle
    max_err = 0.0
    for n in sizes:
        x, y, batch = bufs[n]
        idx = torch.arange(0, batch, max(1, batch // 64), device=dev)[:64]
        ref = O.fft_f64(x[idx].cpu().numpy())
        max_err = max(max_err, O.rel_l2(y[idx].cpu().numpy(), ref))

    # end to end through fftoc_c2c_fwd_host, pinned host buffers
    e2e = None
    if not args.no_e2e:
        hb = max(bufs[n][2] * n for n in sizes)
        h_in = torch.empty(hb, dtype=torch.complex128, pin_memory=True)
        h_out = torch.empty(hb, dtype=torch.complex128, pin_memory=True)
        h_in.copy_(bufs[sizes[0]][0].reshape(-1)[:hb].cpu())
        for n in sizes:  # warm-up (allocates staging once)
            F.check(L.fftoc_c2c_fwd_host(n, h_in.data_ptr(), h_out.data_ptr(), bufs[n][2], eng, sptr))
        torch.cuda.synchronize()
        E = max(1, args.e2e_steps)
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(E):
            for n in sizes:
                F.check(L.fftoc_c2c_fwd_host(n, h_in.data_ptr(), h_out.data_ptr(), bufs[n][2], eng, sptr))
            stream.synchronize()
        el = allreduce_max(time.perf_counter() - t0, world)
        bytes_step = sum(bufs[n][2] * n * 16 for n in sizes)
        e2e = {"value": world * E * sum(bufs[n][2] for n in sizes) / el, "unit": "FFT/s",
               "h2d_bytes_per_step": bytes_step, "d2h_bytes_per_step": bytes_step,
               "steps": E, "ms_per_step": 1e3 * el / E, "path": "fftoc_c2c_fwd_host (pinned, 64 MiB chunks)"}
        del h_in, h_out

    forms = {}
    if "split" in args.forms.split(","):
        forms["split"] = bench_split(args, torch, F, dev, stream, world, per_n)
    if "uneven" in args.forms.split(","):
        forms["uneven"] = bench_uneven(args, torch, F, dev, stream, world)
    if "serve" in args.forms.split(",") and rank == 0:
        forms["serve"] = bench_serve(args, torch, F)
    if "onchip" in args.forms.split(",") and rank == 0:
        forms["onchip"] = bench_onchip(args, torch, F)
    if "config1" in args.forms.split(","):
        forms["config1"] = bench_config1(args, torch, F, dev, stream, world)
    if "cufft" in args.forms.split(","):
        forms["cufft"] = bench_cufft(args, torch, sizes, bufs, stream, per_n)

    cpu = None
    if rank == 0 and not args.no_cpu:
        v, cores, per, extra = cpu_sample_rate(sizes, args.cpu_seconds)
        cpu = {"value": v, "unit": "FFT/s", "cores": cores, "kind": "port",
               "sample": "oracle FP64 Stockham (radix-8/4/2) on 1/%d of each size's 1 GiB batch, every size once "
                         "per round (the weighting of value and of the reference arm), rounds for >= %.1f s"
                         % (CPU_FRACTION, args.cpu_seconds),
               "per_n": per}
        cpu.update(extra)

    if rank == 0:
        resolved = sorted({F.plan_query(n, eng)["engine"] for n in sizes})
        names = {F.ENGINE_FX: "int64 block fixed point (complex128 in/out)", F.ENGINE_F64: "f64",
                 F.ENGINE_SPLIT_BF16X3: "bf16x3 split on tensor cores, fp32 accumulation (complex128 in/out)",
                 F.ENGINE_SPLIT_TF32X2: "tf32x2 split on tensor cores, fp32 accumulation (complex128 in/out)",
                 F.ENGINE_DMMA: "f64 (FP64 tensor cores)",
                 F.ENGINE_SPLIT_EXACT: "int64 block fixed point, 8-bit digit slices exact on bf16 tensor cores "
                                       "(complex128 in/out)"}
        dtype = names.get(resolved[0], "mixed") if len(resolved) == 1 else "mixed"
        line = {
            "metric": METRIC, "value": value, "unit": "FFT/s", "n_gpus": world, "steps": K,
            "warmup": max(3, args.warmup), "ms_per_step": t_ms / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": dtype, "data": "synthetic",
            "config": {"workload": WORKLOAD, "sizes": sizes, "engine": args.engine,
                       "plans": {str(n): _plan_str(F.plan_query(n, eng)) for n in sizes},
                       "bytes_per_step": sum(32 * n * bufs[n][2] for n in sizes),
                       "l2": "inputs and outputs (1 GiB each per size) larger than L2; no flush",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "per_n": per_n, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": K * len(sizes), "clocks": clocks, "max_rel_err_vs_oracle": max_err,
            "forms": forms,
        }
        print(json.dumps(line), flush=True)


def bench_split(args, torch, F, dev, stream, world, per_n):
    """Split-precision form, N in {256, 512, 4096}, 1 GiB of complex128 per N:
    throughput of BF16x3, TF32x2 and the exact-slice form against the plain
    form (the sweep's default engine) and the IEEE binary64 engine on the
    same buffers; error
    against the binary64 oracle on 64-transform samples of two input
    families, (a) re/im N(0,1) and (b) |z| log-uniform in [1e-6, 1e6] with
    uniform phase."""
    from fft_onchip_gb300 import inputs
    from oracle import oracle as O
    L = F.load()
    hbm, _ = peaks()
    K = max(3, args.steps)
    out = {"workload": "split-precision form: N in {256,512,4096}, 1 GiB complex128 per N; errors on 64-transform "
                       "samples of families (a) N(0,1) and (b) log-uniform magnitudes [1e-6,1e6], uniform phase",
           "gate_rel_l2": 1e-11, "per_n": {}}
    sptr = stream.cuda_stream

    def timed(n, x, y, batch, eng):
        for _ in range(3):
            F.check(L.fftoc_c2c_fwd_ex(n, x.data_ptr(), y.data_ptr(), batch, eng, sptr))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(K):
            F.check(L.fftoc_c2c_fwd_ex(n, x.data_ptr(), y.data_ptr(), batch, eng, sptr))
        b.record(stream)
        torch.cuda.synchronize()
        return allreduce_max(a.elapsed_time(b), world) / K

    for n in (256, 512, 4096):
        batch = GIB // (16 * n)
        g = torch.Generator(device=dev).manual_seed(77 + n)
        x = torch.randn(batch, n, dtype=torch.complex128, device=dev, generator=g)
        y = torch.empty_like(x)
        row = {"batch": batch}
        for name, eng in (("plain", F.ENGINE_AUTO), ("f64", F.ENGINE_F64), ("split_bf16x3", F.ENGINE_SPLIT_BF16X3),
                          ("split_tf32x2", F.ENGINE_SPLIT_TF32X2), ("split_exact", F.ENGINE_SPLIT_EXACT)):
            ms = timed(n, x, y, batch, eng)
            gbs = 32.0 * n * batch / (ms * 1e-3) / 1e9
            row[name] = {"ms": round(ms, 4), "fft_per_s": world * batch / (ms * 1e-3), "hbm_gbs": round(gbs, 1),
                         "frac_hbm": round(gbs / hbm, 4)}
        for name in ("split_bf16x3", "split_tf32x2", "split_exact"):
            eng = F.ENGINES[name]
            errs = {}
            for fam, gen in (("a_normal", inputs.normal), ("b_loguniform", inputs.loguniform)):
                xs = gen(n, 64, seed=n)
                d = torch.from_numpy(xs).to(dev)
                ys = F.fft(d, engine=eng).cpu().numpy()
                ref = O.fft_f64(xs)
                errs[fam] = {"rel_l2": O.rel_l2(ys, ref), "max_abs": float(np.max(np.abs(ys - ref))),
                             "max_abs_ref": float(np.max(np.abs(ref)))}
            row[name]["error"] = errs
            row[name]["meets_gate"] = all(v["rel_l2"] <= 1e-11 for v in errs.values())
            row[name]["speedup_vs_plain"] = round(row["plain"]["ms"] / row[name]["ms"], 3)
            row[name]["speedup_vs_f64_engine"] = round(row["f64"]["ms"] / row[name]["ms"], 3)
        out["per_n"][str(n)] = row
        del x, y
    return out


def bench_config1(args, torch, F, dev, stream, world):
    """The small plain configuration: N = 64, batch 65,536 (64 MiB of
    complex128 in, L2-sized), re/im uniform [-1, 1) from seed 0, through the
    per-size entry point.  Cold: a 512 MiB write flushes L2 before each
    launch, and only the launch is timed (CUDA events around it).  Warm:
    launches back to back on L2-resident buffers.  The reference times its
    own driver with and without transfers (src/gpu_fft.cu:33-69)."""
    from fft_onchip_gb300 import inputs
    from oracle import oracle as O
    L = F.load()
    hbm, _ = peaks()
    n, batch = 64, 65536
    xh = inputs.uniform(n, batch, seed=0)
    x = torch.from_numpy(xh).to(dev)
    y = torch.empty_like(x)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    sptr = stream.cuda_stream
    K = max(10, args.steps)

    def launch():
        F.check(L.fftoc_c2c_fwd_n64(x.data_ptr(), y.data_ptr(), batch, sptr))

    for _ in range(3):
        launch()
    cold = []
    for r in range(K):
        flush.fill_(r & 0xFF)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        launch()
        b.record(stream)
        torch.cuda.synchronize()
        cold.append(a.elapsed_time(b))
    for _ in range(3):
        launch()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(K):
        launch()
    b.record(stream)
    torch.cuda.synchronize()
    warm = a.elapsed_time(b) / K
    idx = np.arange(0, batch, batch // 64)
    err = O.rel_l2(y.cpu().numpy()[idx], O.fft_f64(xh[idx]))
    out = {"workload": "N=64, batch 65536 (64 MiB in), uniform[-1,1) seed 0, fftoc_c2c_fwd_n64",
           "rel_l2_vs_oracle_64_samples": err}
    for name, ms in (("cold_l2_flushed", allreduce_max(float(np.median(cold)), world)),
                     ("warm_back_to_back", allreduce_max(warm, world))):
        gbs = 32.0 * n * batch / (ms * 1e-3) / 1e9
        out[name] = {"ms": round(ms, 5), "fft_per_s": world * batch / (ms * 1e-3), "hbm_gbs": round(gbs, 1),
                     "frac_hbm": round(gbs / hbm, 4)}
    del x, y, flush
    return out


def bench_cufft(args, torch, sizes, bufs, stream, per_n):
    """The device library on the same buffers: cuFFT's batched Z2Z forward
    transform (through torch.fft.fft), the stand-in for the reference's
    cuFFTDx path; CUDA events, 1 GiB per size, same algorithmic bytes."""
    hbm, _ = peaks()
    out = {"workload": "cuFFT Z2Z forward (torch.fft.fft) on the sweep's buffers", "per_n": {}}
    K = max(3, args.steps)
    for n in sizes:
        x, _, batch = bufs[n]
        for _ in range(3):
            y = torch.fft.fft(x, dim=-1)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(K):
            y = torch.fft.fft(x, dim=-1)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / K
        gbs = 32.0 * n * batch / (ms * 1e-3) / 1e9
        out["per_n"][str(n)] = {"ms": round(ms, 4), "hbm_gbs": round(gbs, 1), "frac_hbm": round(gbs / hbm, 4),
                                "fftoc_speedup": round(per_n[str(n)]["hbm_gbs"] / gbs, 3)}
        del y
    return out


def bench_onchip(args, torch, F):
    """On-chip repeat mode (the reference's own timing method,
    includes/testing.cuh:94-127): microseconds per in-shared-memory pass over
    32 x SMs transforms, t(1100 repeats) - t(100 repeats) over 1000."""
    from fft_onchip_gb300 import onchip
    out = {"workload": "on-chip repeat mode: (32 x SMs) transforms per pass resident in shared memory, "
                       "(t(1100) - t(100)) / 1000 per pass, no HBM traffic in the difference", "per_n": {}}
    for n in (8, 16, 64, 128, 256, 512, 4096):
        r = onchip.time_onchip(n, F.ENGINE_AUTO)
        out["per_n"][str(n)] = {k: r[k] for k in ("us_per_pass", "ffts_per_s", "transforms_per_block", "blocks")}
    return out


def bench_uneven(args, torch, F, dev, stream, world):
    """Mixed-size batch: `count` transforms, N in 8..4096 with P ~ 1/log2 N,
    packed back to back with an int64 offset table, re/im uniform [-1, 1).
    One CUDA graph per batch (device bucketing + one persistent kernel per
    size) against one launch per size after a host read of the counts."""
    from fft_onchip_gb300 import inputs
    count = args.uneven_count
    ns = inputs.uneven_sizes(count, seed=0)
    off, total = inputs.uneven_layout(ns)
    g = torch.Generator(device=dev).manual_seed(4)
    x = torch.view_as_complex(torch.rand(total, 2, dtype=torch.float64, device=dev, generator=g) * 2 - 1)
    y = torch.empty_like(x)
    d_off = torch.from_numpy(off).to(dev)
    d_ns = torch.from_numpy(ns).to(dev)
    plan = F.UnevenPlan(count)
    algo_bytes = 32 * int(ns.astype(np.int64).sum())
    out = {"workload": "uneven batch: %d transforms, N in 8..4096 with P ~ 1/log2(N), int64 offset table, "
                       "uniform[-1,1) values, %.2f GiB in" % (count, total * 16 / GIB),
           "count": count, "algorithmic_bytes": algo_bytes,
           "per_size_counts": {str(n): int(np.sum(ns == n)) for n in inputs.SIZES}}
    K = max(3, args.steps)
    for mode, per_size in (("graph", False), ("per_size_launches", True)):
        for _ in range(3):
            plan(x, d_off, d_ns, out=y, stream=stream, per_size=per_size)
        torch.cuda.synchronize()
        barrier(world)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(K):
            plan(x, d_off, d_ns, out=y, stream=stream, per_size=per_size)
        b.record(stream)
        torch.cuda.synchronize()
        ms = allreduce_max(a.elapsed_time(b), world) / K
        hbm, _ = peaks()
        out[mode] = {"ms": round(ms, 4), "fft_per_s": world * count / (ms * 1e-3),
                     "hbm_gbs": round(algo_bytes / (ms * 1e-3) / 1e9, 1),
                     "frac_hbm": round(algo_bytes / (ms * 1e-3) / 1e9 / hbm, 4)}
    out["graph_speedup_vs_per_size"] = round(out["per_size_launches"]["ms"] / out["graph"]["ms"], 3)
    out["graph_grids_set_on_device"] = plan.device_sized()
    out["gpu_launches_per_step"] = {"graph": 1 + 3 + len(inputs.SIZES),
                                    "per_size_launches": 1 + 3 + int(sum(1 for n in inputs.SIZES if np.any(ns == n)))}
    plan.close()
    del x, y
    return out


def bench_serve(args, torch, F):
    """Serving loop: Poisson arrivals at each offered rate, each request 1..4096
    transforms (log-uniform) of one N (uniform over 8..4096), N(0,1)-sized
    values from pinned host memory; 8 GiB device pool with admission by
    bytes; latency = completion - scheduled arrival."""
    from fft_onchip_gb300 import inputs
    from fft_onchip_gb300.serve import Server, latency_summary, make_trace
    arena = 1 << 25  # complex values (512 MiB) per arena; the largest request is 2^24
    h_in = torch.empty(arena, dtype=torch.complex128, pin_memory=True)
    h_in.copy_(torch.randn(arena, dtype=torch.complex128, generator=torch.Generator().manual_seed(5)))
    h_out = torch.empty(arena, dtype=torch.complex128, pin_memory=True)
    srv = Server(pool_bytes=8 << 30, slots=4, max_batch_bytes=256 << 20, max_wait_us=50.0)
    tags = (F.ENGINE_AUTO, F.ENGINE_SPLIT_BF16X3)
    warm, _, _ = make_trace(1e4, 64, arena, seed=99, engines=tags)
    srv.replay(warm, h_in, h_out)
    out = {"workload": "Poisson arrivals; request = 1..4096 transforms (log-uniform) of one N uniform over "
                       "8..4096; N(0,1) values in pinned host memory; 8 GiB device pool, admission by bytes; "
                       "4 batches in flight, 256 MiB per batch, 50 us batching window",
           "tag": "50/50 plain FP64 form (engine auto) / split form BF16x3 (8-point requests always plain)",
           "rates": []}
    for rate in [float(r) for r in args.serve_rates.split(",") if r]:
        m = int(min(2000, max(200, rate * 0.4)))
        items, transforms, nbytes = make_trace(rate, m, arena, seed=int(rate) % 1000003, engines=tags)
        before = srv.stats()
        lat, wall = srv.replay(items, h_in, h_out)
        after = srv.stats()
        row = {"offered_req_per_s": rate, "requests": m, "achieved_req_per_s": m / wall,
               "fft_per_s": transforms / wall, "host_link_gbs_each_way": nbytes / wall / 1e9,
               "batches": after["batches"] - before["batches"], "max_inflight_batches": after["max_inflight_batches"]}
        row.update(latency_summary(lat))
        out["rates"].append(row)
    srv.close()
    return out


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
