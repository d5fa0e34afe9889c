"""The JSON line bench.py prints for this library's arm carries every key of
its contract, with consistent values, on a reduced configuration (two sizes,
small batches, one serving rate, short CPU sample)."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_line_has_the_contract_keys(cuda, fftoc_lib):
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--sizes", "64,4096", "--gib", "0.125", "--steps", "3",
           "--warmup", "3", "--e2e-steps", "1", "--cpu-seconds", "0.2", "--forms", "config1,split,uneven,serve,onchip,cufft",
           "--serve-rates", "1e3", "--uneven-count", "20000"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "roofline", "cpu_baseline", "e2e", "gpu_launches", "clocks"):
        assert k in d, k
    assert d["value"] > 0 and d["unit"] == "FFT/s" and d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] >= 3
    assert d["higher_is_better"] is True and d["scaling"] == "weak"
    assert "workload" in d["config"] and set(d["config"]["plans"]) == {"64", "4096"}
    rl = d["roofline"]
    assert rl["bound"] == "hbm" and rl["unit"] == "GB/s" and rl["peak"] > 0
    assert abs(rl["frac"] - rl["achieved"] / rl["peak"]) < 1e-3
    assert rl["traffic"] is None or rl["traffic"] > 0
    assert set(rl["per_n"]) == {"64", "4096"} and all(0 < v["frac"] < 1.5 for v in rl["per_n"].values())
    cpu = d["cpu_baseline"]
    assert cpu["value"] > 0 and cpu["cores"] >= 1 and cpu["kind"] == "port" and cpu["sample"]
    assert cpu["one_core"]["value"] > 0 and cpu["numpy_fft"]["value"] > 0
    e2e = d["e2e"]
    assert e2e["value"] > 0 and e2e["unit"] == "FFT/s"
    assert e2e["h2d_bytes_per_step"] == e2e["d2h_bytes_per_step"] > 0
    assert d["gpu_launches"] > 0
    assert d["clocks"]["sm_mhz"] > 0
    assert d["max_rel_err_vs_oracle"] < 1e-13
    for n in ("64", "4096"):
        p = d["per_n"][n]
        assert p["fft_per_s"] > 0 and 0 < p["frac_hbm"] < 1.5
    f = d["forms"]
    assert set(f) == {"config1", "split", "uneven", "serve", "onchip", "cufft"}
    c1 = f["config1"]
    assert c1["rel_l2_vs_oracle_64_samples"] < 1e-13
    assert c1["cold_l2_flushed"]["fft_per_s"] > 0 and c1["warm_back_to_back"]["fft_per_s"] > 0
    assert f["split"]["per_n"]["4096"]["split_exact"]["meets_gate"] is True
    assert f["uneven"]["graph"]["fft_per_s"] > 0
    assert f["serve"]["rates"][0]["p99_ms"] >= f["serve"]["rates"][0]["p50_ms"] > 0
