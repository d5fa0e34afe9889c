"""Thread safety of the C ABI: host threads on their own streams call the
entry points concurrently from a cold start (the per-device set-up races),
results match the oracle, and error messages stay per thread.  Runs in a
fresh process so that the library's first use happens under contention."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r'''
import sys, threading
import numpy as np
import torch
sys.path.insert(0, ROOT)
import fft_onchip_gb300 as F
from fft_onchip_gb300 import inputs
from oracle import oracle as O

torch.cuda.set_device(0)
SIZES = [8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096]
start = threading.Barrier(len(SIZES) + 1, timeout=120)
errors = []

def work(i, n):
    try:
        torch.cuda.set_device(0)
        s = torch.cuda.Stream()
        x = inputs.normal(n, max(4, 8192 // n), seed=i)
        ref = O.fft_f64(x)
        d = torch.from_numpy(x).cuda()
        torch.cuda.synchronize()
        start.wait()
        with torch.cuda.stream(s):
            for _ in range(10):
                y = F.fft(d, engine="auto", stream=s)
        s.synchronize()
        assert O.rel_l2(y.cpu().numpy(), ref) < 1e-13, ("device", n)
        h = F.fft_host(x) if i % 2 == 0 else None
        if h is not None:
            assert O.rel_l2(h, ref) < 1e-13, ("host", n)
    except Exception as e:
        errors.append(repr(e))

def bad_caller():
    L = F.load()
    start.wait()
    st = L.fftoc_c2c_fwd(60, None, None, 1, None)
    msg = L.fftoc_last_error_string().decode()
    if st != 1 or "60" not in msg:
        errors.append("bad call: %d %r" % (st, msg))

threads = [threading.Thread(target=work, args=(i, n)) for i, n in enumerate(SIZES)]
threads.append(threading.Thread(target=bad_caller))
for t in threads:
    t.start()
for t in threads:
    t.join()
msg = F.load().fftoc_last_error_string().decode()
if "60" in msg:
    errors.append("another thread's message leaked: %r" % msg)
print("ERRORS" if errors else "OK", errors)
sys.exit(1 if errors else 0)
'''


def test_concurrent_threads_from_cold_start(cuda):
    code = "ROOT = %r\n" % ROOT + CHILD
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0 and "OK" in r.stdout, (r.stdout[-2000:], r.stderr[-3000:])
