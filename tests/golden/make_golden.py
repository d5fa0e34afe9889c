"""Generate the golden vectors in tests/golden/ (run once; outputs committed).

The reference ships no golden vectors or known-answer tests (its only check,
src/gpu_fft.cu:41-66, prints an MSE against cuFFTDx).  These fixtures are the
forward DFT of the reference's convention (includes/reference.cuh:10-12:
C2C, forward, unnormalised, natural order) evaluated in 50-digit arithmetic
(mpmath) and rounded to binary64:

  impulse      x[n] = delta[n]                 -> X[k] = 1
  shift        x[n] = delta[n - m], m = 3      -> X[k] = W^{mk}
  constant     x[n] = 0.5 - 0.25i              -> X[0] = N*c, else 0
  tone         x[n] = exp(+2 pi i k0 n / N)    -> X[k0] = N (k0 = N/4 + 1)
  uniform      two seeded uniform[-1,1) rows (SplitMix64 seed 1234), N <= 512

Usage: python tests/golden/make_golden.py
"""
import os
import sys

import mpmath as mp
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from fft_onchip_gb300 import inputs  # noqa: E402

SIZES = (8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096)
mp.mp.dps = 50


def w(n, e):
    """exp(-2 pi i e / n) at 50 digits."""
    a = -2 * mp.pi * mp.mpf(e % n) / n
    return mp.mpc(mp.cos(a), mp.sin(a))


def dft_exact(x):
    n = len(x)
    tw = [w(n, k) for k in range(n)]
    xs = [mp.mpc(float(v.real), float(v.imag)) for v in x]
    out = np.empty(n, dtype=np.complex128)
    for k in range(n):
        s = mp.mpc(0)
        for j in range(n):
            if xs[j] != 0:
                s += xs[j] * tw[(j * k) % n]
        out[k] = complex(float(s.real), float(s.imag))
    return out


def make(n):
    names, xs, ys = [], [], []
    # impulse
    x = np.zeros(n, np.complex128); x[0] = 1
    names.append("impulse"); xs.append(x); ys.append(np.ones(n, np.complex128))
    # shifted impulse
    m = 3 % n
    x = np.zeros(n, np.complex128); x[m] = 1
    y = np.array([complex(float(w(n, m * k).real), float(w(n, m * k).imag)) for k in range(n)])
    names.append("shift3"); xs.append(x); ys.append(y)
    # constant
    c = 0.5 - 0.25j
    x = np.full(n, c, np.complex128)
    y = np.zeros(n, np.complex128); y[0] = n * c
    names.append("constant"); xs.append(x); ys.append(y)
    # tone (input rounded to binary64; expected output is the analytic N*delta)
    k0 = n // 4 + 1
    x = np.array([complex(float(v.real), float(v.imag)) for v in (w(n, -k0 * j) for j in range(n))])
    y = np.zeros(n, np.complex128); y[k0] = n
    names.append("tone"); xs.append(x); ys.append(y)
    # seeded uniform rows, exact DFT
    if n <= 512:
        u = inputs.uniform(n, 2, seed=1234)
        for r in range(2):
            names.append("uniform%d" % r); xs.append(u[r]); ys.append(dft_exact(u[r]))
    return np.array(names), np.stack(xs), np.stack(ys)


def main():
    for n in SIZES:
        names, x, y = make(n)
        np.savez_compressed(os.path.join(HERE, "kat_%d.npz" % n), names=names, x=x, y=y)
        print("kat_%d.npz" % n, len(names))


if __name__ == "__main__":
    main()
