"""CPU tests pinning the oracle to the reference's ACTUAL outputs.

tests/golden/ref_out_*.npz hold inputs and outputs of the reference's own
executors (includes/tensor_fft_*.cuh, legacy8_fft.cuh, legacy16_fft.cuh)
compiled unmodified from the reference's headers into a cubin and run on a
GB300 by oracle/ref_runner.py (`python -m oracle.ref_runner fixtures`).

Two things are pinned:
  1. the oracle's lane-exact restatements, run with the reference's own
     twiddle sources, reproduce those outputs;
  2. the exact DFT oracle (sign, natural order, no scaling) agrees with every
     reference executor to that executor's own accuracy (FP32 sincospif
     twiddles ~3e-8, the 6-digit table ~6e-7, 12-digit constants ~1e-12),
     except tensor_fft_4096, whose output is not the DFT.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden")

# executor: (restatement, tolerance restatement-vs-reference, DFT accuracy bound)
CASES = {
    "tensor_fft_8": ("tensor", 1e-14, 3e-8),
    "tensor_fft_64": ("tensor", 5e-8, 1e-7),
    "tensor_fft_128": ("tensor", 5e-8, 1e-7),
    "tensor_fft_256": ("tensor", 1e-14, 2e-6),
    "tensor_fft_512": ("tensor", 5e-8, 1e-7),
    "legacy8_fft_8": ("legacy8", 1e-14, 1e-11),
    "legacy8_fft_64": ("legacy8", 1e-14, 1e-11),
    "legacy8_fft_512": ("legacy8", 1e-14, 1e-11),
    "legacy8_fft_4096": ("legacy8", 1e-14, 1e-11),
    "legacy16_fft_16": ("legacy16", 1e-14, 1e-11),
    "legacy16_fft_256": ("legacy16", 1e-14, 1e-11),
    "legacy16_fft_4096": ("legacy16", 1e-14, 1e-11),
}


def load(name):
    d = np.load(os.path.join(GOLD, "ref_out_%s.npz" % name))
    return d["x"], d["y"]


def restate(kind, x):
    return {"tensor": O.ref_tensor, "legacy8": O.ref_legacy8, "legacy16": O.ref_legacy16}[kind](x, exact=False)


@pytest.mark.parametrize("name", sorted(CASES))
def test_restatement_reproduces_reference_outputs(name):
    kind, tol, _ = CASES[name]
    x, y = load(name)
    assert O.rel_l2(restate(kind, x), y) < tol


@pytest.mark.parametrize("name", sorted(CASES))
def test_reference_computes_the_forward_dft(name):
    """Convention pin: the exact oracle agrees with the reference's outputs to
    the reference's own accuracy (no sign flip, reordering or scaling)."""
    _, _, acc = CASES[name]
    x, y = load(name)
    e = O.rel_l2(y, O.fft_ld(x))
    assert e < acc, e
    # and a wrong convention would be O(1) off
    assert O.rel_l2(y, np.fft.ifft(x, axis=1) * x.shape[1]) > 0.5
    assert O.rel_l2(y, O.fft_ld(x) / x.shape[1]) > 0.5


def test_reference_tensor_fft_4096_output_is_not_the_dft():
    """The reference's tensor_fft_4096 (never run upstream) returns O(1)-wrong
    results on the GPU; the lane-exact restatement reproduces exactly that."""
    x, y = load("tensor_fft_4096")
    assert O.rel_l2(y, O.fft_ld(x)) > 0.5
    assert O.rel_l2(O.ref_tensor(x, exact=False), y) < 5e-8
