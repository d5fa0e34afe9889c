"""Seeded synthetic inputs (host side, numpy).

Counter-based SplitMix64: value i of stream `seed` is mix(seed + (i+1)*golden),
so any slice of a stream can be generated independently and identically on
every machine.  Layout of every generator's result: complex128 (batch, n),
re and im drawn from consecutive counter values (2*idx, 2*idx+1).

The reference draws unseeded std::uniform_real_distribution<float>(0, 1)
values (src/gpu_fft.cu:17-25); these generators are seeded so results can be
reproduced and checked.
"""
import numpy as np

_G = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed, start, count):
    """uint64 stream values start..start+count-1."""
    with np.errstate(over="ignore"):
        i = np.arange(start + 1, start + 1 + count, dtype=np.uint64)
        z = np.uint64(seed) + i * _G
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def _u01(seed, start, count):
    """uniform [0, 1) doubles with 53 random bits."""
    return (splitmix64(seed, start, count) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def uniform(n, batch, seed=0):
    """re, im i.i.d. uniform [-1, 1): (z >> 11) * 2^-52 - 1, exact in binary64."""
    v = (splitmix64(seed, 0, 2 * n * batch) >> np.uint64(11)).astype(np.float64) * (2.0 ** -52) - 1.0
    return v.view(np.complex128).reshape(batch, n)


def normal(n, batch, seed=0):
    """re, im i.i.d. N(0, 1) by Box-Muller on two uniform streams."""
    m = n * batch
    u1 = _u01(seed, 0, m)
    u2 = _u01(seed ^ 0x5DEECE66D, 0, m)
    r = np.sqrt(-2.0 * np.log1p(-u1))
    out = np.empty(2 * m, dtype=np.float64)
    out[0::2] = r * np.cos(2 * np.pi * u2)
    out[1::2] = r * np.sin(2 * np.pi * u2)
    return out.view(np.complex128).reshape(batch, n)


def loguniform(n, batch, seed=0, lo=1e-6, hi=1e6):
    """|z| log-uniform in [lo, hi], phase uniform in [0, 2*pi)."""
    m = n * batch
    u1 = _u01(seed, 0, m)
    u2 = _u01(seed ^ 0x2545F4914F6CDD1D, 0, m)
    mag = np.exp(np.log(lo) + u1 * (np.log(hi) - np.log(lo)))
    z = mag * np.exp(2j * np.pi * u2)
    return z.astype(np.complex128).reshape(batch, n)


SIZES = (8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096)


def uneven_sizes(count, seed=0):
    """Transform sizes for an uneven batch: N from {8, ..., 4096} with
    probability proportional to 1/log2(N) (inverse-CDF on a SplitMix64
    uniform stream).  int32 array of length `count`."""
    w = np.array([1.0 / np.log2(n) for n in SIZES])
    cdf = np.cumsum(w / w.sum())
    cdf[-1] = 1.0
    u = _u01(seed ^ 0x1F83D9ABFB41BD6B, 0, count)
    return np.asarray(SIZES, dtype=np.int32)[np.searchsorted(cdf, u, side="right")]


def uneven_layout(ns):
    """Back-to-back packing of transforms of sizes ns: (int64 offsets in
    complex elements, total elements)."""
    ns = np.asarray(ns, dtype=np.int64)
    off = np.zeros(len(ns), dtype=np.int64)
    if len(ns) > 1:
        np.cumsum(ns[:-1], out=off[1:])
    return off, int(ns.sum())


def uniform_flat(total, seed=0):
    """`total` complex values, re and im i.i.d. uniform [-1, 1) (the stream of
    `uniform`)."""
    v = (splitmix64(seed, 0, 2 * total) >> np.uint64(11)).astype(np.float64) * (2.0 ** -52) - 1.0
    return v.view(np.complex128)


FAMILIES = {"uniform": uniform, "normal": normal, "loguniform": loguniform}
