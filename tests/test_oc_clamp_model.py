"""The OC bisection's clamp (oc_clamp in csrc/tp_kernels_design.cu), restated
on bit patterns: max(lo, min(hi, v)) for 0 <= lo <= hi finite as integer
comparisons of the doubles' bit patterns must give exactly what fmax/fmin give
(fmin ignores a NaN v) for every v, including NaN of either sign, +-0 and
+-inf -- the bisection then takes the same decisions as with the FP64 min/max."""
import struct

import numpy as np

INF = 0x7FF0000000000000
MASK = 0x7FFFFFFFFFFFFFFF


def bits(x):
    return struct.unpack("<q", struct.pack("<d", x))[0]


def from_bits(i):
    return struct.unpack("<d", struct.pack("<q", i))[0]


def oc_clamp(lo, hi, v):
    iv = bits(v)
    if iv < 0:
        iv = INF if (iv & MASK) > INF else 0
    elif iv > INF:
        iv = INF
    il, ih = bits(lo), bits(hi)
    iv = min(iv, ih)
    return from_bits(max(iv, il))


def reference(lo, hi, v):
    m = hi if np.isnan(v) else min(hi, v)  # CUDA fmin returns the non-NaN operand
    return max(lo, m)


def test_clamp_matches_fmin_fmax():
    rng = np.random.default_rng(0)
    special = [0.0, -0.0, float("nan"), -float("nan"), float("inf"), -float("inf"), -1.0, 1e-300, 5e-324, 0.3,
               2.0]
    assert bits(-float("nan")) < 0 < bits(float("nan"))  # NaN of both signs is covered
    n = 0
    for _ in range(20000):
        x = float(rng.uniform(0, 1))
        lo, hi = max(0.0, x - 0.2), min(1.0, x + 0.2)
        if rng.uniform() < 0.3:
            v = special[int(rng.integers(len(special)))]
        else:
            v = float(rng.uniform(-1, 2)) * 10.0 ** int(rng.integers(-5, 3))
        a, b = oc_clamp(lo, hi, v), reference(lo, hi, v)
        assert a == b, (lo, hi, v, a, b)
        n += 1
    assert n == 20000


def test_clamp_at_the_bounds():
    for lo, hi in ((0.0, 0.4), (0.1, 0.5), (0.8, 1.0), (0.0, 1.0)):
        for v in (lo, hi, 0.5 * (lo + hi), -0.0, 0.0, 1.0, float("inf"), float("nan")):
            assert oc_clamp(lo, hi, v) == reference(lo, hi, v)
