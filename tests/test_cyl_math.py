"""The portable atan2 of include/cyl_math.h (shared by the FP64 kernel and
the oracle) against libm's atan2: at most 2 ulp apart on a sweep of
quadrants, magnitudes and the small-angle region the deposit uses."""
import math

import numpy as np


def test_atan2_close_to_libm():
    from oracle.oracle import load
    lib = load()
    rng = np.random.default_rng(7)
    ys = np.concatenate([rng.standard_normal(20000), rng.standard_normal(2000) * 1e-12,
                         [0.0, -0.0, 1.0, -1.0, 1e-300, -1e300]])
    xs = np.concatenate([rng.standard_normal(20000), rng.standard_normal(2000),
                         [1.0, -1.0, 0.0, -0.0, 1.0, 1.0]])
    worst = 0.0
    for y, x in zip(ys, xs):
        a = lib.orc_atan2(float(y), float(x))
        b = math.atan2(float(y), float(x))
        if a == b:
            continue
        ulp = math.ulp(b) if b != 0 else 5e-324
        worst = max(worst, abs(a - b) / ulp)
    assert worst <= 2.0, worst


def test_atan2_special_values():
    from oracle.oracle import load
    lib = load()
    for y, x in [(0.0, 1.0), (-0.0, 1.0), (0.0, -1.0), (-0.0, -1.0), (1.0, 0.0), (-1.0, 0.0),
                 (0.0, 0.0), (0.0, -0.0), (-0.0, -0.0)]:
        a = lib.orc_atan2(y, x)
        b = math.atan2(y, x)
        assert a == b and math.copysign(1, a) == math.copysign(1, b), (y, x, a, b)
