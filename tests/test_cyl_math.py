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


def test_sincos_turn_close_to_exact():
    """cyl_sincos_turn(u) = (sin 2 pi u, cos 2 pi u) for the counter stream's
    u = (r + 1/2) 2^-32: within 4e-16 absolute (about two ulp of 1) of the
    values computed to 30 digits, across all four quadrants."""
    import ctypes as C
    import mpmath
    from oracle.oracle import load
    lib = load()
    mpmath.mp.dps = 30
    rng = np.random.default_rng(11)
    rs = np.concatenate([rng.integers(0, 2**32, size=3000), [0, 2**30 - 1, 2**30, 2**31, 3 * 2**30, 2**32 - 1]])
    s, c = C.c_double(), C.c_double()
    worst = 0.0
    for r in rs:
        u = (float(r) + 0.5) * 2.0**-32
        lib.orc_sincos_turn(u, C.byref(s), C.byref(c))
        es = float(mpmath.sin(2 * mpmath.pi * mpmath.mpf(u)))
        ec = float(mpmath.cos(2 * mpmath.pi * mpmath.mpf(u)))
        worst = max(worst, abs(s.value - es), abs(c.value - ec))
    assert worst < 4e-16, worst
