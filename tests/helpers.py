"""Shared helpers of the parity tests (test infrastructure)."""
import numpy as np


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.sqrt(np.sum(np.abs(b) ** 2))
    num = np.sqrt(np.sum(np.abs(a - b) ** 2))
    if den == 0.0:
        return float(num)
    return float(num / den)


def random_fields(deck, seed, scale_e=1.0e9, scale_b=3.0):
    """Smooth-ish random mode fields, same on both sides of a parity test."""
    rng = np.random.default_rng(seed)
    shape = (deck.n_mode, deck.ny + 10, deck.nx + 10)
    out = {}
    for name, s in (("exm", scale_e), ("erm", scale_e), ("etm", scale_e),
                    ("bxm", scale_b), ("brm", scale_b), ("btm", scale_b)):
        a = (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)) * s
        out[name] = a
    return out


def match_by_id(pa, pb):
    a = pa.sorted_by_id()
    b = pb.sorted_by_id()
    assert np.array_equal(a.id, b.id), "particle id sets differ"
    return a, b
