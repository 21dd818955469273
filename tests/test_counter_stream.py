"""The counter stream of device loading and device window injection (CPU).

- The product's Philox4x32-10 block (cyl_counter_block, the host build of
  the device code) equals the oracle's independent restatement, bit for bit.
- The stream's words are uniform and uncorrelated (chi-square and lag-1
  bounds at the 1e-4 tail).
- The oracle's counter loader and counter injector make the reference
  loader's counts, ids and per-cell occupancy exactly (integer particles per
  cell), and its weight and momentum distributions within sampling error:
  total weight within 2e-3 relative (positions move weights by a few % each,
  averaged over > 8000 particles), thermal spread within 5 / sqrt(2 n) of
  sqrt(kB T m), means within 5 sigma / sqrt(n) of the drift.
"""
import ctypes as C

import numpy as np

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi
from cylindrical_epoch_gb300.lib import load

KB = 1.3806488e-23


def _blocks(fn, seed, ctrs):
    out = np.zeros((len(ctrs), 4), dtype=np.uint64)
    o = (C.c_uint32 * 4)()
    for i, c in enumerate(ctrs):
        assert fn(seed, (C.c_uint32 * 4)(*[int(v) for v in c]), o) == 0
        out[i] = list(o)
    return out


def test_counter_block_matches_oracle():
    from oracle.oracle import load as oload
    lib, olib = load(), oload()
    rng = np.random.default_rng(5)
    for _ in range(20):
        seed = int(rng.integers(0, 2**63))
        ctrs = rng.integers(0, 2**32, size=(50, 4), dtype=np.uint64)
        assert np.array_equal(_blocks(lib.cyl_counter_block, seed, ctrs),
                              _blocks(olib.orc_counter_block, seed, ctrs))


def test_counter_words_uniform_and_uncorrelated():
    lib = load()
    n = 1 << 14
    ctrs = np.stack([np.arange(n), np.zeros(n), np.zeros(n), np.ones(n)], axis=1).astype(np.uint64)
    w = _blocks(lib.cyl_counter_block, 7842432, ctrs)
    u = (w.astype(np.float64) + 0.5) * 2.0**-32
    for k in range(4):
        h, _ = np.histogram(u[:, k], bins=64, range=(0.0, 1.0))
        chi2 = float(np.sum((h - n / 64) ** 2 / (n / 64)))
        assert chi2 < 120.0, (k, chi2)  # 63 degrees of freedom: P(chi2 > 120) ~ 1e-5
        c = np.corrcoef(u[:-1, k], u[1:, k])[0, 1]
        assert abs(c) < 4.0 / np.sqrt(n), (k, c)
    assert abs(np.corrcoef(u[:, 0], u[:, 1])[0, 1]) < 4.0 / np.sqrt(n)


def _moments_ok(p, deck):
    s = deck.species[0]
    for k, comp in enumerate(("px", "py", "pz")):
        v = getattr(p, comp)
        sd = np.sqrt(KB * s.temp_k[k] * s.mass)
        if sd == 0.0:
            assert np.all(v == 0.0)
            continue
        assert abs(v.mean()) < 5.0 * sd / np.sqrt(v.size), comp
        assert abs(v.std() / sd - 1.0) < 5.0 / np.sqrt(2 * v.size), comp


def test_counter_loader_matches_reference_loader():
    from oracle.oracle import Oracle
    for deck in (cg.thermal_plasma(nx=64, ny=32, ppc=4), cg.thermal_plasma(nx=64, ny=32, ppc=4.5),
                 cg.wakefield(nx=128, ny=32, ppc=2.5, density=3.0e24, ramp=2.0e-6)):
        k = Oracle(deck, load_species=True)
        c = Oracle(deck, counter_seed=11)
        pk, pc = k.particles(0), c.particles(0)
        assert pc.n == pk.n
        assert np.array_equal(np.sort(pc.id), np.arange(pk.n))
        assert abs(pc.w.sum() / pk.w.sum() - 1.0) < 2e-3
        _moments_ok(pc, deck)
        if float(deck.species[0].npart_per_cell).is_integer():
            kx, ky = k.cell_indices(0)
            cx, cy = c.cell_indices(0)
            assert np.array_equal(np.unique(np.stack([kx, ky]), axis=1, return_counts=True)[1],
                                  np.unique(np.stack([cx, cy]), axis=1, return_counts=True)[1])
        # a different seed gives different particles with the same counts
        c2 = Oracle(deck, counter_seed=12)
        assert c2.particles(0).n == pc.n and not np.array_equal(c2.particles(0).x, pc.x)


def test_counter_injection_matches_reference_injection():
    """A windowed wakefield stepped by the oracle with each stream: the same
    shifts and the same injected count (ids above the loaded range), the
    injected particles' total weight within 2e-3 and their radii uniform in
    their rows."""
    from oracle.oracle import Oracle
    deck = cg.wakefield(nx=128, ny=32, ppc=4, density=3.0e24, ramp=2.0e-6)
    deck.window_start_time = 20 * 5.0e-17
    k = Oracle(deck, load_species=True)
    c = Oracle(deck, counter_seed=3)
    n0 = k.particles(0).n
    for o in (k, c):
        o.initialise()
        o.step(60)
    sk, sc = k.state(), c.state()
    assert sk.n_shifts == sc.n_shifts > 10
    pk, pc = k.particles(0), c.particles(0)
    ik, ic = pk.id >= n0, pc.id >= n0
    assert ik.sum() == ic.sum() == sk.n_shifts * deck.ny * 4
    assert np.array_equal(np.sort(pc.id[ic]), np.arange(n0, n0 + ic.sum()))
    assert abs(pc.w[ic].sum() / pk.w[ik].sum() - 1.0) < 2e-3
    dy = deck.y_max / deck.ny
    r = np.sqrt(pc.y[ic] ** 2 + pc.z[ic] ** 2) / dy
    frac = r - np.floor(r)
    assert abs(frac.mean() - 0.5) < 5.0 / np.sqrt(12.0 * frac.size)
