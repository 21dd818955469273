"""Host-side logic of the product library against the oracle (CPU only).

The loader and the KISS stream of libcylpic.so (host code, no GPU needed)
must reproduce the oracle's loader bit for bit; the decks' time steps follow
set_dt (setup.F90:629-670) and the values quoted for the benchmark decks.
"""
import ctypes as C

import numpy as np
import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi

oracle = pytest.importorskip("oracle.oracle")


@pytest.fixture(scope="module")
def lib():
    from cylindrical_epoch_gb300 import build
    build.build()
    return cg.load()


@pytest.mark.parametrize("name", ["thermal", "wakefield"])
def test_product_loader_bit_exact_vs_oracle(lib, name):
    if name == "thermal":
        deck = cg.thermal_plasma(nx=32, ny=16, ppc=6)
    else:
        deck = cg.wakefield(nx=64, ny=24, ppc=3, density=3.0e24, ramp=1.0e-6)
    parts, rng = cg.host_load(deck)
    orc = oracle.Oracle(deck, load_species=True)
    for i in range(len(deck.species)):
        a = parts[i].sorted_by_id()
        b = orc.particles(i).sorted_by_id()
        assert np.array_equal(a.id, b.id)
        for k in ("x", "y", "z", "px", "py", "pz", "w"):
            assert np.array_equal(getattr(a, k), getattr(b, k)), k
    r = orc.rng_state()
    for k in ("x", "y", "z", "w", "box_muller_cached"):
        assert getattr(rng, k) == getattr(r, k), k


def _grid_deck():
    """A wakefield deck whose density, temperature and drift are given as
    grids (as the Fortran driver evaluates deck expressions): an x- and
    r-dependent density with cells below density_min, a temperature that
    varies per direction and cell, a drift in x."""
    deck = cg.wakefield(nx=48, ny=20, ppc=3, density=3.0e24, ramp=1.0e-6)
    ng, nx, ny = abi.NG, deck.nx, deck.ny
    ix = np.arange(1 - ng, nx + ng + 1)
    iy = np.arange(1 - ng, ny + ng + 1)
    xg = (deck.x_min + deck.dx / 2.0) + (ix - 1.0) * deck.dx
    yg = deck.dy / 2.0 + (iy - 1.0) * deck.dy
    dens = 3.0e24 * (0.5 + np.sin(xg / 0.3e-6)[None, :] ** 2) * np.exp(-(yg[:, None] / 1.5e-6) ** 2)
    dens[:, :8] = 0.0
    temp = np.stack([1.0e5 * (1 + k + np.cos(yg[:, None] / 1e-6) + 0 * xg[None, :]) for k in range(3)])
    drift = np.zeros_like(temp)
    drift[0] = 1.0e-24 * (1.0 + xg[None, :] / deck.x_max)
    deck.load_grids = lambda isp: (dens, temp, drift)
    return deck


def test_grid_loader_bit_exact_vs_oracle(lib):
    """cyl_host_load_species_grid (density, temperature and drift as grids)
    against the oracle's loader given the same grids: bit for bit."""
    deck = _grid_deck()
    parts, rng = cg.host_load(deck)
    orc = oracle.Oracle(deck, load_species=True)
    a = parts[0].sorted_by_id()
    b = orc.particles(0).sorted_by_id()
    assert a.n > 1000 and np.array_equal(a.id, b.id)
    for k in ("x", "y", "z", "px", "py", "pz", "w"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    r = orc.rng_state()
    for k in ("x", "y", "z", "w", "box_muller_cached"):
        assert getattr(rng, k) == getattr(r, k), k
    # the grids were used: no particle in the empty columns, drift visible
    assert a.x.min() >= deck.x_min + 3 * deck.dx and a.px.mean() > 0.5e-24  # columns ix <= 3 are empty


def test_moving_window_deck_loads_like_closed_form(lib):
    """The reference's moving_window.deck: its x-dependent density through
    the grid loader matches the oracle, and a uniform grid equal to the
    closed form loads the same particles as the closed form."""
    deck = cg.moving_window_deck()
    parts, rng = cg.host_load(deck)
    orc = oracle.Oracle(deck, load_species=True)
    a, b = parts[0].sorted_by_id(), orc.particles(0).sorted_by_id()
    assert a.n == 2 * deck.nx * deck.ny
    for k in ("x", "y", "z", "px", "py", "pz", "w"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    plain = cg.wakefield(nx=32, ny=12, ppc=2, density=2.0e24, ramp=1.0)
    p0, _ = cg.host_load(plain)
    ng = abi.NG
    shape = (plain.ny + 2 * ng, plain.nx + 2 * ng)
    ix = np.arange(1 - ng, plain.nx + ng + 1)
    xg = (plain.x_min + plain.dx / 2.0) + (ix - 1.0) * plain.dx
    dens = np.repeat(plain.species[0].density_at(xg)[None, :], shape[0], axis=0)
    plain.load_grids = lambda isp: (dens, None, None)
    p1, _ = cg.host_load(plain)
    for k in ("x", "y", "z", "px", "py", "pz", "w"):
        assert np.array_equal(getattr(p0[0], k), getattr(p1[0], k)), k


def test_kiss_stream_matches_oracle(lib):
    s = abi.RngState()
    lib.cyl_rng_init(C.byref(s), 7842432)
    deck = cg.thermal_plasma(nx=16, ny=8, ppc=1)
    orc = oracle.Oracle(deck)
    r = orc.rng_state()
    for k in ("x", "y", "z", "w"):
        assert getattr(s, k) == getattr(r, k), k
    v = [lib.cyl_rng_random(C.byref(s)) for _ in range(1000)]
    assert all(0.0 <= x < 1.0 for x in v)
    assert abs(np.mean(v) - 0.5) < 0.03


def test_deck_time_steps():
    # thermal plasma: dz = dr = 50 nm, CFL 0.95 -> dt = 0.95 * 0.9 * 50 nm / sqrt(2) / c
    d1 = cg.thermal_plasma()
    assert cg.deck.set_dt(d1) == pytest.approx(1.008e-16, rel=2e-3)
    # wakefield: dz = lambda/32 = 25 nm -> dt ~ 5.04e-17 s
    d2 = cg.wakefield()
    assert cg.deck.set_dt(d2) == pytest.approx(5.04e-17, rel=2e-3)
    # the grid descriptor carries the same value
    assert d2.grid_desc().dt == cg.deck.set_dt(d2)


def test_device_estimate_grows_with_the_run(lib):
    from cylindrical_epoch_gb300 import serve
    small = serve.estimate_bytes(cg.wakefield(nx=256, ny=64, ppc=2))
    wide = serve.estimate_bytes(cg.wakefield(nx=512, ny=64, ppc=2))
    dense = serve.estimate_bytes(cg.wakefield(nx=256, ny=64, ppc=8))
    mixed = serve.estimate_bytes(cg.wakefield(nx=256, ny=64, ppc=2, precision=abi.PREC_MIXED))
    assert small < wide and small < dense and small < mixed
    # C2: 15 FP64 mode arrays of 2058 x 266 x 2 complex plus 4.6 M particle slots
    c2 = serve.estimate_bytes(cg.wakefield())
    assert 0.6e9 < c2 < 1.5e9


def test_server_without_device_reports_status(lib):
    from cylindrical_epoch_gb300 import serve
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(abi.CylError) as e:
        serve.Server(0, 2)
    assert e.value.code == abi.CYL_ERR_NO_DEVICE


def test_compare_runs_of_identical_runs():
    """The run comparison used by the bench and the full-size oracle check:
    two oracle runs of the same deck compare with zero error."""
    oracle = pytest.importorskip("oracle.oracle")
    import cylindrical_epoch_gb300 as cg
    from cylindrical_epoch_gb300.diagnostics import compare_runs
    deck = cg.wakefield(nx=64, ny=16, ppc=2, density=3.0e24, ramp=2.0e-6)
    a = oracle.Oracle(deck, load_species=True)
    b = oracle.Oracle(deck, load_species=True)
    for o in (a, b):
        o.initialise()
        o.step(6)
    r = compare_runs(a, b, deck)
    assert r["ez_rel_l2_per_mode"] == [0.0] * deck.n_mode
    assert r["n_live"]["run"] == r["n_live"]["against"] > 0
    assert r["electron_spectrum"]["rel_err"]["mean_mev"] == 0.0
    assert r["continuity_residual_per_mode"]["run"] == r["continuity_residual_per_mode"]["against"]
    assert r["continuity_residual_per_mode"]["run"][0] < 1e-10  # round-off; the charge barely moves in 6 steps
