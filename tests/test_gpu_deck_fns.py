"""The deck-expression channel of the C ABI (cyl_set_deck_fns,
cyl_host_load_species_grid) on the device against the oracle, which calls
the same callbacks.

- The reference's own example_decks/moving_window.deck, whose species
  density 0.5 + sin(x / 4 um)^2 is a deck expression: loaded from the
  evaluated grid, injected at every window shift from the evaluated column;
  counts, window shifts and positions exact (the species is neutral), fields
  within 1e-10.
- A laser wakefield whose laser time profile, omega (a chirp), profile (a
  waist that grows) and phase (a tilt that oscillates) are all callbacks
  (laser.f90:182-328), against the oracle at 1e-10; and the time-profile
  callback equal to the built-in gauss bit for bit.
- Error paths: a raising callback fails the step with CYL_ERR_CALLBACK; bad
  masks and an inject callback with device injection are refused.
"""
import math

import numpy as np
import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi
from tests.helpers import match_by_id, rel_l2

pytestmark = pytest.mark.gpu

FIELDS = ["exm", "erm", "etm", "bxm", "brm", "btm", "jxm", "jrm", "jtm"]


def _pair(deck):
    from oracle.oracle import Oracle
    parts, rng = cg.host_load(deck)
    gpu = cg.Run(deck, particles=parts, rng=rng)
    orc = Oracle(deck, particles=parts, rng=rng, atan2="shared")
    orc.initialise()
    return gpu, orc


def _cmp(gpu, orc, tol=1e-10):
    for n in FIELDS:
        a, b = gpu.field(n), orc.field(n)
        for m in range(a.shape[0]):
            if np.all(b[m] == 0) and np.all(a[m] == 0):
                continue
            assert rel_l2(a[m], b[m]) < tol, (n, m, rel_l2(a[m], b[m]))


def test_moving_window_deck_parity(gpu_lib):
    deck = cg.moving_window_deck()
    gpu, orc = _pair(deck)
    for chunk in (300, 100, 140):  # the window starts at 30 fs, step 373
        gpu.step(chunk, graph=True)
        orc.step(chunk)
        sg, so = gpu.state(), orc.state()
        assert sg.n_shifts == so.n_shifts and sg.x_grid_min == so.x_grid_min
        assert sg.n_live[0] == so.n_live[0]
    assert so.n_shifts > 40
    a, b = match_by_id(gpu.particles(0), orc.particles(0))
    for k in ("x", "y", "z", "px", "py", "pz", "w"):
        assert rel_l2(getattr(a, k), getattr(b, k)) < 1e-12, k
    # injected particles carry the evaluated column's density in their weight
    fresh = b.id >= 2 * deck.nx * deck.ny
    assert fresh.sum() > 1000 and np.array_equal(a.w[fresh], b.w[fresh])
    _cmp(gpu, orc)
    # the mixed form on the same deck: same shifts and counts
    deck.precision = abi.PREC_MIXED
    parts, rng = cg.host_load(deck)
    mix = cg.Run(deck, particles=parts, rng=rng)
    mix.step(540, graph=True)
    sm = mix.state()
    assert sm.n_shifts == sg.n_shifts and abs(sm.n_live[0] - sg.n_live[0]) <= 2


def test_moving_window_column_callback_is_used(gpu_lib):
    """An inject callback that returns an empty column stops the injection:
    the run loses the removed columns' particles and gains none."""
    deck = cg.moving_window_deck()
    ny = deck.ny
    deck.inject = lambda isp, t, x: (np.zeros(ny + 2), np.full((3, ny + 2), 0.5), np.zeros((3, ny + 2)))
    gpu, orc = _pair(deck)
    gpu.step(480, graph=True)
    orc.step(480)
    sg, so = gpu.state(), orc.state()
    assert sg.n_shifts == so.n_shifts > 30
    assert sg.n_live[0] == so.n_live[0] < 2 * deck.nx * deck.ny


def _laser_deck():
    deck = cg.wakefield(nx=128, ny=32, ppc=2, density=3.0e24, ramp=2.0e-6)
    deck.window_start_time = 20 * 5.0e-17
    las = deck.lasers[0]
    ny = deck.ny
    yv = deck.y_grid(np.arange(0, ny + 1))
    w0 = 10.0e-6

    def t_env(il, t):
        v = (t - las.t0) / las.tw
        return math.exp(-(v * v))

    deck.laser_time = t_env
    deck.laser_omega = lambda il, t: las.omega * (1.0 + 0.05 * t / 1.0e-13)
    deck.omega_fn = frozenset({0})
    deck.laser_profile = lambda il, t: np.exp(-(yv / (w0 * (1.0 + t / 2.0e-14))) ** 2)
    deck.profile_fn = frozenset({0})
    deck.laser_phase = lambda il, t: 0.3 * math.sin(t / 1.0e-15) * yv / w0
    deck.phase_fn = frozenset({0})
    return deck


def test_laser_callbacks_parity(gpu_lib):
    deck = _laser_deck()
    gpu, orc = _pair(deck)
    for chunk in (16, 24):
        gpu.step(chunk, graph=True)
        orc.step(chunk)
    sg, so = gpu.state(), orc.state()
    assert sg.n_shifts == so.n_shifts > 0 and sg.n_live[0] == so.n_live[0]
    _cmp(gpu, orc)


def test_laser_time_callback_equals_closed_form(gpu_lib):
    """laser_time evaluating gauss(time, t0, tw) gives the built-in
    t_profile = 1 run: the same laser sources (both call libm's exp on the
    same value), so the runs differ only by the order of the FP64 atomic
    current adds, as two runs of one deck do."""
    a_deck = cg.wakefield(nx=96, ny=24, ppc=2, density=3.0e24, ramp=2.0e-6)
    b_deck = cg.wakefield(nx=96, ny=24, ppc=2, density=3.0e24, ramp=2.0e-6)
    las = b_deck.lasers[0]

    def t_env(il, t):
        v = (t - las.t0) / las.tw
        return math.exp(-(v * v))

    b_deck.laser_time = t_env
    parts, rng = cg.host_load(a_deck)
    a = cg.Run(a_deck, particles=parts, rng=rng)
    b = cg.Run(b_deck, particles=parts, rng=rng)
    a.step(32, graph=True)
    b.step(32, graph=True)
    for n in ("exm", "erm", "etm", "btm"):
        assert rel_l2(b.field(n), a.field(n)) < 1e-12, n


def test_callback_error_fails_the_step(gpu_lib):
    deck = cg.wakefield(nx=64, ny=16, ppc=1, density=3.0e24, ramp=2.0e-6)

    def bad(il, t):
        raise ValueError("parser error")

    deck.laser_time = bad
    run = cg.Run(deck, initialise=False)
    with pytest.raises(abi.CylError) as e:
        run.step(1)
    assert e.value.code == abi.CYL_ERR_CALLBACK


def test_set_deck_fns_refusals(gpu_lib):
    deck = cg.wakefield(nx=64, ny=16, ppc=1, density=3.0e24, ramp=2.0e-6)
    run = cg.Run(deck, initialise=False)
    f, keep = _laser_deck().deck_fns()
    f.omega_fn_mask = 0b10  # the run has one laser
    assert run.lib.cyl_set_deck_fns(run.h, f) == abi.CYL_ERR_BAD_ARG
    f.omega_fn_mask = 1
    f.laser_omega = abi.LaserOmegaFn()  # a mask bit without its callback
    assert run.lib.cyl_set_deck_fns(run.h, f) == abi.CYL_ERR_BAD_ARG
    mw = cg.moving_window_deck()
    g, keep2 = mw.deck_fns()
    assert run.lib.cyl_set_injection_stream(run.h, abi.RNG_COUNTER, 5) == abi.CYL_OK
    assert run.lib.cyl_set_deck_fns(run.h, g) == abi.CYL_ERR_UNSUPPORTED
    assert run.lib.cyl_set_injection_stream(run.h, abi.RNG_KISS, 5) == abi.CYL_OK
    assert run.lib.cyl_set_deck_fns(run.h, g) == abi.CYL_OK
    assert run.lib.cyl_set_injection_stream(run.h, abi.RNG_COUNTER, 5) == abi.CYL_ERR_UNSUPPORTED
    assert run.lib.cyl_set_deck_fns(run.h, None) == abi.CYL_OK
