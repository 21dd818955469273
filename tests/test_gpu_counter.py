"""Device loading and device window injection (the counter stream) against
the oracle's counter loader and injector, through the C ABI.

Tolerances: counts, ids, cells and window shifts exact.  FP64 form:
loaded positions and weights bit-exact (the same operations, no FMA
contraction on either side, angles through the shared cyl_sincos_turn);
momenta within 1e-13 relative (the device's log against the host libm, a
few ulp); after steps, positions within 1e-12 and fields within 1e-10
relative L2 (the other parity tests' bar).  Mixed form: the FP32 particle
state within 1e-6, and the run within the mixed form's 1e-3 bar on Ez
against FP64.
"""
import numpy as np
import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi
from tests.helpers import match_by_id, rel_l2

pytestmark = pytest.mark.gpu

FIELDS = ["exm", "erm", "etm", "bxm", "brm", "btm", "jxm", "jrm", "jtm"]


def _maxrel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _wake(ppc=4, precision=abi.PREC_FP64):
    deck = cg.wakefield(nx=128, ny=32, ppc=ppc, density=3.0e24, ramp=2.0e-6, precision=precision)
    deck.window_start_time = 20 * 5.0e-17
    return deck


@pytest.mark.parametrize("ppc", [4, 4.5])
def test_device_load_matches_oracle(gpu_lib, ppc):
    from oracle.oracle import Oracle
    deck = cg.thermal_plasma(nx=64, ny=32, ppc=ppc)
    gpu = cg.Run(deck, rng_mode=abi.RNG_COUNTER, counter_seed=11, initialise=False)
    orc = Oracle(deck, counter_seed=11, atan2="shared")
    a, b = match_by_id(gpu.particles(0), orc.particles(0))
    assert a.n == b.n == int(np.floor(ppc * 64 * 32))
    for k in ("x", "y", "z", "w"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    for k in ("px", "py", "pz"):
        assert _maxrel(getattr(a, k), getattr(b, k)) < 1e-13, k
    gx, gy = gpu.cell_indices(0)
    ox, oy = orc.cell_indices(0)
    ga, oa = np.argsort(gpu.particles(0).id), np.argsort(orc.particles(0).id)
    assert np.array_equal(gx[ga], ox[oa]) and np.array_equal(gy[ga], oy[oa])


def test_device_load_mixed_form(gpu_lib):
    from oracle.oracle import Oracle
    deck = cg.wakefield(nx=128, ny=32, ppc=2.5, density=3.0e24, ramp=2.0e-6, precision=abi.PREC_MIXED)
    gpu = cg.Run(deck, rng_mode=abi.RNG_COUNTER, counter_seed=5, initialise=False)
    orc = Oracle(deck, counter_seed=5, atan2="shared")
    a, b = match_by_id(gpu.particles(0), orc.particles(0))
    for k in ("x", "y", "z", "w"):
        assert rel_l2(getattr(a, k), getattr(b, k)) < 1e-6, k


def test_counter_window_parity(gpu_lib):
    from oracle.oracle import Oracle
    deck = _wake()
    gpu = cg.Run(deck, rng_mode=abi.RNG_COUNTER, counter_seed=3, initialise=False)
    orc = Oracle(deck, counter_seed=3, atan2="shared")
    gpu.lib.cyl_initialise(gpu.h)
    orc.initialise()
    for chunk in (1, 15, 24, 40):
        gpu.step(chunk)
        orc.step(chunk)
        sg, so = gpu.state(), orc.state()
        assert sg.step == so.step
        assert sg.n_shifts == so.n_shifts
        assert sg.x_grid_min == so.x_grid_min
        assert sg.n_live[0] == so.n_live[0], (sg.n_live[0], so.n_live[0])
    assert so.n_shifts > 10
    a, b = match_by_id(gpu.particles(0), orc.particles(0))
    for k in ("x", "y", "z"):
        assert rel_l2(getattr(a, k), getattr(b, k)) < 1e-12, k
    for n in FIELDS:
        ga, ob = gpu.field(n), orc.field(n)
        for m in range(ga.shape[0]):
            if np.any(ob[m] != 0):
                assert rel_l2(ga[m], ob[m]) < 1e-10, (n, m)


def test_counter_graph_matches_eager(gpu_lib):
    deck = _wake()
    a = cg.Run(deck, rng_mode=abi.RNG_COUNTER, counter_seed=9)
    b = cg.Run(deck, rng_mode=abi.RNG_COUNTER, counter_seed=9)
    a.step(48, graph=False)
    b.step(48, graph=True)
    sa, sb = a.state(), b.state()
    assert sa.n_live[0] == sb.n_live[0] and sa.n_shifts == sb.n_shifts > 10
    pa, pb = match_by_id(a.particles(0), b.particles(0))
    assert rel_l2(pb.x, pa.x) < 1e-12
    for n in ("exm", "btm", "jxm"):
        assert rel_l2(b.field(n), a.field(n)) < 1e-10


def test_counter_stream_switch_mid_run(gpu_lib):
    """KISS injection for 32 steps, then the counter stream: the switch
    rebuilds the captured step, and injected ids continue without a gap."""
    deck = _wake()
    run = cg.Run(deck)
    run.step(32, graph=True)
    s0 = run.state()
    ids0 = run.particles(0).id.max()
    abi.check("cyl_set_injection_stream", run.lib.cyl_set_injection_stream(run.h, abi.RNG_COUNTER, 21))
    run.step(32, graph=True)
    s1 = run.state()
    assert s1.n_shifts > s0.n_shifts
    ids = np.sort(run.particles(0).id)
    new = ids[ids > ids0]
    assert np.array_equal(new, np.arange(ids0 + 1, ids0 + 1 + new.size))
    assert new.size == (s1.n_shifts - s0.n_shifts) * deck.ny * 4
    assert run.diagnostics().device_error == 0


def test_counter_mixed_vs_fp64(gpu_lib):
    from tests.helpers import rel_l2 as rl
    d64, d32 = _wake(), _wake(precision=abi.PREC_MIXED)
    a = cg.Run(d64, rng_mode=abi.RNG_COUNTER, counter_seed=4)
    b = cg.Run(d32, rng_mode=abi.RNG_COUNTER, counter_seed=4)
    a.step(80, graph=True)
    b.step(80, graph=True)
    sa, sb = a.state(), b.state()
    assert sa.n_shifts == sb.n_shifts
    assert abs(sa.n_live[0] - sb.n_live[0]) <= 1e-3 * sa.n_live[0]
    ea, eb = a.field("exm"), b.field("exm")
    for m in range(ea.shape[0]):
        assert rl(eb[m], ea[m]) < 1e-3, m


def test_counter_runs_in_batch(gpu_lib):
    """Mixed-form runs with device injection stepped as one batch give each
    run its result alone (counts exact, energies within 1e-6)."""
    decks = [_wake(precision=abi.PREC_MIXED), _wake(ppc=3, precision=abi.PREC_MIXED)]
    alone = [cg.Run(d, rng_mode=abi.RNG_COUNTER, counter_seed=30 + i) for i, d in enumerate(decks)]
    for r in alone:
        r.step(48, graph=True)
    batched = [cg.Run(d, rng_mode=abi.RNG_COUNTER, counter_seed=30 + i) for i, d in enumerate(decks)]
    with cg.Batch(4) as bt:
        bt.step(batched, 48)
    for x, y in zip(alone, batched):
        sx, sy = x.state(), y.state()
        assert sx.n_live[0] == sy.n_live[0] and sx.n_shifts == sy.n_shifts
        dx, dy = x.diagnostics(), y.diagnostics()
        for k in ("kinetic_energy", "field_energy_e", "field_energy_b"):
            assert abs(getattr(dy, k) - getattr(dx, k)) <= 1e-6 * abs(getattr(dx, k)), k


def test_counter_two_species_window_parity(gpu_lib):
    """Electrons and mobile ions (fractional ions per cell) in a windowed
    wakefield, loaded and injected from the counter stream: ids continue
    across the species, each species' injection matches the oracle's, and
    the run matches the oracle at the usual bar."""
    from cylindrical_epoch_gb300.deck import Q0, Species
    from oracle.oracle import Oracle
    ions = Species("helium2+", 2.0 * Q0, 4.0 * 1.66053886e-27, 1.5, 0.01 * 3.0e24, density_kind=1,
                   ramp_x0=0.0, ramp_length=2.0e-6, bc=(abi.BC_SIMPLE_LASER, abi.BC_OPEN, abi.BC_OTHER, abi.BC_OPEN))
    deck = cg.wakefield(nx=128, ny=32, ppc=3, density=3.0e24, ramp=2.0e-6, ions=ions)
    deck.window_start_time = 20 * 5.0e-17
    gpu = cg.Run(deck, rng_mode=abi.RNG_COUNTER, counter_seed=17, initialise=False)
    orc = Oracle(deck, counter_seed=17, atan2="shared")
    ids = np.concatenate([gpu.particles(0).id, gpu.particles(1).id])
    assert np.array_equal(np.sort(ids), np.arange(ids.size))
    gpu.lib.cyl_initialise(gpu.h)
    orc.initialise()
    gpu.step(48)
    orc.step(48)
    sg, so = gpu.state(), orc.state()
    assert sg.n_shifts == so.n_shifts > 10
    for i in (0, 1):
        assert sg.n_live[i] == so.n_live[i], i
        a, b = match_by_id(gpu.particles(i), orc.particles(i))
        for k in ("x", "y", "z"):
            assert rel_l2(getattr(a, k), getattr(b, k)) < 1e-12, (i, k)
    for n in FIELDS:
        ga, ob = gpu.field(n), orc.field(n)
        for m in range(ga.shape[0]):
            if np.any(ob[m] != 0):
                assert rel_l2(ga[m], ob[m]) < 1e-10, (n, m)
