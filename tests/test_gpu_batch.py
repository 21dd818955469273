"""Batches (cyl_batch_*): runs of different grids and particle counts stepped
together, with one push launch per step over all their tiles, give each run
the result of stepping it alone -- particle counts and window shifts exact,
energies within 1e-6 relative (the order of the FP64 current additions and
of the per-tile flushes differs) -- including when the membership changes
between calls and for chunks shorter than 16 steps."""
import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi

pytestmark = pytest.mark.gpu

TOL = 1e-6


def _decks():
    a = cg.wakefield(nx=128, ny=32, ppc=2, density=3.0e24, ramp=2.0e-6, precision=abi.PREC_MIXED)
    a.window_start_time = 20 * 5.0e-17
    b = cg.wakefield(nx=192, ny=48, ppc=3, density=2.0e24, ramp=3.0e-6, a0=1.5, precision=abi.PREC_MIXED)
    b.window_start_time = 12 * 5.0e-17
    c = cg.thermal_plasma(nx=64, ny=32, ppc=4, precision=abi.PREC_MIXED)
    return [a, b, c]


def _runs(decks, loads):
    return [cg.Run(d, particles=p, rng=r) for d, (p, r) in zip(decks, loads)]


def _rel(x, y):
    return abs(x - y) / max(abs(y), 1e-300)


def _same(a, b):
    sa, sb = a.state(), b.state()
    assert sa.n_live[0] == sb.n_live[0]
    assert sa.n_shifts == sb.n_shifts
    assert sa.step == sb.step
    da, db = a.diagnostics(), b.diagnostics()
    assert db.device_error == 0
    for k in ("kinetic_energy", "field_energy_e", "field_energy_b"):
        assert _rel(getattr(db, k), getattr(da, k)) < TOL, k


def test_batch_matches_runs_alone(gpu_lib):
    decks = _decks()
    loads = [cg.host_load(d) for d in decks]
    alone = _runs(decks, loads)
    for r in alone:
        r.step(16, graph=True)
        r.step(30, graph=True)
    batched = _runs(decks, loads)
    with cg.Batch(4) as b:
        b.step(batched, 16)  # one graph
        b.step(batched, 30)  # the same graph again, then a 14-step chunk
    for a, r in zip(alone, batched):
        _same(a, r)
    assert alone[0].state().n_shifts > 0 and alone[1].state().n_shifts > 0


def test_batch_membership_changes(gpu_lib):
    decks = _decks()
    loads = [cg.host_load(d) for d in decks]
    alone = _runs(decks, loads)
    for r in alone:
        r.step(48, graph=True)
    batched = _runs(decks, loads)
    with cg.Batch(4) as b:
        b.step(batched, 16)
        b.step(batched[:2], 16)     # the third run leaves ...
        batched[2].step(16, graph=True)
        b.step(batched[1:], 16)     # ... the first leaves, the third joins again
        batched[0].step(16, graph=True)
    for a, r in zip(alone, batched):
        _same(a, r)


def test_batch_rejects_mixed_modes_and_forms(gpu_lib):
    d2 = cg.thermal_plasma(nx=64, ny=32, ppc=2, precision=abi.PREC_MIXED)
    d3 = cg.thermal_plasma(nx=64, ny=32, ppc=2, n_mode=3, precision=abi.PREC_MIXED)
    d64 = cg.thermal_plasma(nx=64, ny=32, ppc=2)
    runs = [cg.Run(d) for d in (d2, d3, d64)]
    with cg.Batch(4) as b:
        with pytest.raises(abi.CylError):
            b.step(runs[:2], 16)
        with pytest.raises(abi.CylError):
            b.step([runs[0], runs[2]], 16)


def test_batch_run_replaced_by_new_run(gpu_lib):
    """A run that leaves and is destroyed, then a new run of the same deck in
    its place (which may get the same handle address): the batch rebuilds its
    graph for the new member instead of reusing the old one."""
    decks = _decks()[:2]
    loads = [cg.host_load(d) for d in decks]
    alone = _runs(decks, loads)
    for r in alone:
        r.step(32, graph=True)
    first = cg.Run(decks[0], particles=loads[0][0], rng=loads[0][1])
    gone = cg.Run(decks[1], particles=loads[1][0], rng=loads[1][1])
    with cg.Batch(4) as b:
        b.step([first, gone], 16)
        gone.close()
        fresh = cg.Run(decks[1], particles=loads[1][0], rng=loads[1][1])
        fresh.step(16, graph=True)
        b.step([first, fresh], 16)
    _same(alone[0], first)
    _same(alone[1], fresh)
