"""The output point inside a step (cyl_step_to_output) and the restart from a
dump taken there (cyl_write_sdf with restart, cyl_restart_sdf), on the device
against the oracle (orc_step_to_output, orc_finish_step, orc_restart).

The deck is a small windowed wakefield whose window has moved before the
dump, with the shift fraction at the dump large enough that a restart which
dropped it would shift a step late.  Its boundaries are the same before and
after the move: a restarted run keeps the deck's boundaries until its first
moving_window, as the reference's does.  Both sides draw window injection
from the counter stream, so the oracle and the device inject the same
particles.  Tolerances are those of the FP64 parity tests: positions 1e-12,
fields 1e-10 relative L2 per mode; step, time, window position, shift
fraction and counts exact.
"""
import numpy as np
import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi
from tests.helpers import match_by_id, rel_l2

pytestmark = pytest.mark.gpu

DUMP_STEP = 31


def _deck(precision=abi.PREC_FP64):
    deck = cg.wakefield(nx=128, ny=32, ppc=4, density=3.0e24, ramp=2.0e-6, precision=precision)
    deck.window_start_time = 20 * 5.0e-17
    deck.bc_after_move = None
    return deck


def _cmp(gpu, orc, tol=1.0e-10):
    sg, so = gpu.state(), orc.state()
    assert (sg.step, sg.time, sg.n_shifts) == (so.step, so.time, so.n_shifts)
    assert (sg.x_grid_min, sg.xb_min, sg.window_shift_fraction) == \
        (so.x_grid_min, so.xb_min, so.window_shift_fraction)
    assert sg.n_live[0] == so.n_live[0], (sg.n_live[0], so.n_live[0])
    a, b = match_by_id(gpu.particles(0), orc.particles(0))
    for k in ("x", "y", "z", "px", "py", "pz"):
        assert rel_l2(getattr(a, k), getattr(b, k)) < 1e-12, k
    for n in abi.FIELD_NAMES:
        ga, ob = gpu.field(n), orc.field(n)
        for m in range(ga.shape[0]):
            if np.any(ob[m] != 0):
                assert rel_l2(ga[m], ob[m]) < tol, (n, m)


def test_output_point_matches_oracle(gpu_lib):
    from oracle.oracle import Oracle
    deck = _deck()
    gpu = cg.Run(deck, rng_mode=abi.RNG_COUNTER, counter_seed=5, initialise=False)
    orc = Oracle(deck, counter_seed=5, atan2="shared")
    gpu.lib.cyl_initialise(gpu.h)
    orc.initialise()
    gpu.step_to_output(DUMP_STEP)
    orc.step_to_output(DUMP_STEP)
    s = gpu.state()
    assert s.step == DUMP_STEP and s.n_shifts > 0 and s.window_shift_fraction > 0.5
    _cmp(gpu, orc)
    # the next stepping call finishes the stopped step, then runs its own
    gpu.step(17, graph=True)
    orc.finish_step()
    orc.step(17)
    _cmp(gpu, orc)


def test_restart_matches_oracle(gpu_lib, tmp_path):
    from oracle.oracle import Oracle
    deck = _deck()
    a = cg.Run(deck, rng_mode=abi.RNG_COUNTER, counter_seed=6)
    a.step_to_output(DUMP_STEP)
    p = tmp_path / "restart.sdf"
    a.write_sdf(p, restart=True)
    sa = a.state()
    assert sa.n_shifts > 0 and sa.window_started and sa.window_shift_fraction > 0.5
    b = cg.Run.from_sdf(deck, p, rng_mode=abi.RNG_COUNTER, counter_seed=6)
    sb = b.state()
    assert (sb.step, sb.time, sb.xb_min, sb.x_grid_min, sb.n_shifts, sb.n_live[0]) == \
        (sa.step, sa.time, sa.xb_min, sa.x_grid_min, sa.n_shifts, sa.n_live[0])
    # the oracle restarted from the same file
    orc = Oracle(deck, atan2="shared")
    orc.lib.orc_set_injection_stream(orc.h, abi.RNG_COUNTER, 6)
    with cg.SdfFile(p) as f:
        for n in abi.FIELD_NAMES:
            orc.set_field(n, f.field(n))
        orc.set_particles(0, f.particles("electron"))
        i = f.info
        orc.restart(i.step, i.time, i.grid_x0, i.x_grid_min,
                    i.window_shift_fraction if i.has_window_shift_fraction else None)
    b.step(20, graph=True)
    orc.step(20)
    _cmp(b, orc)
    # and the run that wrote the dump went the same way
    a.step(20, graph=True)
    sa, sb = a.state(), b.state()
    assert (sa.step, sa.time, sa.n_shifts, sa.n_live[0]) == (sb.step, sb.time, sb.n_shifts, sb.n_live[0])
    for n in ("exm", "erm", "btm"):
        fa, fb = a.field(n), b.field(n)
        for m in range(fa.shape[0]):
            if np.any(fa[m] != 0):
                assert rel_l2(fb[m], fa[m]) < 1e-10, (n, m)


def test_restart_mixed_form(gpu_lib, tmp_path):
    deck = _deck(precision=abi.PREC_MIXED)
    a = cg.Run(deck, rng_mode=abi.RNG_COUNTER, counter_seed=7)
    a.step_to_output(DUMP_STEP)
    p = tmp_path / "restart_mixed.sdf"
    a.write_sdf(p, restart=True)
    b = cg.Run.from_sdf(deck, p, rng_mode=abi.RNG_COUNTER, counter_seed=7)
    a.step(20, graph=True)
    b.step(20, graph=True)
    sa, sb = a.state(), b.state()
    assert (sa.step, sa.n_shifts) == (sb.step, sb.n_shifts)
    assert abs(sa.n_live[0] - sb.n_live[0]) <= 1e-3 * sa.n_live[0]
    ea, eb = a.field("exm"), b.field("exm")
    for m in range(ea.shape[0]):
        assert rel_l2(eb[m], ea[m]) < 1e-3, m


def test_restart_rules(gpu_lib, tmp_path):
    deck = _deck()
    run = cg.Run(deck, rng_mode=abi.RNG_COUNTER, counter_seed=8)
    run.step(3)
    # a restart dump only at the output point
    with pytest.raises(abi.CylError):
        run.write_sdf(tmp_path / "r.sdf", restart=True)
    # a dump without restart data does not restart a run
    run.write_sdf(tmp_path / "plain.sdf")
    with pytest.raises(abi.CylError):
        cg.Run.from_sdf(deck, tmp_path / "plain.sdf")
    # nor does a restart dump of another grid
    run.step_to_output(2)
    run.write_sdf(tmp_path / "r.sdf", restart=True)
    other = cg.wakefield(nx=96, ny=32, ppc=4, density=3.0e24, ramp=2.0e-6)
    with pytest.raises(abi.CylError):
        cg.Run.from_sdf(other, tmp_path / "r.sdf")
    # an initialised run cannot be initialised again at the output point
    with pytest.raises(abi.CylError):
        abi.check("cyl_initialise", run.lib.cyl_initialise(run.h))
    # steps after the output point continue
    run.step(2)
    assert run.state().step == 7


def test_restart_dump_of_loaded_run_keeps_shift_fraction(gpu_lib, tmp_path):
    """A run loaded from a dump restarts its window at its first
    moving_window; a restart dump written before that still carries the
    loaded shift fraction, and the rest of the state as loaded."""
    from oracle.sdf_read import read
    deck = _deck()
    a = cg.Run(deck, rng_mode=abi.RNG_COUNTER, counter_seed=9)
    a.step_to_output(DUMP_STEP)
    p1, p2 = tmp_path / "first.sdf", tmp_path / "second.sdf"
    a.write_sdf(p1, restart=True)
    b = cg.Run.from_sdf(deck, p1, rng_mode=abi.RNG_COUNTER, counter_seed=9)
    b.write_sdf(p2, restart=True)
    h1, _, _, d1 = read(p1)
    h2, _, _, d2 = read(p2)
    assert (h2.step, h2.time, h2.nblocks) == (h1.step, h1.time, h1.nblocks)
    assert d2["window_shift_fraction"] == d1["window_shift_fraction"] > 0.5
    for k in d1:
        if k != "grid":
            assert np.array_equal(np.asarray(d2[k]), np.asarray(d1[k])), k
