"""Request loop (cyl_server_*): each run's result is the same alone and in
the mix, and admission respects the HBM budget.

Tolerance: runs share no state, but the order of the FP64 atomic current
adds differs between executions; over the few tens of steps here that moves
the diagnostics by far less than 1e-8 relative (FP64 form) and 1e-6
(mixed form, which also re-sorts particles)."""
import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi, serve

pytestmark = pytest.mark.gpu


def _jobs():
    w = cg.wakefield(nx=128, ny=32, ppc=2, density=3.0e24, ramp=2.0e-6, precision=abi.PREC_MIXED)
    w.window_start_time = 20 * 5.0e-17
    t64 = cg.thermal_plasma(nx=64, ny=32, ppc=4)
    t32 = cg.thermal_plasma(nx=96, ny=24, ppc=3, precision=abi.PREC_MIXED)
    # 45 and 37 steps: the batched loop takes their last partial chunks alone
    return [(w, 45, 1e-6), (t64, 40, 1e-8), (t32, 37, 1e-6)]


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


def test_results_same_alone_and_in_mix(gpu_lib):
    jobs = _jobs()
    alone = []
    with serve.Server(0, 1) as srv:
        for deck, n, _ in jobs:
            alone.append(srv.wait(srv.submit(deck, n), 300.0))
    with serve.Server(0, len(jobs)) as srv:
        ids = [srv.submit(deck, n) for deck, n, _ in jobs]
        mixed = [srv.wait(i, 300.0) for i in ids]
    # the mix really overlapped: some two jobs were running at the same time
    assert any(a.t_start < b.t_end and b.t_start < a.t_end
               for i, a in enumerate(mixed) for b in mixed[i + 1:])
    for (deck, n, tol), a, b in zip(jobs, alone, mixed):
        assert a.status == abi.JOB_DONE and b.status == abi.JOB_DONE, (a.error, b.error)
        assert a.steps_done == b.steps_done == n
        assert a.state.n_live[0] == b.state.n_live[0]
        assert a.state.n_shifts == b.state.n_shifts
        assert b.diag.device_error == 0
        assert _rel(b.diag.kinetic_energy, a.diag.kinetic_energy) < tol
        assert _rel(b.diag.field_energy_e, a.diag.field_energy_e) < tol
        assert _rel(b.diag.field_energy_b, a.diag.field_energy_b) < tol


def test_admission_respects_budget(gpu_lib):
    jobs = _jobs()
    need = [serve.estimate_bytes(d) for d, _, _ in jobs]
    budget = max(need) + min(need) // 2  # the largest job never runs beside another
    with serve.Server(budget, 3) as srv:
        ids = [srv.submit(d, n) for d, n, _ in jobs]
        res = [srv.wait(i, 300.0) for i in ids]
        with pytest.raises(abi.CylError):
            srv.submit(cg.wakefield(), 1)  # larger than the whole budget
    for r, b in zip(res, need):
        assert r.status == abi.JOB_DONE
        assert r.device_bytes == b
    # at the start of every job, the jobs then running fit the budget together
    for r in res:
        live = [q.device_bytes for q in res if q.t_start <= r.t_start < q.t_end]
        assert sum(live) <= budget
    big = res[need.index(max(need))]
    for q in res:
        if q is not big:
            assert q.t_end <= big.t_start or q.t_start >= big.t_end


def test_batched_server_matches_runs_alone(gpu_lib):
    """The request loop with continuous batching (cyl_server_create_batched):
    the two mixed-form jobs step together in one batch (with the FP64 job
    beside them); each result matches the same deck stepped alone on its own
    handle, within the same tolerances."""
    jobs = _jobs()
    alone = []
    for deck, n, _ in jobs:
        run = cg.Run(deck)
        run.step(n, graph=True)
        alone.append((run.state(), run.diagnostics()))
        run.close()
    with serve.Server(0, 2, batched=True, max_batch=4) as srv:
        ids = [srv.submit(deck, n) for deck, n, _ in jobs]
        res = [srv.wait(i, 300.0) for i in ids]
    for (deck, n, tol), (sa, da), b in zip(jobs, alone, res):
        assert b.status == abi.JOB_DONE, b.error
        assert b.steps_done == n
        assert b.state.n_live[0] == sa.n_live[0]
        assert b.state.n_shifts == sa.n_shifts
        assert b.diag.device_error == 0
        assert _rel(b.diag.kinetic_energy, da.kinetic_energy) < tol
        assert _rel(b.diag.field_energy_e, da.field_energy_e) < tol
        assert _rel(b.diag.field_energy_b, da.field_energy_b) < tol


def test_counter_jobs_in_server(gpu_lib):
    """Jobs loaded and injected on the device (rng_mode = counter): the FP64
    job's result equals the same deck run alone in the counter mode, and
    every job's result is the same alone and in the mix."""
    jobs = _jobs()
    with serve.Server(0, 1) as srv:
        alone = [srv.wait(srv.submit(d, n, rng_mode=abi.RNG_COUNTER), 300.0) for d, n, _ in jobs]
    with serve.Server(0, len(jobs)) as srv:
        ids = [srv.submit(d, n, rng_mode=abi.RNG_COUNTER) for d, n, _ in jobs]
        mixed = [srv.wait(i, 300.0) for i in ids]
    for (deck, n, tol), a, b in zip(jobs, alone, mixed):
        assert a.status == abi.JOB_DONE and b.status == abi.JOB_DONE, (a.error, b.error)
        assert a.state.n_live[0] == b.state.n_live[0]
        assert a.state.n_shifts == b.state.n_shifts
        assert _rel(b.diag.kinetic_energy, a.diag.kinetic_energy) < tol
        assert _rel(b.diag.field_energy_e, a.diag.field_energy_e) < tol
    deck, n, tol = jobs[1]
    run = cg.Run(deck, rng_mode=abi.RNG_COUNTER)
    run.step(n, graph=True)
    s, d = run.state(), run.diagnostics()
    assert s.n_live[0] == alone[1].state.n_live[0]
    assert _rel(alone[1].diag.kinetic_energy, d.kinetic_energy) < tol
    assert _rel(alone[1].diag.field_energy_e, d.field_energy_e) < tol
