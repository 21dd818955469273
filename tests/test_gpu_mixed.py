"""Mixed-precision form (int cell + FP32 offset, FP32 push/deposit into FP64
currents) against the FP64 form and the oracle.

Error bar: per-mode Ez (exm) relative L2 <= 1e-3 against the
FP64 result on the same deck; the other stated results (wake amplitude,
electron energy moments, particle count) are compared with the same
tolerance here.
"""
import numpy as np
import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi
from tests.helpers import rel_l2

pytestmark = pytest.mark.gpu

TOL_EZ = 1.0e-3


def _wake(prec, nx=256, ny=64, ppc=4):
    deck = cg.wakefield(nx=nx, ny=ny, ppc=ppc, density=3.0e24, ramp=4.0e-6, precision=prec)
    deck.window_start_time = 60 * 5.0e-17
    return deck


def test_mixed_roundtrip_conversion(gpu_lib):
    deck = _wake(abi.PREC_MIXED)
    parts, rng = cg.host_load(deck)
    run = cg.Run(deck, particles=parts, rng=rng, initialise=False)
    p = run.particles(0).sorted_by_id()
    q = parts[0].sorted_by_id()
    assert np.array_equal(p.id, q.id)
    assert np.max(np.abs(p.x - q.x)) < 1e-6 * deck.dx
    assert np.max(np.abs(p.y - q.y)) < 1e-6 * deck.y_max
    assert rel_l2(p.w, q.w) < 1e-7


def test_mixed_vs_fp64_wakefield(gpu_lib):
    d64 = _wake(abi.PREC_FP64)
    d32 = _wake(abi.PREC_MIXED)
    parts, rng = cg.host_load(d64)
    a = cg.Run(d64, particles=parts, rng=rng)
    b = cg.Run(d32, particles=parts, rng=rng)
    for k in (16, 16, 32, 32):
        a.step(k)
        b.step(k)
    sa, sb = a.state(), b.state()
    assert sa.n_shifts == sb.n_shifts and sa.n_shifts > 0
    assert abs(sa.n_live[0] - sb.n_live[0]) <= max(2, 1e-4 * sa.n_live[0])
    ea, eb = a.field("exm"), b.field("exm")
    errs = [rel_l2(eb[m], ea[m]) for m in range(d64.n_mode)]
    print("mixed vs fp64 Ez rel L2 per mode:", errs)
    for m, e in enumerate(errs):
        assert e < TOL_EZ, (m, e)
    da, db = a.diagnostics(), b.diagnostics()
    assert abs(db.kinetic_energy - da.kinetic_energy) <= TOL_EZ * da.kinetic_energy
    assert db.device_error == 0


def test_mixed_thermal_energy(gpu_lib):
    d64 = cg.thermal_plasma(nx=64, ny=32, ppc=8)
    d32 = cg.thermal_plasma(nx=64, ny=32, ppc=8, precision=abi.PREC_MIXED)
    parts, rng = cg.host_load(d64)
    a = cg.Run(d64, particles=parts, rng=rng)
    b = cg.Run(d32, particles=parts, rng=rng)
    a.step(40)
    b.step(40)
    da, db = a.diagnostics(), b.diagnostics()
    assert da.n_live == db.n_live
    assert abs(db.kinetic_energy - da.kinetic_energy) < 1e-3 * da.kinetic_energy
    for n in ("exm", "erm"):
        x, y = a.field(n), b.field(n)
        assert rel_l2(y[0], x[0]) < 5e-3, n


def test_mixed_continuity_residual(gpu_lib):
    """Discrete continuity residual of one mixed-form step, evaluated in FP64
    from the stored state: m = 0 within the form's 1e-3 error bar (the FP64
    form is at round-off), m = 1 within 1e-3 of the FP64 form's value."""
    from cylindrical_epoch_gb300.diagnostics import continuity_residual
    d64 = cg.thermal_plasma(nx=64, ny=32, ppc=8)
    d32 = cg.thermal_plasma(nx=64, ny=32, ppc=8, precision=abi.PREC_MIXED)
    parts, rng = cg.host_load(d64)
    res = []
    for d in (d64, d32):
        run = cg.Run(d, particles=parts, rng=rng)
        run.step(2)
        r0 = run.charge_density()
        run.step(1)
        r1 = run.charge_density()
        res.append(continuity_residual(d, r0, r1, run.field("jxm"), run.field("jrm"), run.field("jtm"),
                                       d.grid_desc().dt)[0])
        run.close()
    print("continuity residual per mode: fp64", res[0], "mixed", res[1])
    assert res[0][0] < 1e-12
    assert res[1][0] < TOL_EZ
    assert abs(res[1][1] - res[0][1]) < TOL_EZ


def test_tile_shapes_agree(gpu_lib):
    """Every tile shape of the mixed push gives the same run: the shape only
    changes how particles are grouped into the exact per-tile sums, whose
    FP32 flush rounds differently.  After 96 steps of a laser wakefield with
    the window moving: particle count within 2, Ez per mode and kinetic
    energy within 1e-4 relative of shape 0 (the form's error bar against
    FP64 is 1e-3)."""
    deck = _wake(abi.PREC_MIXED)
    parts, rng = cg.host_load(deck)
    ref = None
    for k in range(abi.N_TILE_SHAPES):
        run = cg.Run(deck, particles=parts, rng=rng)
        idx, (tx, ty) = run.tune_tiles(k)
        assert idx == k and tx * ty > 0
        run.step(48)
        run.step(48, graph=True)
        s, d, ez = run.state(), run.diagnostics(), run.field("exm")
        assert d.device_error == 0
        run.close()
        if ref is None:
            ref = (s, d, ez)
            assert s.n_shifts > 0
            continue
        assert s.n_shifts == ref[0].n_shifts
        assert abs(s.n_live[0] - ref[0].n_live[0]) <= 2
        assert abs(d.kinetic_energy - ref[1].kinetic_energy) <= 1e-4 * ref[1].kinetic_energy, k
        for m in range(deck.n_mode):
            assert rel_l2(ez[m], ref[2][m]) < 1e-4, (k, m)


def test_tune_tiles_keeps_state(gpu_lib):
    """cyl_tune_tiles in timing mode pushes copies of the state: the run's
    particles are the same set afterwards (same ids, positions, momenta),
    and its currents and later steps are those of a run set to the chosen
    shape.  The FP64 form has no tiles and refuses."""
    deck = _wake(abi.PREC_MIXED)
    parts, rng = cg.host_load(deck)
    a = cg.Run(deck, particles=parts, rng=rng)
    a.step(20)
    before = a.particles(0).sorted_by_id()
    j0 = a.field("jxm")
    k, _ = a.tune_tiles()
    assert 0 <= k < abi.N_TILE_SHAPES
    after = a.particles(0).sorted_by_id()
    for name in ("id", "x", "y", "z", "px", "py", "pz", "w"):
        assert np.array_equal(getattr(before, name), getattr(after, name)), name
    assert np.array_equal(j0, a.field("jxm"))
    a.step(20)
    assert a.diagnostics().device_error == 0
    a.close()
    d64 = _wake(abi.PREC_FP64)
    b = cg.Run(d64, particles=parts, rng=rng)
    with pytest.raises(abi.CylError):
        b.tune_tiles()
    b.close()


def test_mixed_number_density(gpu_lib):
    """The mixed form's number density (evaluated in FP64 from its stored
    state) against the FP64 form's after a windowed wakefield run."""
    d64 = _wake(abi.PREC_FP64)
    d32 = _wake(abi.PREC_MIXED)
    parts, rng = cg.host_load(d64)
    a = cg.Run(d64, particles=parts, rng=rng)
    b = cg.Run(d32, particles=parts, rng=rng)
    a.step(96)
    b.step(96)
    na, nb = a.number_density(), b.number_density()
    for m in range(d64.n_mode):
        e = rel_l2(nb[m], na[m])
        assert e < TOL_EZ, (m, e)


def test_mixed_large_deck_physics(gpu_lib):
    """The large deck's physics on a small grid: modes m = 0..3, circular
    polarisation (two lasers), mobile helium ions.  Per-mode Ez against the
    FP64 form within 1e-3, relative to the mode itself or, for modes whose
    norm is below 1e-3 of the largest, to the largest mode's norm."""
    from cylindrical_epoch_gb300.deck import M0, Q0, Species
    def deck(prec):
        ions = Species("helium2+", 2.0 * Q0, 4.0 * 1.66053886e-27, 1, 0.01 * 3.0e24, density_kind=1,
                       ramp_x0=0.0, ramp_length=4.0e-6,
                       bc=(abi.BC_SIMPLE_LASER, abi.BC_OPEN, abi.BC_OTHER, abi.BC_OPEN))
        d = cg.wakefield(nx=256, ny=64, n_mode=4, ppc=4, a0=4.0, waist=8.0e-6, density=3.0e24, ramp=4.0e-6,
                         circular=True, ions=ions, precision=prec)
        d.window_start_time = 60 * 5.0e-17
        return d
    d64, d32 = deck(abi.PREC_FP64), deck(abi.PREC_MIXED)
    parts, rng = cg.host_load(d64)
    a = cg.Run(d64, particles=parts, rng=rng)
    b = cg.Run(d32, particles=parts, rng=rng)
    b.tune_tiles()
    for k in (32, 32, 32):
        a.step(k)
        b.step(k)
    assert a.state().n_shifts == b.state().n_shifts > 0
    ea, eb = a.field("exm"), b.field("exm")
    norms = [np.linalg.norm(ea[m]) for m in range(4)]
    errs = []
    for m in range(4):
        ref = norms[m] if norms[m] >= 1e-3 * max(norms) else max(norms)
        errs.append(float(np.linalg.norm(eb[m] - ea[m]) / ref))
    print("M=4 mixed vs fp64 Ez error per mode:", errs, "mode norms:", norms)
    assert max(errs) < TOL_EZ
    assert b.diagnostics().device_error == 0


@pytest.mark.parametrize("kind", ["wakefield", "thermal", "thermal3"])
def test_merged_e_half_steps(gpu_lib, kind):
    """Inside a chunk, the mixed form merges each step's closing E half-step
    with the next step's opening one; the edge cells that the E boundary rules
    touch between them take the halves one at a time.  Against runs with
    every half-step separate (cyl_set_merge_e_halves(h, 0)), under the x_min
    laser and outflow boundaries, periodic x with a conducting r_max, and the
    axis rule of modes m >= 2.  The arithmetic is the same, but the mixed form
    is not bit-reproducible from run to run (the order of its FP64 current
    atomics), so the bar is the spread of two separate-half-step runs: a
    mistake at the edge cells would put O(1) errors on whole rows or columns
    (relative L2 of order 1e-2)."""
    if kind == "wakefield":
        deck = _wake(abi.PREC_MIXED)
    else:
        deck = cg.thermal_plasma(nx=128, ny=32, ppc=4, n_mode=3 if kind == "thermal3" else 2,
                                 precision=abi.PREC_MIXED)
    parts, rng = cg.host_load(deck)
    runs = [cg.Run(deck, particles=parts, rng=rng) for _ in range(3)]
    runs[0].merge_e_halves(False)
    runs[1].merge_e_halves(False)
    for k in (16, 16, 8):
        for r in runs:
            r.step(k, graph=True)
    sep, sep2, merged = runs
    assert sep.state().n_live[0] == merged.state().n_live[0]
    for n in ("exm", "erm", "etm", "bxm", "brm", "btm"):
        fa, fb, fm_ = sep.field(n), sep2.field(n), merged.field(n)
        for m in range(fa.shape[0]):
            if not np.any(fa[m] != 0):
                continue
            spread = rel_l2(fb[m], fa[m])
            assert rel_l2(fm_[m], fa[m]) <= max(1e3 * spread, 1e-9), (n, m, spread)
    for r in runs:
        assert r.diagnostics().device_error == 0
