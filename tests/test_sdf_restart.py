"""The restart reader (cyl_sdf_open, cyl_sdf_read_field, cyl_sdf_read_particles)
and the restart sequence, on the CPU.

- Round trip: a restart dump written by cyl_sdf_write reads back through the
  product's reader as restart_data reads it (setup.F90:777-1569): every mode
  array zero outside the interior, the rows of the Ex-staggered arrays moved
  back down by one (setup.F90:1237-1247), particles by species, the
  constants dt, window_shift_fraction and x_grid_min, the grid extents.
- Malformed input: a file that is not SDF, a point variable whose count
  differs from its mesh's (setup.F90:1411-1425).
- The oracle's restart (orc_restart: restart_data's scalars, then the
  start-up of epoch2d.F90:143-153) from a dump taken at the output point
  continues exactly as the run that wrote it, on a windowed wakefield deck
  whose window has moved before the dump.
"""
import numpy as np
import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi

NX, NY, M = 20, 10, 2
SHIFTED = {"exm", "etm", "brm", "jxm", "jtm", "brm_old", "jxm_old", "jtm_old"}


def _arrays(seed):
    rng = np.random.default_rng(seed)
    shape = (M, NY + 2 * abi.NG, NX + 2 * abi.NG)
    return {n: rng.standard_normal(shape) + 1j * rng.standard_normal(shape) for n in abi.FIELD_NAMES}


def _particles(n, seed):
    rng = np.random.default_rng(seed)
    p = cg.Particles(n)
    for k in ("x", "y", "z", "px", "py", "pz", "w"):
        setattr(p, k, rng.standard_normal(n))
    p.id = rng.integers(0, 2**40, n)
    return p


def _expected_read(a, name):
    """What the reader gives for array a: the interior rows the file holds,
    zero elsewhere."""
    ng = abi.NG
    s = 1 if name in SHIFTED else 0
    out = np.zeros_like(a)
    out[:, ng - s:ng - s + NY, ng:ng + NX] = a[:, ng - s:ng - s + NY, ng:ng + NX]
    return out


def test_reader_round_trip(tmp_path):
    arrays = _arrays(1)
    species = [("electron", _particles(700, 2)), ("empty", _particles(0, 3)), ("ion", _particles(41, 4))]
    p = tmp_path / "restart.sdf"
    cg.sdf_write_arrays(p, NX, NY, M, arrays, step=12, time=6.5e-15, xb_min=2.5e-7, dx=2.5e-8, dy=1.0e-7,
                        restart=True, species=species, dt=5.0e-17, x_grid_min=2.625e-7,
                        window_shift_fraction=0.375)
    with cg.SdfFile(p) as f:
        i = f.info
        assert (i.step, i.restart, i.time, i.code_name) == (12, 1, 6.5e-15, b"Epoch2d")
        assert (i.nx, i.ny, i.n_mode) == (NX, NY, M)
        assert i.has_dt and i.dt == 5.0e-17
        assert i.has_x_grid_min and i.x_grid_min == 2.625e-7
        assert i.has_window_shift_fraction and i.window_shift_fraction == 0.375
        assert i.has_grid and i.grid_x0 == 2.5e-7 and i.grid_y0 == 0.0
        assert i.grid_x1 == 2.5e-7 + NX * 2.5e-8 and i.grid_y1 == NY * 1.0e-7
        for name in abi.FIELD_NAMES:
            assert np.array_equal(f.field(name), _expected_read(arrays[name], name)), name
        for name, q in species:
            if q.n == 0:
                assert f.species_count(name) == -1
                continue
            assert f.species_count(name) == q.n
            r = f.particles(name)
            for k in q.__slots__:
                assert np.array_equal(getattr(r, k), getattr(q, k)), (name, k)
        assert f.species_count("proton") == -1
        with pytest.raises(KeyError):
            f.particles("proton")


def test_reader_plain_dump_defaults(tmp_path):
    """A dump without restart data: no constants, absent arrays read as zero."""
    arrays = {n: a for n, a in _arrays(5).items() if n in abi.FIELD_NAMES[:9]}
    p = tmp_path / "plain.sdf"
    cg.sdf_write_arrays(p, NX, NY, M, arrays, step=3, time=1.0e-15, dx=1.0e-7, dy=1.0e-7)
    with cg.SdfFile(p) as f:
        i = f.info
        assert i.restart == 0 and not i.has_dt and not i.has_x_grid_min and not i.has_window_shift_fraction
        assert np.array_equal(f.field("exm"), _expected_read(arrays["exm"], "exm"))
        assert not np.any(f.field("jxm_old"))


def test_reader_rejects_bad_files(tmp_path):
    bad = tmp_path / "not.sdf"
    bad.write_bytes(b"NOTSDF" + bytes(200))
    with pytest.raises(abi.CylError):
        cg.SdfFile(bad)
    with pytest.raises(abi.CylError):
        cg.SdfFile(tmp_path / "missing.sdf")
    # a point variable whose count is not its mesh's
    from oracle.sdf_read import read
    p = tmp_path / "bad_count.sdf"
    cg.sdf_write_arrays(p, NX, NY, M, {}, dx=1.0, dy=1.0, species=[("electron", _particles(9, 6))])
    _, inline, _, _ = read(p)
    b = next(b for b in inline if b["id"] == "px/electron")
    raw = bytearray(p.read_bytes())
    at = b["start"] + 200 + 8 + 2 * 32  # mult, units, mesh id, then npoints
    assert int.from_bytes(raw[at:at + 8], "little") == 9
    raw[at:at + 8] = (8).to_bytes(8, "little")
    p.write_bytes(bytes(raw))
    with cg.SdfFile(p) as f:
        with pytest.raises(abi.CylError):
            f.particles("electron")


def _restart_deck():
    deck = cg.wakefield(nx=64, ny=16, ppc=2, density=3.0e24, ramp=1.0e-6)
    deck.window_start_time = 20 * 5.0e-17
    # the restart starts with the deck's boundaries until its first
    # moving_window (as the reference's); equal boundaries before and after
    # the move make that the boundaries the continuing run has
    deck.bc_after_move = None
    return deck


def test_oracle_restart_continues_run(tmp_path):
    from oracle.oracle import Oracle
    deck = _restart_deck()
    parts, rng = cg.host_load(deck)
    a = Oracle(deck, particles=parts, rng=rng)
    a.initialise()
    a.step_to_output(31)
    s = a.state()
    # a moved window, and a shift fraction large enough that dropping it
    # would move the next shift by a step
    assert s.n_shifts > 0 and s.window_started and s.window_shift_fraction > 0.5
    p = tmp_path / "dump.sdf"
    dx = (deck.x_max - deck.x_min) / deck.nx
    dy = deck.y_max / deck.ny
    cg.sdf_write_arrays(p, deck.nx, deck.ny, deck.n_mode, {n: a.field(n) for n in abi.FIELD_NAMES},
                        step=s.step, time=s.time, xb_min=s.xb_min, dx=dx, dy=dy, restart=True,
                        species=[("electron", a.particles(0))], dt=deck.grid_desc().dt,
                        x_grid_min=s.x_grid_min, window_shift_fraction=s.window_shift_fraction)
    b = Oracle(deck, rng=a.rng_state())
    with cg.SdfFile(p) as f:
        for n in abi.FIELD_NAMES:
            b.set_field(n, f.field(n))
        b.set_particles(0, f.particles("electron"))
        i = f.info
        b.restart(i.step, i.time, i.grid_x0, i.x_grid_min, i.window_shift_fraction)
    a.finish_step()
    a.step(12)
    b.step(12)
    sa, sb = a.state(), b.state()
    assert (sa.step, sa.time, sa.n_shifts, sa.x_grid_min, sa.xb_min) == \
        (sb.step, sb.time, sb.n_shifts, sb.x_grid_min, sb.xb_min)
    assert sa.window_shift_fraction == sb.window_shift_fraction and sa.n_live[0] == sb.n_live[0]
    for n in abi.FIELD_NAMES:
        assert np.array_equal(a.field(n), b.field(n)), n
    pa, pb = a.particles(0), b.particles(0)
    for k in pa.__slots__:
        assert np.array_equal(getattr(pa, k), getattr(pb, k)), k


def test_reader_argument_checks(tmp_path):
    p = tmp_path / "particles_only.sdf"
    cg.sdf_write_arrays(p, NX, NY, M, {}, dx=1.0, dy=1.0, species=[("electron", _particles(5, 7))])
    with cg.SdfFile(p) as f:
        assert (f.info.nx, f.info.ny, f.info.n_mode) == (0, 0, 0)
        # no mode arrays: the file does not say their shape
        with pytest.raises(abi.CylError):
            f.field("exm")
        assert f.particles("electron").n == 5
    p2 = tmp_path / "fields.sdf"
    cg.sdf_write_arrays(p2, NX, NY, M, {"exm": _arrays(8)["exm"]}, dx=1.0, dy=1.0)
    with cg.SdfFile(p2) as f:
        with pytest.raises(abi.CylError):
            f.field(abi.NFIELDS)
        with pytest.raises(abi.CylError):
            f.field(-1)
