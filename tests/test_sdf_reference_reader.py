"""This package's SDF dumps read by the reference's own SDF C library
(SDF/C, built by oracle/sdf_ref.py into oracle/_ref/), not by a restatement:
the header, the order, ids, names, types, dims, staggers, mesh ids and units
of every block, and every value, against what was written.  Skipped where
the reference's sources are absent (the library is built from them)."""
import numpy as np
import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi
from tests.test_sdf import (CONST_NAMES, M, META, NX, NY, PVARS, _arrays, _expected_order, _interior,
                            _particles)


@pytest.fixture(scope="module")
def ref():
    from oracle import sdf_ref
    try:
        exe = sdf_ref.build()
    except RuntimeError as e:
        pytest.fail(str(e))
    if exe is None:
        pytest.skip("the reference's SDF C sources are not available here")
    return sdf_ref


BT_PLAIN_MESH, BT_POINT_MESH, BT_PLAIN_VAR, BT_POINT_VAR, BT_CONST = 1, 2, 3, 4, 5
DT_INT8, DT_REAL8 = 2, 4


def _check_with_reference(ref, path, arrays, restart, step, time, xb_min, dx, dy, species=(), consts=None):
    h, blocks = ref.read(path)
    consts = consts if consts is not None else ({"x_grid_min": xb_min + 0.5 * dx} if restart else {})
    order = _expected_order(restart, species, consts)
    assert h["code_name"] == "Epoch2d" and h["step"] == step and h["time"] == time
    assert h["restart"] == (1 if restart else 0) and h["nblocks"] == len(order)
    assert [b["id"] for b in blocks] == order
    by_sp = dict(species)
    for b in blocks:
        assert not b.get("read_error"), b["id"]
        if b["blocktype"] == BT_CONST:
            assert b["name"] == CONST_NAMES[b["id"]] and b["constant"] == consts[b["id"]]
        elif b["blocktype"] == BT_PLAIN_VAR:
            name, part = b["id"].rsplit("_", 1)
            title, units, stagger = META[name]
            assert (b["name"], b["units"], b["stagger"], b["mesh_id"]) == (f"{title}/{part}", units, stagger,
                                                                            "mode_grid")
            assert b["datatype"] == DT_REAL8 and b["dims"] == [NX, NY, M]
            got = b["data"].reshape(M, NY, NX)
            assert np.array_equal(got, _interior(arrays[name], name, part)), b["id"]
        elif b["blocktype"] == BT_PLAIN_MESH:
            assert b["id"] == "grid" and b["name"] == "Grid/Grid" and b["dims"] == [NX + 1, NY + 1]
            x, y = b["grids"]
            assert np.array_equal(x, xb_min + np.arange(NX + 1) * dx)
            assert np.array_equal(y, np.arange(NY + 1) * dy)
        elif b["blocktype"] == BT_POINT_MESH:
            sp = b["id"].split("/", 1)[1]
            p = by_sp[sp]
            assert b["name"] == f"Grid/Particles/{sp}" and b["dims"][0] == p.n
            assert all(np.array_equal(g, v) for g, v in zip(b["grids"], (p.x, p.y, p.z)))
        elif b["blocktype"] == BT_POINT_VAR:
            var, sp = b["id"].split("/", 1)
            title, units, attr, dt = PVARS[var]
            assert b["name"] == f"Particles/{title}/{sp}" and b["units"] == units and b["datatype"] == dt
            assert b["mesh_id"] == f"grid/{sp}"
            assert np.array_equal(b["data"], getattr(by_sp[sp], attr)), b["id"]
        else:
            raise AssertionError(("unexpected block type", b))


def test_reference_reads_field_dump(tmp_path, ref):
    arrays = _arrays(abi.FIELD_NAMES[:9])
    p = tmp_path / "fields.sdf"
    cg.sdf_write_arrays(p, NX, NY, M, arrays, step=17, time=1.25e-14, xb_min=-3.0e-6, dx=2.5e-8, dy=1.0e-7)
    _check_with_reference(ref, p, arrays, False, 17, 1.25e-14, -3.0e-6, 2.5e-8, 1.0e-7)


def test_reference_reads_restart_dump_with_particles(tmp_path, ref):
    arrays = _arrays(abi.FIELD_NAMES, seed=9)
    species = [("electron", _particles(513, 10)), ("empty", _particles(0, 3)), ("ion", _particles(29, 4))]
    p = tmp_path / "restart_p.sdf"
    consts = {"dt": 4.0e-17, "window_shift_fraction": 0.375, "x_grid_min": 1.5e-6}
    cg.sdf_write_arrays(p, NX, NY, M, arrays, step=40, time=8.0e-15, xb_min=1.49e-6, dx=2.0e-8, dy=4.0e-8,
                        restart=True, species=species, dt=consts["dt"], x_grid_min=consts["x_grid_min"],
                        window_shift_fraction=consts["window_shift_fraction"])
    _check_with_reference(ref, p, arrays, True, 40, 8.0e-15, 1.49e-6, 2.0e-8, 4.0e-8, species, consts)


def test_reference_reads_run_dump(tmp_path, ref):
    """A dump written by cyl_sdf_write from host arrays shaped like a run's
    (the path cyl_write_sdf takes after downloading the device state)."""
    arrays = _arrays(abi.FIELD_NAMES[:9], seed=21)
    species = [("electron", _particles(2000, 22))]
    p = tmp_path / "run.sdf"
    cg.sdf_write_arrays(p, NX, NY, M, arrays, step=120, time=6.0e-15, xb_min=2.5e-7, dx=2.5e-8, dy=1.0e-7,
                        species=species)
    _check_with_reference(ref, p, arrays, False, 120, 6.0e-15, 2.5e-7, 2.5e-8, 1.0e-7, species)
