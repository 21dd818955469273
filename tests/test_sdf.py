"""SDF output of the mode fields (cyl_sdf_write), read back on the CPU with
the independent reader of oracle/sdf_read.py.

Checks, all exact: the header fields the reference's writer sets; the
inline block chain and the summary chain give the same blocks; the block
order, ids, names, units, mesh id and staggers of the reference's field dump
(diagnostics.F90:498-560); the data of every block against the source array,
with the rows of the arrays with Ex's or Etheta's stagger shifted up by one
(write_mode_field, diagnostics.F90:2088-2099); the edge grid; the restart
variant with the _old arrays; the particle blocks (diagnostics.F90:614-762,
write_particle_variable and write_particle_grid): per variable one point
variable per species, then one 3D point mesh per species, species without
particles left out.  The same dumps are read by the reference's own SDF C
library in tests/test_sdf_reference_reader.py, which pins the layout; this
file checks the byte-level details (block headers, summary, offsets) that a
reader does not expose.
"""
import numpy as np

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi

NX, NY, M = 24, 12, 3
SHIFTED = {"exm", "etm", "brm", "jxm", "jtm", "brm_old", "jxm_old", "jtm_old"}
META = {
    "exm": ("Electric Field Modes/Exm", "V/m", 2), "erm": ("Electric Field Modes/Erm", "V/m", 1),
    "etm": ("Electric Field Modes/Etm", "V/m", 3), "bxm": ("Magnetic Field Modes/Bxm", "T", 1),
    "brm": ("Magnetic Field Modes/Brm", "T", 2), "btm": ("Magnetic Field Modes/Btm", "T", 4),
    "jxm": ("Current Modes/Jxm", "A/m^2", 2), "jrm": ("Current Modes/Jrm", "A/m^2", 1),
    "jtm": ("Current Modes/Jtm", "A/m^2", 3),
    "bxm_old": ("Magnetic Field Modes/Bxm_old", "T", 1), "brm_old": ("Magnetic Field Modes/Brm_old", "T", 2),
    "btm_old": ("Magnetic Field Modes/Btm_old", "T", 4), "jxm_old": ("Current Modes/Jxm_old", "A/m^2", 2),
    "jrm_old": ("Current Modes/Jrm_old", "A/m^2", 1), "jtm_old": ("Current Modes/Jtm_old", "A/m^2", 3),
}


def _arrays(names, seed=3):
    rng = np.random.default_rng(seed)
    shape = (M, NY + 2 * abi.NG, NX + 2 * abi.NG)
    return {n: rng.standard_normal(shape) + 1j * rng.standard_normal(shape) for n in names}


def _expected_order(restart, species=(), consts=()):
    out = list(consts) if restart else []
    groups = [["exm", "erm", "etm"], ["bxm", "brm", "btm"]]
    if restart:
        groups.append(["bxm_old", "brm_old", "btm_old"])
    groups.append(["jxm", "jrm", "jtm"])
    if restart:
        groups.append(["jxm_old", "jrm_old", "jtm_old"])
    for g in groups:
        out += [n + "_real" for n in g] + [n + "_imag" for n in g]
    live = [name for name, p in species if p.n > 0]
    for v in ("weight", "px", "py", "pz", "id"):
        out += [f"{v}/{name}" for name in live]
    out += [f"grid/{name}" for name in live]
    return out + ["grid"]


def _interior(a, name, part):
    ng = abi.NG
    v = a.real if part == "real" else a.imag
    s = 1 if name in SHIFTED else 0
    return v[:, ng - s:ng - s + NY, ng:ng + NX]


CONST_NAMES = {"dt": "Time increment", "window_shift_fraction": "Window Shift Fraction",
               "x_grid_min": "Minimum grid position"}


def _check(path, arrays, restart, step, time, xb_min, dx, dy, species=(), consts=None):
    """consts: the restart constants expected, {id: value} in file order."""
    from oracle.sdf_read import read
    h, inline, summary, data = read(path)
    consts = consts if consts is not None else ({"x_grid_min": xb_min + 0.5 * dx} if restart else {})
    nconst = len(consts)
    for b in inline[:nconst]:
        assert b["blocktype"] == 5 and b["datatype"] == 4 and b["ndims"] == 1 and b["data_length"] == 0
        assert b["name"] == CONST_NAMES[b["id"]] and b["value"] == consts[b["id"]]
    inline_all, inline = inline, inline[nconst:]
    nfield = len(_expected_order(restart)) - 1
    assert h.magic == b"SDF1" and h.endianness == 16911887 and (h.version, h.revision) == (1, 4)
    assert h.code_name == "Epoch2d" and h.code_io_version == 1
    assert h.first_block_location == 112 and h.block_header_length == 200 and h.string_length == 128
    assert h.step == step and h.time == time and h.restart_flag == (1 if restart else 0)
    order = _expected_order(restart, species, consts)
    assert h.nblocks == len(order)
    assert [b["id"] for b in inline_all] == order == [b["id"] for b in summary]
    assert h.summary_location == inline_all[-1]["next_block_location"]
    assert h.file_size == h.summary_location + h.summary_size
    for bi, bs in zip(inline_all, summary):
        for k in bi:
            if k not in ("start", "next_block_location"):
                assert bi[k] == bs[k], (bi["id"], k)
        assert bi["data_location"] == bi["start"] + 200 + bi["info_length"]
    for b in inline[:nfield]:
        name, part = b["id"].rsplit("_", 1)
        title, units, stagger = META[name]
        assert b["name"] == f"{title}/{part}" and b["units"] == units and b["stagger"] == stagger
        assert b["blocktype"] == 3 and b["datatype"] == 4 and b["ndims"] == 3
        assert b["mesh_id"] == "mode_grid" and b["mult"] == 1.0 and b["dims"] == [NX, NY, M]
        assert np.array_equal(data[b["id"]], _interior(arrays[name], name, part)), b["id"]
    g = inline[-1]
    assert g["name"] == "Grid/Grid" and g["blocktype"] == 1 and g["dims"] == [NX + 1, NY + 1]
    assert g["labels"] == ["X", "Y"] and g["units"] == ["m", "m"] and g["geometry"] == 1
    x, y = data["grid"]
    assert np.array_equal(x, xb_min + np.arange(NX + 1) * dx)
    assert np.array_equal(y, np.arange(NY + 1) * dy)
    assert g["extents"] == [x[0], y[0], x[-1], y[-1]]
    _check_particles(inline[nfield:-1], data, species)


PVARS = {"weight": ("Weight", "", "w", 4), "px": ("Px", "kg.m/s", "px", 4), "py": ("Py", "kg.m/s", "py", 4),
         "pz": ("Pz", "kg.m/s", "pz", 4), "id": ("ID", "#", "id", 2)}


def _check_particles(blocks, data, species):
    by_name = dict(species)
    for b in blocks:
        var, sp = b["id"].split("/", 1)
        p = by_name[sp]
        assert b["species_id"] == sp and b["npoints"] == p.n
        if var == "grid":
            assert b["name"] == f"Grid/Particles/{sp}" and b["blocktype"] == 2 and b["datatype"] == 4
            assert b["ndims"] == 3 and b["geometry"] == 1 and b["mults"] == [1.0] * 3
            assert b["labels"] == ["X", "Y", "Z"] and b["units"] == ["m"] * 3
            xyz = np.stack([p.x, p.y, p.z])
            assert np.array_equal(data[b["id"]], xyz)
            assert b["extents"] == list(xyz.min(axis=1)) + list(xyz.max(axis=1))
        else:
            title, units, attr, dt = PVARS[var]
            assert b["name"] == f"Particles/{title}/{sp}" and b["units"] == units and b["mult"] == 1.0
            assert b["blocktype"] == 4 and b["datatype"] == dt and b["ndims"] == 1
            assert b["mesh_id"] == f"grid/{sp}"
            assert np.array_equal(data[b["id"]], getattr(p, attr)), b["id"]


def _particles(n, seed):
    rng = np.random.default_rng(seed)
    p = cg.Particles(n)
    for k in ("x", "y", "z", "px", "py", "pz", "w"):
        setattr(p, k, rng.standard_normal(n))
    p.id = rng.integers(-2**62, 2**62, n)
    return p


def test_sdf_field_dump(tmp_path):
    arrays = _arrays(abi.FIELD_NAMES[:9])
    p = tmp_path / "fields.sdf"
    cg.sdf_write_arrays(p, NX, NY, M, arrays, step=17, time=1.25e-14, xb_min=-3.0e-6, dx=2.5e-8, dy=1.0e-7)
    _check(p, arrays, False, 17, 1.25e-14, -3.0e-6, 2.5e-8, 1.0e-7)


def test_sdf_restart_dump(tmp_path):
    arrays = _arrays(abi.FIELD_NAMES, seed=4)
    p = tmp_path / "restart.sdf"
    cg.sdf_write_arrays(p, NX, NY, M, arrays, step=3, time=2.0e-15, xb_min=0.0, dx=5.0e-8, dy=5.0e-8, restart=True)
    _check(p, arrays, True, 3, 2.0e-15, 0.0, 5.0e-8, 5.0e-8)


def test_sdf_particle_dump(tmp_path):
    arrays = _arrays(abi.FIELD_NAMES[:9], seed=5)
    species = [("electron", _particles(1000, 6)), ("empty", _particles(0, 7)), ("ion", _particles(37, 8))]
    p = tmp_path / "particles.sdf"
    cg.sdf_write_arrays(p, NX, NY, M, arrays, step=9, time=3.0e-15, xb_min=1.0e-6, dx=2.0e-8, dy=4.0e-8,
                        species=species)
    _check(p, arrays, False, 9, 3.0e-15, 1.0e-6, 2.0e-8, 4.0e-8, species)


def test_sdf_restart_with_particles(tmp_path):
    arrays = _arrays(abi.FIELD_NAMES, seed=9)
    species = [("electron", _particles(513, 10))]
    p = tmp_path / "restart_p.sdf"
    cg.sdf_write_arrays(p, NX, NY, M, arrays, step=40, time=8.0e-15, xb_min=0.0, dx=2.0e-8, dy=4.0e-8,
                        restart=True, species=species)
    _check(p, arrays, True, 40, 8.0e-15, 0.0, 2.0e-8, 4.0e-8, species)


def test_sdf_rejects_bad_input(tmp_path):
    import pytest
    with pytest.raises(abi.CylError):
        cg.sdf_write_arrays(tmp_path / "x.sdf", NX, NY, M, {}, dx=0.0)
    with pytest.raises(abi.CylError):
        cg.sdf_write_arrays(tmp_path / "no_such_dir" / "x.sdf", NX, NY, M, {}, dx=1.0, dy=1.0)
    with pytest.raises(abi.CylError):
        cg.sdf_write_arrays(tmp_path / "x.sdf", NX, NY, M, {}, dx=1.0, dy=1.0, species=[("", _particles(3, 1))])
