"""SDF output of the mode fields (cyl_sdf_write), read back on the CPU with
the independent reader of oracle/sdf_read.py.

Checks, all exact: the header fields the reference's writer sets; the
inline block chain and the summary chain give the same blocks; the block
order, ids, names, units, mesh id and staggers of the reference's field dump
(diagnostics.F90:498-560); the data of every block against the source array,
with the rows of the arrays with Ex's or Etheta's stagger shifted up by one
(write_mode_field, diagnostics.F90:2088-2099); the edge grid; the restart
variant with the _old arrays.  Parity status: unpinned (no reference SDF
files or buildable reference reader here); the layout is restated from the
reference's SDF library sources.
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


def _expected_order(restart):
    groups = [["exm", "erm", "etm"], ["bxm", "brm", "btm"]]
    if restart:
        groups.append(["bxm_old", "brm_old", "btm_old"])
    groups.append(["jxm", "jrm", "jtm"])
    if restart:
        groups.append(["jxm_old", "jrm_old", "jtm_old"])
    out = []
    for g in groups:
        out += [n + "_real" for n in g] + [n + "_imag" for n in g]
    return out + ["grid"]


def _interior(a, name, part):
    ng = abi.NG
    v = a.real if part == "real" else a.imag
    s = 1 if name in SHIFTED else 0
    return v[:, ng - s:ng - s + NY, ng:ng + NX]


def _check(path, arrays, restart, step, time, xb_min, dx, dy):
    from oracle.sdf_read import read
    h, inline, summary, data = read(path)
    assert h.magic == b"SDF1" and h.endianness == 16911887 and (h.version, h.revision) == (1, 4)
    assert h.code_name == "Epoch2d" and h.code_io_version == 1
    assert h.first_block_location == 112 and h.block_header_length == 200 and h.string_length == 128
    assert h.step == step and h.time == time and h.restart_flag == (1 if restart else 0)
    order = _expected_order(restart)
    assert h.nblocks == len(order)
    assert [b["id"] for b in inline] == order == [b["id"] for b in summary]
    assert h.summary_location == inline[-1]["next_block_location"]
    assert h.file_size == h.summary_location + h.summary_size
    for bi, bs in zip(inline, summary):
        for k in bi:
            if k not in ("start", "next_block_location"):
                assert bi[k] == bs[k], (bi["id"], k)
        assert bi["data_location"] == bi["start"] + 200 + bi["info_length"]
    for b in inline[:-1]:
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


def test_sdf_rejects_bad_input(tmp_path):
    import pytest
    with pytest.raises(abi.CylError):
        cg.sdf_write_arrays(tmp_path / "x.sdf", NX, NY, M, {}, dx=0.0)
    with pytest.raises(abi.CylError):
        cg.sdf_write_arrays(tmp_path / "no_such_dir" / "x.sdf", NX, NY, M, {}, dx=1.0, dy=1.0)
