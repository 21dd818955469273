"""The ctypes mirrors of the header's structs (cylindrical_epoch_gb300/abi.py)
have the C layout: a small C program compiled against include/cylpic.h
prints sizeof and every member's offsetof, and each must equal the ctypes
figure."""
import ctypes as C
import os
import shutil
import subprocess

import pytest

from cylindrical_epoch_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PAIRS = {
    "cyl_grid_desc": abi.GridDesc, "cyl_species_desc": abi.SpeciesDesc, "cyl_laser_desc": abi.LaserDesc,
    "cyl_rng_state": abi.RngState, "cyl_run_state": abi.RunState, "cyl_diag": abi.Diag,
    "cyl_sdf_desc": abi.SdfDesc, "cyl_sdf_species": abi.SdfSpecies, "cyl_sdf_info": abi.SdfInfo,
    "cyl_job_desc": abi.JobDesc, "cyl_job_result": abi.JobResult, "cyl_deck_fns": abi.DeckFns,
}


def test_ctypes_structs_match_header(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "cylpic.h"', "int main(void) {"]
    expect = []
    for cname, cls in PAIRS.items():
        lines.append(f'  printf("%zu\\n", sizeof({cname}));')
        expect.append((cname, "sizeof", C.sizeof(cls)))
        for f in cls._fields_:
            lines.append(f'  printf("%zu\\n", offsetof({cname}, {f[0]}));')
            expect.append((cname, f[0], getattr(cls, f[0]).offset))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = [int(v) for v in subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split()]
    assert len(got) == len(expect)
    bad = [(c, f, e, g) for (c, f, e), g in zip(expect, got) if e != g]
    assert not bad, bad
