"""The C-ABI library loads without a GPU and exports every function that
include/*.h declares; entry points that need a device fail with a status,
not a crash."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        txt = open(os.path.join(ROOT, "include", fn)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        txt = re.sub(r"//[^\n]*", "", txt)
        # prototypes only (inline helpers such as cyl_atan2 have bodies)
        for m in re.finditer(r"\b(?:int|void|double)\s+(cyl_\w+)\s*\([^)]*\)\s*;", txt):
            names.append(m.group(1))
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("cyl_create", "cyl_step", "cyl_destroy", "cyl_upload_particles", "cyl_initialise"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from cylindrical_epoch_gb300 import build
    path = build.build()
    lib = C.CDLL(path)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_create_without_device_reports_status():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import cylindrical_epoch_gb300 as cg
    from cylindrical_epoch_gb300 import abi
    lib = cg.load()
    deck = cg.thermal_plasma(nx=16, ny=8, ppc=1)
    g = deck.grid_desc()
    sp = deck.species_descs()
    h = C.c_void_p()
    rc = lib.cyl_create(C.byref(g), sp, 1, None, 0, None, C.byref(h))
    assert rc == abi.CYL_ERR_NO_DEVICE


def test_wait_timeout_setter():
    """cyl_set_wait_timeout touches no device: NaN is refused, other values
    (<= 0 meaning no limit) are taken."""
    import cylindrical_epoch_gb300 as cg
    from cylindrical_epoch_gb300 import abi
    lib = cg.load()
    assert lib.cyl_set_wait_timeout(float("nan")) == abi.CYL_ERR_BAD_ARG
    assert lib.cyl_set_wait_timeout(0.0) == abi.CYL_OK
    cg.set_wait_timeout(600.0)
