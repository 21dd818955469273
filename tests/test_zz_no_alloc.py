"""cyl_cell_indices_noalloc (fixed static scratch, no allocation) against
cyl_cell_indices (per-call scratch), through the C ABI, over two calls in a
row after each of two pushes.  Collected last so that it also runs after
every other GPU test in the same process."""
import ctypes as C

import numpy as np
import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi
from tests.helpers import random_fields

pytestmark = pytest.mark.gpu

PI32 = C.POINTER(C.c_int32)


def _noalloc(run, isp=0):
    n = C.c_int64(0)
    abi.check("cyl_cell_indices_noalloc", run.lib.cyl_cell_indices_noalloc(run.h, isp, None, None, C.byref(n)))
    cx = np.zeros(max(1, n.value), dtype=np.int32)
    cy = np.zeros(max(1, n.value), dtype=np.int32)
    abi.check("cyl_cell_indices_noalloc",
              run.lib.cyl_cell_indices_noalloc(run.h, isp, cx.ctypes.data_as(PI32), cy.ctypes.data_as(PI32),
                                               C.byref(n)))
    return cx[:n.value], cy[:n.value]


@pytest.mark.parametrize("prec", [abi.PREC_FP64, abi.PREC_MIXED])
def test_noalloc_matches_allocating_entry_point(gpu_lib, prec):
    deck = cg.thermal_plasma(nx=40, ny=20, ppc=5, precision=prec)
    parts, rng = cg.host_load(deck)
    run = cg.Run(deck, particles=parts, rng=rng, fields=random_fields(deck, 7), initialise=False)
    try:
        for _ in range(2):
            run.push_only()
            ref_x, ref_y = run.cell_indices(0)
            for _call in range(2):  # two calls in a row reuse the same scratch
                gx, gy = _noalloc(run)
                assert np.array_equal(gx, ref_x)
                assert np.array_equal(gy, ref_y)
    finally:
        run.close()


def test_noalloc_rejects_oversize_species(gpu_lib):
    ppc = abi.NOALLOC_MAX_PARTICLES // (64 * 32) + 1
    deck = cg.thermal_plasma(nx=64, ny=32, ppc=ppc)
    parts, rng = cg.host_load(deck)
    assert parts[0].n > abi.NOALLOC_MAX_PARTICLES
    run = cg.Run(deck, particles=parts, rng=rng, initialise=False)
    try:
        cx = np.zeros(parts[0].n, dtype=np.int32)
        cy = np.zeros(parts[0].n, dtype=np.int32)
        n = C.c_int64(parts[0].n)
        rc = run.lib.cyl_cell_indices_noalloc(run.h, 0, cx.ctypes.data_as(PI32), cy.ctypes.data_as(PI32),
                                              C.byref(n))
        assert rc == abi.CYL_ERR_SCRATCH
    finally:
        run.close()
