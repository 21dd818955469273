"""cyl_cell_indices_noalloc (fixed static scratch, no allocation) against
cyl_cell_indices (per-call scratch), through the C ABI, over two calls in a
row after each of two pushes, and on a species whose slots hold removed
particles (holes) that no sort has compacted yet.  Collected last so that it
also runs after every other GPU test in the same process."""
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


@pytest.mark.parametrize("prec", [abi.PREC_FP64, abi.PREC_MIXED])
def test_noalloc_with_removed_particles(gpu_lib, prec):
    """A drifting plasma with open x boundaries: the push of the last step
    removes the particles that crossed x_max, and stopping at that step's
    output point (no sort since the push) leaves their slots as holes."""
    deck = cg.thermal_plasma(nx=40, ny=20, ppc=5, precision=prec)
    deck.bc_field = (abi.BC_SIMPLE_OUTFLOW, abi.BC_SIMPLE_OUTFLOW, abi.BC_OTHER, abi.BC_CONDUCT)
    e = deck.species[0]
    e.bc = (abi.BC_OPEN, abi.BC_OPEN, abi.BC_OTHER, abi.BC_CONDUCT)
    e.drift = (0.5 * cg.deck.M0 * cg.deck.CL, 0.0, 0.0)
    parts, rng = cg.host_load(deck)
    run = cg.Run(deck, particles=parts, rng=rng)
    try:
        run.step(19)
        n_before = run.state().n_live[0]
        run.step_to_output(1)
        n_after = run.state().n_live[0]
        assert n_after < n_before, (n_before, n_after)  # holes left by this push
        ref_x, ref_y = run.cell_indices(0)
        assert ref_x.size == n_after
        for _call in range(2):
            gx, gy = _noalloc(run)
            assert np.array_equal(gx, ref_x)
            assert np.array_equal(gy, ref_y)
    finally:
        run.close()


def test_cell_indices_reject_one_null_array(gpu_lib):
    deck = cg.thermal_plasma(nx=16, ny=8, ppc=2)
    parts, rng = cg.host_load(deck)
    run = cg.Run(deck, particles=parts, rng=rng, initialise=False)
    try:
        cx = np.zeros(parts[0].n, dtype=np.int32)
        n = C.c_int64(parts[0].n)
        for fn in (run.lib.cyl_cell_indices, run.lib.cyl_cell_indices_noalloc):
            assert fn(run.h, 0, cx.ctypes.data_as(PI32), None, C.byref(n)) == abi.CYL_ERR_BAD_ARG
            assert fn(run.h, 0, None, cx.ctypes.data_as(PI32), C.byref(n)) == abi.CYL_ERR_BAD_ARG
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
