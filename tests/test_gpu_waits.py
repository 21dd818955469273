"""Bounded host waits (cyl_set_wait_timeout).  A wait that runs out returns
CYL_ERR_TIMEOUT without a GPU fault: the queued steps keep running, the run's
host state is the one before the wait, and a later call picks the run up
where it is.  The limit is made to run out by a 1 us limit on calls whose
device work takes milliseconds."""
import ctypes as C

import pytest

import cylindrical_epoch_gb300 as cg
from cylindrical_epoch_gb300 import abi
from tests.helpers import match_by_id, rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [abi.PREC_FP64, abi.PREC_MIXED])
def test_wait_runs_out_then_resumes(gpu_lib, precision):
    deck = cg.wakefield(nx=512, ny=128, ppc=8, precision=precision)
    parts, rng = cg.host_load(deck)
    a = cg.Run(deck, particles=parts, rng=rng)
    b = cg.Run(deck, particles=parts, rng=rng)
    try:
        b.step(64, graph=True)
        a.state()  # nothing queued on a before the limit is set
        cg.set_wait_timeout(1e-6)
        try:
            rc = a.lib.cyl_step_graph(a.h, 64)
        finally:
            cg.set_wait_timeout(600.0)
        assert rc == abi.CYL_ERR_TIMEOUT
        done = a.state().step
        assert done % 16 == 0 and 0 < done <= 64, done
        if done < 64:
            a.step(64 - done, graph=True)
        sa, sb = a.state(), b.state()
        assert sa.step == sb.step == 64
        assert list(sa.n_live) == list(sb.n_live) and sa.n_shifts == sb.n_shifts
        # two runs of the same deck differ by the order of the FP64 atomic
        # current additions: at rounding level in the FP64 form, and through
        # the FP32 fields at ~1e-7 in the mixed form
        tol = 1e-9 if precision == abi.PREC_FP64 else 1e-6
        pa, pb = match_by_id(a.particles(0), b.particles(0))
        for k in ("x", "y", "z", "px", "py", "pz"):
            assert rel_l2(getattr(pa, k), getattr(pb, k)) < tol, k
        for n in ("exm", "bxm", "jxm"):
            fa, fb = a.field(n), b.field(n)
            assert rel_l2(fa[0], fb[0]) < tol, n
    finally:
        a.close()
        b.close()


def test_wait_limit_on_reads(gpu_lib):
    """A state read whose wait runs out returns CYL_ERR_TIMEOUT; the same read
    with the limit lifted returns the run's state."""
    deck = cg.wakefield(nx=512, ny=128, ppc=8)
    parts, rng = cg.host_load(deck)
    a = cg.Run(deck, particles=parts, rng=rng)
    try:
        a.state()
        assert a.lib.cyl_step_async(a.h, 64) == abi.CYL_OK
        cg.set_wait_timeout(1e-6)
        try:
            st = abi.RunState()
            rc = a.lib.cyl_get_run_state(a.h, C.byref(st))
        finally:
            cg.set_wait_timeout(600.0)
        assert rc == abi.CYL_ERR_TIMEOUT
        assert a.state().step == 64
    finally:
        a.close()
