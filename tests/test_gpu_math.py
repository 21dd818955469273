"""The FP64 kernel's atan2 on the device (cyl_eval_atan2) against the same
routine built for the host (the oracle's orc_atan2_many): bit for bit on the
million-point sweep of tests/test_cyl_math.py, whose CPU tests show that the
routine is correctly rounded."""
import ctypes as C

import numpy as np
import pytest

from cylindrical_epoch_gb300 import abi
from tests.test_cyl_math import _ours, _sweep

pytestmark = pytest.mark.gpu


def test_device_atan2_equals_host(gpu_lib):
    y, x = _sweep(1_000_000, 5)
    host = _ours(y, x)
    dev = np.empty_like(host)
    PD = C.POINTER(C.c_double)
    abi.check("cyl_eval_atan2", gpu_lib.cyl_eval_atan2(y.size, y.ctypes.data_as(PD), x.ctypes.data_as(PD),
                                                       dev.ctypes.data_as(PD)))
    diff = np.nonzero(dev.view(np.int64) != host.view(np.int64))[0]
    assert diff.size == 0, (diff.size, y[diff[:3]], x[diff[:3]], dev[diff[:3]], host[diff[:3]])
