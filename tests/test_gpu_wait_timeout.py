"""The bounded device wait gives up as designed.

Every wait of the patch kernels on an mbarrier (bulk copies landing, sub-rounds
completing) is bounded in time on the GPU's nanosecond timer.  The self-test
entry point waits, through that same wait, on an mbarrier that nothing
arrives at and no copy targets: the wait must give up after about one second,
record AXG_ERR_TIMEOUT, and leave the context usable.  Nothing faults, traps
or hangs.
"""
import ctypes as C

import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import random_gvec, structured_mesh
from axisem_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_with_timeout_status(gpu_lib, orc):
    status = C.c_int32(-99)
    elapsed = C.c_double(0.0)
    rc = gpu_lib.axg_selftest_wait_timeout(C.byref(status), C.byref(elapsed))
    assert rc == _abi.AXG_OK, gpu_lib.axg_last_error(None).decode()
    assert status.value == _abi.AXG_ERR_TIMEOUT
    assert 0.9 <= elapsed.value <= 5.0, elapsed.value
    # the context is still usable: a stiffness evaluation agrees with the oracle
    m = structured_mesh(9, 7, 2, seed=3)
    u = random_gvec(m, seed=4)
    with Solver(m) as s:
        f = s.stiffness_assembled(u)
    ref = orc.stiffness_assembled(m, u, np.float64)
    assert np.linalg.norm(f - ref) / np.linalg.norm(ref) < 1e-5
