"""The stiffness + assembly entry point that allocates no device memory.

Callers such as code running inside another runtime's memory pool or with all
device memory reserved up front cannot call cudaMalloc; for them
axg_stiffness_assembled_noalloc keeps every device buffer in a fixed 32 MiB
static device array.  These tests call it through the C-ABI and compare it
with the allocating entry point (axg_stiffness_assembled) on the same inputs,
two calls in a row (the second call must not see the first call's data), and
check that a mesh larger than the array is refused with a clear message.
"""
import ctypes as C

import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import random_gvec, structured_mesh
from axisem_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def _fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _noalloc(lib, mesh, u):
    d = mesh.desc()
    uu = np.asfortranarray(u, dtype=np.float32)
    f = np.full_like(uu, np.nan, order="F")
    rc = lib.axg_stiffness_assembled_noalloc(C.byref(d), _fp(uu), _fp(f))
    assert rc == _abi.AXG_OK, lib.axg_last_error(None).decode()
    return f


def _rel(a, b):
    return float(np.linalg.norm(a.astype(np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("pole", [0, 1, 2])
def test_noalloc_matches_allocating_entry_point(gpu_lib, pole):
    m = structured_mesh(48, 40, pole, seed=900 + pole, axial="random1pct")
    u = random_gvec(m, seed=31)
    v = random_gvec(m, seed=32)
    with Solver(m) as s:
        fu = s.stiffness_assembled(u)
        fv = s.stiffness_assembled(v)
    a = _noalloc(gpu_lib, m, u)
    b = _noalloc(gpu_lib, m, v)
    # same tolerance as the stiffness parity tests (relative L2 <= 1e-5)
    assert np.isfinite(a).all() and np.isfinite(b).all()
    assert _rel(a, fu) <= 1e-5
    assert _rel(b, fv) <= 1e-5


def test_noalloc_rejects_meshes_beyond_the_array(gpu_lib):
    m = structured_mesh(160, 160, 2, terms="pole")
    u = random_gvec(m, seed=1)
    f = np.zeros_like(u, order="F")
    rc = gpu_lib.axg_stiffness_assembled_noalloc(C.byref(m.desc()), _fp(u), _fp(f))
    assert rc == _abi.AXG_ERR_BAD_ARG
    msg = gpu_lib.axg_last_error(None).decode()
    assert "no-allocation" in msg and "bytes" in msg
