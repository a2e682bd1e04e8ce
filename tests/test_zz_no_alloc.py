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


def _refused(lib, mesh, u):
    f = np.zeros_like(u, order="F")
    rc = lib.axg_stiffness_assembled_noalloc(C.byref(mesh.desc()), _fp(u), _fp(f))
    assert rc in (_abi.AXG_OK, _abi.AXG_ERR_BAD_ARG), lib.axg_last_error(None).decode()
    return rc == _abi.AXG_ERR_BAD_ARG


def test_noalloc_at_the_size_limit_matches_the_oracle(gpu_lib, orc):
    """A one-element-wide strip of quadrupole elements grown until the next
    row no longer fits: the mesh fills the static array to within one
    element's bytes (about 3 KiB), so its last region (the force) ends at the
    array's end.  Two calls in a row against the FP64 oracle."""
    lo, hi = 2000, 20000
    small = structured_mesh(1, lo, 2, terms="pole")
    assert not _refused(gpu_lib, small, random_gvec(small, seed=1))
    while hi - lo > 1:
        mid = (lo + hi) // 2
        mm = structured_mesh(1, mid, 2, terms="pole")
        if _refused(gpu_lib, mm, random_gvec(mm, seed=1)):
            hi = mid
        else:
            lo = mid
    m = structured_mesh(1, lo, 2, terms="pole", seed=77)
    big = structured_mesh(1, lo + 1, 2, terms="pole", seed=77)
    assert _refused(gpu_lib, big, random_gvec(big, seed=1))
    for seed in (41, 42):
        u = random_gvec(m, seed=seed)
        f = _noalloc(gpu_lib, m, u)
        ref = orc.stiffness_assembled(m, u, np.float64)
        assert np.isfinite(f).all()
        assert _rel(f, ref) <= 1e-5


def test_noalloc_unreferenced_points_read_zero(gpu_lib):
    """Global points that no element refers to get a zero force, whatever an
    earlier call left in the shared array."""
    m = structured_mesh(30, 24, 1, seed=5)
    u = random_gvec(m, seed=3)
    f1 = _noalloc(gpu_lib, m, u)
    extra = 64
    m2 = structured_mesh(30, 24, 1, seed=5)
    m2.nglob_solid = m.nglob_solid + extra
    u2 = np.asfortranarray(np.vstack([u, np.ones((extra, 3), np.float32)]))
    big = structured_mesh(40, 40, 1, seed=6)   # leaves nonzero data across the array
    _noalloc(gpu_lib, big, random_gvec(big, seed=4))
    f2 = _noalloc(gpu_lib, m2, u2)
    assert not f2[m.nglob_solid:].any()
    assert np.array_equal(f2[:m.nglob_solid], f1)
