"""ctypes wrapper of the CPU oracle (oracle/axisem_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference legs of bench.py, never by the product.  The oracle
restates the reference's hot-path routines (file:line citations in
axisem_oracle.c) in float (the realkind = sp build) and double (realkind = dp).
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

_lib = None


def build():
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
    return _lib


def _t(dtype):
    return ("f32", C.c_float, np.float32) if np.dtype(dtype) == np.float32 else ("f64", C.c_double, np.float64)


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def stiffness_assembled(mesh, u_gvec: np.ndarray, dtype=np.float32) -> np.ndarray:
    """pdistsum_solid(mask(glob_stiffness(mask(u)))) in gvec layout (nglob, 3)."""
    tag, ct, nt = _t(dtype)
    d = mesh.desc()
    u = np.asfortranarray(u_gvec, dtype=nt)
    f = np.zeros_like(u, order="F")
    getattr(lib(), f"orc_{tag}_stiffness_assembled")(C.byref(d), _p(u, ct), _p(f, ct))
    return f


def stiffness_solid(mesh, u_elem: np.ndarray, dtype=np.float32) -> np.ndarray:
    """glob_stiffness_<pole> element-local (no masks, no assembly)."""
    tag, ct, nt = _t(dtype)
    d = mesh.desc()
    u = np.asfortranarray(u_elem, dtype=nt)
    f = np.zeros_like(u, order="F")
    getattr(lib(), f"orc_{tag}_stiffness_solid")(C.byref(d), _p(u, ct), _p(f, ct))
    return f


def gradient_cg4(mesh, f_elem: np.ndarray, dtype=np.float64) -> np.ndarray:
    """axisym_gradient_solid_el_cg4 for every element: (4, 2, nel)."""
    tag, ct, nt = _t(dtype)
    d = mesh.desc()
    f = np.asfortranarray(f_elem, dtype=nt)
    out = np.zeros((4, 2, mesh.nel_solid), dtype=nt, order="F")
    getattr(lib(), f"orc_{tag}_gradient_cg4_all")(C.byref(d), _p(f, ct), _p(out, ct))
    return out


class TimeLoop:
    """sf_time_loop_newmark on element-local state, as the reference holds it."""

    def __init__(self, mesh, dtype=np.float32):
        self.mesh = mesh
        self.tag, self.ct, self.nt = _t(dtype)
        self.d = mesh.desc()
        m = mesh
        self.disp = np.zeros((5, 5, m.nel_solid, 3), dtype=self.nt, order="F")
        self.velo = np.zeros_like(self.disp)
        self.acc0 = np.zeros_like(self.disp)
        nf = max(m.nel_fluid, 1)
        self.chi = np.zeros((5, 5, nf), dtype=self.nt, order="F")
        self.dchi = np.zeros_like(self.chi)
        self.ddchi0 = np.zeros_like(self.chi)
        nsls = 0 if m.anel is None else len(m.anel["y_j"])
        self.memvar = np.zeros((4, 6, max(nsls, 1), m.nel_solid), dtype=self.nt, order="F")
        self.src_tr_tm1 = np.zeros((4, m.nel_solid), dtype=self.nt, order="F")
        self.src_dev_tm1 = np.zeros((4, 6, m.nel_solid), dtype=self.nt, order="F")
        self.nseismo = m.niter // max(m.seis_it, 1) + 1
        self.rec = np.zeros((self.nseismo, 3, max(m.num_rec, 1)), dtype=np.float32, order="F")
        self.iseismo = C.c_int32(1)  # sample 0 is the iter-0 (zero) wavefield
        self.blowup_iter = C.c_int32(0)

    def run(self, first_iter: int, n_iter: int) -> int:
        ct = self.ct
        fn = getattr(lib(), f"orc_{self.tag}_time_loop")
        fn.restype = C.c_int
        return fn(C.byref(self.d), _p(self.disp, ct), _p(self.velo, ct), _p(self.acc0, ct),
                  _p(self.chi, ct), _p(self.dchi, ct), _p(self.ddchi0, ct), _p(self.memvar, ct),
                  _p(self.src_tr_tm1, ct), _p(self.src_dev_tm1, ct), C.c_int32(first_iter),
                  C.c_int32(n_iter), _p(self.rec, C.c_float), C.c_int32(self.nseismo),
                  C.byref(self.iseismo), C.byref(self.blowup_iter))

    def receivers(self) -> np.ndarray:
        return self.rec[:, :, : self.mesh.num_rec]
