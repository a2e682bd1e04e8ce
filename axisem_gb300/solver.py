"""Host-side mirror of the reference's time-loop interface over the C-ABI.

``Solver`` stands where ``time_loop`` (SOLVER/time_evol_wave.F90:231) is
called from ``SOLVER/main.f90:92``: it is created from the module arrays the
Fortran setup produced (here: a ``Mesh``), runs the Newmark loop on the GPU
and returns the seismograms in the reference's ``(nseismo, 3, num_rec)``
layout.  Errors are raised as ``AxgError`` carrying the library's status code
and message (the reference stops through ``pcheck``, SOLVER/commun.F90:578).
There is no CPU fallback: without the CUDA library or a GPU this raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from .mesh import Mesh


class AxgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"axg error {code}: {msg}")
        self.code = code


def _check(lib, h, rc):
    if rc != _abi.AXG_OK:
        msg = lib.axg_last_error(h).decode()
        raise AxgError(rc, msg)


def _fp(a):
    if a is None:
        return C.cast(None, C.POINTER(C.c_float))
    return a.ctypes.data_as(C.POINTER(C.c_float))


def symplectic_coefficients(scheme: int, deltat: float, lib=None):
    """(coefd, coefv, coeff) of a symplectic scheme times deltat
    (axg_symplectic_coefficients)."""
    lib = lib or _abi.load_library()
    a, b, c = (C.c_double * 40)(), (C.c_double * 40)(), (C.c_double * 40)()
    n = C.c_int32()
    _check(lib, None, lib.axg_symplectic_coefficients(scheme, deltat, a, b, c, C.byref(n)))
    n = n.value
    return np.array(a[: n + 1]), np.array(b[:n]), np.array(c[:n])


def plan_shape(mesh: Mesh, ctas: int = 0, lib=None) -> tuple[int, int]:
    """The patch shape (patch_elems, growth) the planner picks for `mesh` on
    a device with `ctas` resident CTAs of the solid kernel
    (axg_plan_check_ctas, host only).  ctas = 0: the choice for launches the
    mesh fills, as when concurrent solves share the GPU; axg_create tunes for
    the device's own CTAs, which favours smaller patches on small meshes."""
    lib = lib or _abi.load_library()
    inf = _abi.Info()
    _check(lib, None, lib.axg_plan_check_ctas(C.byref(mesh.desc()), 0, -1, ctas, C.byref(inf)))
    return inf.patch_elems_solid, inf.growth_solid


class Solver:
    """One solve on one GPU (one axg_handle)."""

    def __init__(self, mesh: Mesh, lib=None, patch_elems: int = 0, growth: int = -1,
                 share_with: "Solver | None" = None):
        """patch_elems / growth: the patch shape (axg_create_tuned); 0 / -1
        let the planner's tuner choose, as axg_create does.  share_with: an
        open Solver on the same mesh whose device mesh data this solve shares
        (axg_create_sharing); only the source, receivers and run length of
        `mesh` are then this solve's."""
        self.lib = lib or _abi.load_library()
        self.mesh = mesh
        self._desc = mesh.desc()
        h = C.c_void_p()
        if share_with is not None:
            rc = self.lib.axg_create_sharing(share_with.h, C.byref(self._desc), C.byref(h))
        else:
            rc = self.lib.axg_create_tuned(C.byref(self._desc), patch_elems, growth, C.byref(h))
        _check(self.lib, None, rc)
        self.h = h
        self.nseismo = (mesh.niter // max(mesh.seis_it, 1)) + 1

    # -- lifecycle --------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self.lib.axg_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- time loop ----------------------------------------------------------
    def reset(self):
        _check(self.lib, self.h, self.lib.axg_reset(self.h))

    def run(self, first_iter: int = 1, n_iter: int | None = None):
        if n_iter is None:
            n_iter = self.mesh.niter - first_iter + 1
        _check(self.lib, self.h, self.lib.axg_run(self.h, first_iter, n_iter))

    def run_async(self, first_iter: int = 1, n_iter: int | None = None):
        """Queue steps on the solve's stream and return (axg_run_async)."""
        if n_iter is None:
            n_iter = self.mesh.niter - first_iter + 1
        _check(self.lib, self.h, self.lib.axg_run_async(self.h, first_iter, n_iter))

    def poll(self) -> bool:
        """True once the queued steps have finished (axg_poll)."""
        done = C.c_int32(0)
        _check(self.lib, self.h, self.lib.axg_poll(self.h, C.byref(done)))
        return bool(done.value)

    def wait(self):
        _check(self.lib, self.h, self.lib.axg_wait(self.h))

    def receivers(self) -> np.ndarray:
        out = np.zeros((self.nseismo, 3, max(self.mesh.num_rec, 1)), dtype=np.float32, order="F")
        n = C.c_int32()
        _check(self.lib, self.h, self.lib.axg_get_receivers(self.h, _fp(out), self.nseismo, C.byref(n)))
        return out[:, :, : self.mesh.num_rec]

    def get_state(self, field: int) -> np.ndarray:
        m = self.mesh
        nsls = max(int(m.anel.get("y_j").size), 1) if m.anel else 1
        # memory variables at the cg4 points (1:4), or at every GLL point (0:4,0:4)
        npt = 25 if (m.anel is not None and "Y" in m.anel) else 4
        if field in (_abi.FIELD_DISP, _abi.FIELD_VELO, _abi.FIELD_ACC0, _abi.FIELD_DISP_COMP,
                     _abi.FIELD_VELO_COMP):
            out = np.zeros((5, 5, m.nel_solid, 3), dtype=np.float32, order="F")
        elif field == _abi.FIELD_MEMVAR:      # memory_var[_cg4](points,6,n_sls,nel_solid)
            out = np.zeros((npt, 6, nsls, m.nel_solid), dtype=np.float32, order="F")
        elif field == _abi.FIELD_ATT_SRC_TR:  # src_tr_tm1_glob[_cg4](points,nel_solid)
            out = np.zeros((npt, m.nel_solid), dtype=np.float32, order="F")
        elif field == _abi.FIELD_ATT_SRC_DEV:  # src_dev_tm1_glob[_cg4](points,6,nel_solid)
            out = np.zeros((npt, 6, m.nel_solid), dtype=np.float32, order="F")
        else:
            out = np.zeros((5, 5, m.nel_fluid), dtype=np.float32, order="F")
        _check(self.lib, self.h, self.lib.axg_get_state(self.h, field, _fp(out)))
        return out

    def set_state(self, field: int, arr: np.ndarray):
        a = np.asfortranarray(arr, dtype=np.float32)
        _check(self.lib, self.h, self.lib.axg_set_state(self.h, field, _fp(a)))

    # -- stiffness + assembly (micro-benchmark operation) ------------------
    def stiffness_assembled(self, u_gvec: np.ndarray) -> np.ndarray:
        u = np.asfortranarray(u_gvec, dtype=np.float32)
        f = np.zeros_like(u, order="F")
        _check(self.lib, self.h, self.lib.axg_stiffness_assembled(self.h, _fp(u), _fp(f)))
        return f

    def upload_disp(self, u_gvec: np.ndarray):
        u = np.asfortranarray(u_gvec, dtype=np.float32)
        _check(self.lib, self.h, self.lib.axg_upload_gvec_disp(self.h, _fp(u)))

    def download_force(self) -> np.ndarray:
        f = np.zeros((self.mesh.nglob_solid, 3), dtype=np.float32, order="F")
        _check(self.lib, self.h, self.lib.axg_download_gvec_force(self.h, _fp(f)))
        return f

    def stiffness_device(self, stream: int | None = None):
        _check(self.lib, self.h, self.lib.axg_stiffness_assembled_device(self.h, stream))

    def time_stiffness(self, n: int) -> float:
        ms = C.c_float()
        _check(self.lib, self.h, self.lib.axg_time_stiffness(self.h, n, C.byref(ms)))
        return ms.value

    def set_time_scheme(self, scheme: int, stf_stages: np.ndarray | None = None):
        """axg_set_time_scheme.  For a symplectic scheme without stf_stages,
        the mesh's Gaussian stf (period 20 deltat, as the test meshes use) is
        evaluated at the stage times t_(iter-1) + coeff(i)."""
        if scheme != _abi.SCHEME_NEWMARK2 and stf_stages is None:
            from .mesh import gauss_at
            _, _, coeff = symplectic_coefficients(scheme, self.mesh.deltat, self.lib)
            t = (np.arange(self.mesh.niter)[:, None] * self.mesh.deltat + coeff[None, :])
            stf_stages = gauss_at(t, 20 * self.mesh.deltat)
        ptr = None if stf_stages is None else _fp(np.asfortranarray(stf_stages, dtype=np.float32))
        self._stf_stages = stf_stages
        _check(self.lib, self.h, self.lib.axg_set_time_scheme(self.h, scheme, ptr))

    def set_compensated(self, on: bool = True):
        """Kahan-compensated predictor / corrector (axg_set_compensated)."""
        _check(self.lib, self.h, self.lib.axg_set_compensated(self.h, int(bool(on))))

    def set_wavefield_dump(self, dump_type: int, strain_it: int = 1, capacity: int = 1, ibeg: int = 0,
                           iend: int = 4, jbeg: int = 0, jend: int = 4, out: np.ndarray | None = None, kwf=None,
                           src_mask: bool = False):
        """axg_set_wavefield_dump with the mesh's data_pointwise arrays
        (mesh.add_pointwise).  Returns the snapshot buffer, (capacity,
        floats_per_snapshot) float32 (`out` if given: page-locked memory lets
        the copies overlap the steps).  src_mask: src_dump_type = 'mask'."""
        from .mesh import dump_desc
        probe = np.zeros(1, dtype=np.float32)
        dd = dump_desc(self.mesh, dump_type, strain_it, probe, 1, ibeg, iend, jbeg, jend, kwf, src_mask)
        _check(self.lib, self.h, self.lib.axg_set_wavefield_dump(self.h, C.byref(dd)))
        if dump_type == _abi.DUMP_NONE:
            self._dump = None
            return None
        floats = self.dump_layout()[2]
        if out is None:
            out = np.zeros((capacity, floats), dtype=np.float32)
        if out.dtype != np.float32 or not out.flags.c_contiguous or out.size < capacity * floats:
            raise ValueError(f"out must be C-contiguous float32 with room for {capacity} x {floats}")
        dd = dump_desc(self.mesh, dump_type, strain_it, out, capacity, ibeg, iend, jbeg, jend, kwf, src_mask)
        _check(self.lib, self.h, self.lib.axg_set_wavefield_dump(self.h, C.byref(dd)))
        self._dump = (out, dd)
        return out

    def dump_layout(self):
        """(solid fields, fluid fields, floats per snapshot, field names)."""
        ns, nf, fl = C.c_int32(), C.c_int32(), C.c_int64()
        names = C.create_string_buffer(4096)
        _check(self.lib, self.h, self.lib.axg_wavefield_dump_layout(self.h, C.byref(ns), C.byref(nf), C.byref(fl),
                                                                    names, len(names)))
        nm = names.value.decode()
        return ns.value, nf.value, fl.value, nm.split(",") if nm else []

    def set_seismogram_checkpoint(self, check_it: int, out: np.ndarray | None = None):
        """Checkpoint the seismograms into `out` (nseismo_cap, 3, num_rec),
        F-ordered float32, every check_it steps (0: off); the array must stay
        alive while runs use it."""
        if check_it and out is not None:
            assert out.dtype == np.float32 and out.flags["F_CONTIGUOUS"] and out.shape[1:] == (3, self.mesh.num_rec)
        self._ckpt = out
        cap = 0 if out is None else out.shape[0]
        _check(self.lib, self.h, self.lib.axg_set_seismogram_checkpoint(self.h, check_it, _fp(out), cap))

    def checkpoint_samples(self) -> int:
        n = C.c_int32(0)
        _check(self.lib, self.h, self.lib.axg_seismogram_checkpoint_samples(self.h, C.byref(n)))
        return n.value

    def autotune(self) -> int:
        """axg_autotune: the measured steps per CUDA graph (the solve's state
        is left as it was)."""
        k = C.c_int32()
        _check(self.lib, self.h, self.lib.axg_autotune(self.h, C.byref(k)))
        return k.value

    def set_tuning(self, patch_elems: int = 0, steps_per_graph: int = 0):
        _check(self.lib, self.h, self.lib.axg_set_tuning(self.h, patch_elems, steps_per_graph))

    def info(self) -> dict:
        inf = _abi.Info()
        _check(self.lib, self.h, self.lib.axg_get_info(self.h, C.byref(inf)))
        return {k: getattr(inf, k) for k, _ in _abi.Info._fields_}

    def solid_colouring(self):
        inf = self.info()
        pe = np.zeros(self.mesh.nel_solid, dtype=np.int32)
        cp = np.zeros(inf["n_patches_solid"], dtype=np.int32)
        _check(self.lib, self.h, self.lib.axg_get_solid_colouring(
            self.h, pe.ctypes.data_as(C.POINTER(C.c_int32)), cp.ctypes.data_as(C.POINTER(C.c_int32)),
            len(cp)))
        return pe, cp


class Batch:
    """Several solves advanced together (axg_batch_*): one launch per colour
    and kernel class covers all of them, and the step is replayed from one
    CUDA graph.  Each solve's results are bit-for-bit those it gets alone.
    The solvers must stay open while the batch exists."""

    def __init__(self, solvers: "list[Solver]"):
        if not solvers:
            raise ValueError("a batch needs at least one solve")
        self.lib = solvers[0].lib
        self.solvers = list(solvers)
        hs = (C.c_void_p * len(solvers))(*[s.h for s in solvers])
        b = C.c_void_p()
        rc = self.lib.axg_batch_create(hs, len(solvers), C.byref(b))
        if rc != _abi.AXG_OK:
            raise AxgError(rc, self.lib.axg_batch_last_error(None).decode())
        self.b = b

    def _check(self, rc):
        if rc != _abi.AXG_OK:
            raise AxgError(rc, self.lib.axg_batch_last_error(self.b).decode())

    def run_async(self, first_iters, n_iter: int):
        """Queue n_iter steps; solve k starts at first_iters[k]."""
        fi = (C.c_int32 * len(self.solvers))(*[int(x) for x in first_iters])
        self._check(self.lib.axg_batch_run_async(self.b, fi, int(n_iter)))

    def poll(self) -> bool:
        done = C.c_int32(0)
        self._check(self.lib.axg_batch_poll(self.b, C.byref(done)))
        return bool(done.value)

    def wait(self):
        self._check(self.lib.axg_batch_wait(self.b))

    def run(self, first_iters, n_iter: int):
        self.run_async(first_iters, n_iter)
        self.wait()

    def launches_per_step(self) -> int:
        n = C.c_int64()
        self._check(self.lib.axg_batch_launches_per_step(self.b, C.byref(n)))
        return n.value

    def close(self):
        if getattr(self, "b", None):
            self.lib.axg_batch_destroy(self.b)
            self.b = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
