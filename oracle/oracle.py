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


def stiffness_fluid(mesh, chi_elem: np.ndarray, dtype=np.float64) -> np.ndarray:
    """glob_fluid_stiffness element-local (no masks, no assembly)."""
    tag, ct, nt = _t(dtype)
    d = mesh.desc()
    c = np.asfortranarray(chi_elem, dtype=nt)
    f = np.zeros_like(c, order="F")
    getattr(lib(), f"orc_{tag}_stiffness_fluid")(C.byref(d), _p(c, ct), _p(f, ct))
    return f


def _mask_axis(mesh, a, comps, fluid=False):
    """apply_axis_mask_* on an element-local array (a copy)."""
    a = np.array(a, dtype=np.float64, order="F", copy=True)
    ax = (mesh.ax_el_fluid if fluid else mesh.ax_el_solid)
    if ax is None or len(ax) == 0:
        return a
    e = np.asarray(ax) - 1
    if a.ndim == 3:
        a[0, :, e] = 0.0
    else:
        for c in comps:
            a[0, :, e, c] = 0.0
    return a


def energy(mesh, disp, velo, dchi=None, ddchi=None) -> dict:
    """The total energy of `energy` (SOLVER/time_evol_wave.F90:1424-1526) in
    FP64: elastic 2 pi sum(u K u) and kinetic 2 pi sum(v^2 m) of the solid,
    with the unassembled mass rho J s w (the dipole's z twice), and in the
    fluid 2 pi sum(ddchi^2 m / lambda) and 2 pi sum(dchi K_f dchi); the
    total is half their sum.  The unassembled masses come from
    mesh.meta['unassem_mass_rho_solid'] and ['unassem_mass_lam_fluid']."""
    pole = mesh.src_type
    comps = {0: [0], 1: [1, 2], 2: [0, 1, 2]}[pole]
    u = _mask_axis(mesh, disp, comps)
    if pole == 0:
        u[..., 1] = 0.0
    ku = stiffness_solid(mesh, u, np.float64)
    ku = _mask_axis(mesh, ku, comps)
    epot_sol = 2.0 * np.pi * float(np.sum(ku * u))
    m = np.asarray(mesh.meta["unassem_mass_rho_solid"], dtype=np.float64)
    v2 = np.asarray(velo, dtype=np.float64) ** 2
    kin = v2[..., 0] * m + v2[..., 1] * m + v2[..., 2] * m * (2.0 if pole == 1 else 1.0)
    if pole == 0:
        kin = v2[..., 0] * m + v2[..., 2] * m
    ekin_sol = 2.0 * np.pi * float(np.sum(kin))
    epot_flu = ekin_flu = 0.0
    if mesh.nel_fluid > 0 and dchi is not None:
        mf = np.asarray(mesh.meta["unassem_mass_lam_fluid"], dtype=np.float64)
        epot_flu = 2.0 * np.pi * float(np.sum(np.asarray(ddchi, np.float64) ** 2 * mf))
        dc = np.array(dchi, dtype=np.float64, order="F", copy=True)
        if pole != 0:
            dc = _mask_axis(mesh, dc, None, fluid=True)
        kf = stiffness_fluid(mesh, dc, np.float64)
        if pole != 0:
            kf = _mask_axis(mesh, kf, None, fluid=True)
        ekin_flu = 2.0 * np.pi * float(np.sum(kf * dc))
    return {"epot_sol": epot_sol, "ekin_sol": ekin_sol, "epot_flu": epot_flu, "ekin_flu": ekin_flu,
            "total": 0.5 * (epot_sol + ekin_sol + epot_flu + ekin_flu)}


def gradient_cg4(mesh, f_elem: np.ndarray, dtype=np.float64) -> np.ndarray:
    """axisym_gradient_solid_el_cg4 for every element: (4, 2, nel)."""
    tag, ct, nt = _t(dtype)
    d = mesh.desc()
    f = np.asfortranarray(f_elem, dtype=nt)
    out = np.zeros((4, 2, mesh.nel_solid), dtype=nt, order="F")
    getattr(lib(), f"orc_{tag}_gradient_cg4_all")(C.byref(d), _p(f, ct), _p(out, ct))
    return out


def wavefield_dump(mesh, dd, disp, velo, chi, dchi, dtype=np.float64) -> np.ndarray:
    """One snapshot of dump_stuff's fields (compute_strain, dump_*_global,
    SOLVER/time_evol_wave.F90:1201-1410, SOLVER/wavefields_io.f90:840-1115)
    from element-local state, in the layout of axg_wavefield_dump_layout;
    dd is the axg_dump_desc (its out and capacity are not used)."""
    tag, ct, nt = _t(dtype)
    d = mesh.desc()
    np_el = (dd.iend - dd.ibeg + 1) * (dd.jend - dd.jbeg + 1)
    out = np.zeros(12 * np_el * (mesh.nel_solid + max(mesh.nel_fluid, 0)), dtype=nt)
    args = [np.asfortranarray(a, dtype=nt) for a in (disp, velo, chi, dchi)]
    fn = getattr(lib(), f"orc_{tag}_wavefield_dump")
    fn.restype = C.c_int
    nfld = fn(C.byref(d), C.byref(dd), *[_p(a, ct) for a in args], _p(out, ct))
    return out, nfld


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
        # memory variables at the cg4 points, or at every GLL point
        npt = 25 if (m.anel is not None and "Y" in m.anel) else 4
        self.memvar = np.zeros((npt, 6, max(nsls, 1), m.nel_solid), dtype=self.nt, order="F")
        self.src_tr_tm1 = np.zeros((npt, m.nel_solid), dtype=self.nt, order="F")
        self.src_dev_tm1 = np.zeros((npt, 6, m.nel_solid), dtype=self.nt, order="F")
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

    def run_symplectic(self, first_iter: int, n_iter: int, scheme: int, stf_stages: np.ndarray) -> int:
        """symplectic_time_loop (with attenuation if the mesh has it) for iterations first_iter..; the
        scheme's coefficients are this module's restatement
        (symplectic_coefficients), stf_stages (niter, nstages) the source time
        function at the stage times."""
        ct = self.ct
        cd, cv, _ = symplectic_coefficients(scheme, self.mesh.deltat)
        stf = np.asfortranarray(stf_stages, dtype=np.float32)
        fn = getattr(lib(), f"orc_{self.tag}_time_loop_symplectic")
        fn.restype = C.c_int
        return fn(C.byref(self.d), C.c_int32(len(cv)), _p(cd, C.c_double), _p(cv, C.c_double),
                  _p(stf, C.c_float), _p(self.disp, ct), _p(self.velo, ct), _p(self.chi, ct), _p(self.dchi, ct),
                  _p(self.memvar, ct), _p(self.src_tr_tm1, ct), _p(self.src_dev_tm1, ct),
                  C.c_int32(first_iter), C.c_int32(n_iter), _p(self.rec, C.c_float), C.c_int32(self.nseismo),
                  C.byref(self.iseismo), C.byref(self.blowup_iter))

    def receivers(self) -> np.ndarray:
        return self.rec[:, :, : self.mesh.num_rec]


def _sp(x: float) -> float:
    """A Fortran literal without kind suffix: a single-precision value."""
    return float(np.float32(x))


def _ss_scheme(g):
    """SS_scheme (SOLVER/time_evol_wave.F90:972-992) as Fortran evaluates it:
    its middle drift 1 / 2 - sum(a(1:n)) has the integer quotient 1 / 2 = 0."""
    n = len(g)
    a = [0.0] * (2 * n + 2)
    b = [0.0] * (2 * n + 1)
    a[0] = g[0] / 2.0
    for i in range(1, n):
        a[i] = (g[i - 1] + g[i]) / 2.0
    sa = 0.0
    for i in range(n):
        sa += a[i]
    a[n] = 0 - sa
    for i in range(n + 1, 2 * n + 2):
        a[i] = a[2 * n + 1 - i]
    sg = 0.0
    for i in range(n):
        b[i] = g[i]
        sg += g[i]
    b[n] = 1.0 - 2.0 * sg
    for i in range(n + 1, 2 * n + 1):
        b[i] = b[2 * n - i]
    return a, b


def symplectic_coefficients(scheme: int, deltat: float):
    """symplectic_coefficients (SOLVER/time_evol_wave.F90:749-967): drifts
    coefd(1:n+1), kicks coefv(1:n) times deltat and the stage times coeff."""
    if scheme == 1:    # symplec4, PEFRL
        zeta, iota, kappa = _sp(+0.1786178958448091), _sp(-0.2123418310626054), _sp(-0.06626458266981849)
        cd = [zeta, kappa, 1.0 - 2.0 * (zeta + kappa), kappa, zeta]
        cv = [0.5 - iota, iota, iota, 0.5 - iota]
    elif scheme == 2:  # ML_SO4m5
        rho = (14.0 - np.sqrt(19.0)) / 108.0
        theta = (20.0 - 7.0 * np.sqrt(19.0)) / 108.0
        nu, lam = 2.0 / 5.0, -1.0 / 10.0
        cd = [rho, theta, 0.5 - rho - theta, 0.5 - rho - theta, theta, rho]
        cv = [nu, lam, 1.0 - 2.0 * (nu + lam), lam, nu]
    elif scheme == 3:  # ML_SO6m7
        d = [_sp(x) for x in (-1.01308797891717472981, 1.18742957373254270702, -0.01833585209646059034,
                              0.34399425728109261313)]
        v = [_sp(x) for x in (0.00016600692650009894, -0.37962421426377360608, 0.68913741185181063674,
                              0.38064159097092574080)]
        cd = d + d[::-1]
        cv = v + v[2::-1]
    elif scheme == 4:  # KL_O8m17
        cd, cv = _ss_scheme([_sp(x) for x in (
            0.13020248308889008088, 0.56116298177510838456, -0.38947496264484728641, 0.15884190655515560090,
            -0.39590389413323757734, 0.18453964097831570709, 0.25837438768632204729, 0.29501172360931029887)])
    elif scheme == 5:  # SS_35o10
        cd, cv = _ss_scheme([_sp(x) for x in (
            0.078795722521686419263907679337684, 0.31309610341510852776481247192647,
            0.027918383235078066109520273275299, -0.22959284159390709415121339679655,
            0.13096206107716486317465685927961, -0.26973340565451071434460973222411,
            0.074973343155891435666137105641410, 0.11199342399981020488957508073640,
            0.36613344954622675119314812353150, -0.39910563013603589787862981058340,
            0.10308739852747107731580277001372, 0.41143087395589023782070411897608,
            -0.0048663605831352617621956593099771, -0.39203335370863990644808193642610,
            0.051942502962449647037182904015976, 0.050665090759924496335874344156866,
            0.049674370639729879054568800279461)])
    else:
        raise ValueError(f"unknown symplectic scheme {scheme}")
    cd = np.array(cd, dtype=np.float64) * deltat
    cv = np.array(cv, dtype=np.float64) * deltat
    coeff = np.cumsum(cd[:-1])
    return cd, cv, coeff


# ---------------------------------------------------------------- timing build
FAST_LIB = HERE / "_build" / "liboracle_fast.so"
_fast = None


def fast_lib():
    """The FP32 restatement built for speed (-O3, the host's instruction set,
    OpenMP): the CPU baseline's timing build, not a parity reference."""
    global _fast
    if _fast is None:
        if not FAST_LIB.exists():
            build()
        _fast = C.CDLL(str(FAST_LIB))
        _fast.orc_fast_colour_elements.restype = C.c_int
    return _fast


class CpuStiffness:
    """Threaded stiffness + assembly of one mesh on the host cores: elements
    coloured once (no two elements of a colour share a point), then per
    colour threads over disjoint element ranges, each element gathering,
    masking, applying glob_stiffness_<pole>_4 and adding into the assembled
    force."""

    def __init__(self, mesh):
        self.mesh = mesh
        self.d = mesh.desc()
        self.order = np.zeros(mesh.nel_solid, dtype=np.int32)
        self.cstart = np.zeros(33, dtype=np.int32)
        self.ncol = fast_lib().orc_fast_colour_elements(C.byref(self.d), _p(self.order, C.c_int32),
                                                        _p(self.cstart, C.c_int32))
        if self.ncol < 0:
            raise RuntimeError("element colouring needs more than 32 colours")

    def __call__(self, u_gvec: np.ndarray, f_gvec: np.ndarray, threads: int = 0):
        fast_lib().orc_fast_stiffness_assembled_coloured(
            C.byref(self.d), _p(self.order, C.c_int32), _p(self.cstart, C.c_int32), C.c_int(self.ncol),
            _p(u_gvec, C.c_float), _p(f_gvec, C.c_float), C.c_int(threads))
        return f_gvec
