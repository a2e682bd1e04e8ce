"""Host-side mesh container and seeded synthetic meshes.

``Mesh`` holds every array the time loop reads, in the reference's Fortran
column-major layouts and ``realkind = 4`` precision, and fills the C-ABI
descriptor ``axg_mesh_desc`` from them.  It plays the role of the Fortran
module arrays (``data_mesh``, ``data_matr``, ``data_source``, ``data_spec``)
that ``SOLVER/main.f90:56-80`` has set up before ``time_loop``.

``structured_mesh`` builds the structured quad grids used for the stiffness /
assembly micro-benchmark (1024 x 1024 elements, 1 % axial elements) and for
the time-loop tests.  The global numbering follows the lattice of GLL points
of the grid: element (I, J), point (ipol, jpol) -> global point
(4 J + jpol) * (4 NI + 1) + 4 I + ipol + 1, the element-local walk being ipol
fastest as in ``igloc_solid`` (SOLVER/commun.F90:101-128).

Metric terms: the stiffness kernels are data-oblivious (their loads, flops and
memory traffic do not depend on the values), so the synthetic metric arrays
are seeded random values in a physical range (a Lame modulus times a
geometric factor).  Element geometry is a seeded bilinear map whose Jacobian
determinant lies in [0.5, 2]; materials are lambda, mu ~ U[1e10, 3e11] Pa and
rho ~ U[2500, 13000] kg/m^3.  The geometry and materials set the scale of the
metric arrays and of the inverse mass.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from ._abi import AXIAL_TERMS, FLUID_TERMS, SOLID_TERMS
from .spectral import Spectral

F32 = np.float32
I32 = np.int32


def _f(a) -> np.ndarray:
    return np.asfortranarray(np.asarray(a, dtype=F32))


def _i(a) -> np.ndarray:
    return np.asfortranarray(np.asarray(a, dtype=I32))


@dataclass
class Mesh:
    """Arrays of one solve, named as the reference's module variables."""

    src_type: int
    nel_solid: int
    nglob_solid: int
    igloc_solid: np.ndarray                       # (25*nel_solid,) 1-based
    ax_el_solid: np.ndarray                       # (naxel_solid,) 1-based
    spec: Spectral
    m_solid: dict                                 # name -> (5,5,nel_solid) F-order
    m0_solid: dict                                # name -> (5,nel_solid)
    inv_mass_rho: np.ndarray                      # (5,5,nel_solid)
    nel_fluid: int = 0
    nglob_fluid: int = 0
    igloc_fluid: np.ndarray | None = None
    ax_el_fluid: np.ndarray | None = None
    m_fluid: dict = field(default_factory=dict)
    m0_w_fl: np.ndarray | None = None
    inv_mass_fluid: np.ndarray | None = None
    fluid_free_surface_mask: np.ndarray | None = None
    # solid-fluid boundary
    bdry_matr: np.ndarray | None = None            # (5, nel_bdry, 2)
    bdry_solid_el: np.ndarray | None = None
    bdry_fluid_el: np.ndarray | None = None
    bdry_jpol_solid: np.ndarray | None = None
    bdry_jpol_fluid: np.ndarray | None = None
    # source / time
    fluid_src: int = 0
    ielsrc: np.ndarray | None = None               # (8,)
    nelsrc: int = 0
    source_term_el: np.ndarray | None = None       # (5,5,8,3)
    source_term_fl: np.ndarray | None = None       # (5,5,8)
    stf: np.ndarray | None = None                  # (niter,)
    deltat: float = 1.0e-3
    magnitude: float = 1.0e20
    seis_it: int = 1
    recfile_el: np.ndarray | None = None           # (num_rec, 3)
    # attenuation (cg4)
    anel: dict | None = None
    pointwise: dict = field(default_factory=dict)  # data_pointwise arrays (add_pointwise)
    # absorbing boundaries
    solid_absorbing_gamma: np.ndarray | None = None
    fluid_absorbing_gamma: np.ndarray | None = None
    # FP64 copies the compensated mode applies in FP64 (optional)
    inv_mass_rho_dp: np.ndarray | None = None      # (5,5,nel_solid) float64
    inv_mass_fluid_dp: np.ndarray | None = None    # (5,5,nel_fluid) float64
    source_term_el_dp: np.ndarray | None = None    # (5,5,8,3) float64
    # bookkeeping for tests: element grid shape, geometry
    meta: dict = field(default_factory=dict)

    # ------------------------------------------------------------------
    @property
    def niter(self) -> int:
        return 0 if self.stf is None else int(self.stf.shape[0])

    @property
    def num_rec(self) -> int:
        return 0 if self.recfile_el is None else int(self.recfile_el.shape[0])

    def desc(self) -> _abi.MeshDesc:
        """Fill an axg_mesh_desc; the returned struct keeps the arrays alive."""
        d = _abi.MeshDesc()
        keep = []

        def fp(a):
            if a is None:
                return C.cast(None, C.POINTER(C.c_float))
            a = np.asfortranarray(a, dtype=F32)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(C.c_float))

        def ip(a):
            if a is None:
                return C.cast(None, C.POINTER(C.c_int32))
            a = np.asfortranarray(a, dtype=I32)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(C.c_int32))

        def dp(a):
            if a is None:
                return C.cast(None, C.POINTER(C.c_double))
            a = np.asfortranarray(a, dtype=np.float64) if np.ndim(a) > 1 else np.ascontiguousarray(a, np.float64)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(C.c_double))

        d.abi_version = _abi.ABI_VERSION
        d.npol = 4
        d.src_type = self.src_type
        d.fluid_src = self.fluid_src
        d.nel_solid = self.nel_solid
        d.nel_fluid = self.nel_fluid
        d.nglob_solid = self.nglob_solid
        d.nglob_fluid = self.nglob_fluid
        d.naxel_solid = len(self.ax_el_solid)
        d.naxel_fluid = 0 if self.ax_el_fluid is None else len(self.ax_el_fluid)
        d.nel_bdry = 0 if self.bdry_solid_el is None else len(self.bdry_solid_el)
        d.nelsrc = self.nelsrc
        d.niter = self.niter
        d.seis_it = self.seis_it
        d.num_rec = self.num_rec
        d.have_absorbing_bc = int(self.solid_absorbing_gamma is not None)
        d.deltat = self.deltat
        d.magnitude = self.magnitude
        d.igloc_solid = ip(self.igloc_solid)
        d.igloc_fluid = ip(self.igloc_fluid)
        d.ax_el_solid = ip(self.ax_el_solid)
        d.ax_el_fluid = ip(self.ax_el_fluid)
        d.G0 = fp(self.spec.f32("G0"))
        d.G1 = fp(self.spec.f32("G1"))
        d.G1T = fp(self.spec.f32("G1T"))
        d.G2 = fp(self.spec.f32("G2"))
        d.G2T = fp(self.spec.f32("G2T"))
        for k, name in enumerate(SOLID_TERMS):
            d.m_solid[k] = fp(self.m_solid.get(name))
        for k, name in enumerate(AXIAL_TERMS):
            d.m0_solid[k] = fp(self.m0_solid.get(name))
        for k, name in enumerate(FLUID_TERMS):
            d.m_fluid[k] = fp(self.m_fluid.get(name))
        d.m0_w_fl = fp(self.m0_w_fl)
        d.inv_mass_rho = fp(self.inv_mass_rho)
        d.inv_mass_fluid = fp(self.inv_mass_fluid)
        d.fluid_free_surface_mask = fp(self.fluid_free_surface_mask)
        d.solid_absorbing_gamma = fp(self.solid_absorbing_gamma)
        d.fluid_absorbing_gamma = fp(self.fluid_absorbing_gamma)
        d.bdry_matr = fp(self.bdry_matr)
        d.bdry_solid_el = ip(self.bdry_solid_el)
        d.bdry_fluid_el = ip(self.bdry_fluid_el)
        d.bdry_jpol_solid = ip(self.bdry_jpol_solid)
        d.bdry_jpol_fluid = ip(self.bdry_jpol_fluid)
        d.ielsrc = ip(self.ielsrc)
        d.source_term_el = fp(self.source_term_el)
        d.source_term_fl = fp(self.source_term_fl)
        d.stf = fp(self.stf)
        d.recfile_el = ip(self.recfile_el)
        a = self.anel
        if a is not None:
            d.anel_true = 1
            d.n_sls = len(a["y_j"])
            d.do_corr_lowq = int(a.get("do_corr_lowq", 0))
            full = "Y" in a  # attenuation at every GLL point (att_coarse_grained = .false.)
            d.att_coarse_grained = 0 if full else 1
            d.y_j_attenuation = dp(a["y_j"])
            d.exp_w_j_deltat = dp(a["exp_w_j_deltat"])
            d.ts_fac_t = dp(a["ts_fac_t"])
            d.ts_fac_tm1 = dp(a["ts_fac_tm1"])
            names = FULL_ATTENUATION if full else CG4_ATTENUATION
            for nm in ("Q_mu", "Q_kappa", "inv_s_solid") + names:
                setattr(d, nm, fp(a[nm]))
        d.inv_mass_rho_dp = dp(self.inv_mass_rho_dp)
        d.inv_mass_fluid_dp = dp(self.inv_mass_fluid_dp)
        d.source_term_el_dp = dp(self.source_term_el_dp)
        d._keep = keep  # type: ignore[attr-defined]
        return d


# ---------------------------------------------------------------------------
def structured_igloc(ni: int, nj: int, base: int = 0) -> tuple[np.ndarray, int]:
    """igloc for an ni x nj element grid (element e = J*ni + I) on the
    (4 ni + 1) x (4 nj + 1) GLL lattice; returns (igloc 1-based, nglob)."""
    ncol = 4 * ni + 1
    I = np.arange(ni)
    J = np.arange(nj)
    ip = np.arange(5)
    # shape (nj, ni, jpol, ipol) then flattened element-major, ipol fastest
    g = ((4 * J[:, None, None, None] + ip[None, None, :, None]) * ncol
         + 4 * I[None, :, None, None] + ip[None, None, None, :])
    return (g.reshape(-1) + 1 + base).astype(I32), ncol * (4 * nj + 1)


def _bilinear_geometry(rng, ni, nj, h=1.0, s0=0.0):
    """Seeded bilinear maps of an ni x nj grid: lattice corners perturbed by at
    most 0.1 h in each coordinate, which bounds det J / det J_0 to [0.6, 1.48]
    (inside the required [0.5, 2]); the bound is checked at all GLL points."""
    spec = Spectral()
    eta = spec.eta
    xs = s0 + h * np.arange(ni + 1, dtype=np.float64)
    zs = h * np.arange(nj + 1, dtype=np.float64)
    S, Z = np.meshgrid(xs, zs)  # (nj+1, ni+1)
    for _ in range(3):
        pert = rng.uniform(-0.1 * h, 0.1 * h, size=(2, nj + 1, ni + 1))
        s = S + pert[0]
        z = Z + pert[1]
        if s0 == 0.0:
            s[:, 0] = 0.0  # the axis stays straight
        # corners of each element (counter-clockwise)
        c = np.stack([
            np.stack([s[:-1, :-1], z[:-1, :-1]], -1), np.stack([s[:-1, 1:], z[:-1, 1:]], -1),
            np.stack([s[1:, 1:], z[1:, 1:]], -1), np.stack([s[1:, :-1], z[1:, :-1]], -1)], 2)
        # d(s,z)/dxi, d/deta of the bilinear map at GLL points (xi, eta)
        xi = eta[:, None]
        et = eta[None, :]
        dxi = 0.25 * ((c[..., 1, None, None, :] - c[..., 0, None, None, :]) * (1 - et)[..., None]
                      + (c[..., 2, None, None, :] - c[..., 3, None, None, :]) * (1 + et)[..., None])
        deta = 0.25 * ((c[..., 3, None, None, :] - c[..., 0, None, None, :]) * (1 - xi)[..., None]
                       + (c[..., 2, None, None, :] - c[..., 1, None, None, :]) * (1 + xi)[..., None])
        detj = (dxi[..., 0] * deta[..., 1] - dxi[..., 1] * deta[..., 0]) / (0.25 * h * h)
        if detj.min() >= 0.5 and detj.max() <= 2.0:
            return c, detj
    raise RuntimeError("bilinear geometry rejection sampling failed")


def structured_mesh(ni: int, nj: int, src_type: int = _abi.QUADPOLE, *, seed: int = 20261203,
                    axial: str = "random1pct", field_seed: int = 20261204,
                    terms: str = "all") -> Mesh:
    """A solid-only structured mesh of ni x nj elements.

    axial: "random1pct" marks a seeded 1 % of the elements axial (a kernel-path
    stand-in: the axial branch with G1/G1T and the M0 vectors, as in the
    stiffness micro-benchmark); "column" marks the I = 0 column (the s = 0
    axis of the grid); "none" marks none.
    terms: "all" fills every metric array, "pole" only those the pole reads.
    """
    rng = np.random.default_rng(seed)
    nel = ni * nj
    igloc, nglob = structured_igloc(ni, nj)
    spec = Spectral()

    if axial == "random1pct":
        nax = max(1, int(round(0.01 * nel)))
        ax = np.sort(rng.choice(nel, size=nax, replace=False)) + 1
    elif axial == "column":
        ax = np.arange(nj) * ni + 1
    elif axial == "none":
        ax = np.zeros(0, dtype=I32)
    else:
        raise ValueError(axial)
    ax = ax.astype(I32)

    # geometry and materials fix the scale of the terms
    _, detj = _bilinear_geometry(rng, ni, nj)
    lam = rng.uniform(1e10, 3e11, size=(nj, ni, 5, 5))
    mu = rng.uniform(1e10, 3e11, size=(nj, ni, 5, 5))
    rho = rng.uniform(2500.0, 13000.0, size=(nj, ni, 5, 5))
    # (nj, ni, ipol, jpol) -> Fortran (ipol, jpol, e)
    def to_f(a):
        return _f(np.transpose(a.reshape(nel, 5, 5), (1, 2, 0)))

    wt2 = np.outer(spec.wt, spec.wt)
    scale = (lam + 2 * mu) * detj * wt2[None, None]
    used = set(_abi.SOLID_TERMS_USED[src_type]) if terms == "pole" else set(SOLID_TERMS)
    m_solid = {}
    for name in SOLID_TERMS:
        if name in used:
            m_solid[name] = to_f(scale * rng.uniform(-1.0, 1.0, size=scale.shape))
    used0 = set(_abi.AXIAL_TERMS_USED[src_type]) if terms == "pole" else set(AXIAL_TERMS)
    m0 = {}
    for name in AXIAL_TERMS:
        if name in used0:
            m0[name] = _f(1e11 * rng.uniform(-1.0, 1.0, size=(5, nel)))
    inv_mass = to_f(1.0 / (rho * detj * wt2[None, None]))

    mesh = Mesh(src_type=src_type, nel_solid=nel, nglob_solid=nglob, igloc_solid=igloc,
                ax_el_solid=ax, spec=spec, m_solid=m_solid, m0_solid=m0,
                inv_mass_rho=inv_mass)
    mesh.meta.update(ni=ni, nj=nj, seed=seed, field_seed=field_seed, axial=axial)
    return mesh


def random_gvec(mesh: Mesh, seed: int | None = None, sigma: float = 1e-6) -> np.ndarray:
    """3-component FP32 displacement ~ N(0, sigma) on the global points,
    gvec layout (nglob_solid, 3) column-major."""
    rng = np.random.default_rng(mesh.meta.get("field_seed", 0) if seed is None else seed)
    return np.asfortranarray(rng.normal(0.0, sigma, size=(mesh.nglob_solid, 3)).astype(F32))


def gvec_to_elemental(mesh: Mesh, g: np.ndarray, fluid: bool = False) -> np.ndarray:
    """Scatter a gvec-layout field to the element-local layout (0:4,0:4,nel[,nc])."""
    ig = (mesh.igloc_fluid if fluid else mesh.igloc_solid) - 1
    nel = mesh.nel_fluid if fluid else mesh.nel_solid
    if g.ndim == 1:
        return np.asfortranarray(g[ig].reshape(nel, 5, 5).transpose(2, 1, 0))
    out = np.empty((5, 5, nel, g.shape[1]), dtype=g.dtype, order="F")
    for c in range(g.shape[1]):
        out[..., c] = g[ig, c].reshape(nel, 5, 5).transpose(2, 1, 0)
    return out


def gauss_at(t: np.ndarray, period: float) -> np.ndarray:
    """The Gaussian source time function of gauss_stf at times t (FP64 in,
    realkind out), for the stage times of a symplectic step
    (compute_stf_t, SOLVER/source.f90:208-233)."""
    decay, shift = 3.5, 1.5 * period
    return np.exp(-((decay / period) * (np.asarray(t, np.float64) - shift)) ** 2).astype(F32)


def gauss_stf(niter: int, deltat: float, period: float) -> np.ndarray:
    """Gaussian source time function sampled at t = iter * deltat (the
    reference's `gauss` STF shape, SOLVER/source.f90:587-600: exp(-(decay/period
    (t - shift))^2) with decay 3.5 and a shift of 1.5 periods), evaluated in
    FP64 and cast to realkind as the reference does."""
    t = deltat * np.arange(1, niter + 1, dtype=np.float64)
    decay = 3.5
    shift = 1.5 * period
    return np.exp(-((decay / period) * (t - shift)) ** 2).astype(F32)


def set_source_receivers(m: Mesh, ni: int, nj_solid: int, nj_fluid: int, val, *, src_row: int = 1,
                         num_rec: int = 6, niter: int = 60, deltat: float = 2e-6, seis_it: int = 2) -> Mesh:
    """The solve-specific part of a coupled mesh: a point source on the
    lattice corner (ni // 2, src_row) of the solid (moment vector `val`; None
    puts a pressure source in the fluid, near the solid-fluid boundary),
    stored in the four elements holding the point; `num_rec` receivers on the
    top surface; the Gaussian stf of `niter` steps of `deltat`."""
    ic = ni // 2
    m.ielsrc = np.zeros(8, dtype=I32)
    if val is None:
        jc = nj_fluid - 1
        els = [(jc - 1) * ni + ic - 1, (jc - 1) * ni + ic, jc * ni + ic - 1, jc * ni + ic]
        pts = [(4, 4), (0, 4), (4, 0), (0, 0)]
        st = np.zeros((5, 5, 8), dtype=F32, order="F")
        for k, (e, (ip, jp)) in enumerate(zip(els, pts)):
            m.ielsrc[k] = e + 1
            st[ip, jp, k] = 1e-3
        m.source_term_fl = st
        m.fluid_src = 1
        m.nelsrc = 4
    else:
        jc = min(max(int(src_row), 1), nj_solid - 1)
        els = [(jc - 1) * ni + ic - 1, (jc - 1) * ni + ic, jc * ni + ic - 1, jc * ni + ic]
        pts = [(4, 4), (0, 4), (4, 0), (0, 0)]
        st = np.zeros((5, 5, 8, 3), dtype=F32, order="F")
        for k, (e, (ip, jp)) in enumerate(zip(els, pts)):
            m.ielsrc[k] = e + 1
            st[ip, jp, k, :] = val
        m.source_term_el = st
        m.nelsrc = 4
    m.deltat = deltat
    m.stf = gauss_stf(niter, deltat, 20 * deltat)   # niter and num_rec follow from stf and recfile_el
    m.seis_it = seis_it
    top = nj_solid - 1
    recs = np.linspace(0, ni - 1, num_rec).astype(int)
    m.recfile_el = np.asfortranarray(np.stack(
        [top * ni + recs + 1, np.full(num_rec, 2), np.full(num_rec, 4)], axis=1).astype(I32))
    return m


def coupled_mesh(ni: int, nj_solid: int, nj_fluid: int, src_type: int = _abi.MONOPOLE, *,
                 niter: int = 60, seed: int = 7, axial_column: bool = True, fluid_src: bool = False,
                 num_rec: int = 6, seis_it: int = 2, deltat: float = 2e-6,
                 free_surface: bool = False, absorbing: bool = False,
                 bdry_scale: float = 1.0, terms: str = "all", src_row: int = 1) -> Mesh:
    """A solid layer on top of a fluid layer, both ni elements wide, with
    the solid-fluid boundary along the fluid's top edge (jpol = 4) and the
    solid's bottom edge (jpol = 0); the I = 0 column lies on the axis.  A
    point source sits on an interior lattice point shared by four solid (or
    fluid) elements -- the source term is stored in the element-local copies of
    every element holding that point, as the reference does after assembly
    (SOLVER/source.f90:1133); receivers sit on the top surface.  src_row
    (1 .. nj_solid-1) is the lattice row of a solid source: deeper rows lie
    nearer the fluid.  Source, receivers, niter and deltat change no other
    array, so meshes differing only in them are the same mesh."""
    rng = np.random.default_rng(seed)
    m = structured_mesh(ni, nj_solid, src_type, seed=seed, axial="column" if axial_column else "none",
                        terms=terms)
    if nj_fluid > 0:
        igf, ngf = structured_igloc(ni, nj_fluid)
        nelf = ni * nj_fluid
        m.nel_fluid, m.nglob_fluid, m.igloc_fluid = nelf, ngf, igf
        m.ax_el_fluid = (np.arange(nj_fluid) * ni + 1).astype(I32) if axial_column else np.zeros(0, I32)
        wt2 = np.outer(m.spec.wt, m.spec.wt)
        # K / M ~ (v / h)^2 ~ 1e8 as in the solid (metric ~1e11, inverse mass ~1e-3)
        sc = 1e-2 * wt2[:, :, None]
        for name in FLUID_TERMS:
            m.m_fluid[name] = _f(sc * rng.uniform(-1.0, 1.0, size=(5, 5, nelf)))
        m.m0_w_fl = _f(1e-2 * rng.uniform(-1.0, 1.0, size=(5, nelf)))
        m.inv_mass_fluid = _f(1e10 * rng.uniform(0.5, 2.0, size=(5, 5, nelf)))
        # assembled inverse mass: make copies of one point agree
        g = m.inv_mass_fluid.reshape(-1, order="F")
        per = np.zeros(ngf, dtype=F32)
        per[igf - 1] = g
        m.inv_mass_fluid = _f(per[igf - 1].reshape(nelf, 5, 5).transpose(2, 1, 0))
        if free_surface:
            mask = np.ones((5, 5, nelf), dtype=F32, order="F")
            mask[:, 0, :ni] = 0.0   # bottom row of the fluid layer
            m.fluid_free_surface_mask = mask
        # boundary: fluid element (I, nj_fluid-1) top edge <-> solid element (I, 0) bottom edge
        m.bdry_fluid_el = ((nj_fluid - 1) * ni + np.arange(ni) + 1).astype(I32)
        m.bdry_solid_el = (np.arange(ni) + 1).astype(I32)
        m.bdry_jpol_fluid = np.full(ni, 4, dtype=I32)
        m.bdry_jpol_solid = np.zeros(ni, dtype=I32)
        m.bdry_matr = _f(bdry_scale * rng.uniform(-1.0, 1.0, size=(5, ni, 2)))
    # solid inverse mass: consistent copies
    per = np.zeros(m.nglob_solid, dtype=F32)
    per[m.igloc_solid - 1] = m.inv_mass_rho.reshape(-1, order="F")
    m.inv_mass_rho = _f(per[m.igloc_solid - 1].reshape(m.nel_solid, 5, 5).transpose(2, 1, 0))
    if absorbing:
        gs = np.zeros(m.nglob_solid, dtype=F32)
        gs[m.igloc_solid - 1] = 10.0 * rng.uniform(0, 1, size=m.igloc_solid.shape)
        m.solid_absorbing_gamma = _f(gs[m.igloc_solid - 1].reshape(m.nel_solid, 5, 5).transpose(2, 1, 0))
        if nj_fluid > 0:
            gf = np.zeros(m.nglob_fluid, dtype=F32)
            gf[m.igloc_fluid - 1] = 10.0 * rng.uniform(0, 1, size=m.igloc_fluid.shape)
            m.fluid_absorbing_gamma = _f(gf[m.igloc_fluid - 1].reshape(m.nel_fluid, 5, 5).transpose(2, 1, 0))
    # source at lattice corner (I, J) = (ni//2, src_row) of the solid (or fluid) grid
    val = None if (fluid_src and nj_fluid > 1) else rng.uniform(-1.0, 1.0, size=3).astype(F32) * 1e3
    set_source_receivers(m, ni, nj_solid, nj_fluid, val, src_row=src_row, num_rec=num_rec, niter=niter,
                         deltat=deltat, seis_it=seis_it)
    m.magnitude = 1e20
    return m


def add_attenuation(m: Mesh, n_sls: int = 5, seed: int = 77, do_corr_lowq: bool = True,
                    coarse_grained: bool = True) -> Mesh:
    """Seeded coarse-grained (cg4) attenuation data for a mesh, or with
    `coarse_grained` False the same at every GLL point (att_coarse_grained =
    .false.: per point modulus defects and anelastic weights, the axial
    elements' Y0 / V0_* vectors, the strain's mapping terms).

    SLS relaxation frequencies are log-spaced over the mesh's band and the
    coefficients y_j positive; the time-stepping factors follow the exact
    integration of the reference (SOLVER/attenuation.f90:882-887):
        exp_w_j_deltat = exp(-w_j dt)
        ts_fac_tm1     = (1 - exp_w_j_deltat) / (w_j dt) - exp_w_j_deltat
        ts_fac_t       = (exp_w_j_deltat - 1) / (w_j dt) + 1
    Q_mu / Q_kappa take a few PREM-like values per element (the reference's
    Q is constant inside an element).  The per-element cg4 factors (the
    modulus defects delta_mu/kappa, the weights Y and V of the anelastic
    stiffness, the mapping derivatives of the strain and 1/s) are seeded
    values with physical signs and scales."""
    rng = np.random.default_rng(seed)
    nel = m.nel_solid
    dt = m.deltat
    w = np.logspace(-1.3, 0.0, n_sls) / dt   # w_j dt from 0.05 to 1
    y = rng.uniform(0.1, 1.0, n_sls)
    ex = np.exp(-w * dt)
    ts_tm1 = (1 - ex) / (w * dt) - ex
    ts_t = (ex - 1) / (w * dt) + 1
    qmu_vals = np.array([80.0, 143.0, 312.0, 600.0], dtype=F32)
    qka_vals = np.array([1327.7, 57823.0], dtype=F32)
    cg = lambda lo, hi: _f(rng.uniform(lo, hi, size=(4, nel)))  # noqa: E731
    sgn = lambda lo, hi: _f(rng.uniform(lo, hi, size=(4, nel)) * rng.choice([-1.0, 1.0], size=(4, nel)))  # noqa: E731
    inv_s = _f(rng.uniform(0.5, 2.0, size=(5, 5, nel)))
    m.anel = {
        "y_j": y, "exp_w_j_deltat": ex, "ts_fac_t": ts_t, "ts_fac_tm1": ts_tm1,
        "do_corr_lowq": int(do_corr_lowq),
        "Q_mu": qmu_vals[rng.integers(0, len(qmu_vals), nel)],
        "Q_kappa": qka_vals[rng.integers(0, len(qka_vals), nel)],
        "delta_mu_cg4": cg(1e9, 1e10), "delta_kappa_cg4": cg(1e9, 1e10),
        "Y_cg4": cg(0.5, 5.0),
        "V_s_eta_cg4": sgn(0.5, 5.0), "V_s_xi_cg4": sgn(0.5, 5.0),
        "V_z_eta_cg4": sgn(0.5, 5.0), "V_z_xi_cg4": sgn(0.5, 5.0),
        "DsDeta_over_J_sol_cg4": sgn(0.5, 2.0), "DzDeta_over_J_sol_cg4": sgn(0.5, 2.0),
        "DsDxi_over_J_sol_cg4": sgn(0.5, 2.0), "DzDxi_over_J_sol_cg4": sgn(0.5, 2.0),
        "inv_s_solid": inv_s,
    }
    if not coarse_grained:
        pt = lambda lo, hi: _f(rng.uniform(lo, hi, size=(5, 5, nel)))  # noqa: E731
        spt = lambda lo, hi: _f(rng.uniform(lo, hi, size=(5, 5, nel)) * rng.choice([-1.0, 1.0], size=(5, 5, nel)))  # noqa: E731
        ax = np.zeros(nel, dtype=bool)
        ax[np.asarray(m.ax_el_solid, dtype=np.int64) - 1] = True
        ax0 = lambda lo, hi: _f(np.where(ax[None, :], rng.uniform(lo, hi, size=(5, nel)), 0.0))  # noqa: E731
        sax0 = lambda lo, hi: _f(np.where(ax[None, :], rng.uniform(lo, hi, size=(5, nel)) * rng.choice([-1.0, 1.0], size=(5, nel)), 0.0))  # noqa: E731
        for nm in list(m.anel):
            if nm.endswith("_cg4"):
                del m.anel[nm]
        m.anel.update({
            "delta_mu": pt(1e9, 1e10), "delta_kappa": pt(1e9, 1e10), "Y": pt(0.5, 5.0),
            "V_s_eta": spt(0.5, 5.0), "V_s_xi": spt(0.5, 5.0), "V_z_eta": spt(0.5, 5.0), "V_z_xi": spt(0.5, 5.0),
            "Y0": ax0(0.5, 5.0), "V0_s_eta": sax0(0.5, 5.0), "V0_s_xi": sax0(0.5, 5.0),
            "V0_z_eta": sax0(0.5, 5.0), "V0_z_xi": sax0(0.5, 5.0),
            "DsDeta_over_J_sol": spt(0.5, 2.0), "DzDeta_over_J_sol": spt(0.5, 2.0),
            "DsDxi_over_J_sol": spt(0.5, 2.0), "DzDxi_over_J_sol": spt(0.5, 2.0),
        })
    return m


PW_SOLID = ("DsDeta_over_J_sol", "DzDeta_over_J_sol", "DsDxi_over_J_sol", "DzDxi_over_J_sol", "inv_s_solid")
CG4_ATTENUATION = ("delta_mu_cg4", "delta_kappa_cg4", "Y_cg4", "V_s_eta_cg4", "V_s_xi_cg4", "V_z_eta_cg4",
                   "V_z_xi_cg4", "DsDeta_over_J_sol_cg4", "DzDeta_over_J_sol_cg4", "DsDxi_over_J_sol_cg4",
                   "DzDxi_over_J_sol_cg4")
FULL_ATTENUATION = ("delta_mu", "delta_kappa", "Y", "V_s_eta", "V_s_xi", "V_z_eta", "V_z_xi",
                    "Y0", "V0_s_eta", "V0_s_xi", "V0_z_eta", "V0_z_xi",
                    "DsDeta_over_J_sol", "DzDeta_over_J_sol", "DsDxi_over_J_sol", "DzDxi_over_J_sol")
PW_FLUID = ("DsDeta_over_J_flu", "DzDeta_over_J_flu", "DsDxi_over_J_flu", "DzDxi_over_J_flu", "inv_s_fluid",
            "inv_rho_fluid")


def add_pointwise(m: Mesh, seed: int = 91) -> Mesh:
    """Seeded data_pointwise arrays (SOLVER/def_precomp_terms.f90:171-230):
    the mapping derivatives over the Jacobian with physical signs and scales,
    1/s and the fluid's 1/rho, each (0:4,0:4,nel) per point.  The dump
    kernels are data-oblivious, as the stiffness kernels are."""
    rng = np.random.default_rng(seed)

    def sgn(nel):
        return _f(rng.uniform(0.5, 2.0, size=(5, 5, nel)) * rng.choice([-1.0, 1.0], size=(5, 5, nel)))

    pw = {}
    for nm in PW_SOLID[:4]:
        pw[nm] = sgn(m.nel_solid)
    pw["inv_s_solid"] = _f(rng.uniform(0.5, 2.0, size=(5, 5, m.nel_solid)))
    if m.nel_fluid > 0:
        for nm in PW_FLUID[:4]:
            pw[nm] = sgn(m.nel_fluid)
        pw["inv_s_fluid"] = _f(rng.uniform(0.5, 2.0, size=(5, 5, m.nel_fluid)))
        pw["inv_rho_fluid"] = _f(rng.uniform(1.0 / 13000.0, 1.0 / 2500.0, size=(5, 5, m.nel_fluid)))
    m.pointwise = pw
    return m


def kwf_mapping(m: Mesh, ibeg: int = 0, iend: int = 4, jbeg: int = 0, jend: int = 4):
    """The kernel wavefield point layout of the reference's NetCDF output
    (SOLVER/meshes_io.F90:543-630) with every element inside the output
    region: walking the solid elements, then the fluid ones, each over
    jpol = jbeg..jend, ipol = ibeg..iend plus the axis point ipol = 0 of an
    axial element, a global point not met before gets the next position and
    marks that element point in kwf_mask.  Returns (kwf_mask,
    mapping_ijel_ikwf, npoint_solid_kwf, npoint_fluid_kwf); the arrays are
    int32 (5, 5, nel_solid + nel_fluid), Fortran order."""
    nes, nef = m.nel_solid, m.nel_fluid
    mask = np.zeros((5, 5, nes + nef), dtype=I32, order="F")
    mapping = np.zeros((5, 5, nes + nef), dtype=I32, order="F")
    ct = 0
    counts = []
    for dom in range(2 if nef > 0 else 1):
        nel = nes if dom == 0 else nef
        ig = (m.igloc_solid if dom == 0 else m.igloc_fluid).reshape(nel, 25) - 1
        axial = np.zeros(nel, dtype=bool)
        ax = m.ax_el_solid if dom == 0 else m.ax_el_fluid
        if ax is not None and len(ax):
            axial[np.asarray(ax) - 1] = True
        seen = {}
        off = 0 if dom == 0 else nes
        for e in range(nel):
            for j in range(jbeg, jend + 1):
                pts = list(range(ibeg, iend + 1)) + ([0] if axial[e] and ibeg > 0 else [])
                for i in pts:
                    g = int(ig[e, i + 5 * j])
                    if g not in seen:
                        ct += 1
                        seen[g] = ct
                        mask[i, j, off + e] = 1
                    mapping[i, j, off + e] = seen[g]
        counts.append(ct)
    n_sol = counts[0]
    return mask, mapping, n_sol, ct - n_sol


def dump_desc(m: Mesh, dump_type: int, strain_it: int, out: np.ndarray | None, capacity: int,
              ibeg: int = 0, iend: int = 4, jbeg: int = 0, jend: int = 4, kwf=None,
              src_mask: bool = False) -> _abi.DumpDesc:
    """An axg_dump_desc for the mesh's pointwise arrays; keeps them alive.
    kwf: (kwf_mask, mapping_ijel_ikwf, npoint_solid_kwf, npoint_fluid_kwf)
    for the kernel wavefield point layout, or None; src_mask: the
    reference's src_dump_type = 'mask' (the source elements' solid values
    zeroed)."""
    dd = _abi.DumpDesc()
    dd.dump_type, dd.strain_it = dump_type, strain_it
    dd.src_dump_mask = int(src_mask)
    dd.ibeg, dd.iend, dd.jbeg, dd.jend = ibeg, iend, jbeg, jend
    keep = []
    for nm in PW_SOLID + PW_FLUID:
        a = m.pointwise.get(nm)
        if a is not None:
            a = np.asfortranarray(a, dtype=F32)
            keep.append(a)
        setattr(dd, nm, _abi.ptr(a, C.c_float))
    dd.out = _abi.ptr(out, C.c_float)
    dd.capacity = capacity
    if kwf is not None:
        kmask, kmap = np.asfortranarray(kwf[0], dtype=I32), np.asfortranarray(kwf[1], dtype=I32)
        keep += [kmask, kmap]
        dd.kwf_mask = _abi.ptr(kmask, C.c_int32)
        dd.mapping_ijel_ikwf = _abi.ptr(kmap, C.c_int32)
        dd.npoint_solid_kwf, dd.npoint_fluid_kwf = int(kwf[2]), int(kwf[3])
    dd._keep = keep  # type: ignore[attr-defined]
    return dd
