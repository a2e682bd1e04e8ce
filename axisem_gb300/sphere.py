"""Axisymmetric whole-Earth meshes and the precomputed arrays of the time loop.

The reference builds a solve's inputs in two programs: its MESHER writes the
element skeleton (MESHER/main.f90:52-106), and its SOLVER turns the skeleton
and the background model into the time loop's arrays in FP64
(SOLVER/def_precomp_terms.f90).  This module does both for the PREM models of
``axisem_gb300.earth`` and returns a ``Mesh`` whose arrays go through the
C-ABI descriptor like the reference's module arrays.

Skeleton (this module's own layout; the reference's MESHER is not restated):
  * the meridional half-plane (s >= 0) of a sphere of radius 6371 km, north
    hemisphere built first and mirrored (z -> -z, corner order reversed) to the
    south, as MESHER/meshgen.f90:1575-1636 mirrors its skeleton;
  * a central square 0 <= s, z <= a of n_c x n_c bilinear elements, a ring of
    n_ring layers blending the square's edge into the circle r = R1 (straight
    edges, the outermost ones arcs of r = R1), then spheroidal shells
    (edges r = const arcs and theta = const rays) up to the surface, with a
    radial level on every discontinuity of the model;
  * elements per wavelength as the reference's mesher sizes them
    (MESHER/discont_meshing.f90: el_per_lambda = 1.5 over the GLL spacing
    ratio, the period times the slowest velocity of a domain), and the
    number of shell elements doubled outward where the surface needs it by
    conforming coarsening bands: per coarse element three quadrilaterals,
    alternately mirrored so that the bands' split side edges pair up.
Every element edge is a straight segment or an arc of constant radius, and the
element map is the transfinite (Coons) interpolation of its four edges, with
theta linear along arcs.  On spheroidal elements this is the reference's
map_spheroid (SOLVER/analytic_spheroid_mapping.f90); axial elements have their
xi = -1 edge on the axis, as the reference's do.

Precomputed arrays (restated from SOLVER/def_precomp_terms.f90, in FP64,
rounded to FP32 where the reference stores realkind):
  * def_mass_matrix_k (:596-800): massmat_k, massmat_kwts2, the solid and
    fluid inverse masses (assembled in FP32 in pdistsum_solid's walk order,
    then inverted; the dipole's 1/2), inv_rho_fluid;
  * def_solid_stiffness_terms / compute_{monopole,dipole,quadrupole}_stiff_terms
    (:1162-2285) with the elastic tensor c_ijkl_ani (:2291-2335), including
    the axial vectors M0_w* and the cg4 weights Y_cg4, V_*_cg4;
  * def_fluid_stiffness_terms (:2336-2467) and def_solid_fluid_boundary_terms
    (:2474-2799);
  * compute_pointwisederiv_matrices (:148-290);
  * the moment-tensor source (define_moment_tensor, SOLVER/source.f90:985-1226,
    with dsdf/dzdf_elem_solid, SOLVER/pointwise_derivatives.f90:419-476) and
    the Gaussian source time function (gauss, SOLVER/source.f90:587-598);
  * the mesh's own checks: volumes, spherical surfaces and the mass of the
    model (SOLVER/def_grid.f90:992-1332, SOLVER/def_precomp_terms.f90:998-1160).
"""
from __future__ import annotations

import copy
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .earth import CMB, DISCONTINUITIES_KM, FLUID_DOMAIN, ICB, NDISC, R_EARTH, domain_of, velocity
from .mesh import F32, I32, Mesh
from .spectral import Spectral

SP = Spectral()
_h = np.diff(SP.eta)
GLL_SPACING_RATIO = float(_h.max() / _h.mean())   # maxh / aveh of the GLL nodes (1.309 for npol = 4)
EDGE_BOTTOM, EDGE_RIGHT, EDGE_TOP, EDGE_LEFT = 0, 1, 2, 3


# ============================================================== skeleton
@dataclass
class Skeleton:
    """Corner nodes (s, z) and elements of the mesh.  elems[e] = (c1, c2, c3,
    c4) are the corners at (xi, eta) = (-1,-1), (1,-1), (1,1), (-1,1); arc[e, k]
    marks edge k (bottom c1-c2, right c2-c3, top c4-c3, left c1-c4) as an arc
    of constant radius; axis[e] marks the xi = -1 edge on the axis."""

    nodes: np.ndarray
    elems: np.ndarray
    arc: np.ndarray
    axis: np.ndarray
    kind: np.ndarray                  # 0 square, 1 ring, 2 shell, 3 coarsening band
    info: dict = field(default_factory=dict)
    cache: dict = field(default_factory=dict, repr=False)   # geometry and numbering, shared by the pole types


class _Builder:
    def __init__(self):
        self.key = {}
        self.nodes = []
        self.elems = []
        self.arcs = []
        self.kinds = []

    def node(self, s, z):
        s = 0.0 if abs(s) < 1e-3 else float(s)
        z = 0.0 if abs(z) < 1e-3 else float(z)
        k = (int(round(s * 1e3)), int(round(z * 1e3)))
        i = self.key.get(k)
        if i is None:
            i = len(self.nodes)
            self.key[k] = i
            self.nodes.append((s, z))
        return i

    def polar(self, r, th):
        return self.node(r * np.sin(th), r * np.cos(th))

    def elem(self, c, arcs, kind):
        self.elems.append(tuple(c))
        self.arcs.append(tuple(arcs))
        self.kinds.append(kind)


def _vmin(idom: int, r0: float, r1: float, model: str) -> float:
    r = np.linspace(r0, r1, 65)
    v = velocity(r, "v_p" if idom == FLUID_DOMAIN else "v_s", idom, model)
    return float(v.min())


def _layers(period: float, model: str, el_per_lambda: float, r1: float):
    """Radial layers from R1 up to the surface: (r_bottom, r_top, domain,
    target element size), a level on every discontinuity."""
    d = DISCONTINUITIES_KM * 1000.0
    out = []
    tops = list(d) + [r1]
    for k in range(NDISC - 1, -1, -1):      # inner core first
        idom = k + 1
        r_top, r_bot = tops[k], tops[k + 1]
        h = period * _vmin(idom, r_bot, r_top, model) / (el_per_lambda * GLL_SPACING_RATIO)
        n = max(1, int(np.ceil((r_top - r_bot) / h)))
        lv = np.linspace(r_bot, r_top, n + 1)
        for i in range(n):
            out.append((lv[i], lv[i + 1], idom, h, i, n))
    return out


def _plan_counts(layers, n_req, n_min_r1: int, n_surf: int):
    """Outside in from n_surf elements per quarter: a layer becomes a
    coarsening band (count halved below it) when no neighbour is a band, it is
    neither the first nor the last layer of its domain, the halved count is
    even and still resolves every layer below.  Returns (counts at each
    layer's top, band flags, count at R1)."""
    L = len(layers)
    need_below = np.zeros(L)
    m = 0
    for i in range(L):
        need_below[i] = m          # max requirement of the layers below layer i
        m = max(m, n_req[i])
    top = np.zeros(L, dtype=np.int64)
    band = np.zeros(L, dtype=bool)
    N = n_surf
    for i in range(L - 1, -1, -1):
        top[i] = N
        _, _, idom, _, k, n = layers[i]
        inner = 0 < k < n - 1
        if (inner and not (i + 1 < L and band[i + 1]) and N % 4 == 0 and N // 2 >= need_below[i]
                and N // 2 >= max(n_req[i] * 0.5, 1) and N // 2 >= n_min_r1):
            band[i] = True
            N //= 2
    return top, band, N


def build_skeleton(period: float = 50.0, model: str = "prem_iso", el_per_lambda: float = 1.5,
                   r1_frac: float = 0.5, square_frac: float = 0.55) -> Skeleton:
    """The element skeleton of a whole-Earth mesh resolving `period` seconds."""
    r1 = r1_frac * ICB
    layers = _layers(period, model, el_per_lambda, r1)
    h_ic = layers[0][3]
    n_req = np.array([int(np.ceil(0.5 * np.pi * rt / h)) for (_, rt, _, h, _, _) in layers])
    a = square_frac * r1
    n_c_min = max(2, int(np.ceil(a / h_ic)))
    best = None
    for q in range(0, 7):
        n_surf = int(np.ceil(n_req[-1] / 2 ** q)) * 2 ** q
        n_surf += n_surf % 2
        top, band, n_r1 = _plan_counts(layers, n_req, 2 * n_c_min, n_surf)
        if n_r1 % 2 or n_r1 < 2 * n_c_min:
            continue
        if np.any(top < n_req):
            continue
        n_c = n_r1 // 2
        n_ring = max(1, int(round((r1 - a) / (0.5 * np.pi * r1 / n_r1))))
        bot = np.where(band, top // 2, top)
        count = n_c * n_c + n_ring * n_r1 + int(np.sum(np.where(band, 3 * bot, top)))
        if best is None or count < best[0]:
            best = (count, top, band, n_c, n_ring)
    if best is None:
        raise RuntimeError("no element layout satisfies the resolution")
    _, top, band, n_c, n_ring = best

    b = _Builder()
    # central square (north quarter): element (i, j), xi along s, eta along z
    hs = a / n_c
    for j in range(n_c):
        for i in range(n_c):
            c = [b.node(i * hs, j * hs), b.node((i + 1) * hs, j * hs), b.node((i + 1) * hs, (j + 1) * hs),
                 b.node(i * hs, (j + 1) * hs)]
            b.elem(c, (False, False, False, False), 0)
    # ring: square edge -> circle r = R1, 2 n_c columns (xi from the axis to the equator)
    m = 2 * n_c

    def sq(k):
        return (k * hs, a) if k <= n_c else (a, a - (k - n_c) * hs)

    def circ(k):
        th = k * 0.5 * np.pi / m
        return (r1 * np.sin(th), r1 * np.cos(th))

    def ring_pt(k, l):
        t = l / n_ring
        if l == n_ring:
            return circ(k)
        p, q = sq(k), circ(k)
        return ((1 - t) * p[0] + t * q[0], (1 - t) * p[1] + t * q[1])

    for l in range(n_ring):
        for k in range(m):
            c = [b.node(*ring_pt(k, l)), b.node(*ring_pt(k + 1, l)), b.node(*ring_pt(k + 1, l + 1)),
                 b.node(*ring_pt(k, l + 1))]
            b.elem(c, (False, False, l + 1 == n_ring, False), 1)
    # shells and coarsening bands
    for i, (rb, rt, idom, _, _, _) in enumerate(layers):
        N = int(top[i])
        if not band[i]:
            dth = 0.5 * np.pi / N
            for k in range(N):
                c = [b.polar(rb, k * dth), b.polar(rb, (k + 1) * dth), b.polar(rt, (k + 1) * dth),
                     b.polar(rt, k * dth)]
                b.elem(c, (True, False, True, False), 2)
            continue
        nc_ = N // 2
        dc = 0.5 * np.pi / nc_
        df = 0.5 * dc
        rm = 0.5 * (rb + rt)
        for j in range(nc_):
            B0, B1 = b.polar(rb, j * dc), b.polar(rb, (j + 1) * dc)
            T0, T1, T2 = b.polar(rt, j * dc), b.polar(rt, j * dc + df), b.polar(rt, (j + 1) * dc)
            X = b.polar(rm, j * dc + df)
            if j % 2 == 0:   # split side on the left
                Ls = b.polar(rm, j * dc)
                b.elem((B0, B1, X, Ls), (True, False, True, False), 3)
                b.elem((X, B1, T2, T1), (False, False, True, False), 3)
                b.elem((Ls, X, T1, T0), (True, False, True, False), 3)
            else:            # split side on the right
                Rs = b.polar(rm, (j + 1) * dc)
                b.elem((B0, B1, Rs, X), (True, False, True, False), 3)
                b.elem((B0, X, T1, T0), (False, False, True, False), 3)
                b.elem((X, Rs, T2, T1), (True, False, True, False), 3)
    nodes_n = np.array(b.nodes, dtype=np.float64)
    elems_n = np.array(b.elems, dtype=np.int64)
    arcs_n = np.array(b.arcs, dtype=bool)
    kinds_n = np.array(b.kinds, dtype=np.int8)
    # the southern hemisphere: z -> -z, corners reversed (c4, c3, c2, c1)
    for (s, z) in nodes_n:
        b.node(s, -z)
    south = np.array([[b.node(nodes_n[c, 0], -nodes_n[c, 1]) for c in el[::-1]] for el in elems_n],
                     dtype=np.int64)
    nodes = np.array(b.nodes, dtype=np.float64)
    elems = np.concatenate([elems_n, south])
    arcs = np.concatenate([arcs_n, arcs_n[:, [EDGE_TOP, EDGE_RIGHT, EDGE_BOTTOM, EDGE_LEFT]]])
    kinds = np.concatenate([kinds_n, kinds_n])
    axis = (nodes[elems[:, 0], 0] == 0.0) & (nodes[elems[:, 3], 0] == 0.0)
    info = {"period": period, "model": model, "r1": r1, "square": a, "n_c": n_c, "n_ring": n_ring,
            "n_surface_quarter": int(top[-1]), "bands": int(band.sum()),
            "layers": [(float(rb), float(rt), int(idom)) for (rb, rt, idom, _, _, _) in layers],
            "layer_counts": [int(t) for t in top], "band_layers": [int(i) for i in np.flatnonzero(band)],
            "el_per_lambda": el_per_lambda}
    return Skeleton(nodes=nodes, elems=elems, arc=arcs, axis=axis, kind=kinds, info=info)


# ============================================================== mapping
def _edge_map(p, q, arc, t):
    """Points and d/dt of the edges from p (t = -1) to q (t = 1): straight,
    or an arc of constant radius with theta linear in t.  p, q (E, 2); arc
    (E,); t (E, n) or (n,).  Returns (E, n, 2) arrays."""
    t = np.broadcast_to(np.asarray(t, dtype=np.float64), (p.shape[0],) + np.shape(t)[-1:])
    w0 = 0.5 * (1.0 - t)[..., None]
    w1 = 0.5 * (1.0 + t)[..., None]
    pt = w0 * p[:, None, :] + w1 * q[:, None, :]
    dt = np.broadcast_to(0.5 * (q - p)[:, None, :], pt.shape).copy()
    if np.any(arc):
        a = np.flatnonzero(arc)
        rp = np.hypot(p[a, 0], p[a, 1])
        rq = np.hypot(q[a, 0], q[a, 1])
        R = 0.5 * (rp + rq)
        thp = np.arctan2(np.maximum(p[a, 0], 0.0), p[a, 1])
        thq = np.arctan2(np.maximum(q[a, 0], 0.0), q[a, 1])
        th = 0.5 * (1.0 - t[a]) * thp[:, None] + 0.5 * (1.0 + t[a]) * thq[:, None]
        pt[a, :, 0] = R[:, None] * np.sin(th)
        pt[a, :, 1] = R[:, None] * np.cos(th)
        half = 0.5 * (thq - thp) * R
        dt[a, :, 0] = half[:, None] * np.cos(th)
        dt[a, :, 1] = -half[:, None] * np.sin(th)
    return pt, dt


def element_geometry(sk: Skeleton, els: np.ndarray | None = None, gll_only: bool = False):
    """s, z and the partial derivatives ds/dxi, dz/dxi, ds/deta, dz/deta at
    the 5 x 5 points of elements `els`: GLL x GLL, or GLJ(0,1) x GLL on axial
    elements (compute_partial_derivatives, SOLVER/analytic_mapping.f90:680-700).
    Arrays (E, 5 [ipol], 5 [jpol])."""
    els = np.arange(len(sk.elems)) if els is None else els
    el = sk.elems[els]
    c = [sk.nodes[el[:, k]] for k in range(4)]
    arc = sk.arc[els]
    ax = sk.axis[els]
    use_glj = ax & (not gll_only)
    xi = np.where(use_glj[:, None], SP.xi_k[None, :], SP.eta[None, :])   # (E, 5)
    eta = SP.eta
    B, dB = _edge_map(c[0], c[1], arc[:, EDGE_BOTTOM], xi)
    T, dT = _edge_map(c[3], c[2], arc[:, EDGE_TOP], xi)
    Lf, dLf = _edge_map(c[0], c[3], arc[:, EDGE_LEFT], eta)
    Rt, dRt = _edge_map(c[1], c[2], arc[:, EDGE_RIGHT], eta)
    X = xi[:, :, None, None]                      # (E, i, 1, 1)
    Y = eta[None, None, :, None]                  # (1, 1, j, 1)
    C = [ck[:, None, None, :] for ck in c]
    bil = 0.25 * ((1 - X) * (1 - Y) * C[0] + (1 + X) * (1 - Y) * C[1] + (1 + X) * (1 + Y) * C[2]
                  + (1 - X) * (1 + Y) * C[3])
    dbx = 0.25 * (-(1 - Y) * C[0] + (1 - Y) * C[1] + (1 + Y) * C[2] - (1 + Y) * C[3])
    dby = 0.25 * (-(1 - X) * C[0] - (1 + X) * C[1] + (1 + X) * C[2] + (1 - X) * C[3])
    Bi, Ti = B[:, :, None, :], T[:, :, None, :]
    dBi, dTi = dB[:, :, None, :], dT[:, :, None, :]
    Lj, Rj = Lf[:, None, :, :], Rt[:, None, :, :]
    dLj, dRj = dLf[:, None, :, :], dRt[:, None, :, :]
    x = 0.5 * (1 - Y) * Bi + 0.5 * (1 + Y) * Ti + 0.5 * (1 - X) * Lj + 0.5 * (1 + X) * Rj - bil
    dx = 0.5 * (1 - Y) * dBi + 0.5 * (1 + Y) * dTi - 0.5 * Lj + 0.5 * Rj - dbx
    dy = -0.5 * Bi + 0.5 * Ti + 0.5 * (1 - X) * dLj + 0.5 * (1 + X) * dRj - dby
    s = x[..., 0]
    s = np.where(np.abs(s) < 1e-6 * R_EARTH, 0.0, s)   # on the axis (map_spheroid's min_distance_dim)
    return {"s": s, "z": x[..., 1], "dsdxi": dx[..., 0], "dzdxi": dx[..., 1], "dsdeta": dy[..., 0],
            "dzdeta": dy[..., 1], "axis": ax, "xi": xi}


# ============================================================== numbering
def global_numbering(sk: Skeleton, els: np.ndarray):
    """igloc (1-based, walk ipol fastest per element) of the points of
    elements `els`, numbered topologically: a corner by its node, an edge
    point by its edge and its position from the lower node id, an interior
    point by its element.  Returns (igloc, nglob)."""
    el = sk.elems[els]
    E = len(els)
    nn = len(sk.nodes)
    keys = np.zeros((E, 5, 5), dtype=np.int64)   # [e, i, j]
    c1, c2, c3, c4 = (el[:, k] for k in range(4))
    keys[:, 0, 0], keys[:, 4, 0], keys[:, 4, 4], keys[:, 0, 4] = c1, c2, c3, c4
    base = nn

    def ekey(a, b, k):
        lo, hi = np.minimum(a, b), np.maximum(a, b)
        kk = np.where(a < b, k, 4 - k)
        return base + (lo * nn + hi) * 5 + kk

    for k in range(1, 4):
        keys[:, k, 0] = ekey(c1, c2, k)
        keys[:, k, 4] = ekey(c4, c3, k)
        keys[:, 0, k] = ekey(c1, c4, k)
        keys[:, 4, k] = ekey(c2, c3, k)
    ibase = base + nn * nn * 5 + 5
    loc = np.arange(25).reshape(5, 5)
    for i in range(1, 4):
        for j in range(1, 4):
            keys[:, i, j] = ibase + np.asarray(els, dtype=np.int64) * 25 + loc[i, j]
    flat = keys.transpose(0, 2, 1).reshape(-1)    # element-major, then jpol, ipol fastest
    uniq, inv = np.unique(flat, return_inverse=True)
    return (inv + 1).astype(I32), len(uniq)


# ============================================================== precomputed terms
C_COMPONENTS = (("11", (1, 1, 1, 1)), ("12", (1, 1, 2, 2)), ("13", (1, 1, 3, 3)), ("15", (1, 1, 3, 1)),
                ("22", (2, 2, 2, 2)), ("23", (2, 2, 3, 3)), ("25", (2, 2, 3, 1)), ("33", (3, 3, 3, 3)),
                ("35", (3, 3, 3, 1)), ("44", (2, 3, 2, 3)), ("46", (2, 3, 1, 2)), ("55", (3, 1, 3, 1)),
                ("66", (1, 2, 1, 2)))


def elastic_tensor(lam, mu, xi_a, phi_a, eta_a, th_fa, ph_fa=0.0) -> dict:
    """c_ijkl_ani (SOLVER/def_precomp_terms.f90:2291-2335) for the 13
    components the stiffness terms use (C11 = c_1111, C12 = c_1122, ...,
    C66 = c_1212): the elastic tensor of a transversely isotropic medium with
    fast axis (th_fa, ph_fa) (Nolet 2008, eq. 16.2).  The anisotropic terms
    are formed only where the medium is anisotropic (they vanish for
    xi = phi = eta = 1)."""
    d = lambda a, b: 1.0 if a == b else 0.0  # noqa: E731
    out = {nm: lam * d(i, j) * d(k, l) + mu * (d(i, k) * d(j, l) + d(i, l) * d(j, k))
           for nm, (i, j, k, l) in C_COMPONENTS}
    ani = (xi_a != 1.0) | (phi_a != 1.0) | (eta_a != 1.0)
    if not np.any(ani):
        return out
    L, M, X, P, E, T = (np.broadcast_to(a, ani.shape)[ani] for a in (lam, mu, xi_a, phi_a, eta_a, th_fa))
    a1 = (E - 1.0) * L + 2.0 * E * M * (1.0 - 1.0 / X)
    a2 = M * (1.0 / X - 1.0)
    a3 = (1.0 - 2.0 * E + P) * (L + 2.0 * M) + (4.0 * E - 4.0) * M / X
    sv = [np.cos(ph_fa) * np.sin(T), np.sin(ph_fa) * np.sin(T), np.cos(T)]
    s = lambda a: sv[a - 1]  # noqa: E731
    for nm, (i, j, k, l) in C_COMPONENTS:
        add = (a1 * (d(i, j) * s(k) * s(l) + d(k, l) * s(i) * s(j))
               + a2 * (d(i, k) * s(j) * s(l) + d(i, l) * s(j) * s(k) + d(j, k) * s(i) * s(l) + d(j, l) * s(i) * s(k))
               + a3 * (s(i) * s(j) * s(k) * s(l)))
        c = np.array(out[nm], dtype=np.float64, copy=True)
        c[ani] = c[ani] + add
        out[nm] = c
    return out


def _pdistsum_f32(vals_f: np.ndarray, igloc: np.ndarray, nglob: int, dtype=F32) -> np.ndarray:
    """pdistsum_solid / pdistsum_fluid (SOLVER/commun.F90:69-283) of an
    element-local field (5, 5, E): edge points summed in `dtype` (FP32, as
    the reference's realkind build) in the walk order (element by element,
    ipol fastest, interior points skipped), the sums scattered back."""
    E = vals_f.shape[2]
    ig = igloc.reshape(E, 5, 5) - 1                # [e, j, i]
    v = np.asarray(vals_f, dtype=dtype).transpose(2, 1, 0)   # [e, j, i]
    edge = np.zeros((5, 5), dtype=bool)
    edge[0, :] = edge[4, :] = edge[:, 0] = edge[:, 4] = True
    idx = ig[:, edge].reshape(-1)
    g = np.zeros(nglob, dtype=dtype)
    np.add.at(g, idx, v[:, edge].reshape(-1))
    out = v.copy()
    out[:, edge] = g[ig[:, edge]]
    return np.asfortranarray(out.transpose(2, 1, 0))


def _neighbourhood(igloc: np.ndarray, nel: int, elems) -> tuple[np.ndarray, np.ndarray, int]:
    """The elements that share a point with `elems` (sorted, so in the walk
    order of pdistsum), and their igloc renumbered compactly (1-based) with
    the number of points: a field nonzero only on `elems` assembles on them
    with the same sums, in the same order, as over the whole mesh."""
    ig_all = np.asarray(igloc).reshape(nel, 25) - 1
    mark = np.zeros(int(ig_all.max()) + 1, dtype=bool)
    mark[ig_all[list(elems)].reshape(-1)] = True
    near = np.flatnonzero(mark[ig_all].any(axis=1))
    uniq, inv = np.unique(ig_all[near], return_inverse=True)
    return near, inv.reshape(-1).astype(I32) + 1, len(uniq)


def _to_f(a):
    """(E, i, j) FP64 -> Fortran (i, j, E) FP32."""
    return np.asfortranarray(np.transpose(a, (1, 2, 0)).astype(F32))


@dataclass
class Attenuation:
    """Options of the anelastic model (inparam_advanced's attenuation keys,
    SOLVER/attenuation.f90:710-730 defaults): n_sls standard linear solids
    over [f_min, f_max] Hz, moduli given at f_ref Hz, the low-Q correction,
    the coarse-grained (cg4) memory variables or, with coarse_grained False
    (att_coarse_grained = .false.), memory variables at every GLL point."""

    n_sls: int = 5
    f_min: float = 0.001
    f_max: float = 1.0
    f_ref: float = 1.0
    do_corr_lowq: bool = True
    nfsamp: int = 100
    coarse_grained: bool = True


def sls_fit(att: Attenuation):
    """Relaxation frequencies w_j (rad/s) and weights y_j of the SLS for
    Q = 1.  The reference anneals them from random draws
    (invert_linear_solids, SOLVER/attenuation.f90:1183-1330), which no run
    reproduces; here the w_j stay at the annealing's start, log-spaced over
    [f_min, f_max] (its FIX_FREQ mode), and y_j minimise the frequency-weighted
    misfit of the linearised 1/Q(w) = sum_j y_j w w_j / (w^2 + w_j^2)
    (Emmerich & Korn 1987, eq. 22) on the reference's nfsamp log-spaced
    samples, by linear least squares."""
    n = att.n_sls
    if n > 1:
        expo = (np.log10(att.f_max) - np.log10(att.f_min)) / (n - 1.0)
        w_j = 2 * np.pi * 10 ** (np.log10(att.f_min) + np.arange(n) * expo)
    else:
        w_j = np.array([np.sqrt(att.f_max * att.f_min) * 2 * np.pi])
    expo = (np.log10(att.f_max) - np.log10(att.f_min)) / (att.nfsamp - 1.0)
    w = 2 * np.pi * 10 ** (np.log10(att.f_min) + np.arange(att.nfsamp) * expo)
    weights = w / w.sum() * att.nfsamp
    A = (w[:, None] * w_j[None, :]) / (w[:, None] ** 2 + w_j[None, :] ** 2)
    sw = np.sqrt(weights)[:, None]
    y_j, *_ = np.linalg.lstsq(A * sw, sw[:, 0], rcond=None)
    return w_j, y_j


def fast_correct(y: np.ndarray) -> np.ndarray:
    """fast_correct (SOLVER/attenuation.f90:1139-1155): first-order
    correction of the linearised SLS weights, yp_j = y_j dy_j."""
    yp = np.zeros_like(y)
    dy = 1.0 + 0.5 * y[0]
    yp[0] = y[0] * dy
    for k in range(1, len(y)):
        dy = dy + (dy - 0.5) * y[k - 1] + 0.5 * y[k]
        yp[k] = y[k] * dy
    return yp


CG4 = ((1, 1), (1, 3), (3, 1), (3, 3))


def _weights_cg(g):
    """weights_cg of prepare_attenuation (SOLVER/attenuation.f90:968-992): each
    cg4 point stands for its quarter of the element, gamma_w_l = g (the mass
    weights wt wt J s); returns (E, 4) in the cg4 order (1,1), (1,3), (3,1), (3,3)."""
    out = np.zeros((g.shape[0], 4))
    out[:, 0] = (g[:, 0, 0] + g[:, 0, 1] + g[:, 1, 0] + g[:, 1, 1]
                 + 0.5 * (g[:, 0, 2] + g[:, 1, 2] + g[:, 2, 0] + g[:, 2, 1]) + 0.25 * g[:, 2, 2]) / g[:, 1, 1]
    out[:, 1] = (g[:, 0, 3] + g[:, 0, 4] + g[:, 1, 3] + g[:, 1, 4]
                 + 0.5 * (g[:, 0, 2] + g[:, 1, 2] + g[:, 2, 3] + g[:, 2, 4]) + 0.25 * g[:, 2, 2]) / g[:, 1, 3]
    out[:, 2] = (g[:, 3, 0] + g[:, 3, 1] + g[:, 4, 0] + g[:, 4, 1]
                 + 0.5 * (g[:, 2, 0] + g[:, 2, 1] + g[:, 3, 2] + g[:, 4, 2]) + 0.25 * g[:, 2, 2]) / g[:, 3, 1]
    out[:, 3] = (g[:, 3, 3] + g[:, 3, 4] + g[:, 4, 3] + g[:, 4, 4]
                 + 0.5 * (g[:, 2, 3] + g[:, 2, 4] + g[:, 3, 2] + g[:, 4, 2]) + 0.25 * g[:, 2, 2]) / g[:, 3, 3]
    return out


@dataclass
class SphereSolve:
    """Options of one solve on a whole-Earth mesh."""

    pole: int = _abi.MONOPOLE
    source: str = ""                 # explosion / mrr / mtt_p_mpp (mono), mtr / mpr (di), mtp / mtt_m_mpp (quad)
    depth_km: float = 100.0
    magnitude: float = 1e20
    seconds: float = 1800.0
    receivers_deg: np.ndarray | None = None     # colatitudes of surface receivers
    seis_it: int = 1
    courant: float = 0.6


def build_mesh(period: float = 50.0, solve: SphereSolve | None = None, model: str = "prem_iso",
               skeleton: Skeleton | None = None, pointwise: bool = True,
               attenuation: Attenuation | None = None) -> Mesh:
    """A whole-Earth solve on the PREM model at `period` seconds: the skeleton,
    every precomputed array of the time loop, source, receivers and the source
    time function, as a ``Mesh`` (FP32 module arrays, 1-based indices).  With
    `attenuation`, the cg4 anelastic model of prepare_attenuation: the solid's
    moduli become the unrelaxed ones before the stiffness terms are formed."""
    solve = solve or SphereSolve()
    sk = skeleton or build_skeleton(period, model)
    pole = solve.pole
    if "geo" not in sk.cache:            # the pole-independent geometry, computed once per skeleton
        sk.cache["geo"] = element_geometry(sk)
    geo = sk.cache["geo"]
    s, z = geo["s"], geo["z"]
    dsdxi, dzdxi, dsdeta, dzdeta = geo["dsdxi"], geo["dzdxi"], geo["dsdeta"], geo["dzdeta"]
    ax = geo["axis"]
    E = len(sk.elems)
    r = np.hypot(s, z)
    theta = np.arctan2(s, z)
    jac = dsdxi * dzdeta - dsdeta * dzdxi
    if not (jac > 0).all():
        raise RuntimeError(f"mesh has {int((jac <= 0).sum())} points with a non-positive Jacobian")
    idom_el = domain_of(r[:, 2, 2])
    idom = np.broadcast_to(idom_el[:, None, None], r.shape)
    fluid_el = idom_el == FLUID_DOMAIN
    # materials at the GLL points (read_model, SOLVER/get_model.F90:149-200)
    rho = velocity(r, "rho", idom, model)
    vph, vpv = velocity(r, "vph", idom, model), velocity(r, "vpv", idom, model)
    vsh, vsv = velocity(r, "vsh", idom, model), velocity(r, "vsv", idom, model)
    eta_a = velocity(r, "eta", idom, model)
    lam = rho * (vph ** 2 - 2.0 * vsh ** 2)
    mu = rho * vsh ** 2
    xi_a = np.where(vsv > 1e-6 * vph, vsh ** 2 / np.where(vsv > 0, vsv, 1.0) ** 2, 1.0)
    phi_a = vpv ** 2 / vph ** 2

    # ---- weights and the axial s / (1 + xi) (s_over_oneplusxi_axis)
    wti = np.where(ax[:, None], SP.wt_axial_k[None, :], SP.wt[None, :])[:, :, None]   # (E, i, 1)
    wtj = SP.wt[None, None, :]
    xi = geo["xi"][:, :, None]
    onexi = 1.0 + xi
    sox = np.where(ax[:, None, None], np.where(xi == -1.0, dsdxi, s / np.where(onexi == 0, 1.0, onexi)), s)
    inv_j = 1.0 / jac
    # massmat_k and massmat_kwts2 (def_mass_matrix_k)
    massmat = jac * sox * wti * wtj
    with np.errstate(divide="ignore", invalid="ignore"):
        kw_non = jac / s * wti * wtj
        kw_ax = np.where(xi == -1.0, jac / sox, jac / (s * onexi)) * wti * wtj
    massmat_kwts2 = np.where(ax[:, None, None], kw_ax, kw_non)
    # the alpha .. zeta and Ms_* terms times the weights (alpha, alphak, ..., analytic_mapping.f90)
    sfac = sox * wti * wtj        # s wt wt (non-axial); s/(1+xi) wt_ax wt (axial)
    T = {
        "alpha": -inv_j * dsdxi * dsdeta * sfac, "beta": inv_j * dsdxi ** 2 * sfac,
        "gamma": inv_j * dsdeta ** 2 * sfac, "delta": -inv_j * dzdxi * dzdeta * sfac,
        "epsil": inv_j * dzdxi ** 2 * sfac, "zeta": inv_j * dzdeta ** 2 * sfac,
        "Mzes_xi": inv_j * dsdxi * dzdeta * sfac, "Mzes_eta": -inv_j * dsdeta * dzdeta * sfac,
        "Mzxs_eta": inv_j * dsdeta * dzdxi * sfac, "Mzxs_xi": -inv_j * dsdxi * dzdxi * sfac,
    }
    mfac = np.where(ax[:, None, None], np.where(xi == -1.0, 0.0, wti * wtj / np.where(onexi == 0, 1.0, onexi)),
                    wti * wtj)
    Msxi, Mzxi = dsdxi * mfac, -dzdxi * mfac
    Mzeta, Mseta = dzdeta * mfac, -dsdeta * mfac
    # non_diag_fact of axial elements: wt_ax(0) wt(j) J(xi_0, eta_j) / s_over_oneplusxi
    ndf = SP.wt_axial_k[0] * SP.wt[None, :] * jac[:, 0, :] / np.where(ax[:, None], dsdxi[:, 0, :], 1.0)
    ndf = np.where(ax[:, None], ndf, 0.0)

    solid = np.flatnonzero(~fluid_el)
    # the CFL time step, from the elastic P velocities (the mesher's dt)
    vp_el = velocity(r, "v_p", idom, model)
    deltat = _cfl(s, z, vp_el, solve.courant)
    anel = None
    if attenuation is not None:
        anel = _prepare_attenuation(attenuation, solid, lam, mu, massmat, r, idom, model, deltat)
    fluid = np.flatnonzero(fluid_el)
    if "num_solid" not in sk.cache:
        sk.cache["num_solid"] = global_numbering(sk, solid)
    ig_s, ng_s = sk.cache["num_solid"]
    m = Mesh(src_type=pole, nel_solid=len(solid), nglob_solid=ng_s, igloc_solid=ig_s,
             ax_el_solid=(np.flatnonzero(ax[solid]) + 1).astype(I32), spec=SP, m_solid={}, m0_solid={},
             inv_mass_rho=None)
    # ---- solid stiffness terms
    S = solid
    th_fa = theta[S]
    C = elastic_tensor(lam[S], mu[S], xi_a[S], phi_a[S], eta_a[S], th_fa, 0.0)
    t = {k: v[S] for k, v in T.items()}
    kw = massmat_kwts2[S]
    Ms, Mz, Me, Mse = Msxi[S], Mzxi[S], Mzeta[S], Mseta[S]
    axS = ax[S]
    M = {}
    if pole in (_abi.MONOPOLE, _abi.QUADPOLE):
        M["M11s"] = C["11"] * t["delta"] + C["15"] * t["Mzes_xi"] + C["15"] * t["Mzxs_eta"] + C["55"] * t["alpha"]
        M["M21s"] = C["11"] * t["zeta"] + C["15"] * 2.0 * t["Mzes_eta"] + C["55"] * t["gamma"]
        M["M41s"] = C["11"] * t["epsil"] + C["15"] * 2.0 * t["Mzxs_xi"] + C["55"] * t["beta"]
        M["M12s"] = C["15"] * t["delta"] + C["13"] * t["Mzes_xi"] + C["55"] * t["Mzxs_eta"] + C["35"] * t["alpha"]
        M["M22s"] = C["15"] * t["zeta"] + (C["13"] + C["55"]) * t["Mzes_eta"] + C["35"] * t["gamma"]
        M["M32s"] = C["15"] * t["delta"] + C["13"] * t["Mzxs_eta"] + C["55"] * t["Mzes_xi"] + C["35"] * t["alpha"]
        M["M42s"] = C["15"] * t["epsil"] + (C["13"] + C["55"]) * t["Mzxs_xi"] + C["35"] * t["beta"]
        M["M_1"] = C["12"] * Me + C["25"] * Mse
        M["M_2"] = C["12"] * Mz + C["25"] * Ms
        M["M_3"] = C["23"] * Mse + C["25"] * Me
        M["M_4"] = C["23"] * Ms + C["25"] * Mz
    else:  # dipole: the + and - components
        M["M11s"] = (C["11"] + C["66"]) * t["delta"] + (C["15"] + C["46"]) * (t["Mzes_xi"] + t["Mzxs_eta"]) \
            + (C["55"] + C["44"]) * t["alpha"]
        M["M21s"] = (C["11"] + C["66"]) * t["zeta"] + (C["15"] + C["46"]) * 2.0 * t["Mzes_eta"] \
            + (C["55"] + C["44"]) * t["gamma"]
        M["M41s"] = (C["11"] + C["66"]) * t["epsil"] + (C["15"] + C["46"]) * 2.0 * t["Mzxs_xi"] \
            + (C["55"] + C["44"]) * t["beta"]
        M["M12s"] = (C["11"] - C["66"]) * t["delta"] + (C["15"] - C["46"]) * (t["Mzes_xi"] + t["Mzxs_eta"]) \
            + (C["55"] - C["44"]) * t["alpha"]
        M["M22s"] = (C["11"] - C["66"]) * t["zeta"] + (C["15"] - C["46"]) * 2.0 * t["Mzes_eta"] \
            + (C["55"] - C["44"]) * t["gamma"]
        M["M42s"] = (C["11"] - C["66"]) * t["epsil"] + (C["15"] - C["46"]) * 2.0 * t["Mzxs_xi"] \
            + (C["55"] - C["44"]) * t["beta"]
        M["M13s"] = C["15"] * t["delta"] + C["13"] * t["Mzes_xi"] + C["55"] * t["Mzxs_eta"] + C["35"] * t["alpha"]
        M["M32s"] = C["15"] * t["zeta"] + (C["13"] + C["55"]) * t["Mzes_eta"] + C["35"] * t["gamma"]
        M["M33s"] = C["15"] * t["delta"] + C["13"] * t["Mzxs_eta"] + C["55"] * t["Mzes_xi"] + C["35"] * t["alpha"]
        M["M43s"] = C["15"] * t["epsil"] + (C["13"] + C["55"]) * t["Mzxs_xi"] + C["35"] * t["beta"]
        M["M_1"] = (C["12"] + C["66"]) * 2.0 * Me + (C["25"] + C["46"]) * 2.0 * Mse
        M["M_2"] = (C["12"] + C["66"]) * 2.0 * Mz + (C["25"] + C["46"]) * 2.0 * Ms
        M["M_3"] = C["46"] * Me + C["44"] * Mse
        M["M_4"] = C["46"] * Mz + C["44"] * Ms
        M["M_5"] = (C["12"] - C["66"]) * 2.0 * Me + (C["25"] - C["46"]) * 2.0 * Mse
        M["M_6"] = (C["12"] - C["66"]) * 2.0 * Mz + (C["25"] - C["46"]) * 2.0 * Ms
        M["M_7"] = C["25"] * 2.0 * Me + C["23"] * 2.0 * Mse
        M["M_8"] = C["25"] * 2.0 * Mz + C["23"] * 2.0 * Ms
        M["M_w1"] = 4.0 * (C["22"] + C["66"]) * kw
        M["M_w2"] = 2.0 * C["46"] * kw
        M["M_w3"] = C["44"] * kw
    M["M11z"] = C["55"] * t["delta"] + C["35"] * (t["Mzes_xi"] + t["Mzxs_eta"]) + C["33"] * t["alpha"]
    M["M21z"] = C["55"] * t["zeta"] + C["35"] * 2.0 * t["Mzes_eta"] + C["33"] * t["gamma"]
    M["M41z"] = C["55"] * t["epsil"] + C["35"] * 2.0 * t["Mzxs_xi"] + C["33"] * t["beta"]
    if pole == _abi.MONOPOLE:
        M["M11z"] = C["55"] * t["delta"] + C["35"] * t["Mzes_xi"] + C["35"] * t["Mzxs_eta"] + C["33"] * t["alpha"]
        M["M_w1"] = C["22"] * kw
    if pole == _abi.QUADPOLE:
        M["M1phi"] = C["66"] * t["delta"] + C["46"] * t["Mzes_xi"] + C["46"] * t["Mzxs_eta"] + C["44"] * t["alpha"]
        M["M2phi"] = C["66"] * t["zeta"] + C["46"] * 2.0 * t["Mzes_eta"] + C["44"] * t["gamma"]
        M["M4phi"] = C["66"] * t["epsil"] + C["46"] * 2.0 * t["Mzxs_xi"] + C["44"] * t["beta"]
        M["M_5"] = C["66"] * Me + C["46"] * Mse
        M["M_6"] = C["66"] * Mz + C["46"] * Ms
        M["M_7"] = C["44"] * Mse + C["46"] * Me
        M["M_8"] = C["44"] * Ms + C["46"] * Mz
        M["M_w1"] = (C["22"] + 4.0 * C["66"]) * kw
        M["M_w2"] = -2.0 * (C["22"] + C["66"]) * kw
        M["M_w3"] = 2.0 * C["46"] * kw
        M["M_w4"] = (4.0 * C["22"] + C["66"]) * kw
        M["M_w5"] = 4.0 * C["44"] * kw
    # axial masking of the ipol = 0 rows (compute_*_stiff_terms)
    zero_rows = ["M_w1"] + ([] if pole == _abi.MONOPOLE else
                            ["M_1", "M_2", "M_3", "M_4", "M_5", "M_6", "M_7", "M_8", "M_w1", "M_w3"]
                            + (["M_w2", "M_w4", "M_w5"] if pole == _abi.QUADPOLE else []))
    for nm in set(zero_rows):
        M[nm][axS, 0, :] = 0.0
    # axial vectors M0_w* (ipol = 0 of axial elements)
    ndfS = ndf[S]
    C0 = {k: v[:, 0, :] for k, v in C.items()}
    wa0 = SP.wt_axial_k[0] * SP.wt[None, :]
    dsx0, dzx0 = dsdxi[S][:, 0, :], dzdxi[S][:, 0, :]
    M0 = {}
    if pole == _abi.MONOPOLE:
        M0["M0_w1"] = (2.0 * C0["12"] + C0["22"]) * ndfS
        M0["M0_w2"] = C0["25"] * ndfS
        M0["M0_w3"] = C0["23"] * dsx0 * wa0 - C0["25"] * dzx0 * wa0
    elif pole == _abi.DIPOLE:
        M0["M0_w1"] = (C0["12"] + C0["66"]) * 2.0 * ndfS
        M0["M0_w2"] = -(C0["12"] + C0["66"]) * 2.0 * dzx0 * wa0
        M0["M0_w3"] = C0["46"] * ndfS
        M0["M0_w4"] = -C0["46"] * dzx0 * wa0
        M0["M0_w5"] = np.zeros_like(ndfS)
        M0["M0_w6"] = (C0["25"] + C0["46"]) * 2.0 * dsx0 * wa0
        M0["M0_w7"] = C0["44"] * ndfS
        M0["M0_w8"] = C0["44"] * dsx0 * wa0
        M0["M0_w9"] = (C0["12"] + C0["22"]) * 4.0 * ndfS
        M0["M0_w10"] = (2.0 * C0["25"] + C0["46"]) * ndfS
    else:
        M0["M0_w1"] = (2.0 * C0["12"] + C0["22"] + 4.0 * C0["66"]) * ndfS
        M0["M0_w2"] = -2.0 * (C0["12"] + C0["22"]) * ndfS
        M0["M0_w3"] = (C0["25"] + 4.0 * C0["46"]) * ndfS
        M0["M0_w4"] = (4.0 * C0["22"] - C0["66"]) * ndfS
        M0["M0_w5"] = -2.0 * C0["25"] * ndfS
        M0["M0_w6"] = 4.0 * C0["44"] * ndfS
    for k in M0:
        M0[k] = np.where(axS[:, None], M0[k], 0.0)
    used = set(_abi.SOLID_TERMS_USED[pole])
    m.m_solid = {k: _to_f(M[k]) for k in used}
    used0 = set(_abi.AXIAL_TERMS_USED[pole])
    m.m0_solid = {k: np.asfortranarray(M0[k].T.astype(F32)) for k in used0}
    # solid inverse mass (def_mass_matrix_k): FP32 rho * massmat_k, assembled, inverted
    mass_s = _to_f(rho[S] * massmat[S])
    unassem = mass_s * F32(2.0) if pole == _abi.DIPOLE else mass_s
    m.meta["unassem_mass_rho_solid"] = np.asfortranarray(unassem)
    mass_s = _pdistsum_f32(mass_s, ig_s, ng_s)
    inv_s = (F32(1.0) / mass_s).astype(F32)
    if pole == _abi.DIPOLE:
        inv_s = (inv_s * F32(0.5)).astype(F32)
    m.inv_mass_rho = np.asfortranarray(inv_s)
    # the same in FP64 throughout, for the compensated mode's FP64 terms
    mass_d = _pdistsum_f32(np.transpose(rho[S] * massmat[S], (1, 2, 0)), ig_s, ng_s, np.float64)
    m.inv_mass_rho_dp = np.asfortranarray((0.5 if pole == _abi.DIPOLE else 1.0) / mass_d)
    m.meta.update(skeleton=sk.info, kind="sphere", period=period, model=model,
                  massmat_k=massmat, rho=rho, solid=solid, fluid=fluid, r=r, theta=theta)

    # ---- fluid
    if len(fluid):
        if "num_fluid" not in sk.cache:
            sk.cache["num_fluid"] = global_numbering(sk, fluid)
        ig_f, ng_f = sk.cache["num_fluid"]
        Fl = fluid
        m.nel_fluid, m.nglob_fluid, m.igloc_fluid = len(Fl), ng_f, ig_f
        m.ax_el_fluid = (np.flatnonzero(ax[Fl]) + 1).astype(I32)
        rf = rho[Fl]
        m.m_fluid = {"M1chi_fl": _to_f((T["delta"][Fl] + T["alpha"][Fl]) / rf),
                     "M2chi_fl": _to_f((T["zeta"][Fl] + T["gamma"][Fl]) / rf),
                     "M4chi_fl": _to_f((T["epsil"][Fl] + T["beta"][Fl]) / rf)}
        if pole != _abi.MONOPOLE:
            mw = massmat_kwts2[Fl] / rf
            mw[ax[Fl], 0, :] = 0.0
            m0 = np.where(ax[Fl][:, None], ndf[Fl] / rf[:, 0, :], 0.0)
            if pole == _abi.QUADPOLE:
                mw, m0 = 4.0 * mw, 4.0 * m0
            m.m_fluid["M_w_fl"] = _to_f(mw)
            m.m0_w_fl = np.asfortranarray(m0.T.astype(F32))
        lam_f = lam[Fl]
        mass_f = _to_f(massmat[Fl] / lam_f)
        m.meta["unassem_mass_lam_fluid"] = np.asfortranarray(mass_f)
        mass_f = _pdistsum_f32(mass_f, ig_f, ng_f)
        m.inv_mass_fluid = np.asfortranarray((F32(1.0) / mass_f).astype(F32))
        mass_fd = _pdistsum_f32(np.transpose(massmat[Fl] / lam_f, (1, 2, 0)), ig_f, ng_f, np.float64)
        m.inv_mass_fluid_dp = np.asfortranarray(1.0 / mass_fd)
        _boundary(m, sk, geo, solid, fluid)
    if pointwise or anel is not None:
        _pointwise(m, geo, solid, fluid, rho)
    if anel is not None:
        # Y, V_* of def_solid_stiffness_terms (anel_true): wt wt J and s times
        # the M_*_wt_k terms; on axial elements s is taken at the GLL node
        # eta(ipol), as the reference's mapping(eta(ipol), eta(jpol)) call does
        sg = element_geometry(sk, solid, gll_only=True)["s"]
        Yf = jac[S] * mfac[S]
        pw = m.pointwise
        anel["inv_s_solid"] = pw["inv_s_solid"]
        V = {"V_s_eta": sg * Mseta[S], "V_s_xi": sg * Msxi[S], "V_z_eta": sg * Mzeta[S], "V_z_xi": sg * Mzxi[S]}
        if attenuation.coarse_grained:
            cg = lambda a: np.asfortranarray(np.stack([a[:, i, j] for (i, j) in CG4], 0).astype(F32))  # noqa: E731
            anel["Y_cg4"] = cg(Yf)
            for nm, a in V.items():
                anel[nm + "_cg4"] = cg(a)
            for nm in ("DsDeta_over_J_sol", "DzDeta_over_J_sol", "DsDxi_over_J_sol", "DzDxi_over_J_sol"):
                anel[nm + "_cg4"] = cg(np.transpose(pw[nm], (2, 0, 1)))
        else:
            # at every GLL point (mfac is zero at ipol = 0 of axial elements,
            # so Y and V_* are, as the reference sets them); the axial
            # elements' ipol = 0 terms Y0, V0_* (def_solid_stiffness_terms,
            # SOLVER/def_precomp_terms.f90:1504-1526), (0:4, nel_solid)
            axs = ax[S]
            wa0 = SP.wt_axial_k[0] * SP.wt[None, :]
            dsx0 = dsdxi[S][:, 0, :]
            a0 = lambda a: np.asfortranarray(np.where(axs[:, None], a, 0.0).T.astype(F32))  # noqa: E731
            anel["Y"] = _to_f(Yf)
            for nm, a in V.items():
                anel[nm] = _to_f(a)
            anel.update({"Y0": a0(wa0 * jac[S][:, 0, :]), "V0_s_eta": a0(np.zeros_like(dsx0)),
                         "V0_s_xi": a0(wa0 * dsx0 * dsx0), "V0_z_eta": a0(wa0 * dsx0 * dzdeta[S][:, 0, :]),
                         "V0_z_xi": a0(wa0 * dsx0 * (-dzdxi[S][:, 0, :]))})
            for nm in ("DsDeta_over_J_sol", "DzDeta_over_J_sol", "DsDxi_over_J_sol", "DzDxi_over_J_sol"):
                anel[nm] = pw[nm]
        m.anel = anel
    _source_receivers(m, sk, geo, solve, period, deltat)
    return m


def _cfl(s, z, vp, courant: float) -> float:
    """CFL time step: courant times the smallest distance between
    neighbouring GLL points over the P velocity there (the criterion of
    MESHER/discont_meshing.f90:336-339, evaluated on the actual points)."""
    ds_i = np.hypot(np.diff(s, axis=1), np.diff(z, axis=1))
    ds_j = np.hypot(np.diff(s, axis=2), np.diff(z, axis=2))
    vi = np.maximum(vp[:, 1:, :], vp[:, :-1, :])
    vj = np.maximum(vp[:, :, 1:], vp[:, :, :-1])
    return float(courant * min((ds_i / vi).min(), (ds_j / vj).min()))


def _prepare_attenuation(att: Attenuation, solid, lam, mu, massmat, r, idom, model, deltat):
    """prepare_attenuation (SOLVER/attenuation.f90:682-1137): per solid
    element Q from the model at its point (1,1), the SLS weights
    yp_j = y_j / Q (fast_correct'ed), the moduli at the band's central
    frequency, the delta moduli, the unrelaxed moduli (written back into
    lam and mu, which the stiffness terms then use) and the cg4-weighted
    delta moduli (coarse-grained; :1035-1052) or the delta moduli at every
    GLL point (:1053-1063); the time-stepping factors of the exact SLS
    integration."""
    w_j, y_j = sls_fit(att)
    w_0 = att.f_ref * 2 * np.pi
    w_1 = np.sqrt(att.f_min * att.f_max) * 2 * np.pi
    S = solid
    ri = r[S][:, 1, 1]
    dom = idom[S][:, 1, 1]
    Q_mu = velocity(ri, "Qmu", dom, model).astype(F32)
    Q_ka = velocity(ri, "Qka", dom, model).astype(F32)
    cgr = att.coarse_grained
    if cgr:
        wcg = _weights_cg(massmat[S])                   # (E, 4)
        wfull = np.zeros((len(S), 5, 5))
        for k, (i, j) in enumerate(CG4):
            wfull[:, i, j] = wcg[:, k]
    else:
        wfull = np.ones((len(S), 5, 5))
    dmu_cg4 = np.zeros((4, len(S)))
    dka_cg4 = np.zeros((4, len(S)))
    dmu_all = np.zeros((len(S), 5, 5))
    dka_all = np.zeros((len(S), 5, 5))
    for e in range(len(S)):
        qm, qk = float(Q_mu[e]), float(Q_ka[e])
        ypm = fast_correct(y_j / qm) if att.do_corr_lowq else y_j / qm
        ypk = fast_correct(y_j / qk) if att.do_corr_lowq else y_j / qk
        mu_fac = float(np.sum(ypm * w_j ** 2 / (w_1 ** 2 + w_j ** 2))) / float(np.sum(ypm))
        ka_fac = float(np.sum(ypk * w_j ** 2 / (w_1 ** 2 + w_j ** 2))) / float(np.sum(ypk))
        ge = S[e]
        mu_w1 = mu[ge] * (1 + 2.0 / (np.pi * qm) * np.log(w_1 / w_0))
        ka_w1 = (lam[ge] + 2.0 / 3.0 * mu[ge]) * (1 + 2.0 / (np.pi * qk) * np.log(w_1 / w_0))
        dmu0 = mu_w1 / (1.0 / np.sum(ypm) + 1 - mu_fac)
        dka0 = ka_w1 / (1.0 / np.sum(ypk) + 1 - ka_fac)
        mu[ge] = mu_w1 + wfull[e] * dmu0 * mu_fac
        lam[ge] = ka_w1 + wfull[e] * dka0 * ka_fac - 2.0 / 3.0 * mu[ge]
        if cgr:
            for k, (i, j) in enumerate(CG4):
                dmu_cg4[k, e] = wcg[e, k] * dmu0[i, j]
                dka_cg4[k, e] = wcg[e, k] * dka0[i, j]
        else:
            dmu_all[e] = dmu0
            dka_all[e] = dka0
    ex = np.exp(-w_j * deltat)
    out = {"y_j": y_j, "w_j": w_j, "exp_w_j_deltat": ex,
           "ts_fac_tm1": (1 - ex) / (w_j * deltat) - ex, "ts_fac_t": (ex - 1) / (w_j * deltat) + 1,
           "do_corr_lowq": int(att.do_corr_lowq), "Q_mu": Q_mu, "Q_kappa": Q_ka}
    if cgr:
        out["delta_mu_cg4"] = np.asfortranarray(dmu_cg4.astype(F32))
        out["delta_kappa_cg4"] = np.asfortranarray(dka_cg4.astype(F32))
    else:
        out["delta_mu"] = _to_f(dmu_all)
        out["delta_kappa"] = _to_f(dka_all)
    return out


def _boundary(m: Mesh, sk: Skeleton, geo, solid, fluid):
    """The solid-fluid boundary tables and bdry_matr
    (def_solid_fluid_boundary_terms, SOLVER/def_precomp_terms.f90:2474-2799):
    for every solid element edge on the CMB or the ICB, the fluid element
    across it; bdry_matr(ipol, 1:2) = dtheta/2 w sin(theta) (sin, cos)(theta)
    r^2, with the axial L'Hopital point, negative where the fluid lies above
    the solid (the ICB)."""
    def edge_index(els):
        el = sk.elems[els]
        bot = np.stack([np.minimum(el[:, 0], el[:, 1]), np.maximum(el[:, 0], el[:, 1])], 1)
        topk = np.stack([np.minimum(el[:, 3], el[:, 2]), np.maximum(el[:, 3], el[:, 2])], 1)
        return bot, topk
    sb, st = edge_index(solid)
    fb, ft = edge_index(fluid)
    fmap = {}
    for k in range(len(fluid)):
        fmap[tuple(fb[k])] = (k, 0)
        fmap[tuple(ft[k])] = (k, 4)
    rows = []
    for k in range(len(solid)):
        for ed, jp in ((sb[k], 0), (st[k], 4)):
            hit = fmap.get(tuple(ed))
            if hit is not None:
                rows.append((k, jp, hit[0], hit[1]))
    rows.sort()
    nb = len(rows)
    bs = np.array([r[0] for r in rows], dtype=np.int64)
    js = np.array([r[1] for r in rows], dtype=np.int64)
    bf = np.array([r[2] for r in rows], dtype=np.int64)
    jf = np.array([r[3] for r in rows], dtype=np.int64)
    s, z = geo["s"][solid][bs], geo["z"][solid][bs]     # (nb, 5, 5)
    sf, zf = geo["s"][fluid][bf], geo["z"][fluid][bf]
    ip = np.arange(5)
    ss, zs = s[np.arange(nb)[:, None], ip[None, :], js[:, None]], z[np.arange(nb)[:, None], ip[None, :], js[:, None]]
    sff, zff = sf[np.arange(nb)[:, None], ip[None, :], jf[:, None]], zf[np.arange(nb)[:, None], ip[None, :], jf[:, None]]
    if np.max(np.hypot(ss - sff, zs - zff)) > 1e-3:
        raise RuntimeError("solid and fluid boundary points do not coincide")
    r = np.hypot(ss, zs)
    th = np.arctan2(ss, zs)
    dth = 0.5 * np.abs(th[:, 4] - th[:, 0])
    axs = geo["axis"][solid][bs]
    w = np.where(axs[:, None], SP.wt_axial_k[None, :], SP.wt[None, :])
    xi = np.where(axs[:, None], SP.xi_k[None, :], SP.eta[None, :])
    fac = np.where(axs[:, None], 1.0 / np.where(xi == -1.0, 1.0, 1.0 + xi), 1.0)
    b1 = dth[:, None] * w * np.sin(th) * fac * np.sin(th)
    b2 = dth[:, None] * w * np.sin(th) * fac * np.cos(th)
    if axs.any():
        # the axis point: 0 and (1/r) dtheta/2 w_ax(0) s/(1+xi) at xi = -1 (= ds/dxi)
        dsx = geo["dsdxi"][solid][bs][np.arange(nb), 0, js]
        b1[axs, 0] = 0.0
        b2[axs, 0] = (1.0 / r[axs, 0]) * dth[axs] * SP.wt_axial_k[0] * dsx[axs]
    rad = r[:, 0]
    sign = np.where(np.abs(rad - ICB) < 1.0, -1.0, 1.0)
    b1 = b1 * sign[:, None] * rad[:, None] ** 2
    b2 = b2 * sign[:, None] * rad[:, None] ** 2
    m.bdry_solid_el = (bs + 1).astype(I32)
    m.bdry_fluid_el = (bf + 1).astype(I32)
    m.bdry_jpol_solid = js.astype(I32)
    m.bdry_jpol_fluid = jf.astype(I32)
    m.bdry_matr = np.asfortranarray(np.stack([b1.T, b2.T], axis=2).astype(F32))   # (5, nb, 2)
    m.meta["bdry_radius"] = rad


def _pointwise(m: Mesh, geo, solid, fluid, rho):
    """data_pointwise (compute_pointwisederiv_matrices,
    SOLVER/def_precomp_terms.f90:148-290): the mapping derivatives over the
    Jacobian, 1/s (1 on the axis points of axial elements) and the fluid's
    1/rho."""
    jac = geo["dsdxi"] * geo["dzdeta"] - geo["dsdeta"] * geo["dzdxi"]
    pw = {}

    def put(els, suf):
        j = jac[els]
        pw[f"DsDeta_over_J_{suf}"] = _to_f(-geo["dsdeta"][els] / j)
        pw[f"DzDeta_over_J_{suf}"] = _to_f(geo["dzdeta"][els] / j)
        pw[f"DsDxi_over_J_{suf}"] = _to_f(geo["dsdxi"][els] / j)
        pw[f"DzDxi_over_J_{suf}"] = _to_f(-geo["dzdxi"][els] / j)
        sv = geo["s"][els]
        with np.errstate(divide="ignore"):
            inv = np.where(sv > 0, 1.0 / np.where(sv > 0, sv, 1.0), 1.0)
        inv[geo["axis"][els], 0, :] = 1.0
        return inv

    inv_s = put(solid, "sol")
    pw["inv_s_solid"] = _to_f(inv_s)
    if len(fluid):
        pw["inv_s_fluid"] = _to_f(put(fluid, "flu"))
        pw["inv_rho_fluid"] = _to_f(1.0 / rho[fluid])
    m.pointwise = pw


def gauss_stf(niter: int, deltat: float, t0: float, magnitude: float, seis_it: int = 1) -> np.ndarray:
    """The `gauss` source time function (SOLVER/source.f90:587-598): t rounded
    to realkind, exp(-(decay / t0 (t - shift))^2) magnitude decay / (t0
    sqrt(pi)), decay 3.5, shift = seis_dt ceiling(1.5 t0 / seis_dt)
    (SOLVER/parameters.F90:1071)."""
    decay = 3.5
    seis_dt = deltat * seis_it
    shift = seis_dt * np.ceil(1.5 * t0 / seis_dt)
    t = (np.arange(1, niter + 1, dtype=np.float64) * deltat).astype(F32).astype(np.float64)
    stf = np.exp(-((decay / t0 * (t - shift)) ** 2)).astype(F32)
    return (stf.astype(np.float64) * magnitude * decay / t0 / np.sqrt(np.pi)).astype(F32)


def _source_receivers(m: Mesh, sk: Skeleton, geo, solve: SphereSolve, period: float, dt: float):
    """Moment-tensor source on the northern axis at the requested depth
    (find_srcloc / define_moment_tensor, SOLVER/source.f90:435-583, 985-1226),
    receivers at the surface points nearest to the requested colatitudes, the
    time step, niter and the Gaussian source time function at the mesh
    period."""
    solid = m.meta["solid"]
    # the solid points' geometry that every solve on this skeleton searches
    # (axis points, surface points), kept with the skeleton
    key = ("solid_points", id(solid))
    if key not in sk.cache:
        s_, z_ = geo["s"][solid], geo["z"][solid]
        r_ = np.hypot(s_, z_)
        on_axis = (s_ == 0.0) & (z_ > 0.0)
        surf_ = np.argwhere(np.abs(r_ - R_EARTH) < 1.0)
        sk.cache[key] = {"axis_pts": np.argwhere(on_axis), "axis_z": z_[on_axis], "z": z_,
                         "surf": surf_, "surf_th": np.degrees(np.arctan2(s_[tuple(surf_.T)], z_[tuple(surf_.T)]))}
    pc = sk.cache[key]
    m.deltat = dt
    m.seis_it = solve.seis_it
    niter = int(np.ceil((solve.seconds + 1e-11) / dt))
    m.magnitude = solve.magnitude
    m.stf = gauss_stf(niter, dt, period, solve.magnitude, solve.seis_it)
    # ---- source: the northern axis point nearest to the source depth
    zsrc = R_EARTH - solve.depth_km * 1000.0
    cand = pc["axis_pts"]
    dz = np.abs(pc["axis_z"] - zsrc)
    best = dz.min()
    hits = cand[np.abs(dz - best) <= 1e-6 * R_EARTH]
    # the point's elements (at most 2 along the axis), as find_srcloc keeps them
    pts = {}
    for e, i, j in hits:
        pts.setdefault(int(e), (int(i), int(j)))
    src_els = sorted(pts)[:2]
    pole = m.src_type
    kind = solve.source or {0: "explosion", 1: "mtr", 2: "mtp"}[pole]
    nsrc = len(src_els)
    E = m.nel_solid
    # The source term is nonzero only on the source elements' points, so its
    # assembly (pdistsum_solid) involves only the elements that hold one of
    # them: it runs on those, in element order, with the same sums in the
    # same order as over the whole mesh.
    near, ig_near, n_near_pts = _neighbourhood(m.igloc_solid, E, src_els)
    slot = {int(e): k for k, e in enumerate(near)}
    N = len(near)
    st = np.zeros((N, 5, 5, 3))          # [near element, ipol, jpol, comp] FP64
    axis_s = geo["axis"][solid]
    pw = m.pointwise
    for e in src_els:
        li, lj = pts[e]
        G = SP.G1 if axis_s[e] else SP.G2
        jac = geo["dsdxi"][solid][e] * geo["dzdeta"][solid][e] - geo["dsdeta"][solid][e] * geo["dzdxi"][solid][e]
        dzdeta_j = geo["dzdeta"][solid][e] / jac
        dzdxi_j = -geo["dzdxi"][solid][e] / jac
        dsdeta_j = -geo["dsdeta"][solid][e] / jac
        dsdxi_j = geo["dsdxi"][solid][e] / jac
        k = slot[e]
        for ip in range(5):
            for jp in range(5):
                # derivatives at (li, lj) of the Lagrange basis function of (ip, jp)
                dfdxi = G[ip, li] * (1.0 if jp == lj else 0.0)
                dfdeta = (1.0 if ip == li else 0.0) * SP.G2[jp, lj]
                dsdf = dzdeta_j[li, lj] * dfdxi + dzdxi_j[li, lj] * dfdeta
                dzdf = dsdeta_j[li, lj] * dfdxi + dsdxi_j[li, lj] * dfdeta
                if pole == _abi.MONOPOLE:
                    if kind == "explosion":
                        st[k, ip, jp, 0] = 2.0 * dsdf
                        st[k, ip, jp, 2] = dzdf
                    elif kind == "mtt_p_mpp":
                        st[k, ip, jp, 0] = dsdf
                    elif kind == "mrr":
                        st[k, ip, jp, 2] = dzdf
                    else:
                        raise ValueError(f"monopole source {kind}")
                elif pole == _abi.DIPOLE:
                    if kind not in ("mtr", "mpr"):
                        raise ValueError(f"dipole source {kind}")
                    st[k, ip, jp, 0] = dzdf
                    st[k, ip, jp, 2] = dsdf
                else:
                    if kind not in ("mtp", "mtt_m_mpp"):
                        raise ValueError(f"quadrupole source {kind}")
                    st[k, ip, jp, 0] = dsdf
                    st[k, ip, jp, 1] = dsdf
    st = st / nsrc
    # pdistsum_solid in FP32, small values cut (smallval = 1e-6), the pole's axis mask
    stf_ = np.zeros((5, 5, N, 3), dtype=F32, order="F")
    for c in range(3):
        stf_[..., c] = _pdistsum_f32(_to_f(st[..., c]), ig_near, n_near_pts)
    stf_[np.abs(stf_) < 1e-6] = 0.0
    ax_near = np.array([slot[int(e)] for e in m.ax_el_solid - 1 if int(e) in slot], dtype=np.int64)
    comps = {0: [0], 1: [1, 2], 2: [0, 1, 2]}[pole]
    for c in comps:
        stf_[0, :, ax_near, c] = 0.0
    stf_ = stf_ / F32(np.pi if pole == _abi.DIPOLE else 2.0 * np.pi)
    # the same in FP64 (the entries the FP32 term keeps)
    std_ = np.zeros((5, 5, N, 3), order="F")
    for c in range(3):
        std_[..., c] = _pdistsum_f32(np.transpose(st[..., c], (1, 2, 0)), ig_near, n_near_pts, np.float64)
    std_[stf_ == 0] = 0.0
    std_ = std_ / (np.pi if pole == _abi.DIPOLE else 2.0 * np.pi)
    nzk = np.flatnonzero(np.any(stf_ != 0, axis=(0, 1, 3))).tolist()
    if len(nzk) > 8:
        raise RuntimeError(f"source term spans {len(nzk)} elements (8 at most)")
    m.ielsrc = np.zeros(8, dtype=I32)
    m.ielsrc[:len(nzk)] = near[nzk].astype(I32) + 1
    m.nelsrc = len(nzk)
    ste = np.zeros((5, 5, 8, 3), dtype=F32, order="F")
    sted = np.zeros((5, 5, 8, 3), order="F")
    for k, e in enumerate(nzk):
        ste[:, :, k, :] = stf_[:, :, e, :]
        sted[:, :, k, :] = std_[:, :, e, :]
    m.source_term_el = ste
    m.source_term_el_dp = sted
    m.fluid_src = 0
    m.meta["source"] = {"kind": kind, "depth_km": float((R_EARTH - pc["z"][tuple(hits[0])]) / 1000.0),
                        "elements": [int(e) + 1 for e in src_els]}
    # ---- receivers: the surface point nearest to each colatitude
    rec = solve.receivers_deg
    if rec is None:
        rec = np.linspace(0.0, 180.0, 20)
    surf, th = pc["surf"], pc["surf_th"]
    rows = []
    for c in np.asarray(rec, dtype=np.float64):
        k = int(np.argmin(np.abs(th - c)))
        e, i, j = surf[k]
        rows.append((e + 1, i, j))
    m.recfile_el = np.asfortranarray(np.array(rows, dtype=I32).reshape(-1, 3))
    m.meta["receiver_colat_deg"] = np.array([th[int(np.argmin(np.abs(th - c)))] for c in rec])


def long_run_mesh(steps: int = 100_000, period: float = 50.0, model: str = "prem_ani",
                  skeleton: Skeleton | None = None) -> Mesh:
    """The long anelastic run of the precision study: `steps` time steps on
    the `model` mesh at `period` seconds with cg4 attenuation (5 SLS, PREM
    Q), a dipole source (Mrt = 1e20 N m) at 100 km depth and 10 surface
    receivers from 5 to 175 degrees, sampled every 50 steps."""
    sk = skeleton or build_skeleton(period, model)
    solve = SphereSolve(pole=_abi.DIPOLE, source="mtr", depth_km=100.0, seconds=1.0,
                        receivers_deg=np.linspace(5.0, 175.0, 10), seis_it=50)
    m = build_mesh(period, solve, model=model, skeleton=sk, attenuation=Attenuation())
    solve.seconds = (steps - 0.5) * m.deltat
    out = with_solve(m, solve, sk)
    assert out.niter == steps
    return out


def with_solve(m: Mesh, solve: SphereSolve, skeleton: Skeleton) -> Mesh:
    """The mesh `m` (built by build_mesh on `skeleton` for the same pole
    type) with another solve's source depth, receivers, run length and
    sampling: a shallow copy sharing every mesh array, so that meshes that
    differ only in these are the same mesh (axg_create_sharing)."""
    if solve.pole != m.src_type:
        raise ValueError("with_solve keeps the pole type of the mesh")
    out = copy.copy(m)
    out.meta = dict(m.meta)
    _source_receivers(out, skeleton, skeleton.cache["geo"], solve, m.meta["period"], m.deltat)
    return out
