"""Whole-Earth PREM meshes and their precomputed terms, checked against the
reference's own known answers and against physical properties of the
operator (CPU; the oracle in FP64).

The reference's checks (SOLVER/def_grid.f90:377-413, mesh_tests; and
SOLVER/def_precomp_terms.f90):
  * compute_volume: 2 pi sum(massmat) against 4/3 pi r^3 for the whole
    sphere, the solid and the fluid outer core (:1188-1332);
  * compute_spherical_surfaces: the boundary weights of every spherical
    level integrate sin(theta) to 2 (:992-1176);
  * compute_mass_earth: the mesh's mass against the model integrated over
    shells of 100 m (:998-1160);
  * def_solid_fluid_boundary_terms: the boundary weights of the CMB and ICB
    sum to 4 (:2474-2799);
  * test_pntwsdrvtvs_solid / _fluid: the pointwise derivatives of
    f = z s^3 + s z^3 + (s + z) r_outer against the analytic gradient
    (:308-590).
Physical properties of the assembled operator the oracle applies:
  * K is symmetric (u.Kv = v.Ku) for every pole type;
  * K of a rigid translation vanishes (z for the monopole, the first
    dipole component for the dipole), to the FP32 rounding of the spectral
    matrices the descriptor holds;
  * the total energy of `energy` (SOLVER/time_evol_wave.F90:1424-1526) is
    conserved once the source has stopped, while it moves between the solid
    and the fluid.
"""
import numpy as np
import pytest

from axisem_gb300 import earth, sphere
from axisem_gb300.spectral import Spectral


@pytest.fixture(scope="module")
def sk50():
    return sphere.build_skeleton(50.0)


@pytest.fixture(scope="module")
def mesh50(sk50):
    return {p: sphere.build_mesh(50.0, sphere.SphereSolve(pole=p, seconds=700.0), skeleton=sk50) for p in (0, 1, 2)}


def test_layout_honours_discontinuities_and_resolution(sk50):
    info = sk50.info
    radii = {round(rb) for (rb, _, _) in info["layers"]} | {round(rt) for (_, rt, _) in info["layers"]}
    for d in earth.DISCONTINUITIES_KM * 1000.0:
        assert round(d) in radii
    # every shell layer has enough elements per quarter for 1.5 elements per wavelength
    for (rb, rt, idom), n in zip(info["layers"], info["layer_counts"]):
        v = sphere._vmin(idom, rb, rt, "prem_iso")
        h = 50.0 * v / (1.5 * sphere.GLL_SPACING_RATIO)
        assert n >= np.ceil(0.5 * np.pi * rt / h)
    geo = sphere.element_geometry(sk50)
    jac = geo["dsdxi"] * geo["dzdeta"] - geo["dsdeta"] * geo["dzdxi"]
    assert (jac > 0).all()
    # axial elements: the xi = -1 edge lies on the axis
    assert np.all(geo["s"][sk50.axis][:, 0, :] == 0.0)
    assert np.all(geo["s"][~sk50.axis] > 0.0)


def test_global_numbering_identifies_coincident_points(sk50, mesh50):
    geo = sphere.element_geometry(sk50)
    m = mesh50[0]
    for els, ig, ng in ((m.meta["solid"], m.igloc_solid, m.nglob_solid),
                        (m.meta["fluid"], m.igloc_fluid, m.nglob_fluid)):
        s = geo["s"][els].transpose(0, 2, 1).reshape(-1)
        z = geo["z"][els].transpose(0, 2, 1).reshape(-1)
        S, Z = np.zeros(ng), np.zeros(ng)
        S[ig - 1], Z[ig - 1] = s, z
        assert np.max(np.hypot(S[ig - 1] - s, Z[ig - 1] - z)) < 1e-3
        assert len(np.unique(ig)) == ng
        # distinct global points are distinct places (no duplicated node)
        key = np.round(np.stack([S, Z], 1) / 10.0).astype(np.int64)
        assert len(np.unique(key, axis=0)) == ng


def test_volumes(mesh50):
    m = mesh50[0]
    mm = m.meta["massmat_k"]
    v = lambda r: 4.0 / 3.0 * np.pi * r ** 3  # noqa: E731
    tot = 2.0 * np.pi * mm.sum()
    flu = 2.0 * np.pi * mm[m.meta["fluid"]].sum()
    sol = 2.0 * np.pi * mm[m.meta["solid"]].sum()
    assert abs(tot - v(earth.R_EARTH)) / v(earth.R_EARTH) < 1e-10
    assert abs(flu - (v(earth.CMB) - v(earth.ICB))) / (v(earth.CMB) - v(earth.ICB)) < 1e-10
    ex_sol = v(earth.R_EARTH) - v(earth.CMB) + v(earth.ICB)
    assert abs(sol - ex_sol) / ex_sol < 1e-10


def test_spherical_surfaces(sk50):
    """compute_spherical_surfaces: at every radial level, from each side, the
    element arcs on that level give sum(dtheta/2 w_i sin(theta_i)) = 2 (axial
    elements: GLJ weights over (1 + xi), the axis point by L'Hopital)."""
    sp = Spectral()
    geo = sphere.element_geometry(sk50)
    levels = sorted({round(rb) for (rb, _, _) in sk50.info["layers"]}
                    | {round(rt) for (_, rt, _) in sk50.info["layers"]})
    rc = np.hypot(geo["s"][:, 2, 2], geo["z"][:, 2, 2])
    sums = {}
    for e in range(len(sk50.elems)):
        for edge, jp in ((sphere.EDGE_BOTTOM, 0), (sphere.EDGE_TOP, 4)):
            if not sk50.arc[e, edge]:
                continue
            s, z = geo["s"][e, :, jp], geo["z"][e, :, jp]
            r = round(float(np.hypot(s[0], z[0])))
            if r not in levels:
                continue   # the mid-radius arcs inside a coarsening band
            th = np.arctan2(s, z)
            dth = 0.5 * abs(th[4] - th[0])
            if sk50.axis[e]:
                fac = np.where(sp.xi_k == -1.0, 0.0, 1.0 / (1.0 + np.where(sp.xi_k == -1.0, 0.0, sp.xi_k)))
                # the axis point by L'Hopital: sin(theta) / (1 + xi) -> dtheta/2
                val = dth * np.sum(sp.wt_axial_k * np.sin(th) * fac) + dth ** 2 * sp.wt_axial_k[0]
            else:
                val = dth * np.sum(sp.wt * np.sin(th))
            key = (r, "above" if rc[e] > r else "below")
            sums[key] = sums.get(key, 0.0) + val
    assert len(sums) >= 2 * len(levels) - 2
    for k, v in sums.items():
        assert abs(v - 2.0) < 1e-10, (k, v)


def test_mass_of_the_earth(mesh50):
    m = mesh50[0]
    mm, rho = m.meta["massmat_k"], m.meta["rho"]
    ex = earth.exact_mass()
    num = 2.0 * np.pi * float(np.sum(rho * mm))
    assert abs(num - ex["total"]) / ex["total"] < 1e-8
    assert abs(num - 5.97e24) / 5.97e24 < 2e-3          # the mass the reference prints beside it
    sol = 2.0 * np.pi * float(np.sum((rho * mm)[m.meta["solid"]]))
    flu = 2.0 * np.pi * float(np.sum((rho * mm)[m.meta["fluid"]]))
    assert abs(sol - ex["solid"]) / ex["solid"] < 1e-8
    assert abs(flu - ex["fluid"]) / ex["fluid"] < 1e-8


def test_boundary_terms(mesh50):
    """bdry_sum of def_solid_fluid_boundary_terms: the weights of the CMB and
    the ICB integrate sin(theta) to 2 each; bdry_matr carries r^2 and is
    negative on the ICB (fluid above solid)."""
    m = mesh50[0]
    rad = m.meta["bdry_radius"]
    b1, b2 = m.bdry_matr[:, :, 0].astype(np.float64), m.bdry_matr[:, :, 1].astype(np.float64)
    assert set(np.round(rad).astype(int)) == {int(earth.CMB), int(earth.ICB)}
    total = 0.0
    for R in (earth.CMB, earth.ICB):
        sel = np.abs(rad - R) < 1.0
        sign = -1.0 if R == earth.ICB else 1.0
        assert np.all(sign * b1[:, sel] >= -1e-3 * R * R)
        # |(b1, b2)| / r^2 = dtheta/2 w |sin(theta)| (the axis point: its
        # L'Hopital weight), the summand of the reference's bdry_sum
        bs = (b1[:, sel] ** 2 + b2[:, sel] ** 2) ** 0.5 / (R * R)
        total += float(bs.sum())
    assert abs(total - 4.0) < 1e-5
    assert len(m.bdry_solid_el) == len(m.bdry_fluid_el)


def test_pointwise_derivatives(sk50, mesh50):
    """test_pntwsdrvtvs_solid / _fluid on FP32 fields, as the reference runs it."""
    sp = Spectral()
    m = mesh50[0]
    geo = sphere.element_geometry(sk50)
    R = earth.R_EARTH
    f32 = lambda a: a.astype(np.float32).astype(np.float64)  # noqa: E731
    for els, suf in ((m.meta["solid"], "sol"), (m.meta["fluid"], "flu")):
        s, z, ax = geo["s"][els], geo["z"][els], geo["axis"][els]
        f = f32(z * s ** 3 + s * z ** 3 + (s + z) * R)
        P = {k: np.transpose(m.pointwise[f"{k}_{suf}"], (2, 0, 1)).astype(np.float64)
             for k in ("DsDeta_over_J", "DzDeta_over_J", "DsDxi_over_J", "DzDxi_over_J")}
        dxi = np.where(ax[:, None, None], np.einsum("ik,ekj->eij", f32(sp.G1.T), f),
                       np.einsum("ik,ekj->eij", f32(sp.G2.T), f))
        deta = np.einsum("eik,kj->eij", f, f32(sp.G2))
        dsf = P["DzDeta_over_J"] * dxi + P["DzDxi_over_J"] * deta
        dzf = P["DsDeta_over_J"] * dxi + P["DsDxi_over_J"] * deta
        es, ez = 3 * z * s ** 2 + z ** 3 + R, 3 * s * z ** 2 + s ** 3 + R
        rs, rz = np.abs(dsf - es) / np.abs(es), np.abs(dzf - ez) / np.abs(ez)
        assert rs.mean() < 5e-5 and rz.mean() < 5e-5
        assert rs.max() < 1e-2 and rz.max() < 1e-2


def test_stiffness_symmetric_and_rigid_modes(mesh50, orc):
    for pole, m in mesh50.items():
        ng = m.nglob_solid
        rng = np.random.default_rng(pole)
        u, v = rng.normal(size=(ng, 3)), rng.normal(size=(ng, 3))
        if pole == 0:
            u[:, 1] = v[:, 1] = 0.0
        Ku = orc.stiffness_assembled(m, u, np.float64)
        Kv = orc.stiffness_assembled(m, v, np.float64)
        a, b = float(np.sum(u * Kv)), float(np.sum(v * Ku))
        assert abs(a - b) / abs(a) < 1e-12
        if pole == 2:
            continue   # a quadrupole field has no rigid translation
        w = np.zeros((ng, 3))
        w[:, 2 if pole == 0 else 0] = 1.0
        Kw = orc.stiffness_assembled(m, w, np.float64)
        scale = np.linalg.norm(Ku) / np.linalg.norm(u)
        assert np.linalg.norm(Kw) / (scale * np.linalg.norm(w)) < 1e-6


def test_energy_conserved(mesh50, orc):
    """FP64 oracle: after the source, the total energy stays constant to
    1e-6 over 1200 steps although it moves between solid and fluid."""
    m = mesh50[0]
    t = orc.TimeLoop(m, np.float64)
    k0 = int(300.0 / m.deltat)
    assert t.run(1, k0) == 0
    es, flu = [], []
    it = k0
    for _ in range(4):
        assert t.run(it + 1, 300) == 0
        it += 300
        e = orc.energy(m, t.disp, t.velo, t.dchi, t.ddchi0)
        es.append(e["total"])
        flu.append(e["epot_flu"] + e["ekin_flu"])
    es = np.array(es)
    assert (es.max() - es.min()) / es.mean() < 1e-6
    assert flu[-1] > 1.5 * flu[0]   # energy did move into the fluid


def test_source_and_receivers(mesh50):
    m = mesh50[0]
    src = m.meta["source"]
    assert abs(src["depth_km"] - 100.0) < 20.0
    assert 1 <= m.nelsrc <= 8
    # receivers sit on the surface at the requested colatitudes
    assert m.recfile_el.shape == (20, 3)
    assert np.max(np.abs(m.meta["receiver_colat_deg"] - np.linspace(0, 180, 20))) < 5.0
    # 1800 s at the CFL time step of the 9.4 km lower-crust layer
    assert 0.05 < m.deltat < 0.3
    assert m.stf.dtype == np.float32 and np.abs(m.stf).max() > 1e17


def test_source_assembly_on_the_neighbourhood_equals_the_whole_mesh(mesh50):
    """with_solve assembles the source term (pdistsum_solid of a field that
    is nonzero on the source elements only) over the elements sharing a point
    with them: bit-identical to the assembly over the whole mesh, in FP32 and
    FP64, and zero everywhere else."""
    m = mesh50[2]
    E = m.nel_solid
    rng = np.random.default_rng(3)
    axial = np.asarray(m.ax_el_solid) - 1
    for src in ([int(axial[5])], [int(axial[5]), int(axial[6])], [E // 2]):
        near, ig_near, n_pts = sphere._neighbourhood(m.igloc_solid, E, src)
        assert set(src) <= set(near.tolist()) and len(near) < 40
        field = np.zeros((E, 5, 5))
        field[src] = rng.standard_normal((len(src), 5, 5))
        for dtype in (np.float32, np.float64):
            full = sphere._pdistsum_f32(np.transpose(field, (1, 2, 0)), m.igloc_solid, m.nglob_solid, dtype)
            part = sphere._pdistsum_f32(np.transpose(field[near], (1, 2, 0)), ig_near, n_pts, dtype)
            assert np.array_equal(full[:, :, near], part)
            rest = np.ones(E, dtype=bool)
            rest[near] = False
            assert not full[:, :, rest].any()


def test_attenuation_at_every_point_arrays(sk50):
    """att_coarse_grained = .false. on the PREM mesh: Y and V_* at every GLL
    point, equal to the coarse-grained arrays at the four cg points and zero
    at ipol = 0 of axial elements, whose terms are Y0 / V0_* (zero on the
    other elements); per-point modulus defects."""
    solve = sphere.SphereSolve(pole=1, source="mtr", seconds=100.0)
    a_cg = sphere.build_mesh(50.0, solve, skeleton=sk50, attenuation=sphere.Attenuation(), pointwise=False).anel
    m = sphere.build_mesh(50.0, solve, skeleton=sk50, attenuation=sphere.Attenuation(coarse_grained=False),
                          pointwise=False)
    a = m.anel
    E = m.nel_solid
    ax = np.asarray(m.ax_el_solid) - 1
    other = np.setdiff1d(np.arange(E), ax)
    for nm in ("Y", "V_s_eta", "V_s_xi", "V_z_eta", "V_z_xi", "delta_mu", "delta_kappa", "DsDeta_over_J_sol"):
        assert a[nm].shape == (5, 5, E) and a[nm].dtype == np.float32, nm
    for nm in ("Y", "V_s_eta", "V_s_xi", "V_z_eta", "V_z_xi"):
        for k, (i, j) in enumerate(sphere.CG4):
            assert np.array_equal(a[nm][i, j], a_cg[nm + "_cg4"][k]), nm
        assert not a[nm][0, :, ax].any()
    for nm in ("Y0", "V0_s_eta", "V0_s_xi", "V0_z_eta", "V0_z_xi"):
        assert a[nm].shape == (5, E) and not a[nm][:, other].any()
    assert (a["Y0"][:, ax] > 0).all() and (a["V0_s_xi"][:, ax] > 0).all() and not a["V0_s_eta"].any()
    assert (a["delta_mu"] > 0).all() and (a["delta_kappa"] > 0).all()


def test_attenuation_model(sk50, orc):
    """prepare_attenuation on the PREM mesh: the SLS fit reproduces a flat
    Q over the band, the cg4 weights partition each element's mass
    (sum_k w_k gamma(cg_k) = sum gamma), the unrelaxed moduli exceed the
    relaxed ones, and an anelastic run loses energy monotonically once the
    source has stopped while the elastic run keeps it."""
    att = sphere.Attenuation()
    w_j, y_j = sphere.sls_fit(att)
    w = 2 * np.pi * np.logspace(np.log10(att.f_min) + 0.3, np.log10(att.f_max) - 0.3, 50)
    qinv = np.sum(y_j[None, :] * w[:, None] * w_j[None, :] / (w[:, None] ** 2 + w_j[None, :] ** 2), axis=1)
    assert np.max(np.abs(qinv - 1.0)) < 0.05
    m = sphere.build_mesh(50.0, sphere.SphereSolve(pole=0, seconds=700.0), skeleton=sk50, attenuation=att)
    g = m.meta["massmat_k"][m.meta["solid"]]
    wcg = sphere._weights_cg(g)
    part = sum(wcg[:, k] * g[:, i, j] for k, (i, j) in enumerate(sphere.CG4))
    assert np.allclose(part, g.reshape(len(g), -1).sum(1), rtol=1e-12)
    an = m.anel
    assert an["delta_mu_cg4"].min() > 0 and an["delta_kappa_cg4"].min() > 0
    assert set(np.unique(an["Q_mu"]).tolist()) <= {600.0, 80.0, 143.0, 312.0, np.float32(84.6)}
    t = orc.TimeLoop(m, np.float64)
    k0 = int(300.0 / m.deltat)
    assert t.run(1, k0) == 0
    es = []
    it = k0
    for _ in range(4):
        assert t.run(it + 1, 300) == 0
        it += 300
        es.append(orc.energy(m, t.disp, t.velo, t.dchi, t.ddchi0)["total"])
    assert all(b < a for a, b in zip(es, es[1:]))
    assert es[-1] < 0.999 * es[0]
