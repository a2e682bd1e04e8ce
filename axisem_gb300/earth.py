"""The Preliminary Reference Earth Model (Dziewonski & Anderson, 1981) as the
reference's background models state it.

``prem_iso`` is the isotropic PREM without the ocean layer
(SOLVER/background_models.F90:417-533, ``prem_sub``); ``prem_ani`` its
transversely isotropic version (``prem_ani_sub``, :534-673).  A model is
given domain by domain: domain ``idom`` (1-based, as the reference counts
them) lies between discontinuity ``idom`` and ``idom + 1`` of
``DISCONTINUITIES_KM`` (MESHER/model_discontinuities.f90:283-378); the
last domain is the inner core.  Every function takes radii in metres and
returns SI units (kg/m^3, m/s), evaluated in FP64 as the reference does.
"""
from __future__ import annotations

import numpy as np

R_EARTH = 6371000.0
# radii (km) of the discontinuities the mesh honours, surface first
DISCONTINUITIES_KM = np.array([6371.0, 6356.0, 6346.6, 6291.0, 6151.0, 5971.0, 5771.0, 5701.0, 5600.0,
                               3630.0, 3480.0, 1221.5])
NDISC = len(DISCONTINUITIES_KM)
CMB, ICB = 3480000.0, 1221500.0
FLUID_DOMAIN = 11   # the outer core (1-based)

# polynomial coefficients in x = r / 6371 km, per domain (1-based index - 1):
# (rho, vp, vs) in g/cm^3 and km/s, lowest order first
_ISO = [
    ((2.6,), (5.8,), (3.2,)),
    ((2.9,), (6.8,), (3.9,)),
    ((2.691, 0.6924), (4.1875, 3.9382), (2.1519, 2.3481)),
    ((2.691, 0.6924), (4.1875, 3.9382), (2.1519, 2.3481)),
    ((7.1089, -3.8045), (20.3926, -12.2569), (8.9496, -4.4597)),
    ((11.2494, -8.0298), (39.7027, -32.6166), (22.3512, -18.5856)),
    ((5.3197, -1.4836), (19.0957, -9.8672), (9.9839, -4.9324)),
    ((7.9565, -6.4761, 5.5283, -3.0807), (29.2766, -23.6027, 5.5242, -2.5514),
     (22.3459, -17.2473, -2.0834, 0.9783)),
    ((7.9565, -6.4761, 5.5283, -3.0807), (24.9520, -40.4673, 51.4832, -26.6419),
     (11.1671, -13.7818, 17.4575, -9.2777)),
    ((7.9565, -6.4761, 5.5283, -3.0807), (15.3891, -5.3181, 5.5242, -2.5514),
     (6.9254, 1.4672, -2.0834, 0.9783)),
    ((12.5815, -1.2638, -3.6426, -5.5281), (11.0487, -4.0362, 4.8023, -13.5732), (0.0,)),
    ((13.0885, 0.0, -8.8381), (11.2622, 0.0, -6.3640), (3.6678, 0.0, -4.4475)),
]
_QMU = [600.0, 600.0, 600.0, 80.0, 143.0, 143.0, 143.0, 312.0, 312.0, 312.0, 0.0, 84.6]
_QKAPPA = [57827.0] * 11 + [1327.7]
# the anisotropic upper mantle (domains 3 and 4) of prem_ani: vpv, vph, vsv, vsh, eta
_ANI_UM = ((0.8317, 7.2180), (3.5908, 4.6172), (5.8582, -1.4678), (-1.0839, 5.7176), (3.3687, -2.4778))


def _poly(c, x):
    out = np.zeros_like(x)
    for k, a in enumerate(c):
        out = out + a * x ** k
    return out


def velocity(r, param: str, idom, model: str = "prem_iso"):
    """The value of `param` ('rho', 'vpv', 'vph', 'vsv', 'vsh', 'eta', 'v_p',
    'v_s', 'Qmu', 'Qka') at radii r (m) in domains idom (1-based), as
    velocity(r, param, idom, bkgrdmodel) returns it."""
    r = np.asarray(r, dtype=np.float64)
    idom = np.broadcast_to(np.asarray(idom), r.shape)
    x = (r / 1000.0) / 6371.0
    out = np.zeros_like(r)
    for d in np.unique(idom):
        sel = idom == d
        rho_c, vp_c, vs_c = _ISO[d - 1]
        xs = x[sel]
        vpv = vph = _poly(vp_c, xs)
        vsv = vsh = _poly(vs_c, xs)
        eta = np.ones_like(xs)
        if model == "prem_ani" and d in (3, 4):
            vpv, vph, vsv, vsh, eta = (_poly(c, xs) for c in _ANI_UM)
        elif model not in ("prem_iso", "prem_ani"):
            raise ValueError(f"unknown background model {model}")
        if param == "rho":
            v = _poly(rho_c, xs) * 1000.0
        elif param == "vpv":
            v = vpv * 1000.0
        elif param == "vph":
            v = vph * 1000.0
        elif param == "vsv":
            v = vsv * 1000.0
        elif param == "vsh":
            v = vsh * 1000.0
        elif param == "eta":
            v = eta
        elif param == "v_p":
            v = np.maximum(vpv, vph) * 1000.0
        elif param == "v_s":
            v = np.minimum(vsv, vsh) * 1000.0
        elif param == "Qmu":
            v = np.full_like(xs, _QMU[d - 1])
        elif param == "Qka":
            v = np.full_like(xs, _QKAPPA[d - 1])
        else:
            raise ValueError(f"unknown parameter {param}")
        out[sel] = v
    return out


def domain_of(r) -> np.ndarray:
    """Domain (1-based) of radii r (m): idom with discont(idom) > r >
    discont(idom+1), the inner core below the last discontinuity
    (SOLVER/get_model.F90:117-133)."""
    r = np.asarray(r, dtype=np.float64)
    d = DISCONTINUITIES_KM * 1000.0
    idom = np.full(r.shape, NDISC, dtype=np.int64)
    for k in range(NDISC - 1, 0, -1):
        idom = np.where(r > d[k], k, idom)
    return idom


def exact_mass(r_out: float = R_EARTH, model: str = "prem_iso", r_in: float = 0.0, dr: float = 100.0):
    """Mass of the model between r_in and r_out, summed over shells of dr
    metres as compute_mass_earth does (SOLVER/def_precomp_terms.f90:1020-1047),
    split into total, solid (v_s >= 0.1 m/s), fluid and inner core."""
    n = int((r_out - r_in) / dr) + 1
    k = np.arange(1, n + 1, dtype=np.float64)
    r = r_out - (k - 0.5) * dr
    keep = r > r_in
    r, k = r[keep], k[keep]
    vol = (r_out - (k - 1.0) * dr) ** 3 - np.maximum(r_out - k * dr, r_in) ** 3
    idom = domain_of(r)
    rho = velocity(r, "rho", idom, model)
    vs = velocity(r, "v_s", idom, model)
    f = 4.0 / 3.0 * np.pi
    fluid = vs < 0.1
    return {"total": f * float(np.sum(rho * vol)), "solid": f * float(np.sum((rho * vol)[~fluid])),
            "fluid": f * float(np.sum((rho * vol)[fluid])),
            "inner_core": f * float(np.sum((rho * vol)[idom == NDISC]))}
