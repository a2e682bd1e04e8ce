"""ctypes mirror of include/axisem_gb300.h and the loader of the CUDA library.

The library is built in-tree (``axisem_gb300/_build/libaxisem_gb300.so``) by
``axisem_gb300.build``.  Loading fails loudly when it is missing: there is no
CPU fallback for the time loop.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "_build" / "libaxisem_gb300.so"

ABI_VERSION = 3
NPOL = 4

# status codes (enum axg_status)
AXG_OK = 0
AXG_ERR_BAD_DESC = 1
AXG_ERR_OOM = 2
AXG_ERR_CUDA = 3
AXG_ERR_BLOWUP = 4
AXG_ERR_TIMEOUT = 5
AXG_ERR_NO_DEVICE = 6
AXG_ERR_BAD_ARG = 7
AXG_ERR_UNSUPPORTED = 8

MONOPOLE, DIPOLE, QUADPOLE = 0, 1, 2
POLE_NAMES = {"monopole": MONOPOLE, "dipole": DIPOLE, "quadpole": QUADPOLE}

SOLID_TERMS = [
    "M_1", "M_2", "M_3", "M_4", "M_5", "M_6", "M_7", "M_8",
    "M_w1", "M_w2", "M_w3", "M_w4", "M_w5",
    "M11s", "M21s", "M41s", "M12s", "M22s", "M32s", "M42s",
    "M11z", "M21z", "M41z",
    "M13s", "M33s", "M43s",
    "M1phi", "M2phi", "M4phi",
]
AXIAL_TERMS = [f"M0_w{k}" for k in range(1, 11)]
FLUID_TERMS = ["M1chi_fl", "M2chi_fl", "M4chi_fl", "M_w_fl"]

# which solid arrays each pole type reads (SOLVER/stiffness_*_4)
_MONO = ["M_1", "M_2", "M_3", "M_4", "M_w1", "M11s", "M21s", "M41s", "M12s", "M22s",
         "M32s", "M42s", "M11z", "M21z", "M41z"]
SOLID_TERMS_USED = {
    MONOPOLE: _MONO,
    DIPOLE: _MONO + ["M_5", "M_6", "M_7", "M_8", "M_w2", "M_w3", "M13s", "M33s", "M43s"],
    QUADPOLE: _MONO + ["M_5", "M_6", "M_7", "M_8", "M_w2", "M_w3", "M_w4", "M_w5",
                       "M1phi", "M2phi", "M4phi"],
}
AXIAL_TERMS_USED = {
    MONOPOLE: ["M0_w1", "M0_w2", "M0_w3"],
    DIPOLE: ["M0_w1", "M0_w2", "M0_w3", "M0_w4", "M0_w6", "M0_w7", "M0_w8", "M0_w9", "M0_w10"],
    QUADPOLE: ["M0_w1", "M0_w2", "M0_w3", "M0_w4", "M0_w5", "M0_w6"],
}

(SCHEME_NEWMARK2, SCHEME_SYMPLEC4, SCHEME_ML_SO4M5, SCHEME_ML_SO6M7, SCHEME_KL_O8M17,
 SCHEME_SS_35O10) = range(6)
(FIELD_DISP, FIELD_VELO, FIELD_ACC0, FIELD_CHI, FIELD_DCHI, FIELD_DDCHI0, FIELD_MEMVAR, FIELD_ATT_SRC_TR,
 FIELD_ATT_SRC_DEV, FIELD_DISP_COMP, FIELD_VELO_COMP, FIELD_CHI_COMP, FIELD_DCHI_COMP) = range(13)
# enum axg_dump_type (dump_type of the reference's inparam_advanced)
DUMP_NONE, DUMP_DISPL_ONLY, DUMP_STRAIN_ONLY, DUMP_DISPL_VELO, DUMP_FULLFIELDS = range(5)

_fp = C.POINTER(C.c_float)
_ip = C.POINTER(C.c_int32)
_dp = C.POINTER(C.c_double)


class MeshDesc(C.Structure):
    """struct axg_mesh_desc"""

    _fields_ = [
        ("abi_version", C.c_int32), ("npol", C.c_int32), ("src_type", C.c_int32),
        ("fluid_src", C.c_int32),
        ("nel_solid", C.c_int32), ("nel_fluid", C.c_int32),
        ("nglob_solid", C.c_int32), ("nglob_fluid", C.c_int32),
        ("naxel_solid", C.c_int32), ("naxel_fluid", C.c_int32),
        ("nel_bdry", C.c_int32), ("nelsrc", C.c_int32),
        ("niter", C.c_int32), ("seis_it", C.c_int32), ("num_rec", C.c_int32),
        ("have_absorbing_bc", C.c_int32),
        ("deltat", C.c_double), ("magnitude", C.c_double),
        ("igloc_solid", _ip), ("igloc_fluid", _ip),
        ("ax_el_solid", _ip), ("ax_el_fluid", _ip),
        ("G0", _fp), ("G1", _fp), ("G1T", _fp), ("G2", _fp), ("G2T", _fp),
        ("m_solid", _fp * len(SOLID_TERMS)),
        ("m0_solid", _fp * len(AXIAL_TERMS)),
        ("m_fluid", _fp * len(FLUID_TERMS)),
        ("m0_w_fl", _fp),
        ("inv_mass_rho", _fp), ("inv_mass_fluid", _fp), ("fluid_free_surface_mask", _fp),
        ("solid_absorbing_gamma", _fp), ("fluid_absorbing_gamma", _fp),
        ("bdry_matr", _fp),
        ("bdry_solid_el", _ip), ("bdry_fluid_el", _ip),
        ("bdry_jpol_solid", _ip), ("bdry_jpol_fluid", _ip),
        ("ielsrc", _ip), ("source_term_el", _fp), ("source_term_fl", _fp), ("stf", _fp),
        ("recfile_el", _ip),
        ("anel_true", C.c_int32), ("n_sls", C.c_int32), ("do_corr_lowq", C.c_int32),
        ("att_coarse_grained", C.c_int32),
        ("y_j_attenuation", _dp), ("exp_w_j_deltat", _dp),
        ("ts_fac_t", _dp), ("ts_fac_tm1", _dp),
        ("Q_mu", _fp), ("Q_kappa", _fp),
        ("delta_mu_cg4", _fp), ("delta_kappa_cg4", _fp),
        ("Y_cg4", _fp), ("V_s_eta_cg4", _fp), ("V_s_xi_cg4", _fp), ("V_z_eta_cg4", _fp),
        ("V_z_xi_cg4", _fp),
        ("DsDeta_over_J_sol_cg4", _fp), ("DzDeta_over_J_sol_cg4", _fp),
        ("DsDxi_over_J_sol_cg4", _fp), ("DzDxi_over_J_sol_cg4", _fp),
        ("inv_s_solid", _fp),
        ("inv_mass_rho_dp", _dp), ("inv_mass_fluid_dp", _dp), ("source_term_el_dp", _dp),
        ("delta_mu", _fp), ("delta_kappa", _fp),
        ("Y", _fp), ("V_s_eta", _fp), ("V_s_xi", _fp), ("V_z_eta", _fp), ("V_z_xi", _fp),
        ("Y0", _fp), ("V0_s_eta", _fp), ("V0_s_xi", _fp), ("V0_z_eta", _fp), ("V0_z_xi", _fp),
        ("DsDeta_over_J_sol", _fp), ("DzDeta_over_J_sol", _fp),
        ("DsDxi_over_J_sol", _fp), ("DzDxi_over_J_sol", _fp),
    ]


class DumpDesc(C.Structure):
    """struct axg_dump_desc"""

    _fields_ = [
        ("dump_type", C.c_int32), ("strain_it", C.c_int32),
        ("ibeg", C.c_int32), ("iend", C.c_int32), ("jbeg", C.c_int32), ("jend", C.c_int32),
        ("DsDeta_over_J_sol", _fp), ("DzDeta_over_J_sol", _fp), ("DsDxi_over_J_sol", _fp),
        ("DzDxi_over_J_sol", _fp), ("inv_s_solid", _fp),
        ("DsDeta_over_J_flu", _fp), ("DzDeta_over_J_flu", _fp), ("DsDxi_over_J_flu", _fp),
        ("DzDxi_over_J_flu", _fp), ("inv_s_fluid", _fp), ("inv_rho_fluid", _fp),
        ("out", _fp), ("capacity", C.c_int64),
        ("kwf_mask", _ip), ("mapping_ijel_ikwf", _ip), ("npoint_solid_kwf", C.c_int32),
        ("npoint_fluid_kwf", C.c_int32),
        ("src_dump_mask", C.c_int32),
    ]


class Info(C.Structure):
    """struct axg_info"""

    _fields_ = [
        ("n_patches_solid", C.c_int64), ("n_patches_fluid", C.c_int64),
        ("n_colours_solid", C.c_int32), ("n_colours_fluid", C.c_int32),
        ("max_subrounds_solid", C.c_int32), ("max_subrounds_fluid", C.c_int32),
        ("device_bytes", C.c_int64),
        ("kernels_per_step", C.c_int64),
        ("kernels_per_force", C.c_int64),
        ("patch_points_solid", C.c_int64),
        ("patch_elems_solid", C.c_int32), ("growth_solid", C.c_int32),
        ("patch_elems_fluid", C.c_int32), ("growth_fluid", C.c_int32),
        ("ctas_per_sm_force", C.c_int32), ("ctas_per_sm_step", C.c_int32),
        ("mesh_bytes", C.c_int64), ("steps_per_graph", C.c_int32),
    ]


def ptr(a: np.ndarray | None, ctype):
    """Pointer to a contiguous numpy array (or NULL)."""
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    assert a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"], "array must be contiguous"
    return a.ctypes.data_as(C.POINTER(ctype))


# the exported C-ABI: name -> (restype, argtypes)
SIGNATURES = {
    "axg_version": (C.c_char_p, []),
    "axg_device_count": (C.c_int, []),
    "axg_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(C.c_void_p)]),
    "axg_create_tuned": (C.c_int, [C.POINTER(MeshDesc), C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "axg_set_compensated": (C.c_int, [C.c_void_p, C.c_int32]),
    "axg_create_sharing": (C.c_int, [C.c_void_p, C.POINTER(MeshDesc), C.POINTER(C.c_void_p)]),
    "axg_symplectic_coefficients": (C.c_int, [C.c_int32, C.c_double, C.POINTER(C.c_double),
                                              C.POINTER(C.c_double), C.POINTER(C.c_double),
                                              C.POINTER(C.c_int32)]),
    "axg_set_time_scheme": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float)]),
    "axg_run_async": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "axg_poll": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "axg_wait": (C.c_int, [C.c_void_p]),
    "axg_autotune": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "axg_set_wavefield_dump": (C.c_int, [C.c_void_p, C.POINTER(DumpDesc)]),
    "axg_wavefield_dump_layout": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                            C.POINTER(C.c_int64), C.c_char_p, C.c_int32]),
    "axg_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_int32, C.POINTER(C.c_void_p)]),
    "axg_batch_run_async": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.c_int32]),
    "axg_batch_poll": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "axg_batch_wait": (C.c_int, [C.c_void_p]),
    "axg_batch_launches_per_step": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "axg_batch_destroy": (None, [C.c_void_p]),
    "axg_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "axg_reset": (C.c_int, [C.c_void_p]),
    "axg_run": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "axg_get_receivers": (C.c_int, [C.c_void_p, _fp, C.c_int32, _ip]),
    "axg_get_state": (C.c_int, [C.c_void_p, C.c_int32, _fp]),
    "axg_set_state": (C.c_int, [C.c_void_p, C.c_int32, _fp]),
    "axg_stiffness_assembled": (C.c_int, [C.c_void_p, _fp, _fp]),
    "axg_stiffness_assembled_device": (C.c_int, [C.c_void_p, C.c_void_p]),
    "axg_stiffness_assembled_noalloc": (C.c_int, [C.POINTER(MeshDesc), _fp, _fp]),
    "axg_upload_gvec_disp": (C.c_int, [C.c_void_p, _fp]),
    "axg_download_gvec_force": (C.c_int, [C.c_void_p, _fp]),
    "axg_set_tuning": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    "axg_get_info": (C.c_int, [C.c_void_p, C.POINTER(Info)]),
    "axg_get_solid_colouring": (C.c_int, [C.c_void_p, _ip, _ip, C.c_int64]),
    "axg_plan_check": (C.c_int, [C.POINTER(MeshDesc), C.c_int32, C.c_int32, C.POINTER(Info)]),
    "axg_plan_check_ctas": (C.c_int, [C.POINTER(MeshDesc), C.c_int32, C.c_int32, C.c_int32, C.POINTER(Info)]),
    "axg_time_stiffness": (C.c_int, [C.c_void_p, C.c_int32, _fp]),
    "axg_device_check_report": (C.c_int, [_ip]),
    "axg_selftest_wait_timeout": (C.c_int, [_ip, C.POINTER(C.c_double)]),
    "axg_set_seismogram_checkpoint": (C.c_int, [C.c_void_p, C.c_int32, _fp, C.c_int32]),
    "axg_seismogram_checkpoint_samples": (C.c_int, [C.c_void_p, _ip]),
    "axg_destroy": (None, [C.c_void_p]),
    "axg_last_error": (C.c_char_p, [C.c_void_p]),
}

_lib = None


def load_library(path: str | os.PathLike | None = None):
    """Load libaxisem_gb300.so (raising if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    if path is None and os.environ.get("AXG_LIBRARY"):
        path = os.environ["AXG_LIBRARY"]  # e.g. a build with device bounds checks
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"CUDA library {p} is missing; build it with "
            "`python -c 'import axisem_gb300.build as b; b.build()'` (there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib
