"""The C-ABI library on a machine without a GPU: it loads, exports every entry
point include/axisem_gb300.h declares, validates descriptors the way the
reference's setup stops on bad input, and its host-side planner (patches,
colours, sub-rounds) satisfies the invariants the atomic-free assembly needs."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import add_attenuation, coupled_mesh, structured_mesh

HEADER = Path(__file__).resolve().parents[1] / "include" / "axisem_gb300.h"


def declared_functions():
    txt = HEADER.read_text()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(axg_[a-z_]+)\s*\(", txt)))


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
        assert n in _abi.SIGNATURES, f"{n} missing from the Python mirror"


@pytest.mark.parametrize("name,mirror", [("axg_mesh_desc", _abi.MeshDesc), ("axg_dump_desc", _abi.DumpDesc),
                                         ("axg_info", _abi.Info)])
def test_header_struct_matches_mirror(name, mirror):
    # every field of the struct appears in the ctypes mirror, in order
    txt = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    body = txt[txt.index(f"typedef struct {name} {{"):txt.index(f"}} {name};")]
    fields = []
    for decl in body.split(";")[:-1]:
        decl = decl.split("{")[-1]
        for part in decl.split(","):
            nm = re.findall(r"\**\s*([A-Za-z_][A-Za-z0-9_]*)\s*(\[[^\]]*\])?\s*$", part.strip())
            if nm:
                fields.append(nm[0][0])
    assert fields == [f for f, _ in mirror._fields_]


def test_version_and_device_count(lib):
    assert b"sm_103a" in lib.axg_version()
    assert lib.axg_device_count() >= 0


def _create(lib, desc):
    h = C.c_void_p()
    rc = lib.axg_create(C.byref(desc), C.byref(h))
    return rc, lib.axg_last_error(None).decode(), h


@pytest.mark.parametrize("mutate,code,needle", [
    (lambda d: setattr(d, "npol", 3), _abi.AXG_ERR_BAD_DESC, "npol"),
    (lambda d: setattr(d, "abi_version", 99), _abi.AXG_ERR_BAD_DESC, "abi_version"),
    (lambda d: setattr(d, "src_type", 5), _abi.AXG_ERR_BAD_DESC, "src_type"),
    (lambda d: setattr(d, "nelsrc", 9), _abi.AXG_ERR_BAD_DESC, "nelsrc"),
    (lambda d: setattr(d, "seis_it", 0), _abi.AXG_ERR_BAD_DESC, "seis_it"),
    (lambda d: (setattr(d, "anel_true", 1), setattr(d, "att_coarse_grained", 2), setattr(d, "n_sls", 5)),
     _abi.AXG_ERR_BAD_DESC, "att_coarse_grained"),
    (lambda d: (setattr(d, "anel_true", 1), setattr(d, "att_coarse_grained", 0), setattr(d, "n_sls", 5)),
     _abi.AXG_ERR_BAD_DESC, "attenuation arrays"),
    (lambda d: (setattr(d, "anel_true", 1), setattr(d, "att_coarse_grained", 1)), _abi.AXG_ERR_UNSUPPORTED,
     "n_sls"),
    (lambda d: (setattr(d, "anel_true", 1), setattr(d, "att_coarse_grained", 1), setattr(d, "n_sls", 5)),
     _abi.AXG_ERR_BAD_DESC, "attenuation arrays"),
])
def test_descriptor_validation(lib, mutate, code, needle):
    m = coupled_mesh(6, 3, 2, 1, niter=10)
    d = m.desc()
    mutate(d)
    rc, msg, h = _create(lib, d)
    assert rc == code and needle in msg
    assert not h.value


def test_attenuation_descriptor_validation(lib):
    m = add_attenuation(coupled_mesh(6, 3, 2, 2, niter=10))
    d = m.desc()
    d.n_sls = 9
    rc, msg, h = _create(lib, d)
    assert rc == _abi.AXG_ERR_UNSUPPORTED and "n_sls" in msg and not h.value
    m.anel["Q_mu"] = m.anel["Q_mu"].copy()
    m.anel["Q_mu"][3] = 0.0
    rc, msg, h = _create(lib, m.desc())
    assert rc == _abi.AXG_ERR_BAD_DESC and "Q_mu" in msg and not h.value


def test_null_metric_array_rejected(lib):
    m = structured_mesh(4, 4, 2)
    d = m.desc()
    d.m_solid[_abi.SOLID_TERMS.index("M1phi")] = C.cast(None, C.POINTER(C.c_float))
    rc, msg, _ = _create(lib, d)
    assert rc == _abi.AXG_ERR_BAD_DESC and "NULL" in msg


def test_out_of_range_indices_rejected(lib):
    m = coupled_mesh(6, 3, 2, 0, niter=10)
    m.recfile_el = m.recfile_el.copy(order="F")
    m.recfile_el[0, 1] = 7
    rc, msg, _ = _create(lib, m.desc())
    assert rc == _abi.AXG_ERR_BAD_DESC and "recfile_el" in msg
    m = structured_mesh(4, 4, 0)
    m.igloc_solid = m.igloc_solid.copy()
    m.igloc_solid[3] = m.nglob_solid + 1
    inf = _abi.Info()
    rc = lib.axg_plan_check(C.byref(m.desc()), 64, -1, C.byref(inf))
    assert rc == _abi.AXG_ERR_BAD_DESC


def test_create_without_gpu_reports_no_device(lib):
    if lib.axg_device_count() > 0:
        pytest.skip("a GPU is present")
    rc, msg, h = _create(lib, structured_mesh(4, 4, 0).desc())
    assert rc == _abi.AXG_ERR_NO_DEVICE and not h.value


@pytest.mark.parametrize("growth", [0, 1, -1])
@pytest.mark.parametrize("ni,nj,pe", [(64, 48, 64), (33, 17, 64), (20, 20, 16), (7, 3, 5), (1, 1, 64),
                                      (50, 30, 48), (41, 23, 0)])
def test_plan_invariants(lib, ni, nj, pe, growth):
    m = structured_mesh(ni, nj, 2, axial="random1pct")
    inf = _abi.Info()
    rc = lib.axg_plan_check(C.byref(m.desc()), pe, growth, C.byref(inf))
    assert rc == 0, lib.axg_last_error(None)
    assert inf.n_colours_solid >= 1 and inf.max_subrounds_solid <= 12
    assert inf.patch_points_solid >= m.nglob_solid


def test_tuner_picks_square_patches_on_structured_grid(lib):
    """On a structured grid the tuner's cost model prefers layered growth with
    64-element (8 x 8) patches: four conflict-free sub-rounds of 16 elements,
    four colours, no fragments."""
    m = structured_mesh(64, 64, 2, axial="none")
    inf = _abi.Info()
    assert lib.axg_plan_check(C.byref(m.desc()), 0, -1, C.byref(inf)) == 0
    assert (inf.patch_elems_solid, inf.growth_solid) == (64, 1)
    assert (inf.n_patches_solid, inf.n_colours_solid, inf.max_subrounds_solid) == (64, 4, 4)
    # an explicit shape is kept
    assert lib.axg_plan_check(C.byref(m.desc()), 48, 0, C.byref(inf)) == 0
    assert (inf.patch_elems_solid, inf.growth_solid) == (48, 0)
    assert lib.axg_plan_check(C.byref(m.desc()), 65, -1, C.byref(inf)) == _abi.AXG_ERR_BAD_ARG
    assert lib.axg_plan_check(C.byref(m.desc()), 64, 2, C.byref(inf)) == _abi.AXG_ERR_BAD_ARG


def test_plan_on_permuted_numbering(lib):
    """Unstructured numbering: a random permutation of global ids and of the
    element order must still give a valid plan."""
    rng = np.random.default_rng(0)
    m = structured_mesh(24, 18, 1)
    perm = rng.permutation(m.nglob_solid) + 1
    ig = perm[m.igloc_solid - 1].astype(np.int32)
    eperm = rng.permutation(m.nel_solid)
    m.igloc_solid = ig.reshape(m.nel_solid, 25)[eperm].reshape(-1).copy()
    inf = _abi.Info()
    rc = lib.axg_plan_check(C.byref(m.desc()), 64, -1, C.byref(inf))
    assert rc == 0, lib.axg_last_error(None)


def test_plan_coupled(lib):
    m = coupled_mesh(40, 12, 9, 2)
    inf = _abi.Info()
    rc = lib.axg_plan_check(C.byref(m.desc()), 64, -1, C.byref(inf))
    assert rc == 0, lib.axg_last_error(None)
    assert inf.n_patches_fluid > 0


def test_tuner_spreads_small_meshes_over_the_gpu(lib):
    """A mesh of less than two rounds of 64-element patches per colour over
    the device's resident CTAs gets smaller patches (the colour latency
    model); a larger one keeps the full-launch choice.  The PREM 50 s mesh has
    5664 solid elements: about 20 patches of 64 per colour for 304 CTAs."""
    from axisem_gb300 import sphere
    m = sphere.build_mesh(50.0, sphere.SphereSolve(pole=0, seconds=100.0), skeleton=sphere.build_skeleton(50.0))
    inf = _abi.Info()
    assert lib.axg_plan_check_ctas(C.byref(m.desc()), 0, -1, 0, C.byref(inf)) == 0
    assert inf.patch_elems_solid == 64
    assert lib.axg_plan_check_ctas(C.byref(m.desc()), 0, -1, 304, C.byref(inf)) == 0
    assert inf.patch_elems_solid <= 16
    assert inf.n_patches_solid >= 4 * 94
    # an explicit shape is kept
    assert lib.axg_plan_check_ctas(C.byref(m.desc()), 64, 1, 304, C.byref(inf)) == 0
    assert inf.patch_elems_solid == 64
    big = structured_mesh(400, 400, 2, axial="none")
    assert lib.axg_plan_check_ctas(C.byref(big.desc()), 0, -1, 304, C.byref(inf)) == 0
    assert (inf.patch_elems_solid, inf.growth_solid) == (64, 1)
    assert lib.axg_plan_check_ctas(C.byref(m.desc()), 0, -1, -1, C.byref(inf)) == _abi.AXG_ERR_BAD_ARG
