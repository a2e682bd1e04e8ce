"""GPU parity of the attenuation at every GLL point (att_coarse_grained =
.false.: time_step_memvars_4 with compute_strain_att_el_4, and
glob_anel_stiffness_{mono,di,quad}_4) in the Newmark loop.

The CUDA path (anel_full_kernel: the memory variables from the displacement
each step stores, then the next step's anelastic force terms, which the solid
patch kernel adds) against the oracle's time loop on the same seeded meshes,
which have an axial column (L'Hospital's f/s on the axis, the axial Y0 / V0_*
vectors).  Tolerances as for the coarse-grained case: relative L2 <= 1e-4 for
seismograms, wavefields and memory variables; each case also checks that
the attenuation changes the displacement by at least ten times that.
"""
import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import add_attenuation, coupled_mesh
from axisem_gb300.solver import AxgError, Batch, Solver

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def _mesh(pole, n_sls=5, niter=40, shape=(8, 5, 3), seed=7, **kw):
    m = coupled_mesh(*shape, pole, niter=niter, **kw)
    return add_attenuation(m, n_sls=n_sls, seed=seed, coarse_grained=False)


def _memvar_comps(pole):
    return [0, 1, 2, 4] if pole == 0 else list(range(6))


@pytest.mark.parametrize("pole", [0, 1, 2])
@pytest.mark.parametrize("variant", ["plain", "near_axis", "sls3", "compensated"])
def test_full_attenuation_time_loop_parity(gpu_lib, orc, pole, variant):
    kw, nsls = {}, 5
    if variant == "near_axis":
        kw["shape"] = (4, 6, 3)
    if variant == "sls3":
        nsls = 3
    m = _mesh(pole, n_sls=nsls, **kw)
    with Solver(m) as s:
        s.set_compensated(variant == "compensated")
        s.run(1, m.niter)
        rec = s.receivers()
        disp = s.get_state(_abi.FIELD_DISP)
        memvar = s.get_state(_abi.FIELD_MEMVAR)
        src_tr = s.get_state(_abi.FIELD_ATT_SRC_TR)
        src_dev = s.get_state(_abi.FIELD_ATT_SRC_DEV)
    assert memvar.shape[0] == 25
    t32 = orc.TimeLoop(m, np.float32)
    t64 = orc.TimeLoop(m, np.float64)
    assert t32.run(1, m.niter) == 0 and t64.run(1, m.niter) == 0
    assert np.abs(t64.receivers()).max() > 0
    assert rel(rec, t32.receivers()) < TOL
    assert rel(rec, t64.receivers()) < TOL
    comps = [0, 2] if pole == 0 else [0, 1, 2]
    assert rel(disp[..., comps], t64.disp[..., comps]) < TOL
    mc = _memvar_comps(pole)
    assert np.abs(t64.memvar).max() > 0
    assert rel(memvar[:, mc], t64.memvar[:, mc]) < TOL
    assert rel(src_tr, t64.src_tr_tm1) < TOL
    assert rel(src_dev[:, mc], t64.src_dev_tm1[:, mc]) < TOL
    # the attenuation matters at this tolerance, and differs from the cg4 one
    shape = kw.pop("shape", (8, 5, 3))
    el = coupled_mesh(*shape, pole, niter=m.niter, **kw)
    te = orc.TimeLoop(el, np.float64)
    assert te.run(1, el.niter) == 0
    assert rel(te.disp[..., comps], t64.disp[..., comps]) > 10 * TOL


def test_full_attenuation_in_pieces_and_restart(gpu_lib, orc):
    """Runs in pieces equal one run; a run continued from an oracle state
    (wavefields, memory variables, previous sources) set through the ABI."""
    m = _mesh(2, niter=48)
    with Solver(m) as s:
        s.set_tuning(steps_per_graph=8)
        s.run(1, 48)
        a = s.receivers()
        s.reset()
        s.run(1, 13)
        s.run(14, 35)
        assert np.array_equal(a, s.receivers())
    m = _mesh(1, niter=40)
    t = orc.TimeLoop(m, np.float32)
    assert t.run(1, 20) == 0
    with Solver(m) as s:
        for fld, arr in ((_abi.FIELD_DISP, t.disp), (_abi.FIELD_VELO, t.velo), (_abi.FIELD_ACC0, t.acc0),
                         (_abi.FIELD_CHI, t.chi), (_abi.FIELD_DCHI, t.dchi), (_abi.FIELD_DDCHI0, t.ddchi0),
                         (_abi.FIELD_MEMVAR, t.memvar), (_abi.FIELD_ATT_SRC_TR, t.src_tr_tm1),
                         (_abi.FIELD_ATT_SRC_DEV, t.src_dev_tm1)):
            s.set_state(fld, arr)
            assert np.array_equal(s.get_state(fld), arr.astype(np.float32))
        s.run(21, 20)
        d = s.get_state(_abi.FIELD_DISP)
        mv = s.get_state(_abi.FIELD_MEMVAR)
    assert t.run(21, 20) == 0
    assert rel(d, t.disp) < TOL
    assert rel(mv, t.memvar) < TOL


def test_full_attenuation_runs_alone(gpu_lib):
    """Not in batches, not with a symplectic scheme (AXG_ERR_UNSUPPORTED)."""
    m = _mesh(0, niter=10)
    with Solver(m) as s, Solver(coupled_mesh(6, 3, 2, 0, niter=10)) as e:
        with pytest.raises(AxgError) as ei:
            Batch([s, e])
        assert ei.value.code == _abi.AXG_ERR_UNSUPPORTED
        with pytest.raises(AxgError) as ei:
            s.set_time_scheme(_abi.SCHEME_SYMPLEC4, np.zeros((m.niter, 4), np.float32))
        assert ei.value.code == _abi.AXG_ERR_UNSUPPORTED


def test_full_attenuation_on_the_prem_mesh(gpu_lib, orc):
    """The PREM 50 s mesh with memory variables at every GLL point
    (sphere.Attenuation(coarse_grained=False): the restated per-point
    precompute), dipole Mrt source: seismograms and memory variables against
    the FP64 and FP32 oracles over 800 steps (114 s: the P wave has reached
    the nearest receivers)."""
    from axisem_gb300 import sphere
    m = sphere.build_mesh(50.0, sphere.SphereSolve(pole=1, source="mtr", depth_km=100.0, seconds=120.0,
                                                   receivers_deg=np.linspace(5.0, 175.0, 10), seis_it=5),
                          skeleton=sphere.build_skeleton(50.0),
                          attenuation=sphere.Attenuation(coarse_grained=False), pointwise=False)
    n = min(800, m.niter)
    with Solver(m) as s:
        s.run(1, n)
        rec = s.receivers()
        disp = s.get_state(_abi.FIELD_DISP)
        memvar = s.get_state(_abi.FIELD_MEMVAR)
    t64 = orc.TimeLoop(m, np.float64)
    t32 = orc.TimeLoop(m, np.float32)
    assert t64.run(1, n) == 0 and t32.run(1, n) == 0
    assert np.abs(t64.receivers()).max() > 0 and np.abs(t64.memvar).max() > 0
    assert rel(rec, t64.receivers()) < TOL
    assert rel(rec, t32.receivers()) < TOL
    assert rel(disp, t64.disp) < TOL
    assert rel(memvar, t64.memvar) < TOL
