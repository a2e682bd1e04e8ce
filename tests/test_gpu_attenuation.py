"""GPU parity of the coarse-grained (cg4) attenuation in the time loop.

The CUDA path (anelastic stiffness + memory-variable step fused into the solid
patch kernel) against the oracle's time_loop with anel_true, on the same
seeded meshes.  Tolerances as for the elastic time loop: relative L2 <= 1e-4
for seismograms, wavefields and memory variables (the GPU rounds the FP64
coefficient products ts_fac * a_j once to FP32, uses fused multiply-adds and
sums element contributions in patch order).  Every case also checks that
attenuation changes the displacement field by at least ten times that
tolerance, so a missing anelastic term cannot pass.
"""
import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import add_attenuation, coupled_mesh
from axisem_gb300.solver import AxgError, Solver

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def _mesh(pole, n_sls=5, do_corr_lowq=True, niter=50, shape=(10, 5, 4), **kw):
    m = coupled_mesh(*shape, pole, niter=niter, **kw)
    return add_attenuation(m, n_sls=n_sls, do_corr_lowq=do_corr_lowq)


def _memvar_comps(pole):
    # the monopole never writes components 4 and 6 (SOLVER/attenuation.f90:185)
    return [0, 1, 2, 4] if pole == 0 else list(range(6))


@pytest.mark.parametrize("pole", [0, 1, 2])
@pytest.mark.parametrize("variant", ["plain", "near_axis", "near_axis_no_axial", "no_lowq_corr", "sls3",
                                     "absorbing"])
def test_attenuation_time_loop_parity(gpu_lib, orc, pole, variant):
    kw, nsls, corr = {}, 5, True
    if variant.startswith("near_axis"):
        # a mesh four elements wide: the source sits one element from the
        # axial column, whose elements then carry most of the wavefield
        kw["shape"] = (4, 6, 3)
    if variant == "near_axis_no_axial":
        kw["axial_column"] = False
    if variant == "no_lowq_corr":
        corr = False
    if variant == "sls3":
        nsls = 3
    if variant == "absorbing":
        kw["absorbing"] = True
    m = _mesh(pole, n_sls=nsls, do_corr_lowq=corr, **kw)
    with Solver(m) as s:
        s.run(1, m.niter)
        rec = s.receivers()
        disp = s.get_state(_abi.FIELD_DISP)
        memvar = s.get_state(_abi.FIELD_MEMVAR)
        src_tr = s.get_state(_abi.FIELD_ATT_SRC_TR)
        src_dev = s.get_state(_abi.FIELD_ATT_SRC_DEV)
    t32 = orc.TimeLoop(m, np.float32)
    t64 = orc.TimeLoop(m, np.float64)
    assert t32.run(1, m.niter) == 0 and t64.run(1, m.niter) == 0
    assert rel(rec, t32.receivers()) < TOL
    assert rel(rec, t64.receivers()) < TOL
    comps = [0, 2] if pole == 0 else [0, 1, 2]
    assert rel(disp[..., comps], t64.disp[..., comps]) < TOL
    mc = _memvar_comps(pole)
    assert np.abs(t64.memvar).max() > 0
    assert rel(memvar[:, mc], t64.memvar[:, mc]) < TOL
    assert rel(src_tr, t64.src_tr_tm1) < TOL
    assert rel(src_dev[:, mc], t64.src_dev_tm1[:, mc]) < TOL
    if pole == 0:
        assert not memvar[:, [3, 5]].any() and not src_dev[:, [3, 5]].any()
    # attenuation must matter at this tolerance
    shape = kw.pop("shape", (10, 5, 4))
    el = coupled_mesh(*shape, pole, niter=m.niter, **kw)
    te = orc.TimeLoop(el, np.float64)
    assert te.run(1, el.niter) == 0
    assert rel(te.disp[..., comps], t64.disp[..., comps]) > 10 * TOL


def test_attenuation_run_in_pieces_equals_one_run(gpu_lib):
    m = _mesh(2, niter=60)
    with Solver(m) as s:
        s.set_tuning(steps_per_graph=8)
        s.run(1, 60)
        a = s.receivers()
        mv = s.get_state(_abi.FIELD_MEMVAR)
        s.reset()
        assert not s.get_state(_abi.FIELD_MEMVAR).any()
        s.run(1, 13)
        s.run(14, 30)
        s.run(44, 17)
        b = s.receivers()
        mv2 = s.get_state(_abi.FIELD_MEMVAR)
    assert np.array_equal(a, b)
    assert np.array_equal(mv, mv2)


def test_attenuation_state_round_trip_and_restart(gpu_lib, orc):
    """Continue from an oracle state (wavefields, memory variables and the
    previous step's attenuation sources) set through the ABI."""
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


def test_attenuation_fields_need_anel_handle(gpu_lib):
    m = coupled_mesh(6, 3, 2, 0, niter=10)
    with Solver(m) as s:
        with pytest.raises(AxgError) as ei:
            s.get_state(_abi.FIELD_MEMVAR)
        assert ei.value.code == _abi.AXG_ERR_BAD_ARG
