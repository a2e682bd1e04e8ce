"""GPU tests of the compensated (Kahan) time integration (axg_set_compensated).

The mode has no counterpart in the reference: the predictor and the velocity
corrector use compensated FP32 summation, so that the rounding of many small
increments does not accumulate.  Checked here:
  * parity: over a short run it matches the FP64 oracle as closely as the
    plain FP32 path does (relative L2 <= 1e-4);
  * what it is for: from a nonzero state with a tiny time step (4000 steps of
    2e-9 s, each increment ~1e-6 of the field), the plain FP32 path drifts
    from the FP64 oracle by ~5e-6 (displacement) and ~1e-5 (chi); the
    compensated path must stay at least 3x closer;
  * the compensation terms are state: they round-trip through
    axg_get_state / axg_set_state, a run in pieces equals one run bit for
    bit, and axg_reset zeroes them.
"""
import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import add_attenuation, coupled_mesh, gvec_to_elemental
from axisem_gb300.mesh import gauss_at
from axisem_gb300.solver import AxgError, Solver, symplectic_coefficients

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def _comps(pole):
    return [0, 2] if pole == 0 else [0, 1, 2]


@pytest.mark.parametrize("pole", [0, 1, 2])
@pytest.mark.parametrize("anel", [False, True])
def test_compensated_parity(gpu_lib, orc, pole, anel):
    m = coupled_mesh(10, 5, 4, pole, niter=50)
    if anel:
        m = add_attenuation(m)
    with Solver(m) as s:
        s.set_compensated(True)
        s.run(1, m.niter)
        rec = s.receivers()
        disp = s.get_state(_abi.FIELD_DISP)
        chi = s.get_state(_abi.FIELD_CHI)
    t64 = orc.TimeLoop(m, np.float64)
    assert t64.run(1, m.niter) == 0
    assert rel(rec, t64.receivers()) < 1e-4
    c = _comps(pole)
    assert rel(disp[..., c], t64.disp[..., c]) < 1e-4
    assert rel(chi, t64.chi) < 1e-4


def _drift_case(pole, niter=4000, dt=2e-9):
    m = coupled_mesh(8, 4, 3, pole, niter=niter, deltat=dt, seis_it=10)
    rng = np.random.default_rng(3)
    u0 = rng.uniform(0.5, 1.5, (m.nglob_solid, 3)).astype(np.float32) * 1e-6
    v0 = rng.normal(0, 1, (m.nglob_solid, 3)).astype(np.float32) * 1e-3
    c0 = rng.uniform(0.5, 1.5, m.nglob_fluid).astype(np.float32) * 1e-6
    d0 = rng.normal(0, 1, m.nglob_fluid).astype(np.float32) * 1e-3
    if pole == 0:
        u0[:, 1] = 0
        v0[:, 1] = 0
    init = {_abi.FIELD_DISP: gvec_to_elemental(m, u0), _abi.FIELD_VELO: gvec_to_elemental(m, v0),
            _abi.FIELD_CHI: gvec_to_elemental(m, c0, fluid=True),
            _abi.FIELD_DCHI: gvec_to_elemental(m, d0, fluid=True)}
    return m, init


@pytest.mark.parametrize("pole", [0, 1, 2])
def test_compensated_reduces_accumulated_rounding(gpu_lib, orc, pole):
    m, init = _drift_case(pole)
    t64 = orc.TimeLoop(m, np.float64)
    t64.disp[...] = init[_abi.FIELD_DISP]
    t64.velo[...] = init[_abi.FIELD_VELO]
    t64.chi[...] = init[_abi.FIELD_CHI]
    t64.dchi[...] = init[_abi.FIELD_DCHI]
    assert t64.run(1, m.niter) == 0
    err = {}
    for comp in (False, True):
        with Solver(m) as s:
            s.set_compensated(comp)
            for f, a in init.items():
                s.set_state(f, a)
            s.run(1, m.niter)
            c = _comps(pole)
            err[comp] = (rel(s.get_state(_abi.FIELD_DISP)[..., c], t64.disp[..., c]),
                         rel(s.get_state(_abi.FIELD_CHI), t64.chi))
    print(f"pole {pole}: plain disp {err[False][0]:.2e} chi {err[False][1]:.2e}; "
          f"compensated disp {err[True][0]:.2e} chi {err[True][1]:.2e}")
    assert err[False][0] > 1e-6  # the case does exercise accumulated rounding
    assert err[True][0] < err[False][0] / 3
    assert err[True][1] < err[False][1] / 3


def test_compensation_is_state(gpu_lib):
    m, init = _drift_case(2, niter=120, dt=2e-8)
    with Solver(m) as s:
        s.set_compensated(True)
        s.set_tuning(steps_per_graph=8)
        for f, a in init.items():
            s.set_state(f, a)
        s.run(1, 120)
        a = s.get_state(_abi.FIELD_DISP)
        cu = s.get_state(_abi.FIELD_DISP_COMP)
        assert np.abs(cu).max() > 0
        s.reset()
        assert not s.get_state(_abi.FIELD_DISP_COMP).any() and not s.get_state(_abi.FIELD_DCHI_COMP).any()
        for f, arr in init.items():
            s.set_state(f, arr)
        s.run(1, 50)
        mid = {f: s.get_state(f) for f in (_abi.FIELD_DISP, _abi.FIELD_VELO, _abi.FIELD_ACC0, _abi.FIELD_CHI,
                                           _abi.FIELD_DCHI, _abi.FIELD_DDCHI0, _abi.FIELD_DISP_COMP,
                                           _abi.FIELD_VELO_COMP, _abi.FIELD_CHI_COMP, _abi.FIELD_DCHI_COMP)}
        s.run(51, 70)
        b = s.get_state(_abi.FIELD_DISP)
        # restart from the saved state, compensation included
        s.reset()
        for f, arr in mid.items():
            s.set_state(f, arr)
            assert np.array_equal(s.get_state(f), arr)
        s.run(51, 70)
        c = s.get_state(_abi.FIELD_DISP)
    assert np.array_equal(a, b)
    assert np.array_equal(a, c)


def test_compensation_fields_need_the_mode(gpu_lib):
    m = coupled_mesh(6, 3, 2, 0, niter=10)
    with Solver(m) as s:
        with pytest.raises(AxgError) as ei:
            s.get_state(_abi.FIELD_DISP_COMP)
        assert ei.value.code == _abi.AXG_ERR_BAD_ARG


def _stf_stages(m, scheme):
    _, _, coeff = symplectic_coefficients(scheme, m.deltat)
    return gauss_at(np.arange(m.niter)[:, None] * m.deltat + coeff[None, :], 20 * m.deltat)


@pytest.mark.parametrize("pole", [0, 1, 2])
def test_compensated_symplectic_parity(gpu_lib, orc, pole):
    """Compensated drifts and kicks of symplec4 against the FP64 oracle."""
    m = coupled_mesh(10, 5, 4, pole, niter=40)
    stf = _stf_stages(m, _abi.SCHEME_SYMPLEC4)
    with Solver(m) as s:
        s.set_compensated(True)
        s.set_time_scheme(_abi.SCHEME_SYMPLEC4, stf)
        s.run()
        rec, disp, chi = s.receivers(), s.get_state(_abi.FIELD_DISP), s.get_state(_abi.FIELD_CHI)
    t64 = orc.TimeLoop(m, np.float64)
    assert t64.run_symplectic(1, m.niter, _abi.SCHEME_SYMPLEC4, stf) == 0
    c = _comps(pole)
    assert rel(rec, t64.receivers()) < 1e-4
    assert rel(disp[..., c], t64.disp[..., c]) < 1e-4
    assert rel(chi, t64.chi) < 1e-4


@pytest.mark.parametrize("pole", [0, 2])
def test_compensated_symplectic_reduces_accumulated_rounding(gpu_lib, orc, pole):
    m, init = _drift_case(pole, niter=2000)
    stf = _stf_stages(m, _abi.SCHEME_SYMPLEC4)
    t64 = orc.TimeLoop(m, np.float64)
    t64.disp[...] = init[_abi.FIELD_DISP]
    t64.velo[...] = init[_abi.FIELD_VELO]
    t64.chi[...] = init[_abi.FIELD_CHI]
    t64.dchi[...] = init[_abi.FIELD_DCHI]
    assert t64.run_symplectic(1, m.niter, _abi.SCHEME_SYMPLEC4, stf) == 0
    err = {}
    for comp in (False, True):
        with Solver(m) as s:
            s.set_compensated(comp)
            s.set_time_scheme(_abi.SCHEME_SYMPLEC4, stf)
            for f, a in init.items():
                if f in (_abi.FIELD_DISP, _abi.FIELD_VELO, _abi.FIELD_CHI, _abi.FIELD_DCHI):
                    s.set_state(f, a)
            s.run(1, m.niter)
            c = _comps(pole)
            err[comp] = (rel(s.get_state(_abi.FIELD_DISP)[..., c], t64.disp[..., c]),
                         rel(s.get_state(_abi.FIELD_CHI), t64.chi))
    print(f"symplec4 pole {pole}: plain disp {err[False][0]:.2e} chi {err[False][1]:.2e}; "
          f"compensated disp {err[True][0]:.2e} chi {err[True][1]:.2e}")
    assert err[True][0] < err[False][0] / 3
    assert err[True][1] < err[False][1] / 3


def test_compensated_symplectic_in_pieces(gpu_lib):
    m, init = _drift_case(1, niter=60, dt=2e-8)
    stf = _stf_stages(m, _abi.SCHEME_ML_SO4M5)
    with Solver(m) as s:
        s.set_compensated(True)
        s.set_time_scheme(_abi.SCHEME_ML_SO4M5, stf)
        s.set_tuning(steps_per_graph=8)
        for f, a in init.items():
            s.set_state(f, a)
        s.run(1, 60)
        a = s.get_state(_abi.FIELD_DISP)
        assert np.abs(s.get_state(_abi.FIELD_VELO_COMP)).max() > 0
        s.reset()
        for f, arr in init.items():
            s.set_state(f, arr)
        s.run(1, 17)
        s.run(18, 43)
        assert np.array_equal(a, s.get_state(_abi.FIELD_DISP))
