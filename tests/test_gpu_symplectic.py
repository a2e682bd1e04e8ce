"""GPU parity of the symplectic time schemes (symplectic_time_loop,
SOLVER/time_evol_wave.F90:516-742) against the oracle on the same meshes.
Tolerance as for the Newmark loop: relative L2 <= 1e-4."""
import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import add_attenuation, coupled_mesh, gauss_at
from axisem_gb300.solver import AxgError, Solver, symplectic_coefficients

pytestmark = pytest.mark.gpu

TOL = 1e-4


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


def _stf_stages(m, scheme):
    _, _, coeff = symplectic_coefficients(scheme, m.deltat)
    return gauss_at(np.arange(m.niter)[:, None] * m.deltat + coeff[None, :], 20 * m.deltat)


@pytest.mark.parametrize("pole", [0, 1, 2])
@pytest.mark.parametrize("scheme", [_abi.SCHEME_SYMPLEC4, _abi.SCHEME_ML_SO4M5, _abi.SCHEME_ML_SO6M7])
@pytest.mark.parametrize("variant", ["plain", "absorbing"])
def test_symplectic_parity(gpu_lib, orc, pole, scheme, variant):
    m = coupled_mesh(10, 5, 4, pole, niter=30, absorbing=variant == "absorbing")
    stf = _stf_stages(m, scheme)
    with Solver(m) as s:
        s.set_time_scheme(scheme, stf)
        s.run(1, m.niter)
        rec = s.receivers()
        disp = s.get_state(_abi.FIELD_DISP)
        chi = s.get_state(_abi.FIELD_CHI)
    t32, t64 = orc.TimeLoop(m, np.float32), orc.TimeLoop(m, np.float64)
    assert t32.run_symplectic(1, m.niter, scheme, stf) == 0 and t64.run_symplectic(1, m.niter, scheme, stf) == 0
    assert np.abs(t64.receivers()).max() > 0
    assert rel(rec, t32.receivers()) < TOL and rel(rec, t64.receivers()) < TOL
    c = [0, 2] if pole == 0 else [0, 1, 2]
    assert rel(disp[..., c], t64.disp[..., c]) < TOL
    assert rel(chi, t64.chi) < TOL
    # and it is not the Newmark loop
    tn = orc.TimeLoop(m, np.float64)
    assert tn.run(1, m.niter) == 0 and rel(tn.disp[..., c], t64.disp[..., c]) > 10 * TOL


def test_symplectic_near_axis_and_in_pieces(gpu_lib, orc):
    m = coupled_mesh(4, 6, 3, 1, niter=40)
    stf = _stf_stages(m, _abi.SCHEME_SYMPLEC4)
    with Solver(m) as s:
        s.set_time_scheme(_abi.SCHEME_SYMPLEC4, stf)
        s.set_tuning(steps_per_graph=8)
        s.run(1, 40)
        a = s.receivers()
        s.reset()
        s.run(1, 11)
        s.run(12, 29)
        assert np.array_equal(a, s.receivers())
    t = orc.TimeLoop(m, np.float64)
    assert t.run_symplectic(1, 40, _abi.SCHEME_SYMPLEC4, stf) == 0
    assert rel(a, t.receivers()) < TOL


@pytest.mark.parametrize("pole", [0, 1, 2])
@pytest.mark.parametrize("scheme", [_abi.SCHEME_SYMPLEC4, _abi.SCHEME_ML_SO4M5])
def test_symplectic_attenuation_parity(gpu_lib, orc, pole, scheme):
    """Every stage adds the anelastic stiffness of the previous step's memory
    variables; they are updated once per step after the final drift
    (SOLVER/time_evol_wave.F90:620-655, 727-731)."""
    m = add_attenuation(coupled_mesh(10, 5, 4, pole, niter=40))
    stf = _stf_stages(m, scheme)
    with Solver(m) as s:
        s.set_time_scheme(scheme, stf)
        s.run()
        rec = s.receivers()
        disp = s.get_state(_abi.FIELD_DISP)
        mv = s.get_state(_abi.FIELD_MEMVAR)
    t64 = orc.TimeLoop(m, np.float64)
    assert t64.run_symplectic(1, m.niter, scheme, stf) == 0
    comps = [0, 2] if pole == 0 else [0, 1, 2]
    mc = [0, 1, 2, 4] if pole == 0 else list(range(6))
    assert rel(rec, t64.receivers()) < TOL
    assert rel(disp[..., comps], t64.disp[..., comps]) < TOL
    assert np.abs(t64.memvar).max() > 0
    assert rel(mv[:, mc], t64.memvar[:, mc]) < TOL
    el = coupled_mesh(10, 5, 4, pole, niter=40)      # attenuation must matter at this tolerance
    te = orc.TimeLoop(el, np.float64)
    assert te.run_symplectic(1, el.niter, scheme, stf) == 0
    assert rel(te.disp[..., comps], t64.disp[..., comps]) > 10 * TOL


def test_symplectic_attenuation_in_pieces(gpu_lib):
    m = add_attenuation(coupled_mesh(10, 5, 4, 2, niter=36))
    stf = _stf_stages(m, _abi.SCHEME_SYMPLEC4)
    with Solver(m) as s:
        s.set_time_scheme(_abi.SCHEME_SYMPLEC4, stf)
        s.set_tuning(steps_per_graph=8)
        s.run()
        a, mva = s.receivers(), s.get_state(_abi.FIELD_MEMVAR)
        s.reset()
        s.run(1, 11)
        s.run(12, 25)
        assert np.array_equal(a, s.receivers())
        assert np.array_equal(mva, s.get_state(_abi.FIELD_MEMVAR))


def test_symplectic_unsupported_combinations(gpu_lib):
    cases = [coupled_mesh(6, 3, 3, 0, niter=10, fluid_src=True),
             coupled_mesh(6, 3, 2, 0, niter=10, free_surface=True)]
    for m in cases:
        with Solver(m) as s:
            with pytest.raises(AxgError) as ei:
                s.set_time_scheme(_abi.SCHEME_SYMPLEC4)
            assert ei.value.code == _abi.AXG_ERR_UNSUPPORTED
    with Solver(coupled_mesh(6, 3, 2, 0, niter=10)) as s:
        s.set_compensated(True)                   # compensated symplectic updates are supported
        s.set_time_scheme(_abi.SCHEME_SYMPLEC4)
        s.run()
        s.reset()
        s.set_compensated(False)
        s.run()
        s.set_time_scheme(_abi.SCHEME_NEWMARK2)   # and back
        s.run()
