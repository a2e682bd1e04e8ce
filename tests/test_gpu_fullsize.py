"""GPU parity on the configurations the benchmark times, at full size.

* Stiffness + assembly on the benchmark's exact mesh: 1024 x 1024 structured
  quads (2^20 elements, 16 785 409 global points, 1 % axial elements, seed
  20261203) with the benchmark's displacement (seed 20261204), every pole
  type, against the FP64 oracle: relative L2 <= 1e-5
  (SOLVER/stiffness_*_4, SOLVER/commun.F90:69-171).
* Newmark steps on the benchmark's coupled time-loop mesh: 1024 x 768 solid
  over 1024 x 256 fluid elements, quadrupole, 200 receivers, 64 steps, elastic
  and with cg4 attenuation (5 SLS), against the FP64 oracle
  (SOLVER/time_evol_wave.F90:264-502): relative L2 <= 1e-4 for the
  displacement, velocity and chi fields and the seismograms.  The elastic run
  is the benchmark's own configuration (source on the second lattice row); the
  attenuated one moves the source next to the receivers, so that 64 steps
  reach them and the seismograms are compared too.

The oracle's element loops run on all host threads (their arithmetic, and
so the result, does not depend on the thread count).
"""
import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import add_attenuation, coupled_mesh, random_gvec, structured_mesh
from axisem_gb300.solver import Solver

pytestmark = pytest.mark.gpu

BENCH_SIZE = 1024
BENCH_SEED, BENCH_FIELD_SEED = 20261203, 20261204


def rel(a, b):
    return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("pole", [0, 1, 2])
def test_bench_mesh_stiffness_parity(gpu_lib, orc, pole):
    m = structured_mesh(BENCH_SIZE, BENCH_SIZE, pole, terms="pole", seed=BENCH_SEED)
    u = random_gvec(m, seed=BENCH_FIELD_SEED)
    with Solver(m) as s:
        f = s.stiffness_assembled(u)
    ref = orc.stiffness_assembled(m, u, np.float64)
    assert np.isfinite(f).all()
    assert rel(f, ref) <= 1e-5


def _bench_timeloop_mesh(anel: bool):
    n = BENCH_SIZE
    nj_s = 3 * n // 4
    m = coupled_mesh(n, nj_s, n // 4, 2, niter=64, seed=5, num_rec=200, seis_it=4, deltat=2e-6,
                     terms="pole", src_row=nj_s - 2 if anel else 1)
    if anel:
        m = add_attenuation(m, n_sls=5, seed=77)
    return m


@pytest.mark.parametrize("anel", [False, True], ids=["elastic", "cg4_attenuation"])
def test_bench_timeloop_parity(gpu_lib, orc, anel):
    m = _bench_timeloop_mesh(anel)
    with Solver(m) as s:
        s.run()
        rec = s.receivers()
        disp = s.get_state(_abi.FIELD_DISP)
        velo = s.get_state(_abi.FIELD_VELO)
        chi = s.get_state(_abi.FIELD_CHI)
        memvar = s.get_state(_abi.FIELD_MEMVAR) if anel else None
    t = orc.TimeLoop(m, np.float64)
    assert t.run(1, m.niter) == 0
    assert np.abs(t.disp).max() > 0
    if not anel:  # the source sits next to the fluid, which 64 steps reach
        assert np.abs(t.chi).max() > 0
    assert rel(disp, t.disp) <= 1e-4
    assert rel(velo, t.velo) <= 1e-4
    assert rel(chi, t.chi) <= 1e-4
    if anel:
        assert np.abs(t.receivers()).max() > 0
        assert rel(rec, t.receivers()) <= 1e-4
        assert rel(memvar, t.memvar) <= 1e-4
