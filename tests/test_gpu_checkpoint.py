"""Seismogram checkpoints (check_it of the reference, niter / 20 steps:
SOLVER/parameters.F90:932, SOLVER/time_evol_wave.F90:1142-1146).

Every check_it steps the samples recorded so far are copied into the
caller's buffer while the run continues; after a run the buffer holds every
sample up to the last multiple of check_it, equal to axg_get_receivers and to
the oracle's seismograms."""
import numpy as np
import pytest

from axisem_gb300.mesh import coupled_mesh
from axisem_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pole", [0, 1])
def test_checkpoints_follow_the_run(gpu_lib, orc, pole):
    m = coupled_mesh(12, 6, 4, pole, niter=100, seis_it=2, num_rec=5)
    check_it = m.niter // 20
    nseismo = m.niter // m.seis_it + 1
    torch = pytest.importorskip("torch")
    buf = torch.zeros((nseismo * 3 * m.num_rec,), dtype=torch.float32, pin_memory=True).numpy()
    out = buf.reshape((nseismo, 3, m.num_rec), order="F")
    with Solver(m) as s:
        s.set_tuning(steps_per_graph=8)
        s.set_seismogram_checkpoint(check_it, out)
        s.run(1, 37)
        n1 = s.checkpoint_samples()
        assert n1 == 35 // m.seis_it + 1
        rec = s.receivers()
        assert np.array_equal(out[:n1], rec[:n1])
        assert not out[n1:].any()
        s.run(38, 63)
        assert s.checkpoint_samples() == nseismo
        assert np.array_equal(out, s.receivers())
        s.reset()   # a reset restarts them
        assert s.checkpoint_samples() == 0
    t = orc.TimeLoop(m, np.float64)
    assert t.run(1, m.niter) == 0
    ref = t.receivers()
    assert np.linalg.norm(out - ref) / np.linalg.norm(ref) < 1e-4
