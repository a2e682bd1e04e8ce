"""GPU tests of the measured steps-per-graph tuner (axg_autotune): it picks
one of the timed graph sizes and leaves the solve's state as it was, so a run
interrupted by tuning equals an untouched run bit for bit."""
import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import add_attenuation, coupled_mesh
from axisem_gb300.solver import Solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", ["plain", "compensated", "anel"])
def test_autotune_leaves_the_solve_untouched(gpu_lib, mode):
    m = coupled_mesh(16, 12, 4, 2, niter=80, num_rec=6)
    if mode == "anel":
        m = add_attenuation(m)
    with Solver(m) as a, Solver(m) as b:
        for s in (a, b):
            s.set_compensated(mode == "compensated")
        a.run(1, 30)
        k = a.autotune()
        assert k in (2, 4, 8, 16, 32, 64) and a.info()["steps_per_graph"] == k
        a.run(31, 50)
        b.run()
        assert np.array_equal(a.receivers(), b.receivers())
        for f in (_abi.FIELD_DISP, _abi.FIELD_VELO, _abi.FIELD_CHI):
            assert np.array_equal(a.get_state(f), b.get_state(f))
        if mode == "anel":
            assert np.array_equal(a.get_state(_abi.FIELD_MEMVAR), b.get_state(_abi.FIELD_MEMVAR))


def test_autotune_without_room_keeps_the_setting(gpu_lib):
    with Solver(coupled_mesh(6, 3, 2, 0, niter=1)) as s:   # no graph of 2 steps fits
        s.set_tuning(steps_per_graph=8)
        assert s.autotune() == 8
