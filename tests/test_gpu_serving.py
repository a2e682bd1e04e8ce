"""GPU tests of mesh sharing, asynchronous runs and the serving loop.

A solve's kernels depend only on its own data and run in a fixed order on its
stream, so sharing a mesh with other solves and overlapping with them on the
GPU must leave every result bit-for-bit what the solve gives alone.
"""
import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.mesh import coupled_mesh
from axisem_gb300.serve import Request, Server, solve_alone
from axisem_gb300.solver import AxgError, Solver

pytestmark = pytest.mark.gpu


def test_sharing_solve_equals_own_mesh(gpu_lib):
    base = coupled_mesh(16, 12, 4, 2, niter=40, num_rec=8)
    other = coupled_mesh(16, 12, 4, 2, niter=64, num_rec=5, src_row=6)   # same mesh, another source
    with Solver(base) as holder:
        with Solver(other, share_with=holder) as shared, Solver(other) as own:
            inf_s, inf_o = shared.info(), own.info()
            assert inf_s["mesh_bytes"] > 0 and inf_s["mesh_bytes"] == holder.info()["mesh_bytes"]
            assert inf_s["device_bytes"] - inf_s["mesh_bytes"] < inf_o["device_bytes"] / 2
            shared.run()
            own.run()
            assert np.array_equal(shared.receivers(), own.receivers())
            assert np.array_equal(shared.get_state(_abi.FIELD_DISP), own.get_state(_abi.FIELD_DISP))
        holder.run()  # the holder is untouched by the solves that shared its mesh
        with Solver(base) as again:
            again.run()
            assert np.array_equal(holder.receivers(), again.receivers())


def test_sharing_checks_the_mesh(gpu_lib):
    with Solver(coupled_mesh(16, 12, 4, 1, niter=10)) as holder:
        with pytest.raises(AxgError) as ei:
            Solver(coupled_mesh(16, 10, 4, 1, niter=10), share_with=holder)
        assert ei.value.code == _abi.AXG_ERR_BAD_DESC
        with pytest.raises(AxgError):
            Solver(coupled_mesh(16, 12, 4, 2, niter=10), share_with=holder)   # another pole type


def test_mesh_outlives_its_creator(gpu_lib):
    m = coupled_mesh(16, 12, 4, 0, niter=32)
    holder = Solver(m)
    shared = Solver(m, share_with=holder)
    holder.close()
    shared.run()
    rec = shared.receivers()
    shared.close()
    with Solver(m) as own:
        own.run()
        assert np.array_equal(rec, own.receivers())


def test_async_runs_overlap_and_match(gpu_lib):
    meshes = [coupled_mesh(16, 12, 4, p, niter=96, num_rec=6, src_row=r) for p, r in ((0, 3), (1, 5), (2, 7))]
    solvers = [Solver(m) for m in meshes]
    try:
        for s in solvers:
            s.run_async(1, 50)
        for s in solvers:
            s.wait()
        for s in solvers:
            s.run_async(51, 46)
        while not all(s.poll() for s in solvers):
            pass
        for m, s in zip(meshes, solvers):
            with Solver(m) as alone:
                alone.run()
                assert np.array_equal(s.receivers(), alone.receivers())
    finally:
        for s in solvers:
            s.close()


@pytest.mark.parametrize("tuning", ["shared", "alone"])
@pytest.mark.parametrize("batched", [False, True])
def test_served_results_equal_alone(gpu_lib, batched, tuning):
    reqs = [Request(k, 0.002 * k, period, pole, depth, nrec, dur, 0.03)
            for k, (period, pole, depth, nrec, dur) in enumerate(
                [(50, 0, 100, 20, 1800), (25, 2, 400, 60, 2400), (50, 1, 650, 30, 3600),
                 (50, 2, 10, 25, 2000), (25, 0, 300, 40, 1800), (50, 0, 500, 20, 2600)])]
    srv = Server(budget_bytes=8e9, chunk=32, tuning=tuning)
    try:
        stats = srv.run(reqs, batched=batched)
    finally:
        srv.close()
    assert len(stats.results) == len(reqs)
    assert stats.max_concurrent > 1
    for r in reqs:
        assert np.array_equal(stats.results[r.rid].seismograms, solve_alone(r, tuning=tuning)), r


@pytest.mark.parametrize("batched", [False, True])
def test_admission_keeps_to_the_budget(gpu_lib, batched):
    reqs = [Request(k, 0.0, 50, k % 3, 200, 20, 1800, 0.03) for k in range(6)]
    srv = Server(budget_bytes=1, chunk=32)   # nothing fits: one solve at a time
    try:
        stats = srv.run(reqs, batched=batched)
    finally:
        srv.close()
    assert len(stats.results) == 6 and stats.max_concurrent == 1
