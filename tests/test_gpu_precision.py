"""The precision study on the GPU: 1e5 Newmark steps of an anelastic dipole
run (axisem_gb300.sphere.long_run_mesh: prem_ani at 50 s, cg4 attenuation
with 5 SLS, Mrt source at 100 km depth, 10 surface receivers), run plain
(FP32) and compensated (Kahan-compensated FP32 updates with the FP64 inverse
masses and source term), each compared per component with the FP64 oracle's
seismograms of the same mesh (tests/golden/precision_long_run.npz, made by
make_precision_reference.py).  The oracle's own FP32 run, the arithmetic of
the reference's default build, is reported beside them.

Bars: both GPU runs within relative L2 1e-4 of the FP64 oracle on every
component, and the compensated run closer to it than the plain run.
"""
from pathlib import Path

import numpy as np
import pytest

from axisem_gb300 import sphere
from axisem_gb300.solver import Solver

pytestmark = pytest.mark.gpu

FIXTURE = Path(__file__).resolve().parent / "golden" / "precision_long_run.npz"


def per_component(rec, ref):
    """relative L2 misfit of each component over all receivers and samples"""
    rec, ref = np.asarray(rec, np.float64), np.asarray(ref, np.float64)
    return [float(np.linalg.norm(rec[:, c] - ref[:, c]) / np.linalg.norm(ref[:, c])) for c in range(3)]


def long_run_misfits():
    """(misfits of the plain and compensated GPU runs and of the oracle's FP32
    run against the FP64 oracle, per component; GPU seconds of each run)"""
    import time
    fx = np.load(FIXTURE)
    m = sphere.long_run_mesh(int(fx["niter"]))
    assert (m.nel_solid, m.nel_fluid, m.seis_it) == (int(fx["nel_solid"]), int(fx["nel_fluid"]), int(fx["seis_it"]))
    # the mesh is rebuilt here: its FP64 precompute may differ from the
    # fixture's machine in the last bits of transcendental functions
    assert abs(m.deltat - float(fx["deltat"])) <= 1e-12 * m.deltat
    ref = fx["rec_float64"]
    out, secs = {}, {}
    for mode in ("plain", "compensated"):
        with Solver(m) as s:
            s.set_compensated(mode == "compensated")
            t0 = time.perf_counter()
            s.run()
            rec = s.receivers()
            secs[mode] = time.perf_counter() - t0
        out[mode] = per_component(rec, ref)
    out["oracle_fp32"] = per_component(fx["rec_float32"], ref)
    return out, secs


def test_long_run_precision(gpu_lib):
    mis, _ = long_run_misfits()
    print(mis)
    assert max(mis["plain"]) <= 1e-4
    assert max(mis["compensated"]) <= 1e-4
    assert max(mis["compensated"]) < max(mis["plain"])
