"""Generates tests/golden/precision_long_run.npz: the seismograms of the
precision study's long run (axisem_gb300.sphere.long_run_mesh: 1e5 steps on
the prem_ani 50 s mesh, cg4 attenuation with 5 SLS, dipole Mrt source at
100 km depth, 10 surface receivers every 50 steps), computed by the oracle's
time loop (sf_time_loop_newmark, SOLVER/time_evol_wave.F90:264-502) in FP64
and in FP32, the precision of the reference's default build (realkind=4).

    python tests/golden/make_precision_reference.py      # about 30 min on 8 cores

The GPU test and the benchmark compare the GPU's plain and compensated runs
of the same mesh with these.
"""
from pathlib import Path
import sys
import time

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from axisem_gb300 import sphere  # noqa: E402
from oracle import oracle as orc  # noqa: E402

OUT = Path(__file__).resolve().parent / "precision_long_run.npz"
STEPS = 100_000


def main():
    m = sphere.long_run_mesh(STEPS)
    out = {"niter": np.int64(m.niter), "deltat": np.float64(m.deltat), "nel_solid": np.int64(m.nel_solid),
           "nel_fluid": np.int64(m.nel_fluid), "seis_it": np.int64(m.seis_it)}
    for dt in (np.float64, np.float32):
        t0 = time.time()
        t = orc.TimeLoop(m, dt)
        assert t.run(1, m.niter) == 0
        out[f"rec_{np.dtype(dt).name}"] = t.receivers().copy()
        print(f"{np.dtype(dt).name}: {time.time() - t0:.0f} s", flush=True)
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
