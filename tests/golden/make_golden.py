"""Generates tests/golden/oracle_golden.npz: outputs of the FP64 oracle on small
seeded meshes (stiffness + assembly for each pole type; a coupled solid-fluid
Newmark run for each pole type).  The reference itself cannot be compiled here
(no Fortran compiler), so these fixtures pin the oracle restatement against
regressions; the oracle is pinned to the reference through the known-answer
tests in tests/test_oracle.py and tests/test_spectral.py.

    python tests/golden/make_golden.py
"""
from pathlib import Path
import sys

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from axisem_gb300.mesh import coupled_mesh, random_gvec, structured_mesh  # noqa: E402


def make_cases(orc):
    out = {}
    for pole in (0, 1, 2):
        m = structured_mesh(5, 4, pole, seed=11 + pole)
        m.ax_el_solid = np.array([1, 6, 13], dtype=np.int32)
        u = random_gvec(m, seed=21 + pole)
        out[f"force_p{pole}"] = orc.stiffness_assembled(m, u, np.float64)
        cm = coupled_mesh(6, 3, 2, pole, niter=24, seed=31 + pole)
        t = orc.TimeLoop(cm, np.float64)
        assert t.run(1, cm.niter) == 0
        out[f"seis_p{pole}"] = t.receivers().copy()
        out[f"chi_p{pole}"] = t.chi.copy()
    return out


if __name__ == "__main__":
    from oracle import oracle as orc

    orc.build()
    cases = make_cases(orc)
    np.savez_compressed(Path(__file__).resolve().parent / "oracle_golden.npz", **cases)
    print({k: v.shape for k, v in cases.items()})
