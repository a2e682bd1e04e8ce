"""Generates tests/golden/oracle_golden.npz: outputs of the FP64 oracle on small
seeded meshes, for each pole type: stiffness + assembly; a coupled solid-fluid
Newmark run; the same with cg4 attenuation; a symplec4 run with attenuation;
the fullfields wavefield dump of the Newmark run's final state.  The reference itself cannot be compiled here
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

from axisem_gb300 import _abi  # noqa: E402
from axisem_gb300.mesh import (add_attenuation, add_pointwise, coupled_mesh, dump_desc, gauss_at,  # noqa: E402
                               random_gvec, structured_mesh)


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
        pw = add_pointwise(cm, seed=41 + pole)
        full, _ = orc.wavefield_dump(pw, dump_desc(pw, _abi.DUMP_FULLFIELDS, 1, None, 1), t.disp, t.velo, t.chi,
                                     t.dchi, np.float64)
        out[f"dump_full_p{pole}"] = full
        am = add_attenuation(coupled_mesh(6, 3, 2, pole, niter=24, seed=51 + pole), seed=61 + pole)
        ta = orc.TimeLoop(am, np.float64)
        assert ta.run(1, am.niter) == 0
        out[f"anel_seis_p{pole}"] = ta.receivers().copy()
        out[f"anel_memvar_p{pole}"] = ta.memvar.copy()
        _, _, coeff = orc.symplectic_coefficients(_abi.SCHEME_SYMPLEC4, am.deltat)
        stf = gauss_at(np.arange(am.niter)[:, None] * am.deltat + np.asarray(coeff)[None, :], 20 * am.deltat)
        ts = orc.TimeLoop(am, np.float64)
        assert ts.run_symplectic(1, am.niter, _abi.SCHEME_SYMPLEC4, stf) == 0
        out[f"symp_anel_seis_p{pole}"] = ts.receivers().copy()
        out[f"symp_anel_memvar_p{pole}"] = ts.memvar.copy()
    return out


if __name__ == "__main__":
    from oracle import oracle as orc

    orc.build()
    cases = make_cases(orc)
    np.savez_compressed(Path(__file__).resolve().parent / "oracle_golden.npz", **cases)
    print({k: v.shape for k, v in cases.items()})
