"""Symplectic time-scheme coefficients (no GPU): the library's tables against
the oracle's independent restatement of symplectic_coefficients
(SOLVER/time_evol_wave.F90:749-992)."""
import numpy as np
import pytest

from axisem_gb300 import _abi
from axisem_gb300.solver import AxgError, symplectic_coefficients


@pytest.mark.parametrize("scheme,nstages", [(1, 4), (2, 5), (3, 7), (4, 17), (5, 35)])
def test_coefficients_equal_the_oracle(lib, orc, scheme, nstages):
    cd, cv, ce = symplectic_coefficients(scheme, 0.37, lib)
    ocd, ocv, oce = orc.symplectic_coefficients(scheme, 0.37)
    assert len(cv) == nstages and len(cd) == nstages + 1
    assert np.array_equal(cd, ocd) and np.array_equal(cv, ocv) and np.array_equal(ce, oce)
    assert abs(cv.sum() / 0.37 - 1.0) < 1e-6            # the kicks span one step
    assert np.allclose(cd, cd[::-1]) and np.allclose(cv, cv[::-1])   # symmetric compositions


def test_drift_sums_as_the_reference_computes_them(lib):
    """The three explicit schemes drift one step in total.  The two built by
    SS_scheme drift zero: the reference writes the middle drift as
    1 / 2 - sum(a(1:n)), and Fortran's integer 1 / 2 is 0; the library
    reproduces that."""
    for scheme in (1, 2, 3):
        assert abs(symplectic_coefficients(scheme, 1.0, lib)[0].sum() - 1.0) < 1e-6
    for scheme in (4, 5):
        assert abs(symplectic_coefficients(scheme, 1.0, lib)[0].sum()) < 1e-12


def test_unknown_scheme_is_refused(lib):
    with pytest.raises(AxgError) as ei:
        symplectic_coefficients(6, 1.0, lib)
    assert ei.value.code == _abi.AXG_ERR_BAD_ARG
