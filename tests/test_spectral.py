"""Spectral matrices against the closed forms of the reference.

GLL nodes/weights for npol = 4 are the published values (0, +-sqrt(3/7), +-1;
32/45, 49/90, 1/10).  The axial GLJ(0,1) derivative matrix is checked entry
by entry against the reference's closed-form expressions of
lag_interp_deriv_wgl (MESHER/splib.f90:71-129), restated here, with m_N the
polynomial of vamnpo (MESHER/splib.f90:534-577).
"""
import numpy as np
from numpy.polynomial import polynomial as P

from axisem_gb300.spectral import Spectral, _m_poly


def test_gll_closed_form():
    s = Spectral()
    r = np.sqrt(3.0 / 7.0)
    np.testing.assert_allclose(s.eta, [-1, -r, 0, r, 1], atol=1e-15)
    np.testing.assert_allclose(s.wt, [1 / 10, 49 / 90, 32 / 45, 49 / 90, 1 / 10], rtol=1e-14)


def test_glj_axial_rule_exactness():
    """sum_j w_j x_j^k = int_{-1}^{1} (1+x) x^k dx for k <= 2N-1 (Lobatto-Jacobi(0,1))."""
    s = Spectral()
    for k in range(0, 8):
        exact = (1 - (-1) ** (k + 1)) / (k + 1) + (1 - (-1) ** (k + 2)) / (k + 2)
        assert abs(np.sum(s.wt_axial_k * s.xi_k ** k) - exact) < 1e-13


def test_g1_matches_reference_closed_forms():
    s = Spectral()
    N = 4
    xi = s.xi_k
    mn = P.polyval(xi, _m_poly(N))
    dl = np.zeros((5, 5))
    for i in range(5):
        for j in range(5):
            if i == 0:
                if j == 0:
                    v = -N * (N + 2) / 6.0
                elif j < N:
                    v = 2 * (-1) ** N * mn[j] / ((1 + xi[j]) * (N + 1))
                else:
                    v = (-1) ** N / (N + 1.0)
            elif i == N:
                if j == 0:
                    v = (-1) ** (N + 1) * (N + 1) / 4.0
                elif j < N:
                    v = -mn[j] / (1 - xi[j])
                else:
                    v = (N * (N + 2) - 1) / 4.0
            else:
                if j == 0:
                    v = (-1) ** (N + 1) * (N + 1) / (2 * mn[i] * (1 + xi[i]))
                elif j < N and j != i:
                    v = (1 / (xi[j] - xi[i])) * mn[j] / mn[i]
                elif j < N:
                    v = -0.5 / (1 + xi[j])
                else:
                    v = 1.0 / (mn[i] * (1 - xi[i]))
            dl[i, j] = v
    # G1(ishp, :) = dl for ishp (MESHER/gllmeshgen.f90:84-88)
    np.testing.assert_allclose(s.G1, dl, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(s.G0, dl[:, 0], rtol=1e-12)


def test_g2_differentiates_polynomials_exactly():
    s = Spectral()
    for k in range(5):
        f = s.eta ** k
        df = k * s.eta ** (k - 1) if k else np.zeros(5)
        # mxm_4(G2T, f): df/dxi at node i = sum_k G2(k, i) f(k)
        np.testing.assert_allclose(s.G2T @ f, df, atol=1e-12)
        np.testing.assert_allclose(s.G1T @ (s.xi_k ** k), k * s.xi_k ** (k - 1) if k else 0, atol=1e-12)
