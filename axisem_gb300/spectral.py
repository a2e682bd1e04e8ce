"""GLL / GLJ(0,1) points, weights and Lagrange-derivative matrices for npol = 4.

These are the spectral matrices the reference mesher writes into the mesh
database (G0, G1, G1T, G2, G2T; MESHER/gllmeshgen.f90:60-92).  They are
recomputed here from the mathematics so that synthetic meshes can be built
without the mesher:

* eta, wt   : Gauss-Lobatto-Legendre nodes and weights
              (MESHER/splib.f90 zelegl / get_welegl: w_j = 2 / (N (N+1) P_N(x_j)^2)).
* xi_k, wt_axial_k : the axial Gauss-Lobatto-Jacobi(0,1) nodes of Azaiez,
              Bernardi, Dauge & Maday (eigenvalues of the symmetric tridiagonal
              matrix of MESHER/splib.f90 zemngl2) and weights
              w_j = 4 / (N (N+2) m_N(x_j)^2), doubled at x_0 = -1, with
              m_N = (P_N + P_{N+1}) / (1 + x) (get_welegl_axial iflag = 2, vamnpo).
* G2(i, q) = l_i'(eta_q) on the GLL nodes, G1(i, q) = lbar_i'(xi_q) on the axial
  nodes (hn_jprime, lag_interp_deriv_wgl), G0 = G1(:, 0).

Derivatives of the Lagrange basis are evaluated with the barycentric formula,
which gives the same values as the reference's closed forms up to rounding.
"""
from __future__ import annotations

import numpy as np
from numpy.polynomial import legendre as L
from numpy.polynomial import polynomial as P

NPOL = 4


def gll_points(n: int = NPOL) -> np.ndarray:
    """Nodes of the GLL rule: -1, 1 and the roots of P_n'."""
    dp = L.legder(np.eye(n + 1)[n])
    inner = np.sort(L.legroots(dp).real)
    return np.concatenate([[-1.0], inner, [1.0]])


def gll_weights(x: np.ndarray, n: int = NPOL) -> np.ndarray:
    pn = L.legval(x, np.eye(n + 1)[n])
    return 2.0 / (n * (n + 1) * pn ** 2)


def glj_axial_points(n: int = NPOL) -> np.ndarray:
    """Axial GLJ(0,1) nodes: -1, 1 and the eigenvalues of the tridiagonal
    matrix with d_i = 3 / (4 (i+1/2)(i+3/2)), e_{i+1} = sqrt(i(i+3)) / (2 (i+3/2))."""
    i = np.arange(1, n, dtype=np.float64)
    d = 3.0 / (4.0 * (i + 0.5) * (i + 1.5))
    e = np.sqrt(i[:-1] * (i[:-1] + 3.0)) / (2.0 * (i[:-1] + 1.5))
    t = np.diag(d) + np.diag(e, 1) + np.diag(e, -1)
    inner = np.sort(np.linalg.eigvalsh(t))
    return np.concatenate([[-1.0], inner, [1.0]])


def _m_poly(n: int) -> np.ndarray:
    """Power-basis coefficients of m_n = (P_n + P_{n+1}) / (1 + x)."""
    num = L.leg2poly(np.eye(n + 2)[n] + np.eye(n + 2)[n + 1])
    q, r = P.polydiv(num, np.array([1.0, 1.0]))
    assert np.allclose(r, 0.0, atol=1e-12)
    return q


def glj_axial_weights(x: np.ndarray, n: int = NPOL) -> np.ndarray:
    m = P.polyval(x, _m_poly(n))
    w = 4.0 / (n * (n + 2)) / (m * m)
    w[0] *= 2.0
    return w


def lagrange_derivative(nodes: np.ndarray) -> np.ndarray:
    """D[i, q] = l_i'(x_q) for the Lagrange basis on `nodes`."""
    n = len(nodes)
    w = np.array([1.0 / np.prod([nodes[j] - nodes[k] for k in range(n) if k != j])
                  for j in range(n)])
    D = np.zeros((n, n))
    for q in range(n):
        for i in range(n):
            if i != q:
                D[i, q] = (w[i] / w[q]) / (nodes[q] - nodes[i])
        D[q, q] = -np.sum(D[np.arange(n) != q, q])
    return D


class Spectral:
    """The spectral matrices of one npol = 4 element family (FP64 and FP32)."""

    def __init__(self, n: int = NPOL):
        self.eta = gll_points(n)
        self.wt = gll_weights(self.eta, n)
        self.xi_k = glj_axial_points(n)
        self.wt_axial_k = glj_axial_weights(self.xi_k, n)
        self.G2 = lagrange_derivative(self.eta)
        self.G2T = self.G2.T.copy()
        self.G1 = lagrange_derivative(self.xi_k)
        self.G1T = self.G1.T.copy()
        self.G0 = self.G1[:, 0].copy()

    def f32(self, name: str) -> np.ndarray:
        """FP32 Fortran-ordered copy of a matrix (what the mesh database holds)."""
        return np.asfortranarray(getattr(self, name).astype(np.float32))
