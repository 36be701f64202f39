"""Drop-in for the reference's Linear_Matrix_Operators.py: the single-mode (Legendre degree l) operators of
the linear stability problem about the conductive state.  These are small dense matrices (3(N_r-1) square)
assembled on the host, as in the reference; the eigenproblem built from them seeds the nonlinear solves.

Operator formulas follow the reference line by line (cited per function); the radial grid of this module
runs from the outer to the inner radius (Linear_Matrix_Operators.py:44-60), the opposite orientation of
Matrix_Operators.cheb_radial."""
import numpy as np


def cheb_radial(N, d):
    """Linear_Matrix_Operators.py:44-60: Chebyshev points R from r_o = (1+d)/d down to r_i = 1/d and the
    differentiation matrix D."""
    r_i, r_o = 1.0 / d, (1.0 + d) / d
    if N == 0:
        return 0.0, 1.0
    n = np.arange(N + 1)
    x = 0.5 * (r_o + r_i) + 0.5 * (r_o - r_i) * np.cos(np.pi * n / N)
    c = np.hstack(([2.0], np.ones(N - 1), [2.0])) * (-1.0) ** n
    dX = x[:, None] - x[None, :]
    D = np.outer(c, 1.0 / c) / (dX + np.eye(N + 1))
    D -= np.diag(D.sum(axis=1))
    return D, x


def laplacian_SP(D, r, l):
    """Linear_Matrix_Operators.py:63-71: D^2 + (2/r) D - l(l+1)/r^2, interior rows/columns."""
    A = D @ D + np.diag(2.0 / r) @ D - l * (l + 1.0) * np.diag(1.0 / r ** 2)
    return A[1:-1, 1:-1]


def Stokes_D2_SP(D, r, l):
    """Linear_Matrix_Operators.py:74-82: D^2 - l(l+1)/r^2, interior."""
    A = D @ D - l * (l + 1.0) * np.diag(1.0 / r ** 2)
    return A[1:-1, 1:-1]


def Stokes_D2D2_SP(D, r, l):
    """Linear_Matrix_Operators.py:85-109: the clamped D^2 D^2 operator (the psi = (r - r_i)(r - r_o) v
    substitution of the fourth derivative, then the l terms), interior."""
    r_i, r_o = r[-1], r[0]
    b, c = -(r_i + r_o), r_i * r_o
    q = r ** 2 + b * r + c
    S = np.diag(np.where(np.arange(len(r)) % (len(r) - 1) == 0, 0.0, 1.0 / np.where(q == 0, 1.0, q)))
    D2 = D @ D
    D3 = D @ D2
    D4 = D2 @ D2
    L = np.diag(q) @ D4 + 4.0 * np.diag(2.0 * r + b) @ D3 + 12.0 * D2
    ll = l * (l + 1.0)
    A = (L @ S - 2.0 * ll * np.diag(1.0 / r ** 2) @ D2 + 4.0 * ll * np.diag(1.0 / r ** 3) @ D
         + (ll ** 2 - 6.0 * ll) * np.diag(1.0 / r ** 4))
    return A[1:-1, 1:-1]


def Bouyancy_Ra_SP(r, d):
    """Linear_Matrix_Operators.py:135-158: R_1^2 / r^2 (without Ra), interior."""
    return np.diag((1.0 / d) ** 2 / r ** 2)[1:-1, 1:-1]


def temp_SP(r, l, d):
    """Linear_Matrix_Operators.py:161-189: l(l+1)/r^2 * A_T/r^2 (the base temperature gradient), interior."""
    R_1, R_2 = 1.0 / d, (1.0 + d) / d
    A_T = (R_1 * R_2) / (R_1 - R_2)
    return np.diag(l * (l + 1.0) / r ** 2 * (A_T / r ** 2))[1:-1, 1:-1]


def ML_0(D, r, l):
    """Linear_Matrix_Operators.py:192-200: block diag(D^2 - l(l+1)/r^2, I, I)."""
    D2L = Stokes_D2_SP(D, r, l)
    n = D2L.shape[0]
    M = np.zeros((3 * n, 3 * n))
    M[:n, :n] = D2L
    M[n:, n:] = np.eye(2 * n)
    return M


def Ll_0(D, r, d, l, Ra, Ra_s, Pr, Tau):
    """Linear_Matrix_Operators.py:233-258: [[Pr D2D2, Pr Ra B, -Pr Ra_s B], [TT, Nabla, 0], [TT, 0, Tau Nabla]]
    (the coupling blocks vanish for l = 0)."""
    D2D2 = Pr * Stokes_D2D2_SP(D, r, l)
    B = Bouyancy_Ra_SP(r, d)
    NAB = laplacian_SP(D, r, l)
    n = D2D2.shape[0]
    L = np.zeros((3 * n, 3 * n))
    L[:n, :n] = D2D2
    L[n:2 * n, n:2 * n] = NAB
    L[2 * n:, 2 * n:] = Tau * NAB
    if l != 0:
        TT = temp_SP(r, l, d)
        L[:n, n:2 * n] = Pr * Ra * B
        L[:n, 2 * n:] = -Pr * Ra_s * B
        L[n:2 * n, :n] = TT
        L[2 * n:, :n] = TT
    return L
