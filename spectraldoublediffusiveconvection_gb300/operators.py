"""Host-side FP64 assembly of the radial operators (set-up, not timed).

These are the reference's formulas, evaluated with numpy so that the pre-inverted blocks are the same
matrices the reference inverts:

* ``cheb_radial``        Matrix_Operators.py:10-28
* ``Nabla2`` / ``Nabla4`` Matrix_Operators.py:31-76
* A4 pieces (D2, A2, IR2, IR4)                    Main.py:209-214 / Matrix_Operators.py:1093-1101
* Linv blocks of A4_TSTEP_MATS / NAB2_TSTEP_MATS  Matrix_Operators.py:1089-1112 / 1014-1030
* DT0 = A_T/r^2                                    Main.py:23-38, 201-202
* R2 / kGR_RT diagonals (r^2, R_1^2/r^2)           Matrix_Operators.py:79-128
"""
import numpy as np


def cheb_radial(N, d):
    """Gauss-Lobatto Chebyshev differentiation matrix D and points R on [1/d, (1+d)/d]
    (Matrix_Operators.py:10-28)."""
    r_i = 1.0 / d
    r_o = (1.0 + d) / d
    if N == 0:
        return 0.0, 1.0
    n = np.arange(0, N + 1)
    x = np.cos(np.pi * n / N).reshape(N + 1, 1)
    x = 0.5 * (r_i + r_o) + 0.5 * (r_i - r_o) * x
    c = (np.hstack(([2.0], np.ones(N - 1), [2.0])) * (-1) ** n).reshape(N + 1, 1)
    X = np.tile(x, (1, N + 1))
    dX = X - X.T
    D = np.dot(c, 1.0 / c.T) / (dX + np.eye(N + 1))
    D -= np.diag(np.sum(D.T, axis=0))
    return D, x.reshape(N + 1)


def Nabla2(D, r):
    """r^2 d2/dr2 + 2 r d/dr without the boundary rows/columns (Matrix_Operators.py:31-45)."""
    D2 = np.diag(r[:] ** 2) @ (D @ D)
    RD = np.diag(2.0 * r[:]) @ D
    return (D2 + RD)[1:-1, 1:-1]


def Nabla4(D, r):
    """Clamped fourth-derivative operator (Matrix_Operators.py:48-76)."""
    I = np.ones(len(r))
    r_i, r_o = r[0], r[-1]
    b = -(r_i + r_o)
    c = r_i * r_o
    with np.errstate(divide="ignore"):
        S = np.diag(1.0 / ((r ** 2) + b * r + c * I))
    S[0, 0] = 0.0
    S[-1, -1] = 0.0
    D2 = D @ D
    D3 = D @ D2
    D4 = D2 @ D2
    L4 = np.diag(r ** 2 + b * r + c * I) @ D4 + 4.0 * np.diag(2.0 * r + b * I) @ D3 + 12.0 * D2
    return (L4 @ S)[1:-1, 1:-1]


def a4_pieces(D, R):
    """(D2, A2, IR2, IR4) of the psi operator (Main.py:209-214, Matrix_Operators.py:1093-1101)."""
    IR = np.diag(1.0 / R)
    IR2 = IR @ IR
    D_sq = D @ D
    D2 = (IR2 @ (2 * D_sq - 4 * (IR @ D) + 6 * IR2))[1:-1, 1:-1]
    A2 = D_sq[1:-1, 1:-1]
    IR2 = IR2[1:-1, 1:-1]
    IR4 = IR2 @ IR2
    return D2, A2, IR2, IR4


def a4_tstep_mats(dt, N_fm, nr, D, R):
    """Inverses of (A2 + b_j IR2) - dt(D4 + b_j(D2 + b_j IR4)), j = N_fm - jj
    (Matrix_Operators.py:1089-1112)."""
    D4 = Nabla4(D, R)
    D2, A2, IR2, IR4 = a4_pieces(D, R)
    out = np.empty((N_fm, nr, nr))
    for jj in range(N_fm):
        j = N_fm - jj
        bj = -j * (j + 1)
        L1 = D2 + bj * IR4
        out[jj] = np.linalg.inv((A2 + bj * IR2) - dt * (D4 + bj * L1))
    return out


def nab2_tstep_mats(dt, N_fm, nr, D, R):
    """Inverses of r^2 - dt(r^2 Lap_r + b_j I), j = N_fm - 1 - jj (Matrix_Operators.py:1014-1030)."""
    I = np.eye(nr)
    R2 = np.diag(R[1:-1] ** 2)
    R2_Nab2 = Nabla2(D, R)
    out = np.empty((N_fm, nr, nr))
    for jj in range(N_fm):
        j = N_fm - (jj + 1)
        bj = -j * (j + 1)
        out[jj] = np.linalg.inv(R2 - dt * (R2_Nab2 + bj * I))
    return out


def base_state_coeffs(d):
    """A_T, B_T of T0 = -A_T/r + B_T (Main.py:23-38)."""
    R_1 = 1.0 / d
    R_2 = (1.0 + d) / d
    return (R_1 * R_2) / (R_1 - R_2), R_1 / (R_1 - R_2)


def theta_operators(D, R):
    """Operators of the theta recurrences and the nonlinear term (FP64, contiguous)."""
    Rin = R[1:-1]
    return dict(
        Dr=np.ascontiguousarray(D[1:-1, 1:-1]),
        D2_r2=np.ascontiguousarray((np.diag(1.0 / R ** 2) @ (D @ D))[1:-1, 1:-1]),   # A2_SINE_R2 :498
        ir4_r2=np.ascontiguousarray(1.0 / (Rin ** 4)),                              # :496
        D2_sine=np.ascontiguousarray((D @ D)[1:-1, 1:-1]),                          # A2_SINE :217
        ir2_sine=np.ascontiguousarray(1.0 / (Rin ** 2)),                            # :216
    )


def plan_arrays(N_fm, N_r, d, dt, Pr, Tau):
    """Every host array a plan needs for (N_fm, N_r, d, dt, Pr, Tau)."""
    D, R = cheb_radial(N_r, d)
    nr = N_r - 1
    ops = theta_operators(D, R)
    D2, _, IR2, IR4 = a4_pieces(D, R)
    A_T = base_state_coeffs(d)[0]
    ops.update(
        D=D, R=R,
        D2_A4=np.ascontiguousarray(D2),
        ir2_A4=np.ascontiguousarray(np.diag(IR2)),
        ir4_A4=np.ascontiguousarray(np.diag(IR4)),
        rsq=np.ascontiguousarray(R[1:-1] ** 2),
        dT0=np.ascontiguousarray(A_T / (R[1:-1] ** 2)),
        gr=np.ascontiguousarray(((1.0 / d) ** 2) / (R[1:-1] ** 2)),
        Linv_A4=a4_tstep_mats(Pr * dt, N_fm, nr, D, R),
        Linv_T=nab2_tstep_mats(dt, N_fm, nr, D, R),
        Linv_S=nab2_tstep_mats(Tau * dt, N_fm, nr, D, R),
        nu_w=np.ascontiguousarray((R[0] ** 2 / A_T) * D[0, 1:-1]),
        r_int=np.ascontiguousarray(R[1:-1]),
    )
    return ops
