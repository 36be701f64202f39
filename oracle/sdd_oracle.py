"""CPU oracle: a numpy restatement of the reference's pseudospectral time-step and Newton path.

TEST INFRASTRUCTURE ONLY.  This module is the checker: ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it.  The product package never imports it.

It restates mannixp/SpectralDoubleDiffusiveConvection (``Transforms.py``, ``Matrix_Operators.py``,
``Main.py``) in vectorised numpy, with the same formulas and, where the reference accumulates
sequentially (parity suffix sums, back-substitution chains), the same accumulation order.  Every function
cites the reference lines it follows.  Parity with the reference itself is pinned by the golden vectors
in ``tests/golden`` (generated by running the reference; see ``tests/golden/make_golden.py``).

State layout (``Matrix_Operators.py:530-575``): X has length 3*N_fm*nr; block f in (psi, T, S) starts at
f*N_fm*nr, and inside a block mode k occupies [k*nr, (k+1)*nr) (radial index contiguous).
psi slot k holds the coefficient of sin((k+1)theta); T/S slot k holds cos(k theta).
"""
import numpy as np
import scipy.fft as sfft

# ---------------------------------------------------------------------------------------------------
# theta transforms  (Transforms.py:8-129)
# ---------------------------------------------------------------------------------------------------


def grid(N):
    """Transforms.py:8-13: midpoint grid theta_i = pi(2i+1)/(2N)."""
    return np.pi / N * (2.0 * np.arange(N) + 1.0) / 2.0


def IDCT(f_hat, n=None, axis=-1):
    """Transforms.py:116-129 (+ sinusoid_to_IDCT :16-26): f(theta_i) = a0 + sum_k a_k cos(k theta_i),
    evaluated on grid(n) (zero-padded when n > N)."""
    a = np.array(f_hat, dtype=float, copy=True)
    a = np.moveaxis(a, axis, -1)
    a[..., 1:] *= 0.5
    out = sfft.dct(a, type=3, n=n, axis=-1)
    return np.moveaxis(out, -1, axis)


def IDST(g_hat, n=None, axis=-1):
    """Transforms.py:87-100 (+ sinusoid_to_IDST :41-54): g(theta_i) = sum_{w=1}^{N-1} b_w sin(w theta_i);
    index = wavenumber, [0] ignored, the top (Nyquist) slot dropped."""
    b = np.array(g_hat, dtype=float, copy=True)
    b = np.moveaxis(b, axis, -1)
    b *= 0.5
    s = np.zeros_like(b)
    s[..., :-1] = b[..., 1:]
    out = sfft.dst(s, type=3, n=n, axis=-1)
    return np.moveaxis(out, -1, axis)


def DCT(f, n=None, axis=-1):
    """Transforms.py:102-114 (+ DCT_to_sinusoid :28-39): a_k = (2/N) sum_i f_i cos(k theta_i), a_0 halved;
    truncated to the first n outputs."""
    y = sfft.dct(np.moveaxis(np.asarray(f, dtype=float), axis, -1), type=2, axis=-1)
    N = y.shape[-1]
    y = y * (1.0 / N)
    y[..., 0] *= 0.5
    if n is not None:
        y = y[..., :n]
    return np.moveaxis(y, -1, axis)


def DST(g, n=None, axis=-1):
    """Transforms.py:73-85 (+ DST_to_sinusoid :56-70): b_w = (2/N) sum_i g_i sin(w theta_i) at index w,
    [0] = 0; truncated to the first n outputs."""
    y = sfft.dst(np.moveaxis(np.asarray(g, dtype=float), axis, -1), type=2, axis=-1)
    N = y.shape[-1]
    s = np.zeros_like(y)
    s[..., 1:] = y[..., :-1]
    s *= 1.0 / N
    if n is not None:
        s = s[..., :n]
    return np.moveaxis(s, -1, axis)


# ---------------------------------------------------------------------------------------------------
# radial operators  (Matrix_Operators.py:10-128)
# ---------------------------------------------------------------------------------------------------


def cheb_radial(N, d):
    """Matrix_Operators.py:10-28: Gauss-Lobatto Chebyshev differentiation matrix on [1/d, (1+d)/d]."""
    r_i = 1.0 / d
    r_o = (1.0 + d) / d
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
    """Matrix_Operators.py:31-45: r^2 d2/dr2 + 2r d/dr, Dirichlet rows/cols removed."""
    D2 = np.diag(r[:] ** 2) @ (D @ D)
    RD = np.diag(2.0 * r[:]) @ D
    return (D2 + RD)[1:-1, 1:-1]


def Nabla4(D, r):
    """Matrix_Operators.py:48-76: clamped fourth-derivative operator (interior)."""
    I = np.ones(len(r))
    r_i, r_o = r[0], r[-1]
    b = -(r_i + r_o)
    c = r_i * r_o
    with np.errstate(divide="ignore"):   # the reference sets np.seterr(divide='ignore') (:7)
        S = np.diag(1.0 / ((r ** 2) + b * r + c * I))
    S[0, 0] = 0.0
    S[-1, -1] = 0.0
    D2 = D @ D
    D3 = D @ D2
    D4 = D2 @ D2
    L4 = np.diag(r ** 2 + b * r + c * I) @ D4 + 4.0 * np.diag(2.0 * r + b * I) @ D3 + 12.0 * D2
    D4 = L4 @ S
    return D4[1:-1, 1:-1]


def base_state_AT(d):
    """Main.py:23-38: A_T of T0 = -A_T/r + B_T."""
    R_1 = 1.0 / d
    R_2 = (1.0 + d) / d
    return (R_1 * R_2) / (R_1 - R_2)


def NAB2_TSTEP_MATS(dt, N_fm, nr, D, R):
    """Matrix_Operators.py:1014-1030: inverses of r^2 - dt(r^2 Lap_r + b_j I), b_j=-j(j+1), j=N_fm-1-jj."""
    I = np.eye(nr)
    R2 = np.diag(R[1:-1] ** 2)
    R2_Nab2 = Nabla2(D, R)
    out = np.empty((N_fm, nr, nr))
    for jj in range(N_fm):
        j = N_fm - (jj + 1)
        bj = -j * (j + 1)
        out[jj] = np.linalg.inv(R2 - dt * (R2_Nab2 + bj * I))
    return out


def A4_operator_pieces(D, R):
    """Main.py:209-214 / Matrix_Operators.py:1093-1101: (D2_A4, A2, IR2, IR4) for the psi equation."""
    IR = np.diag(1.0 / R)
    IR2 = IR @ IR
    D_sq = D @ D
    D2 = (IR2 @ (2 * D_sq - 4 * (IR @ D) + 6 * IR2))[1:-1, 1:-1]
    A2 = D_sq[1:-1, 1:-1]
    IR2 = IR2[1:-1, 1:-1]
    IR4 = IR2 @ IR2
    return D2, A2, IR2, IR4


def A4_TSTEP_MATS(dt, N_fm, nr, D, R):
    """Matrix_Operators.py:1089-1112: inverses of (A2 + b_j IR2) - dt(D4 + b_j(D2 + b_j IR4)), j=N_fm-jj."""
    D4 = Nabla4(D, R)
    D2, A2, IR2, IR4 = A4_operator_pieces(D, R)
    out = np.empty((N_fm, nr, nr))
    for jj in range(N_fm):
        j = N_fm - jj
        bj = -j * (j + 1)
        L1 = D2 + bj * IR4
        L = (A2 + bj * IR2) - dt * (D4 + bj * L1)
        out[jj] = np.linalg.inv(L)
    return out


class Operators:
    """Main.py:179-225 (Build_Matrix_Operators) restated as a plain record.

    Attributes follow the reference's names; the sparse R2 / kGR_RT operators (Matrix_Operators.py:79-128)
    are kept as their diagonals ``rsq`` (r^2) and ``gr`` (R_1^2/r^2), applied mode-wise."""

    def __init__(self, N_fm, N_r, d, dt, Pr, Tau):
        self.N_fm, self.N_r, self.d, self.dt, self.Pr, self.Tau = N_fm, N_r, d, dt, Pr, Tau
        D, R = cheb_radial(N_r, d)
        self.D, self.R = D, R
        nr = N_r - 1
        self.nr = nr
        self.Dr = np.ascontiguousarray(D[1:-1, 1:-1])
        self.rsq = R[1:-1] ** 2                                   # R2, Matrix_Operators.py:85
        self.gr = ((1.0 / d) ** 2) / (R[1:-1] ** 2)               # kGR_RT GR, Matrix_Operators.py:113
        self.DT0 = base_state_AT(d) / (R[1:-1] ** 2)              # Main.py:201-202
        self.Linv_A4 = A4_TSTEP_MATS(Pr * dt, N_fm, nr, D, R)     # Main.py:205
        self.Linv_T = NAB2_TSTEP_MATS(dt, N_fm, nr, D, R)         # Main.py:206
        self.Linv_S = NAB2_TSTEP_MATS(Tau * dt, N_fm, nr, D, R)   # Main.py:207
        self.D2_A4, _, IR2, IR4 = A4_operator_pieces(D, R)        # Main.py:209-214
        self.IR2_A4 = np.diag(IR2).copy()
        self.IR4_A4 = np.diag(IR4).copy()
        # A2_SINE operators (Matrix_Operators.py:216-217) and A2_SINE_R2 (:496-498)
        self.IR2_sine = 1.0 / (R[1:-1] ** 2)
        self.D2_sine = (D @ D)[1:-1, 1:-1]
        self.IR4_r2 = 1.0 / (R[1:-1] ** 4)
        self.D2_r2 = (np.diag(1.0 / R ** 2) @ (D @ D))[1:-1, 1:-1]


# ---------------------------------------------------------------------------------------------------
# layout  (Matrix_Operators.py:529-627, Main.py:137-176)
# ---------------------------------------------------------------------------------------------------


def Vecs_to_X(PSI, T, C, N_fm, nr, symmetric):
    """Matrix_Operators.py:530-575: three (nr, N_fm) arrays -> flat X; symmetric keeps psi odd slots and
    T/S even slots."""
    NX = np.zeros((3, N_fm, nr))
    if symmetric:
        NX[0, 1::2] = PSI.T[1::2]
        NX[1, 0::2] = T.T[0::2]
        NX[2, 0::2] = C.T[0::2]
    else:
        NX[0], NX[1], NX[2] = PSI.T, T.T, C.T
    return NX.reshape(-1)


def X_to_Vecs(X, N_fm, nr, symmetric):
    """Matrix_Operators.py:579-627: flat X -> (PSI, T, C), each (nr, N_fm)."""
    V = np.asarray(X, dtype=float).reshape(3, N_fm, nr)
    PSI, T, C = (np.array(V[f].T) for f in range(3))
    if symmetric:
        PSI[:, 0::2] = 0.0
        T[:, 1::2] = 0.0
        C[:, 1::2] = 0.0
    return PSI, T, C


def Eq_SYM(X1, R):
    """Main.py:137-176: mask that zeroes psi even slots and T/S odd slots."""
    nr = len(R[1:-1])
    N_fm = int(X1.shape[0] / (3 * nr))
    m = np.ones((3, N_fm, nr))
    m[0, 0::2] = 0.0
    m[1, 1::2] = 0.0
    m[2, 1::2] = 0.0
    return m.reshape(-1)


# ---------------------------------------------------------------------------------------------------
# theta-coupling recurrences  (Matrix_Operators.py:131-245, 436-526)
# ---------------------------------------------------------------------------------------------------


def _parity_suffix(G):
    """S[m] = sum_{m' >= m, m' = m (mod 2)} G[m'] accumulated from the top mode downwards, the order the
    reference's running sums use (Matrix_Operators.py:159-167, 223-231)."""
    S = np.empty_like(G)
    for p in (0, 1):
        S[p::2] = np.cumsum(G[p::2][::-1], axis=0)[::-1]
    return S


def _parity_mask(N_fm, sym_keep_parity, symmetric):
    keep = np.ones(N_fm, dtype=bool)
    if symmetric:
        keep[:] = False
        keep[sym_keep_parity::2] = True
    return keep[:, None]


def J_theta_RT(g, nr, N_fm, symmetric):
    """Matrix_Operators.py:436-472: J_theta(psi) = (1/sin)d(psi sin)/dtheta in the cosine basis.
    f_j = (j+1) g_{j-1} + 2 b_j (j>=1), f_0 = b_0, b_j = sum_{m>j, m-j odd} g_m."""
    G = np.asarray(g, dtype=float).reshape(N_fm, nr)
    S = _parity_suffix(G)
    b = np.zeros_like(G)
    b[:-1] = S[1:]
    j = np.arange(N_fm, dtype=float)[:, None]
    f = np.empty_like(G)
    f[1:] = (j[1:] + 1.0) * G[:-1] + 2.0 * b[1:]
    f[0] = 1.0 * b[0]
    if symmetric:
        f[1::2] = 0.0      # only even cosine rows are formed (:457)
    return f.reshape(-1)


def DT0_theta(g, dT0, N_fm, nr, symmetric):
    """Matrix_Operators.py:131-189: r^2 J(psi, T0) = T0' J_theta(psi)."""
    G = np.asarray(g, dtype=float).reshape(N_fm, nr)
    S = _parity_suffix(G)
    b = np.zeros_like(G)
    b[:-1] = S[1:]
    j = np.arange(N_fm, dtype=float)[:, None]
    f = np.empty_like(G)
    f[1:] = dT0 * ((j[1:] + 1.0) * G[:-1] + 2.0 * b[1:])
    f[0] = dT0 * 1.0 * b[0]
    if symmetric:
        f[1::2] = 0.0
    return f.reshape(-1)


def _a2_like(G, D2, IRx, N_fm, symmetric):
    """Shared body of A2_SINE (:192-245) and A2_SINE_R2 (:475-526): slot s <-> sine wavenumber j=s+1,
    f_s = D2 g_s - j IRx ((j+1) g_s + 2 f_e), f_e = sum of same-parity slots above s."""
    S = _parity_suffix(G)
    fe = np.zeros_like(G)
    fe[:-2] = S[2:]
    j = np.arange(1, N_fm + 1, dtype=float)[:, None]
    f = G @ D2.T - j * IRx * ((j + 1.0) * G + 2.0 * fe)
    if symmetric:
        f[0::2] = 0.0      # only the odd rows (even wavenumbers) are formed (:233)
    return f


def A2_SINE(g, D, R, N_fm, nr, symmetric):
    """Matrix_Operators.py:192-245: A^2 psi with D2=(D@D)[1:-1,1:-1], IR2=1/r^2."""
    G = np.asarray(g, dtype=float).reshape(N_fm, nr)
    IR2 = 1.0 / (R[1:-1] ** 2)
    D2 = (D @ D)[1:-1, 1:-1]
    return _a2_like(G, D2, IR2, N_fm, symmetric).reshape(-1)


def A2_SINE_R2(g, N_fm, nr, D, R, symmetric):
    """Matrix_Operators.py:475-526: (1/r^2) A^2 psi with D2=(diag(1/R^2) D@D)[1:-1,1:-1], IR4=1/r^4."""
    G = np.asarray(g, dtype=float).reshape(N_fm, nr)
    IR4 = 1.0 / (R[1:-1] ** 4)
    D2 = (np.diag(1.0 / R ** 2) @ (D @ D))[1:-1, 1:-1]
    return _a2_like(G, D2, IR4, N_fm, symmetric).reshape(-1)


# ---------------------------------------------------------------------------------------------------
# nonlinear term  (Matrix_Operators.py:630-898)
# ---------------------------------------------------------------------------------------------------


def Derivatives(X_hat, JPSI, OMEGA, Dr, N_fm, nr, symmetric):
    """Matrix_Operators.py:630-740: the nine spectral fields, each (nr, N_fm), sine fields shifted to the
    sinusoid convention (index = wavenumber, :734-737)."""
    N = N_fm * nr
    V = np.asarray(X_hat, dtype=float).reshape(3, N_fm, nr)
    PSI, T, C = V[0].T, V[1].T, V[2].T                      # (nr, N_fm)
    JP = np.asarray(JPSI).reshape(N_fm, nr).T
    OM = np.asarray(OMEGA).reshape(N_fm, nr).T
    k_s = np.arange(1, N_fm + 1, dtype=float)[None, :]
    k_c = np.arange(0, N_fm, dtype=float)[None, :]
    Dpsi = Dr @ PSI
    kDpsi = k_s * Dpsi
    omega = np.array(OM)
    komega = k_s * omega
    JT_psi = np.array(JP)
    DT = Dr @ T
    kT = -k_c * T
    DC = Dr @ C
    kC = -k_c * C
    if symmetric:
        odd = np.zeros(N_fm, dtype=bool)
        odd[1::2] = True
        for A in (Dpsi, kDpsi, omega, komega):
            A[:, ~odd] = 0.0
        for A in (JT_psi, DT, kT, DC, kC):
            A[:, odd] = 0.0

    def shift(A):
        B = np.zeros_like(A)
        B[:, 1:] = A[:, :-1]
        return B

    Dpsi, kDpsi, omega, komega = shift(Dpsi), shift(kDpsi), shift(omega), shift(komega)
    _ = N
    return JT_psi, kDpsi, komega, DT, DC, omega, Dpsi, kT, kC


def grid_fields(X_hat, D, R, N_fm, nr, symmetric):
    """Matrix_Operators.py:761-786: the nine fields on the 3/2-padded grid, each (nr, 3*N_fm/2)."""
    N = nr * N_fm
    JPSI = J_theta_RT(X_hat[0:N], nr, N_fm, symmetric)
    OMEGA = A2_SINE_R2(X_hat[0:N], N_fm, nr, D, R, symmetric)
    Dr = D[1:-1, 1:-1]
    JT_psi_h, kDpsi_h, komega_h, DT_h, DC_h, omega_h, Dpsi_h, kT_h, kC_h = Derivatives(
        X_hat, JPSI, OMEGA, Dr, N_fm, nr, symmetric)
    P = (3 * N_fm) // 2
    cos_in = np.stack([JT_psi_h, komega_h, kDpsi_h, DT_h, DC_h])
    sin_in = np.stack([omega_h, Dpsi_h, kT_h, kC_h])
    JT_psi, komega, kDpsi, DT, DC = IDCT(cos_in, n=P)
    omega, Dpsi, kT, kC = IDST(sin_in, n=P)
    return dict(JT_psi=JT_psi, komega=komega, kDpsi=kDpsi, DT=DT, DC=DC, omega=omega, Dpsi=Dpsi,
                kT=kT, kC=kC)


def _finish(NJ_PSI, NJ_T, NJ_C, N_fm, nr, symmetric):
    """Matrix_Operators.py:795-804: forward transforms, un-pad, psi shifted back to slot = wavenumber-1."""
    J_PSI_hat = DST(NJ_PSI, axis=-1)[:, 0:N_fm]
    J_T_hat = DCT(NJ_T, axis=-1)[:, 0:N_fm]
    J_C_hat = DCT(NJ_C, axis=-1)[:, 0:N_fm]
    J_PSI_hat[:, 0:-1] = J_PSI_hat[:, 1:]
    J_PSI_hat[:, -1] = 0.0
    return Vecs_to_X(J_PSI_hat, J_T_hat, J_C_hat, N_fm, nr, symmetric)


def NLIN_FX(X_hat, D, R, N_fm, nr, symmetric):
    """Matrix_Operators.py:743-804: F(X, X) = u.grad(omega), u.grad(T), u.grad(S), 3/2-dealiased."""
    if N_fm % 2 != 0:
        raise ValueError('The number of Fourier modes is not even %d' % N_fm)
    g = grid_fields(X_hat, D, R, N_fm, nr, symmetric)
    Dr = D[1:-1, 1:-1]
    NJ_PSI = Dr @ (g["JT_psi"] * g["omega"]) - (g["kDpsi"] * g["omega"] + g["Dpsi"] * g["komega"])
    NJ_T = g["JT_psi"] * g["DT"] - g["Dpsi"] * g["kT"]
    NJ_C = g["JT_psi"] * g["DC"] - g["Dpsi"] * g["kC"]
    return _finish(NJ_PSI, NJ_T, NJ_C, N_fm, nr, symmetric)


def NLIN_DFX(dv_hat, X_hat, D, R, N_fm, nr, symmetric, base=None):
    """Matrix_Operators.py:807-898: DF(X) dv = F(X, dv) + F(dv, X).  ``base`` may carry the grid fields
    of X (they depend on X only)."""
    if N_fm % 2 != 0:
        raise ValueError('The number of Fourier modes is not even %d' % N_fm)
    a = base if base is not None else grid_fields(X_hat, D, R, N_fm, nr, symmetric)
    b = grid_fields(dv_hat, D, R, N_fm, nr, symmetric)
    Dr = D[1:-1, 1:-1]
    NJ_PSI = Dr @ (a["JT_psi"] * b["omega"]) - (a["kDpsi"] * b["omega"] + a["Dpsi"] * b["komega"])
    NJ_PSI += Dr @ (b["JT_psi"] * a["omega"]) - (b["kDpsi"] * a["omega"] + b["Dpsi"] * a["komega"])
    NJ_T = (b["JT_psi"] * a["DT"] - b["Dpsi"] * a["kT"]) + (a["JT_psi"] * b["DT"] - a["Dpsi"] * b["kT"])
    NJ_C = (b["JT_psi"] * a["DC"] - b["Dpsi"] * a["kC"]) + (a["JT_psi"] * b["DC"] - a["Dpsi"] * b["kC"])
    return _finish(NJ_PSI, NJ_T, NJ_C, N_fm, nr, symmetric)


# ---------------------------------------------------------------------------------------------------
# implicit back-substitution chains  (Matrix_Operators.py:1033-1194)
# ---------------------------------------------------------------------------------------------------


def NAB2_BSub_TSTEP_V2(g, L_inv, N_fm, nr, dt, symmetric):
    """Matrix_Operators.py:1033-1086: solve (r^2 - dt r^2 Lap) f = g by two parity chains over cosine
    modes j (descending); b accumulates 2 dt (j+2) f_{j+2}; row j=0 uses 0.5 b."""
    G = np.asarray(g, dtype=float).reshape(N_fm, nr)
    F = np.zeros_like(G)
    starts = (1,) if symmetric else (0, 1)
    for start in starts:
        b = np.zeros(nr)
        for jj in range(start, N_fm, 2):
            j = N_fm - (jj + 1)
            if j < N_fm - 2:
                bk = -2.0 * (j + 2.0)
                bk = -dt * bk
                b += bk * F[j + 2]
            if j == 0:
                F[j] = L_inv[jj] @ (G[j] - 0.5 * b)
            else:
                F[j] = L_inv[jj] @ (G[j] - b)
    return F.reshape(-1)


def A4_BSub_TSTEP_V2(g, L_inv, D2, IR4, IR2, N_fm, nr, dt, symmetric):
    """Matrix_Operators.py:1115-1194: solve (A^2 - dt Pr A^4) psi = g by two parity chains over sine modes
    (rows descending) with running sums f_e, bf_e.  IR4/IR2 may be the diagonal matrices the reference
    passes or their diagonals."""
    IR4 = np.diag(IR4) if np.ndim(IR4) == 2 else np.asarray(IR4)
    IR2 = np.diag(IR2) if np.ndim(IR2) == 2 else np.asarray(IR2)
    G = np.asarray(g, dtype=float).reshape(N_fm, nr)
    F = np.zeros_like(G)
    starts = (0,) if symmetric else (0, 1)
    for start in starts:
        f_e = np.zeros(nr)
        bf_e = np.zeros(nr)
        for jj in range(start, N_fm, 2):
            row = N_fm - (jj + 1)
            j = N_fm - jj
            bj = -j * (j + 1)
            bjt = -2 * j
            if row < N_fm - 2:
                f_e += F[row + 2]
                L1f = D2 @ f_e + bj * IR4 * f_e
                b_test = dt * bjt * (L1f + IR4 * bf_e) - bjt * IR2 * f_e
                F[row] = L_inv[jj] @ (G[row] + b_test)
                bf_e += bj * F[row] + bjt * f_e
            else:
                F[row] = L_inv[jj] @ G[row]
                bf_e += bj * F[row]
    return F.reshape(-1)


# ---------------------------------------------------------------------------------------------------
# step, Newton residual and Jacobian  (Main.py:255-283, 473-521)
# ---------------------------------------------------------------------------------------------------


def _gr_apply(ops, v):
    """kGR_RT (Matrix_Operators.py:97-128) applied to a cosine-indexed field: psi slot k <- -(k+1) GR v_{k+1};
    the top psi slot receives nothing."""
    V = v.reshape(ops.N_fm, ops.nr)
    out = np.zeros_like(V)
    k1 = np.arange(1, ops.N_fm, dtype=float)[:, None]
    out[:-1] = (-k1 * ops.gr) * V[1:]
    return out.reshape(-1)


def linear_solve(ops, Xn, NX, Ra, Ra_s, symmetric):
    """Main.py:266-283: add the linear explicit terms to NX (= -dt F) and run the three chains."""
    N_fm, nr, dt, Pr, Tau = ops.N_fm, ops.nr, ops.dt, ops.Pr, ops.Tau
    N = N_fm * nr
    psi, T, S = Xn[0:N], Xn[N:2 * N], Xn[2 * N:3 * N]
    NX = np.array(NX, dtype=float, copy=True)
    psi_T0 = DT0_theta(psi, ops.DT0, N_fm, nr, symmetric)
    Om = A2_SINE(psi, ops.D, ops.R, N_fm, nr, symmetric)
    NX[0:N] += Om + dt * Pr * _gr_apply(ops, Ra * T - Ra_s * S)
    a = A4_BSub_TSTEP_V2(NX[0:N], ops.Linv_A4, ops.D2_A4, ops.IR4_A4, ops.IR2_A4, N_fm, nr, Pr * dt,
                         symmetric)
    rsq = np.tile(ops.rsq, N_fm)
    NX[N:2 * N] += rsq * T - dt * psi_T0
    b = NAB2_BSub_TSTEP_V2(NX[N:2 * N], ops.Linv_T, N_fm, nr, dt, symmetric)
    NX[2 * N:3 * N] += rsq * S - dt * psi_T0
    c = NAB2_BSub_TSTEP_V2(NX[2 * N:3 * N], ops.Linv_S, N_fm, nr, Tau * dt, symmetric)
    return np.hstack((a, b, c))


def step(ops, Xn, Ra, Ra_s, symmetric, linear=False):
    """Main.py:255-283 (Step_Python): one IMEX-Euler ("CNAB1") step."""
    if linear:
        NX = np.zeros(3 * ops.N_fm * ops.nr)
    else:
        NX = -1 * ops.dt * NLIN_FX(Xn, ops.D, ops.R, ops.N_fm, ops.nr, symmetric)
    return linear_solve(ops, Xn, NX, Ra, Ra_s, symmetric)


def time_step(ops, X, Ra, Ra_s, symmetric, n_steps, linear=False, every=None):
    """Main.py:286-329 without diagnostics/IO: X <- X_SYM * step(X) repeated; returns final state and
    optionally the states after every ``every`` steps."""
    X_SYM = Eq_SYM(X, ops.R) if symmetric else 1.0
    X = np.array(X, dtype=float, copy=True)
    snaps = []
    Xn = X
    for it in range(n_steps):
        Xn = step(ops, X, Ra, Ra_s, symmetric, linear)
        if every and it % every == 0:
            snaps.append(Xn.copy())
        X = X_SYM * Xn
    return (Xn, snaps) if every else Xn


def step_cnab2(ops_half, Xn, E_prev, Ra, Ra_s, symmetric, dt):
    """A Crank-Nicolson / Adams-Bashforth-2 step of dt composed of the reference's own operations
    (NLIN_FX Matrix_Operators.py:743, DT0_theta :131, A2_SINE :192, kGR_RT :97, A4_BSub_TSTEP_V2 :1115,
    NAB2_BSub_TSTEP_V2 :1033), with ops_half the operators of dt/2 (Main.py:179-225 at dt/2):
      psi' = A4_BSub_{dt/2}(2 A2_SINE(psi) + dt E~_psi) - psi,   T' = NAB2_BSub_{dt/2}(2 r^2 T + dt E~_T) - T,
    E the explicit terms per unit time (psi: -F_psi + Pr gr_k(Ra T - Ra_s S); T/S: -F_T/S - DT0_theta(psi)),
    E~ = 3/2 E - 1/2 E_prev (E_prev None: E).  Returns (X', E)."""
    N_fm, nr, Pr, Tau = ops_half.N_fm, ops_half.nr, ops_half.Pr, ops_half.Tau
    h = ops_half.dt
    N = N_fm * nr
    psi, T, S = Xn[0:N], Xn[N:2 * N], Xn[2 * N:3 * N]
    F = NLIN_FX(Xn, ops_half.D, ops_half.R, N_fm, nr, symmetric)
    psi_T0 = DT0_theta(psi, ops_half.DT0, N_fm, nr, symmetric)
    E = np.hstack((-F[0:N] + Pr * _gr_apply(ops_half, Ra * T - Ra_s * S), -F[N:2 * N] - psi_T0,
                   -F[2 * N:3 * N] - psi_T0))
    Et = E if E_prev is None else 1.5 * E - 0.5 * E_prev
    rsq = np.tile(ops_half.rsq, N_fm)
    Om = A2_SINE(psi, ops_half.D, ops_half.R, N_fm, nr, symmetric)
    a = A4_BSub_TSTEP_V2(2.0 * Om + dt * Et[0:N], ops_half.Linv_A4, ops_half.D2_A4, ops_half.IR4_A4,
                         ops_half.IR2_A4, N_fm, nr, Pr * h, symmetric) - psi
    b = NAB2_BSub_TSTEP_V2(2.0 * rsq * T + dt * Et[N:2 * N], ops_half.Linv_T, N_fm, nr, h, symmetric) - T
    c = NAB2_BSub_TSTEP_V2(2.0 * rsq * S + dt * Et[2 * N:], ops_half.Linv_S, N_fm, nr, Tau * h, symmetric) - S
    return np.hstack((a, b, c)), E


def PFX(ops, Xn, Ra, Ra_s, symmetric):
    """Main.py:473-496: Newton residual F(X) = Phi_dt(X) - X."""
    NX = -1.0 * ops.dt * NLIN_FX(Xn, ops.D, ops.R, ops.N_fm, ops.nr, symmetric)
    return linear_solve(ops, Xn, NX, Ra, Ra_s, symmetric) - Xn


def PDFX(ops, dv, Xn, Ra, Ra_s, symmetric, base=None):
    """Main.py:498-521: Jacobian-vector product of PFX."""
    NX = -1.0 * ops.dt * NLIN_DFX(dv, Xn, ops.D, ops.R, ops.N_fm, ops.nr, symmetric, base=base)
    return linear_solve(ops, dv, NX, Ra, Ra_s, symmetric) - dv


def newton_gmres(ops, X, Ra, Ra_s, symmetric, tol=1e-10, restart=50, max_newton=20, gmres_rtol=1e-4,
                 maxiter=40):
    """Main.py:523-536 with the stopping rule made absolute: Newton on PFX with a GMRES(restart) inner
    solve (inner tolerance gmres_rtol*|F|), stop when |F(X)|_2 <= tol.  Returns (X, |F| history, matvecs)."""
    import scipy.sparse.linalg as spla
    X = np.array(X, dtype=float, copy=True)
    n = X.shape[0]
    hist = []
    mv = [0]
    for _ in range(max_newton):
        fx = PFX(ops, X, Ra, Ra_s, symmetric)
        nf = np.linalg.norm(fx)
        hist.append(nf)
        if nf <= tol:
            break
        base = grid_fields(X, ops.D, ops.R, ops.N_fm, ops.nr, symmetric)

        def mvf(v, X=X, base=base):
            mv[0] += 1
            return PDFX(ops, v, X, Ra, Ra_s, symmetric, base=base)

        A = spla.LinearOperator((n, n), matvec=mvf, dtype="float64")
        dv, _ = spla.gmres(A, fx, restart=restart, maxiter=maxiter, rtol=0.0, atol=gmres_rtol * nf)
        X = X - dv
    return X, hist, mv[0]


# ---------------------------------------------------------------------------------------------------
# diagnostics  (Main.py:41-134)
# ---------------------------------------------------------------------------------------------------


def Nusselt(T_hat, d, R, D, N_fm, nr):
    """Main.py:41-68: convective Nusselt number at the inner wall (value returned is NuM1[0])."""
    A_T = base_state_AT(d)
    NuM1 = 0.0 * R
    for k in range(0, N_fm, 2):
        TT = 0 * R
        TT[1:-1] = T_hat[k * nr:(k + 1) * nr]
        NuM1 += (D @ TT) / (1.0 - (k ** 2))
    NuM1 = ((R ** 2) / A_T) * NuM1
    return NuM1[0]


def Kinetic_Energy(X_hat, R, D, N_fm, nr, symmetric):
    """Main.py:71-134: volume-averaged kinetic energy on the 3*N_fm grid with trapezoidal quadrature."""
    N = N_fm * nr
    Dr = D[1:-1, 1:-1]
    JPSI = J_theta_RT(X_hat[0:N], nr, N_fm, symmetric).reshape(N_fm, nr)
    PSI = np.asarray(X_hat[0:N]).reshape(N_fm, nr)
    Dpsi_h = (PSI @ Dr.T).T
    Jpsi_h = (JPSI / R[1:-1][None, :]).T
    Dpsi_s = np.zeros_like(Dpsi_h)
    Dpsi_s[:, 1:] = Dpsi_h[:, :-1]
    th = grid(3 * N_fm)
    Jpsi = IDCT(Jpsi_h, n=3 * N_fm)
    Dpsi = IDST(Dpsi_s, n=3 * N_fm)
    KE_rt = Jpsi ** 2 + Dpsi ** 2
    KE_t = np.trapezoid(KE_rt, x=R[1:-1], axis=0)
    KE = np.trapezoid(KE_t * np.sin(th), x=th, axis=-1)
    V = (2.0 / 3.0) * (R[-1] ** 3 - R[0] ** 3)
    return (0.5 / V) * KE


# ---------------------------------------------------------------------------------------------------
# resolution changes  (Matrix_Operators.py:901-1011)
# ---------------------------------------------------------------------------------------------------


def INTERP_RADIAL(N_n, N_o, X_o, d):
    """Matrix_Operators.py:901-941: polyfit of degree len(R_o) through (R_o, [0, X, 0]), polyval on R_n."""
    import warnings
    if N_n == N_o:
        return X_o
    _, R_n = cheb_radial(N_n, d)
    _, R_o = cheb_radial(N_o, d)
    nr_n, nr_o = len(R_n[1:-1]), len(R_o[1:-1])
    N_fm = len(X_o) // (3 * nr_o)
    X_n = np.zeros(3 * nr_n * N_fm)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for k in range(N_fm):
            for f in range(3):
                io = f * N_fm * nr_o + nr_o * k
                poly = np.polyfit(R_o, np.hstack(([0.0], X_o[io:io + nr_o], [0.0])), len(R_o))
                i_n = f * N_fm * nr_n + nr_n * k
                X_n[i_n:i_n + nr_n] = np.polyval(poly, R_n[1:-1])
    return X_n


def INTERP_THETAS(N_fm_n, N_fm_o, X_o):
    """Matrix_Operators.py:944-1011: IDST/IDCT of the (zero-padded) modes, DST/DCT back with n = N_fm_n
    (psi rows in storage order, as the reference)."""
    if N_fm_n == N_fm_o:
        return X_o
    nr = len(X_o) // (3 * N_fm_o)
    Mx = max(N_fm_n, N_fm_o)
    V = np.asarray(X_o, dtype=float).reshape(3, N_fm_o, nr)
    F = np.zeros((3, nr, Mx))
    for f in range(3):
        F[f, :, :N_fm_o] = V[f].T
    out = np.stack([DST(IDST(F[0]), n=N_fm_n), DCT(IDCT(F[1]), n=N_fm_n), DCT(IDCT(F[2]), n=N_fm_n)])
    return np.ascontiguousarray(out.transpose(0, 2, 1)).reshape(-1)


# ---------------------------------------------------------------------------------------------------
# seeded synthetic states
# ---------------------------------------------------------------------------------------------------


def seeded_state(N_fm, nr, seed, symmetric=False):
    """Seeded Gaussian coefficients, amplitude 1e-3*exp(-k/8)*exp(-n/4) for n in [0,nr), k in [0,N_fm),
    drawn for psi, T, S in that order from numpy.random.default_rng(seed)."""
    rng = np.random.default_rng(seed)
    k = np.arange(N_fm)[None, :]
    n = np.arange(nr)[:, None]
    amp = 1e-3 * np.exp(-k / 8.0) * np.exp(-n / 4.0)
    P, T, S = [rng.standard_normal((nr, N_fm)) * amp for _ in range(3)]
    return Vecs_to_X(P, T, S, N_fm, nr, symmetric)


def Full_Eig_Vec(f, l, N_fm, nr, symmetric=False):
    """Linear_Problem.py:295-317: radial profiles f = [psi; T; S] times -sin(theta) C^{3/2}_{l-1}(cos theta)
    (psi) and P_l(cos theta) (T, S), transformed (DST/DCT with n = N_fm; psi shifted to the code's sine
    convention) and laid out by Vecs_to_X."""
    from scipy.special import eval_gegenbauer, eval_legendre
    th = grid(N_fm)
    Gl_hat = np.array(DST(-np.sin(th) * eval_gegenbauer(l - 1, 1.5, np.cos(th)), n=N_fm), dtype=float)
    Pl_hat = np.array(DCT(eval_legendre(l, np.cos(th)), n=N_fm), dtype=float)
    Gl_hat[:-1] = Gl_hat[1:].copy()
    Gl_hat[-1] = 0.0
    f = np.asarray(f, dtype=float).reshape(-1)
    return Vecs_to_X(np.outer(f[:nr], Gl_hat), np.outer(f[nr:2 * nr], Pl_hat), np.outer(f[2 * nr:3 * nr], Pl_hat),
                     N_fm, nr, symmetric)
