"""Drop-in for the eigen-seed functions of the reference's Linear_Problem.py (Linear_Problem.py:16-85,
295-317): eigenvalues and eigenvectors of the single-mode linear problem M^-1 L (a 3(N_r-1) square dense
eigenproblem, solved on the host with LAPACK as in the reference), and the full state X built from an
eigenvector, whose theta transforms run on the GPU.  Used to seed Newton / continuation on a nontrivial
branch near the linear onset."""
import numpy as np

from .Linear_Matrix_Operators import ML_0, Ll_0, cheb_radial


def _sorted_eig(Ra1, l, d, Ra_s, Pr, Tau, Nr, vectors):
    D, R = cheb_radial(Nr, d)
    AA = np.linalg.solve(ML_0(D, R, l), Ll_0(D, R, d, l, Ra1, Ra_s, Pr, Tau))
    if vectors:
        w, V = np.linalg.eig(AA)
    else:
        w, V = np.linalg.eigvals(AA), None
    idx = w.real.argsort()[::-1]
    return w[idx], (V[:, idx] if V is not None else None)


def Eig_Vals(Ra1, l, d, Nvals, Ra_s=150, Pr=1, Tau=1. / 15., Nr=20):
    """Linear_Problem.py:16-53: eigenvalues sorted by decreasing real part; Nvals in {0, 1, 2} returns
    the real part of that one, otherwise the first Nvals (complex)."""
    w, _ = _sorted_eig(Ra1, l, d, Ra_s, Pr, Tau, Nr, False)
    if Nvals in (0, 1, 2):
        return w[Nvals].real
    return w[:Nvals]


def Eig_Vec(Ra1, l, d, k, Ra_s=150, Pr=1, Tau=1. / 15., Nr=20):
    """Linear_Problem.py:56-85: the real part of the k-th eigenvector (same ordering), a column of
    length 3(Nr-1): [psi; T; S] radial profiles.  Its sign and scale are LAPACK's (unit 2-norm)."""
    _, V = _sorted_eig(Ra1, l, d, Ra_s, Pr, Tau, Nr, True)
    return V[:, k].real.reshape(-1, 1)


def Full_Eig_Vec(f, l, N_fm, nr, symmetric=False):
    """Linear_Problem.py:295-317: the state with radial profiles f = [psi; T; S] times the theta profiles
    -sin(theta) C^{3/2}_{l-1}(cos theta) (psi) and P_l(cos theta) (T, S), transformed to the code's
    sine/cosine coefficients (psi in the shifted sine convention) and laid out by Vecs_to_X."""
    from scipy.special import eval_gegenbauer, eval_legendre
    from .Transforms import DCT, DST, grid
    from .Matrix_Operators import Vecs_to_X
    th = grid(N_fm)
    Gl = -np.sin(th) * eval_gegenbauer(l - 1, 1.5, np.cos(th))
    Pl = eval_legendre(l, np.cos(th))
    Gl_hat = np.asarray(DST(Gl, n=N_fm), dtype=np.float64).copy()
    Pl_hat = np.asarray(DCT(Pl, n=N_fm), dtype=np.float64)
    Gl_hat[:-1] = Gl_hat[1:].copy()
    Gl_hat[-1] = 0.0
    f = np.asarray(f, dtype=np.float64).reshape(-1)
    PSI = np.outer(f[0:nr], Gl_hat)
    T = np.outer(f[nr:2 * nr], Pl_hat)
    C = np.outer(f[2 * nr:3 * nr], Pl_hat)
    return Vecs_to_X(PSI, T, C, N_fm, nr, symmetric)
