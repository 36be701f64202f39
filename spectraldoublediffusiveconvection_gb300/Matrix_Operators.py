"""Drop-in for the reference's ``Matrix_Operators.py``.

Same names, argument order and return conventions.  The hot functions run on the GPU through
libsdd_gb300: ``NLIN_FX``/``NLIN_DFX`` (fused transform + product row kernels), ``J_theta_RT``,
``A2_SINE_R2``, ``A2_SINE``, ``DT0_theta`` (parity-scan row kernels), ``A4_BSub_TSTEP_V2`` and
``NAB2_BSub_TSTEP_V2`` (back-substitution chain kernels).  Operator builders (``cheb_radial``,
``Nabla2``, ``Nabla4``, ``R2``, ``kGR_RT``, ``*_TSTEP_MATS``) are set-up and stay FP64 numpy, as are
the layout helpers ``Vecs_to_X``/``X_to_Vecs`` for numpy input.

Operators handed in as arrays are uploaded once per distinct content and cached in a device plan.
"""
import hashlib
import warnings

import numpy as np

from . import operators as _ops
from ._dev import back, is_tensor, to_dev, torch
from .plan import Plan

# ---- set-up operators (host FP64) --------------------------------------------------------------
cheb_radial = _ops.cheb_radial
Nabla2 = _ops.Nabla2
Nabla4 = _ops.Nabla4


def R2(R, N_fm):
    """Matrix_Operators.py:79-94: block-diagonal r^2 (scipy sparse csr)."""
    from scipy.sparse import block_diag, diags
    GR = diags((R[1:-1] ** 2), 0, format="csr")
    return block_diag([GR] * N_fm, format="csr")


def kGR_RT(R, N_fm, d):
    """Matrix_Operators.py:97-128: buoyancy map, psi slot jj <- -(jj+1) (R_1^2/r^2) T slot jj+1."""
    from scipy.sparse import bmat, diags
    nr = len(R[1:-1])
    R_1 = 1.0 / d
    GR = diags((R_1 ** 2) / (R[1:-1] ** 2), 0, format="csr")
    Z = diags(0.0 * np.ones(nr), 0, format="csr")
    rows = []
    for jj in range(N_fm):
        j = jj + 1
        rows.append([(-k * GR) if k == j else Z for k in range(N_fm)])
    return bmat(rows, format="csr")


def NAB2_TSTEP_MATS(dt, N_fm, nr, D, R):
    """Matrix_Operators.py:1014-1030 (list of N_fm inverses)."""
    return list(_ops.nab2_tstep_mats(dt, N_fm, nr, D, R))


def A4_TSTEP_MATS(dt, N_fm, nr, D, R):
    """Matrix_Operators.py:1089-1112 (list of N_fm inverses)."""
    return list(_ops.a4_tstep_mats(dt, N_fm, nr, D, R))


# ---- device plans keyed by operator content ----------------------------------------------------
_plans = {}


def _digest(*arrs):
    h = hashlib.sha1()
    for a in arrs:
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def _dummy_arrays(N_fm, nr):
    z = np.zeros(nr)
    zz = np.zeros((nr, nr))
    return dict(Dr=zz, D2_r2=zz, ir4_r2=z, D2_sine=zz, ir2_sine=z, D2_A4=zz, ir2_A4=z, ir4_A4=z, rsq=z,
                dT0=z, gr=z, Linv_A4=np.zeros((N_fm, nr, nr)), Linv_T=np.zeros((N_fm, nr, nr)),
                Linv_S=np.zeros((N_fm, nr, nr)))


def _plan_from(N_fm, nr, symmetric, dt=1.0, **arrays):
    key = (N_fm, nr, bool(symmetric), float(dt), _digest(*[arrays[k] for k in sorted(arrays)]),
           tuple(sorted(arrays)))
    p = _plans.get(key)
    if p is None:
        A = _dummy_arrays(N_fm, nr)
        A.update({k: np.asarray(v, dtype=np.float64) for k, v in arrays.items()})
        p = Plan(N_fm, nr + 1, 1.0, dt, 1.0, 1.0, symmetric=symmetric, arrays=A)
        _plans[key] = p
    return p


def _theta_plan(D, R, N_fm, nr, symmetric, dT0=None):
    ops = _ops.theta_operators(np.asarray(D, dtype=np.float64), np.asarray(R, dtype=np.float64))
    if dT0 is not None:
        ops["dT0"] = np.asarray(dT0, dtype=np.float64)
    return _plan_from(N_fm, nr, symmetric, **ops)


def _check_even(N_fm):
    if N_fm % 2 != 0:
        raise ValueError('The number of Fourier modes is not even %d' % N_fm)


# ---- theta recurrences --------------------------------------------------------------------------
def _theta(op, g, plan):
    gt, was_np = to_dev(g)
    out = plan.theta_op(op, gt.reshape(1, -1)).reshape(gt.shape)
    return back(out, was_np)


def J_theta_RT(g, nr, N_fm, symmetric):
    """Matrix_Operators.py:436-472."""
    _check_even(N_fm)
    z = np.zeros((nr + 2, nr + 2))
    r = np.ones(nr + 2)
    return _theta(0, g, _theta_plan(z, r, N_fm, nr, symmetric))


def A2_SINE_R2(g, N_fm, nr, D, R, symmetric):
    """Matrix_Operators.py:475-526."""
    _check_even(N_fm)
    return _theta(1, g, _theta_plan(D, R, N_fm, nr, symmetric))


def A2_SINE(g, D, R, N_fm, nr, symmetric):
    """Matrix_Operators.py:192-245."""
    _check_even(N_fm)
    return _theta(2, g, _theta_plan(D, R, N_fm, nr, symmetric))


def DT0_theta(g, dT0, N_fm, nr, symmetric):
    """Matrix_Operators.py:131-189."""
    _check_even(N_fm)
    z = np.zeros((nr + 2, nr + 2))
    r = np.ones(nr + 2)
    return _theta(3, g, _theta_plan(z, r, N_fm, nr, symmetric, dT0=dT0))


# ---- nonlinear term -----------------------------------------------------------------------------
def NLIN_FX(X_hat, D, R, N_fm, nr, symmetric):
    """Matrix_Operators.py:743-804: F(X, X)."""
    _check_even(N_fm)
    plan = _theta_plan(D, R, N_fm, nr, symmetric)
    Xt, was_np = to_dev(X_hat)
    out = plan.nlin_fx(Xt.reshape(1, -1)).reshape(Xt.shape)
    return back(out, was_np)


def NLIN_DFX(dv_hat, X_hat, D, R, N_fm, nr, symmetric):
    """Matrix_Operators.py:807-898: F(X, dv) + F(dv, X)."""
    _check_even(N_fm)
    plan = _theta_plan(D, R, N_fm, nr, symmetric)
    dvt, was_np = to_dev(dv_hat)
    Xt, _ = to_dev(X_hat)
    out = plan.nlin_dfx(dvt.reshape(1, -1), Xt.reshape(1, -1)).reshape(dvt.shape)
    return back(out, was_np)


# ---- implicit solves ----------------------------------------------------------------------------
def NAB2_BSub_TSTEP_V2(g, L_inv, N_fm, nr, dt, symmetric):
    """Matrix_Operators.py:1033-1086."""
    Linv = np.asarray(L_inv, dtype=np.float64).reshape(N_fm, nr, nr)
    plan = _plan_from(N_fm, nr, symmetric, dt=dt, Linv_T=Linv)
    gt, was_np = to_dev(g)
    out = plan.nab2_bsub(1, gt.reshape(1, -1)).reshape(gt.shape)
    return back(out, was_np)


def A4_BSub_TSTEP_V2(g, L_inv, D2, IR4, IR2, N_fm, nr, dt, symmetric):
    """Matrix_Operators.py:1115-1194 (dt here is the reference's dt*Pr)."""
    Linv = np.asarray(L_inv, dtype=np.float64).reshape(N_fm, nr, nr)
    IR4 = np.diag(IR4) if np.ndim(IR4) == 2 else np.asarray(IR4)
    IR2 = np.diag(IR2) if np.ndim(IR2) == 2 else np.asarray(IR2)
    plan = _plan_from(N_fm, nr, symmetric, dt=dt, Linv_A4=Linv, D2_A4=np.asarray(D2), ir4_A4=IR4, ir2_A4=IR2)
    gt, was_np = to_dev(g)
    out = plan.a4_bsub(gt.reshape(1, -1)).reshape(gt.shape)
    return back(out, was_np)


# ---- layout ---------------------------------------------------------------------------------------
def Vecs_to_X(PSI, T, C, N_fm, nr, symmetric):
    """Matrix_Operators.py:529-575."""
    if is_tensor(PSI):
        t = torch()
        X = t.stack([PSI.T, T.T, C.T]).clone()
        if symmetric:
            X[0, 0::2] = 0.0
            X[1:, 1::2] = 0.0
        return X.reshape(-1)
    NX = np.zeros((3, N_fm, nr))
    if symmetric:
        NX[0, 1::2] = np.asarray(PSI).T[1::2]
        NX[1, 0::2] = np.asarray(T).T[0::2]
        NX[2, 0::2] = np.asarray(C).T[0::2]
    else:
        NX[0], NX[1], NX[2] = np.asarray(PSI).T, np.asarray(T).T, np.asarray(C).T
    return NX.reshape(-1)


def X_to_Vecs(X, N_fm, nr, symmetric):
    """Matrix_Operators.py:578-627."""
    if is_tensor(X):
        V = X.reshape(3, N_fm, nr)
        out = [V[f].T.clone() for f in range(3)]
    else:
        V = np.asarray(X, dtype=np.float64).reshape(3, N_fm, nr)
        out = [np.array(V[f].T) for f in range(3)]
    if symmetric:
        out[0][:, 0::2] = 0.0
        out[1][:, 1::2] = 0.0
        out[2][:, 1::2] = 0.0
    return tuple(out)


# ---- resolution changes (load-time) ----------------------------------------------------------------
def INTERP_RADIAL(N_n, N_o, X_o, d):
    """Matrix_Operators.py:901-941: per mode and field, a polynomial through the old collocation values
    (with the zero boundary values), evaluated on the new interior points.  Load-time host code (numpy
    polyfit/polyval, as the reference)."""
    if N_n == N_o:
        return X_o
    X_o = np.asarray(X_o.cpu() if hasattr(X_o, "cpu") else X_o, dtype=np.float64)
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
    """Matrix_Operators.py:944-1011: theta resolution change by a transform to the grid and back (the
    transforms run on the GPU).  Like the reference, the psi rows go through IDST/DST in storage order."""
    from .Transforms import DCT, DST, IDCT, IDST
    if N_fm_n == N_fm_o:
        return X_o
    X_o = np.asarray(X_o.cpu() if hasattr(X_o, "cpu") else X_o, dtype=np.float64)
    nr = len(X_o) // (3 * N_fm_o)
    Mx = max(N_fm_n, N_fm_o)
    V = X_o.reshape(3, N_fm_o, nr)
    F = np.zeros((3, nr, Mx))
    for f in range(3):
        F[f, :, :N_fm_o] = V[f].T
    PSI_X, T_X, S_X = IDST(F[0]), IDCT(F[1]), IDCT(F[2])
    out = np.stack([DST(PSI_X, n=N_fm_n), DCT(T_X, n=N_fm_n), DCT(S_X, n=N_fm_n)])   # (3, nr, N_fm_n)
    return np.ascontiguousarray(out.transpose(0, 2, 1)).reshape(-1)
