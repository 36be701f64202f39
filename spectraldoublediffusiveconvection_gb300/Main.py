"""Drop-in for the drivers of the reference's ``Main.py``.

``Build_Matrix_Operators``, ``_Time_Step`` and ``_Newton`` keep the reference's signatures
(Main.py:179, 228, 430).  Time integration and Newton-GMRES run on the GPU through a cached device
plan: the state stays resident for the whole call and comes back to the host once at the end (and at
the save points).

Differences from the reference, by design:
* ``_Newton`` stops on the absolute FP64 residual |F(X)|_2 <= tol_newton.  The reference's relative
  step test |dv|/|X| < tol (Main.py:536) cannot be met when the steady state is X = 0, where the seeded
  states of the benchmark converge.  GMRES restarts every min(Krylov_Space_Size, 50) vectors.
* ``_Time_Step`` evaluates Norm/KE/Nu at the save points (every N_iters/10 steps) rather than after every
  step, and writes the HDF5 file only when h5py is importable.
"""
import os
import time
import warnings

import numpy as np

from . import Matrix_Operators as MO
from . import operators as _ops
from .Transforms import IDCT, IDST, grid
from .plan import get_plan


def uniquify(path):
    """Main.py:12-20: next free file name of the form name_<n>.ext."""
    filename, extension = os.path.splitext(path)
    counter = int(filename.split('_')[1])
    while os.path.exists(path):
        path = filename.split('_')[0] + "_" + str(counter) + extension
        counter += 1
    return path


def Base_State_Coeffs(d):
    """Main.py:23-38."""
    return _ops.base_state_coeffs(d)


def Nusselt(T_hat, d, R, D, N_fm, nr, check=True):
    """Main.py:41-68: convective Nusselt number from the even cosine modes of T (or S)."""
    T_hat = np.asarray(T_hat.cpu() if hasattr(T_hat, "cpu") else T_hat, dtype=np.float64)
    A_T = _ops.base_state_coeffs(d)[0]
    TT = np.zeros((N_fm // 2 + N_fm % 2, len(R)))
    ks = np.arange(0, N_fm, 2)
    TT[:, 1:-1] = T_hat.reshape(N_fm, nr)[ks]
    NuM1 = ((TT @ D.T) / (1.0 - ks[:, None] ** 2)).sum(axis=0)
    NuM1 = ((R ** 2) / A_T) * NuM1
    error = abs(NuM1[-1] - NuM1[0]) / abs(NuM1[-1])
    if check and error > 1e-03:
        raise ValueError("|Nu(R_1) - Nu(R_2)|/|Nu(R_1)| = ", error, " > .1%, Increase Nr \n")
    return NuM1[0]


def Kinetic_Energy(X_hat, R, D, N_fm, nr, symmetric):
    """Main.py:71-134: volume-averaged kinetic energy; the transforms run on the GPU."""
    X_hat = np.asarray(X_hat.cpu() if hasattr(X_hat, "cpu") else X_hat, dtype=np.float64)
    N = N_fm * nr
    Dr = D[1:-1, 1:-1]
    JPSI = np.asarray(MO.J_theta_RT(X_hat[0:N], nr, N_fm, symmetric)).reshape(N_fm, nr)
    PSI = X_hat[0:N].reshape(N_fm, nr)
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


def Eq_SYM(X1, R):
    """Main.py:137-176: mask keeping psi odd slots and T/S even slots."""
    nr = len(R[1:-1])
    N_fm = int(X1.shape[0] / (3 * nr))
    m = np.ones((3, N_fm, nr))
    m[0, 0::2] = 0.0
    m[1:, 1::2] = 0.0
    return m.reshape(-1)


def Build_Matrix_Operators(N_fm, N_r, d, dt, Pr, Tau):
    """Main.py:179-225: the reference's operator tuple (host FP64; the device copies live in the plan)."""
    D, R = _ops.cheb_radial(N_r, d)
    Rsq = MO.R2(R, N_fm)
    gr_K = MO.kGR_RT(R, N_fm, d)
    A_T = _ops.base_state_coeffs(d)[0]
    DT0 = A_T / (R[1:-1] ** 2)
    nr = len(R[1:-1])
    L_inv_A4 = MO.A4_TSTEP_MATS(Pr * dt, N_fm, nr, D, R)
    L_inv_NAB2_T = MO.NAB2_TSTEP_MATS(dt, N_fm, nr, D, R)
    L_inv_NAB2_S = MO.NAB2_TSTEP_MATS(Tau * dt, N_fm, nr, D, R)
    D2, _, IR2, IR4 = _ops.a4_pieces(D, R)
    args_A4 = (np.ascontiguousarray(D2), np.ascontiguousarray(IR4), np.ascontiguousarray(IR2), N_fm, nr)
    args_FXS = (np.ascontiguousarray(D), R, N_fm, nr)
    return D, R, Rsq, DT0, gr_K, L_inv_A4, L_inv_NAB2_T, L_inv_NAB2_S, args_A4, args_FXS


def _to_state(X, plan):
    import torch
    if isinstance(X, torch.Tensor):
        return X.to(device=plan.device, dtype=torch.float64).reshape(1, -1).contiguous(), False
    return torch.from_numpy(np.ascontiguousarray(X, dtype=np.float64)).to(plan.device).reshape(1, -1), True


def _diagnostics(plan, Xd):
    """|X|_2, Kinetic_Energy, Nusselt(T), Nusselt(S) of a device state (Main.py:41-134, on the device)."""
    return tuple(float(v) for v in plan.diagnostics(Xd.reshape(1, -1))[0].tolist())


def _Time_Step(X, Ra, Ra_s, Tau, Pr, d, N_fm, N_r, symmetric, save_filename='TimeStep_0.h5', start_time=0,
               Total_time=1, dt=1e-04, linear=False, Verbose=False):
    """Main.py:228-329: int(Total_time/dt) IMEX ("CNAB1") steps on the GPU; returns X_new.  As the
    reference, it records |X|_2, KE, Nu_T and Nu_S after every step (computed on the device,
    sdd_step_diag) and the state at every N_iters/10-th step, and writes them to save_filename when h5py
    is available (the file holds the series up to the last save point, as the reference's last write)."""
    plan = get_plan(N_fm, N_r, d, dt, Pr, Tau, symmetric)
    Xd, was_np = _to_state(X, plan)
    N_iters = int(Total_time / dt)
    N_save = max(1, int(N_iters / 10))
    rec = dict(X_DATA=[], Norm=[], KE=[], Nu_T=[], Nu_S=[], Time=[])
    diags = []
    t0 = time.time()
    done = 0
    last_save = -1
    while done < N_iters:
        # the reference saves after iterations 0, N_save, 2 N_save, ...  (Main.py:301)
        nxt = 1 if done == 0 else min(N_iters, done + N_save)
        Xd, dg = plan.step_diag(Xd, Ra, Ra_s, nsteps=nxt - done, linear=linear)
        diags.append(dg[:, 0, :])
        done = nxt
        if (done - 1) % N_save == 0:
            rec["X_DATA"].append(Xd.cpu().numpy().ravel())
            last_save = done - 1
            if Verbose:
                ke, nut = dg[-1, 0, 1].item(), dg[-1, 0, 2].item()
                print("Iteration =%i, Time = %e, Energy = %e, NuT = %e \n " % (done - 1, start_time + dt * (done - 1),
                                                                              ke, nut))
    import torch
    series = torch.cat(diags).cpu().numpy() if diags else np.zeros((0, 4))
    n_rec = last_save + 1
    rec["Norm"], rec["KE"], rec["Nu_T"], rec["Nu_S"] = (series[:n_rec, q].copy() for q in range(4))
    rec["Time"] = start_time + dt * np.arange(n_rec)
    _Time_Step.last_record = dict(rec, series=series)
    if save_filename:
        _write_h5(save_filename, rec, dict(Ra=Ra, Ra_s=Ra_s, Tau=Tau, Pr=Pr, d=d, N_r=N_r, N_fm=N_fm, dt=dt,
                                           start_time=start_time, symmetric=symmetric))
    if Verbose:
        print("Avg time = %e \n" % ((time.time() - t0) / max(1, N_iters)))
    return Xd.cpu().numpy().ravel() if was_np else Xd.reshape(-1)


def _write_h5(filename, rec, params):
    try:
        import h5py
    except ImportError:
        warnings.warn("h5py is not installed: %s was not written" % filename)
        return
    with h5py.File(filename, 'w') as f:
        f.create_group("Checkpoints")['X_DATA'] = rec["X_DATA"]
        g = f.create_group("Scalar_Data")
        for k in ("Norm", "KE", "Nu_T", "Nu_S", "Time"):
            g[k] = rec[k]
        p = f.create_group("Parameters")
        for k, v in params.items():
            p[k] = v


def _Newton(X, Ra, Ra_s, Tau, Pr, d, N_fm, N_r, symmetric, dt=1, tol_newton=1e-08, tol_gmres=1e-04,
            Krylov_Space_Size=300, max_newton=20):
    """Main.py:430-554: steady state of Phi_dt(X) - X by Newton-GMRES on the GPU.

    Returns (X, Norm, KE, NuT, NuS, True) on convergence (|F(X)|_2 <= tol_newton) and
    (None, None, None, None, None, False) otherwise, as the reference does (Main.py:541-544)."""
    plan = get_plan(N_fm, N_r, d, dt, Pr, Tau, symmetric)
    Xd, was_np = _to_state(X, plan)
    Xd = Xd.clone()
    res = plan.newton(Xd, Ra, Ra_s, tol=tol_newton, restart=min(int(Krylov_Space_Size), 50),
                      gmres_rtol=tol_gmres, max_newton=max_newton)[0]
    if not res["converged"]:
        print('Newton iteration could not converge')
        return None, None, None, None, None, False
    Xh = Xd.cpu().numpy().ravel()
    Norm, KE, NuT, NuS = _diagnostics(plan, Xd)
    return (Xh if was_np else Xd.reshape(-1)), Norm, KE, NuT, NuS, True


class result():
    """Main.py:677-714: record of a continuation run."""

    def __init__(self):
        self.NuT = []
        self.NuS = []
        self.KE = []
        self.Norm = []
        self.Ra = []
        self.Ra_dot = []
        self.Y_FOLD = []
        self.X_DATA = []
        self.Ra_DATA = []
        self.Iterations = 0

    def __str__(self):
        i = self.Iterations
        return ('Continuation succeed \n' + 'Total iterations  = ' + str(i) + '\n' + 'Ra                = '
                + str(self.Ra[i]) + '\n' + 'Ra_dot            = ' + str(self.Ra_dot[i]) + '\n'
                + 'NuT               = ' + str(self.NuT[i]) + '\n' + 'NuS               = ' + str(self.NuS[i])
                + '\n' + 'KE                = ' + str(self.KE[i]) + '\n')


def _NewtonC(Y, sign, ds, **kwargs_f):
    """Main.py:717-739: natural-parameter step Ra -> Ra + sign*ds solved by Newton; ds doubles on success
    and halves on failure."""
    Y = np.asarray(Y.cpu() if hasattr(Y, "cpu") else Y, dtype=np.float64)
    X = Y[0:-1].copy()
    Ra = Y[-1] + sign * ds
    kwargs_f = dict(kwargs_f)
    kwargs_f["Ra"] = Ra
    kwargs_f.setdefault("tol_newton", 1e-08)
    X_new, Norm, KE, NuT, NuS, exitcode = _Newton(X, **kwargs_f)
    if exitcode:
        return np.hstack((X_new, Ra)), sign, ds * 2, Norm, KE, NuT, NuS, exitcode
    return Y, sign, ds * 0.5, Norm, KE, NuT, NuS, exitcode


def _ContinC(Y_0_dot, Y_0, sign, ds, Ra, Ra_s, Tau, Pr, d, N_fm, N_r, symmetric, dt=1, tol_newton=1e-08,
             tol_gmres=1e-04, Krylov_Space_Size=300):
    """Main.py:742-955: one pseudo-arclength step on the GPU (sdd_contin_step).

    Returns (Y_dot, Y, sign, ds, Norm, KE, NuT, NuS, True) like the reference.  The corrector stops on the
    absolute residuals |F(X,Ra)|_2 <= tol_newton and |arclength residual| <= tol_newton; a step that cannot be
    corrected after ds has been halved raises ValueError as the reference does (Main.py:895)."""
    import torch
    plan = get_plan(N_fm, N_r, d, dt, Pr, Tau, symmetric)
    Y_0 = np.asarray(Y_0.cpu() if hasattr(Y_0, "cpu") else Y_0, dtype=np.float64)
    X = torch.from_numpy(Y_0[0:-1].copy()).to(plan.device).reshape(1, -1)
    if symmetric:
        X = X * torch.from_numpy(Eq_SYM(Y_0[0:-1], plan.arrays["R"])).to(plan.device).reshape(1, -1)
    Ra_d = torch.tensor([float(Y_0[-1])], dtype=torch.float64, device=plan.device)
    Xd, res = plan.contin_step(X, Ra_d, Ra_s, sign, ds, tol=tol_newton, restart=min(int(Krylov_Space_Size), 50),
                               gmres_rtol=tol_gmres, tangent_rtol=tol_newton)
    r = res[0]
    if not r["converged"]:
        raise ValueError("\n Step-size ds has become too small terminating \n")
    Xh = X.cpu().numpy().ravel()
    Y = np.hstack((Xh, float(Ra_d.item())))
    Y_dot = np.hstack((Xd.cpu().numpy().ravel(), r["Ra_dot"]))
    Norm, KE, NuT, NuS = _diagnostics(plan, X)
    return Y_dot, Y, sign, r["ds"], Norm, KE, NuT, NuS, True


def _Continuation(filename, N_steps, sign, Y, **kwargs):
    """Main.py:958-1045: branch following; natural-parameter Newton steps while ds > 1, pseudo-arclength
    steps otherwise, fold detection by a sign change of Ra_dot.  Returns the ``result`` record (the reference
    returns None and writes it to ``filename``; the file is written here only if h5py is importable)."""
    Y = np.array(Y, dtype=np.float64, copy=True)
    Y_dot = 0.0 * Y
    ds, ds_min, ds_max = 0.01, 1.0, 10.0
    Result = result()
    while Result.Iterations < N_steps:
        Y_dot_new = None
        if ds > ds_min:
            OUT = _NewtonC(Y, sign, ds, **kwargs)
            if OUT[-1] is False:
                print('Switching to arc-length \n')
                Y_dot_new, Y_new, sign, ds, Norm, KE, NuT, NuS, _ = _ContinC(Y_dot, Y, sign, ds, **kwargs)
            else:
                Y_new, sign, ds, Norm, KE, NuT, NuS = OUT[0], OUT[1], OUT[2], OUT[3], OUT[4], OUT[5], OUT[6]
            if ds > ds_max:
                ds = ds_max
        else:
            Y_dot_new, Y_new, sign, ds, Norm, KE, NuT, NuS, _ = _ContinC(Y_dot, Y, sign, ds, **kwargs)
            if (Y_dot_new[-1] * Y_dot[-1]) < 0:
                Result.Y_FOLD.append(Y_new)
            sign = 1.0 if Y_new[-1] > Y[-1] else -1.0
        Y = Y_new.copy()
        Y_dot = Y_dot_new.copy() if Y_dot_new is not None else 0.0 * Y
        Result.Ra.append(Y[-1])
        Result.Ra_dot.append(Y_dot[-1])
        Result.Norm.append(Norm)
        Result.KE.append(KE)
        Result.NuT.append(NuT)
        Result.NuS.append(NuS)
        if Result.Iterations % 5 == 0:
            Result.X_DATA.append(Y[0:-1])
            Result.Ra_DATA.append(Y[-1])
            if filename:
                _write_continuation_h5(filename, Result, kwargs)
        print(Result, flush=True)
        Result.Iterations += 1
    return Result


def _write_continuation_h5(filename, Result, kwargs):
    try:
        import h5py
    except ImportError:
        warnings.warn("h5py is not installed: %s was not written" % filename)
        return
    with h5py.File(filename, 'w') as f:
        c = f.create_group("Checkpoints")
        c['X_DATA'] = Result.X_DATA
        c['Ra_DATA'] = Result.Ra_DATA
        p = f.create_group("Parameters")
        for k, v in kwargs.items():
            p[k] = v
        b = f.create_group("Bifurcation")
        for k, v in vars(Result).items():
            b.create_dataset(k, data=v)
