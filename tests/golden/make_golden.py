"""Generate the golden vectors in ``tests/golden/*.npz`` by running the reference itself.

The reference (mannixp/SpectralDoubleDiffusiveConvection, Python + numpy + scipy + numba) is imported
read-only from REF_DIR.  Its pinned third-party packages that are not installed here are replaced by
shims, so that the reference's own source runs unmodified:

* ``numba.njit``           -> identity decorator (the reference then runs un-JIT'd, same arithmetic
                               up to fastmath reassociation, i.e. ~1e-16 relative);
* ``numba.typed.List``     -> ``list``;
* ``matplotlib``/``pyplot``-> empty stub modules (plotting only);
* ``h5py``                 -> an in-memory fake whose ``File`` objects keep what ``_Time_Step`` writes
                               (``Checkpoints/X_DATA``, ``Scalar_Data/*``), so trajectories and per-step
                               diagnostics can be read back;
* ``np.RankWarning`` / ``np.trapz`` -> numpy-2 aliases (``Matrix_Operators.py:6``, ``Main.py:9,129``).

Run:  python tests/golden/make_golden.py REF_DIR [--only-<case>]
(or with REF_DIR in the environment variable SDD_REFERENCE_DIR).  It writes small ``.npz`` fixtures beside this script.  They are inputs/outputs of the reference's own
functions on seeded synthetic states (amplitude 1e-3*exp(-k/8)*exp(-n/4), default_rng seeds below).
"""
import os
import sys
import types

sys.dont_write_bytecode = True      # never write __pycache__ into the (read-only) reference tree
import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = sys.argv[1] if len(sys.argv) > 1 and not sys.argv[1].startswith("--") else \
    os.environ.get("SDD_REFERENCE_DIR")
if not REF_DIR:
    sys.exit("usage: make_golden.py REF_DIR [--only-<case>]  (or set SDD_REFERENCE_DIR)")
OPTS = [a for a in sys.argv[1:] if a.startswith("--")]


# ----------------------------------------------------------------------------------------------
# shims
# ----------------------------------------------------------------------------------------------
def _install_shims():
    if not hasattr(np, "RankWarning"):
        np.RankWarning = np.exceptions.RankWarning
    if not hasattr(np, "trapz"):
        np.trapz = np.trapezoid

    numba = types.ModuleType("numba")

    def njit(*a, **k):
        if len(a) == 1 and callable(a[0]) and not k:
            return a[0]
        return lambda f: f

    numba.njit = njit
    typed = types.ModuleType("numba.typed")
    typed.List = list
    numba.typed = typed
    sys.modules["numba"] = numba
    sys.modules["numba.typed"] = typed

    mpl = types.ModuleType("matplotlib")
    plt = types.ModuleType("matplotlib.pyplot")
    plt.rcParams = {}                  # Linear_Problem.py:5 updates it at import
    mpl.pyplot = plt
    sys.modules["matplotlib"] = mpl
    sys.modules["matplotlib.pyplot"] = plt

    h5py = types.ModuleType("h5py")

    class _Group(dict):
        def create_group(self, name):
            g = _Group()
            self[name] = g
            return g

        def create_dataset(self, name, data=None):
            self[name] = np.asarray(data)

        def __setitem__(self, key, value):
            if not isinstance(value, _Group):
                value = np.array(value, copy=True)
            dict.__setitem__(self, key, value)

    class File(_Group):
        files = {}

        def __init__(self, name, mode="r"):
            super().__init__()
            File.files[name] = self

        def close(self):
            pass

    h5py.File = File
    sys.modules["h5py"] = h5py
    return h5py


H5 = _install_shims()
sys.path.insert(0, REF_DIR)
import Transforms as Tr  # noqa: E402
import Matrix_Operators as MO  # noqa: E402
import Main  # noqa: E402

PARAMS = dict(d=2.0, Pr=1.0, Tau=0.01, Ra=8000.0, Ra_s=500.0)


def seeded_state(N_fm, nr, seed, symmetric=False):
    """Seeded Gaussian coefficients of amplitude 1e-3*exp(-k/8)*exp(-n/4) per field (psi, T, S)."""
    rng = np.random.default_rng(seed)
    k = np.arange(N_fm)[None, :]
    n = np.arange(nr)[:, None]
    amp = 1e-3 * np.exp(-k / 8.0) * np.exp(-n / 4.0)
    P, T, S = [rng.standard_normal((nr, N_fm)) * amp for _ in range(3)]
    return MO.Vecs_to_X(P, T, S, N_fm, nr, symmetric)


def linear_parts(Xn, NX, ops, N, N_fm, nr, dt, Pr, Tau, Ra, Ra_s, symmetric, subtract):
    """Main.py:255-283 / 473-496: the linear half of one step after NX = -dt*F has been formed."""
    D, R, Rsq, DT0, gr_k, LA4, LT, LS, args_A4, args_FX = ops
    psi, T, S = Xn[0:N], Xn[N:2 * N], Xn[2 * N:3 * N]
    psi_T0 = MO.DT0_theta(psi, DT0, N_fm, nr, symmetric)
    Om = MO.A2_SINE(psi, D, R, N_fm, nr, symmetric)
    NX[0:N] += Om + dt * Pr * gr_k.dot(Ra * T - Ra_s * S)
    a = MO.A4_BSub_TSTEP_V2(NX[0:N], LA4, *args_A4, Pr * dt, symmetric)
    NX[N:2 * N] += Rsq.dot(T) - dt * psi_T0
    b = MO.NAB2_BSub_TSTEP_V2(NX[N:2 * N], LT, N_fm, nr, dt, symmetric)
    NX[2 * N:3 * N] += Rsq.dot(S) - dt * psi_T0
    c = MO.NAB2_BSub_TSTEP_V2(NX[2 * N:3 * N], LS, N_fm, nr, Tau * dt, symmetric)
    if subtract:
        a, b, c = a - psi, b - T, c - S
    return np.hstack((a, b, c))


def operator_case(tag, N_r, N_fm, dt, symmetric, seed, store_linv=False):
    d, Pr, Tau, Ra, Ra_s = (PARAMS[k] for k in ("d", "Pr", "Tau", "Ra", "Ra_s"))
    nr = N_r - 1
    N = nr * N_fm
    out = {}
    ops = Main.Build_Matrix_Operators(N_fm, N_r, d, dt, Pr, Tau)
    D, R, Rsq, DT0, gr_k, LA4, LT, LS, args_A4, args_FX = ops
    X = seeded_state(N_fm, nr, seed, symmetric)
    dv = seeded_state(N_fm, nr, seed + 1, symmetric)
    if symmetric:
        X_SYM = Main.Eq_SYM(X, R)
        X = X_SYM * X
        dv = X_SYM * dv
    psi = X[0:N]
    out.update(D=D, R=R, X=X, dv=dv, DT0=DT0,
               params=np.array([N_r, N_fm, dt, d, Pr, Tau, Ra, Ra_s, float(symmetric)]))
    out["J_theta_RT"] = MO.J_theta_RT(psi, nr, N_fm, symmetric)
    out["A2_SINE_R2"] = MO.A2_SINE_R2(psi, N_fm, nr, D, R, symmetric)
    out["A2_SINE"] = MO.A2_SINE(psi, D, R, N_fm, nr, symmetric)
    out["DT0_theta"] = MO.DT0_theta(psi, DT0, N_fm, nr, symmetric)
    out["NLIN_FX"] = MO.NLIN_FX(X, *args_FX, symmetric)
    out["NLIN_DFX"] = MO.NLIN_DFX(dv, X, *args_FX, symmetric)
    g = dv[0:N] * 1e3
    out["A4_g"] = g
    out["A4_BSub"] = MO.A4_BSub_TSTEP_V2(g, LA4, *args_A4, Pr * dt, symmetric)
    out["NAB2_T"] = MO.NAB2_BSub_TSTEP_V2(g, LT, N_fm, nr, dt, symmetric)
    out["NAB2_S"] = MO.NAB2_BSub_TSTEP_V2(g, LS, N_fm, nr, Tau * dt, symmetric)
    # one IMEX ("CNAB1") step, Main.py:255-283
    NX = -1 * dt * MO.NLIN_FX(X, *args_FX, symmetric)
    out["step1"] = linear_parts(X, NX, ops, N, N_fm, nr, dt, Pr, Tau, Ra, Ra_s, symmetric, False)
    NX = np.zeros(3 * N)
    out["step1_linear"] = linear_parts(X, NX, ops, N, N_fm, nr, dt, Pr, Tau, Ra, Ra_s, symmetric, False)
    # Newton residual and Jacobian with the dt=1 operator set, Main.py:473-521
    ops1 = Main.Build_Matrix_Operators(N_fm, N_r, d, 1.0, Pr, Tau)
    NX = -1.0 * MO.NLIN_FX(X, *ops1[9], symmetric)
    out["PFX"] = linear_parts(X, NX, ops1, N, N_fm, nr, 1.0, Pr, Tau, Ra, Ra_s, symmetric, True)
    NX = -1.0 * MO.NLIN_DFX(dv, X, *ops1[9], symmetric)
    out["PDFX"] = linear_parts(dv, NX, ops1, N, N_fm, nr, 1.0, Pr, Tau, Ra, Ra_s, symmetric, True)
    # diagnostics, Main.py:41-134
    out["KE"] = np.array(Main.Kinetic_Energy(X, R, D, N_fm, nr, symmetric))
    out["NuT"] = np.array(Main.Nusselt(X[N:2 * N], d, R, D, N_fm, nr, check=False))
    out["NuS"] = np.array(Main.Nusselt(X[2 * N:3 * N], d, R, D, N_fm, nr, check=False))
    if store_linv:
        out["Linv_A4"] = np.array(LA4)
        out["Linv_T"] = np.array(LT)
        out["Linv_S"] = np.array(LS)
        out["D2_A4"], out["IR4_A4"], out["IR2_A4"] = args_A4[0], args_A4[1], args_A4[2]
    np.savez(os.path.join(HERE, f"ops_{tag}.npz"), **out)
    print("wrote", tag, {k: np.shape(v) for k, v in out.items() if np.ndim(v) > 0 and np.size(v) > 40})


def trajectory_case(tag, N_r, N_fm, dt, n_steps, symmetric, seed, linear=False):
    """Main._Time_Step run as written; X_DATA every n_steps/10 steps and the scalar series come back
    through the fake h5py File."""
    d, Pr, Tau, Ra, Ra_s = (PARAMS[k] for k in ("d", "Pr", "Tau", "Ra", "Ra_s"))
    nr = N_r - 1
    X0 = seeded_state(N_fm, nr, seed, symmetric)
    fname = f"golden_{tag}.h5"
    total = n_steps * dt
    assert int(total / dt) == n_steps, (total, dt)
    XN = Main._Time_Step(X0.copy(), Ra, Ra_s, Tau, Pr, d, N_fm, N_r, symmetric, save_filename=fname,
                         start_time=0, Total_time=total, dt=dt, linear=linear, Verbose=False)
    f = H5.File.files[fname]
    out = dict(X0=X0, X_final=XN, X_DATA=np.asarray(f["Checkpoints"]["X_DATA"]),
               Norm=np.asarray(f["Scalar_Data"]["Norm"]), KE=np.asarray(f["Scalar_Data"]["KE"]),
               NuT=np.asarray(f["Scalar_Data"]["Nu_T"]), NuS=np.asarray(f["Scalar_Data"]["Nu_S"]),
               params=np.array([N_r, N_fm, dt, d, Pr, Tau, Ra, Ra_s, float(symmetric), n_steps]))
    np.savez(os.path.join(HERE, f"traj_{tag}.npz"), **out)
    print("wrote", tag, out["X_DATA"].shape)


def continuation_case(tag, N_r, N_fm, Ra0, Tau, ds, n_steps, dt_ts, seed):
    """A nontrivial steady convective state (Tau = 1, the reference's validation regime: critical Ra_T
    near 7270 at d = 2, Tests/Run_Tests.py:55-65) and one pseudo-arclength step from it, both by the
    reference: _Time_Step to saturation, _Newton to polish, then _ContinC (Main.py:742-955)."""
    d, Pr, Ra_s = PARAMS["d"], PARAMS["Pr"], PARAMS["Ra_s"]
    nr = N_r - 1
    X0 = seeded_state(N_fm, nr, seed)
    fname = f"golden_cont_{tag}.h5"
    Xt = Main._Time_Step(X0.copy(), Ra0, Ra_s, Tau, Pr, d, N_fm, N_r, False, save_filename=fname,
                         start_time=0, Total_time=n_steps * dt_ts, dt=dt_ts, linear=False, Verbose=False)
    Xs, Norm, KE, NuT, NuS, ok = Main._Newton(Xt, Ra0, Ra_s, Tau, Pr, d, N_fm, N_r, False, dt=1,
                                              tol_newton=1e-10, tol_gmres=1e-6, Krylov_Space_Size=300)
    assert ok, "reference _Newton did not converge"
    Y0 = np.hstack((Xs, Ra0))
    out = Main._ContinC(0.0 * Y0, Y0, 1.0, ds, Ra0, Ra_s, Tau, Pr, d, N_fm, N_r, False, dt=1,
                        tol_newton=1e-8, tol_gmres=1e-4, Krylov_Space_Size=300)
    Y_dot, Y, sign, ds_new, Norm1, KE1, NuT1, NuS1, flag = out
    res = dict(X_steady=Xs, Ra0=np.array(Ra0), Y=Y, Y_dot=Y_dot, ds_new=np.array(ds_new), ds=np.array(ds),
               Norm=np.array(Norm1), KE=np.array(KE1), NuT=np.array(NuT1), NuS=np.array(NuS1),
               steady_diag=np.array([Norm, KE, NuT, NuS]),
               params=np.array([N_r, N_fm, 1.0, d, Pr, Tau, Ra0, Ra_s, 0.0]))
    np.savez(os.path.join(HERE, f"cont_{tag}.npz"), **res)
    print("wrote cont", tag, "|X_s| %.4e" % np.linalg.norm(Xs), "Ra %.6f -> %.6f" % (Ra0, Y[-1]))


def interp_case():
    """Matrix_Operators.py:901-1011 INTERP_RADIAL / INTERP_THETAS on a seeded state (up and down)."""
    X = seeded_state(16, 11, 41)                         # N_r = 12, N_fm = 16
    out = dict(X=X,
               rad_up=MO.INTERP_RADIAL(20, 12, X, 2.0),
               rad_down=MO.INTERP_RADIAL(8, 12, X, 2.0),
               th_up=MO.INTERP_THETAS(32, 16, X),
               th_down=MO.INTERP_THETAS(8, 16, X))
    np.savez(os.path.join(HERE, "interp.npz"), **out)
    print("wrote interp")


def eigen_case():
    """Linear_Problem.py:16-85 and 295-317: eigenvalues and eigenvectors of the single-mode linear
    problem (Linear_Matrix_Operators.py ML_0 / Ll_0), and the full-state vector built from one."""
    import Linear_Matrix_Operators as LMO
    # Linear_Problem.py does not parse as Python: an IPython "%matplotlib inline" line sits inside a
    # function (Linear_Problem.py:594).  Compile it in memory with that line replaced by "pass" (the file
    # itself is not touched); nothing on the path of the functions recorded here changes.
    src_path = os.path.join(REF_DIR, "Linear_Problem.py")
    lines = open(src_path).read().split("\n")
    lines = [ln[:len(ln) - len(ln.lstrip())] + "pass" if ln.lstrip().startswith("%") else ln for ln in lines]
    LP = types.ModuleType("Linear_Problem")
    LP.__file__ = src_path
    exec(compile("\n".join(lines), src_path, "exec"), LP.__dict__)
    out = {}
    for tag, (Ra, l, d, Ra_s, Pr, Tau, Nr) in {"a": (9000.0, 2.0, 2.0, 500.0, 1.0, 1.0, 20),
                                               "b": (4525.9, 13.0, 0.31325, 150.0, 1.0, 1.0 / 15.0, 16)}.items():
        D, R = LMO.cheb_radial(Nr, d)
        out[f"D_{tag}"], out[f"R_{tag}"] = D, R
        out[f"ML0_{tag}"] = np.asarray(LMO.ML_0(D, R, l))
        out[f"Ll0_{tag}"] = np.asarray(LMO.Ll_0(D, R, d, l, Ra, Ra_s, Pr, Tau))
        out[f"vals_{tag}"] = LP.Eig_Vals(Ra, l, d, 5, Ra_s=Ra_s, Pr=Pr, Tau=Tau, Nr=Nr)
        out[f"val1_{tag}"] = LP.Eig_Vals(Ra, l, d, 1, Ra_s=Ra_s, Pr=Pr, Tau=Tau, Nr=Nr)
        for k in (0, 1):
            out[f"vec{k}_{tag}"] = LP.Eig_Vec(Ra, l, d, k, Ra_s=Ra_s, Pr=Pr, Tau=Tau, Nr=Nr)
        out[f"params_{tag}"] = np.array([Ra, l, d, Ra_s, Pr, Tau, Nr])
    f = out["vec0_a"]
    for N_fm in (16, 32):
        out[f"full_{N_fm}"] = LP.Full_Eig_Vec(f, 2.0, N_fm, 19, symmetric=False)
    out["full_sym_16"] = LP.Full_Eig_Vec(f, 2.0, 16, 19, symmetric=True)
    np.savez(os.path.join(HERE, "eigen.npz"), **out)
    print("wrote eigen")


def transform_case():
    """Transforms.py:73-129 on seeded rows, with and without the 3/2 zero-padding length n."""
    rng = np.random.default_rng(7)
    out = {}
    for M in (8, 10, 16, 64):
        P = (3 * M) // 2
        a = rng.standard_normal((3, M))
        g = rng.standard_normal((3, P))
        out[f"IDCT_in_{M}"] = a
        out[f"IDCT_{M}"] = Tr.IDCT(a, n=P)
        out[f"IDST_{M}"] = Tr.IDST(a, n=P)
        out[f"IDCT_nonpad_{M}"] = Tr.IDCT(a)
        out[f"IDST_nonpad_{M}"] = Tr.IDST(a)
        out[f"DCT_in_{M}"] = g
        out[f"DCT_{M}"] = Tr.DCT(g)
        out[f"DST_{M}"] = Tr.DST(g)
        out[f"DCT_trunc_{M}"] = Tr.DCT(g, n=M)
        out[f"DST_trunc_{M}"] = Tr.DST(g, n=M)
        out[f"grid_{M}"] = Tr.grid(P)
    np.savez(os.path.join(HERE, "transforms.npz"), **out)
    print("wrote transforms")


def trajectory_c2_case():
    """The production-size plain configuration: N_r = 30, N_fm = 256, dt = 5e-4, 10^4 steps of the reference's
    own _Time_Step (Main.py:228-329) from the seed-1234 state.  Kept small: the seed, the saved states after
    steps 1, 5001 and 9001 (X_DATA[0], [5], [9]), the final state, and every 10th entry of the per-step
    Norm / KE / Nu_T / Nu_S series."""
    d, Pr, Tau, Ra, Ra_s = (PARAMS[k] for k in ("d", "Pr", "Tau", "Ra", "Ra_s"))
    N_r, N_fm, dt, n_steps = 30, 256, 5e-4, 10000
    nr = N_r - 1
    X0 = seeded_state(N_fm, nr, 1234)
    fname = "golden_c2.h5"
    assert int(n_steps * dt / dt) == n_steps
    XN = Main._Time_Step(X0.copy(), Ra, Ra_s, Tau, Pr, d, N_fm, N_r, False, save_filename=fname,
                         start_time=0, Total_time=n_steps * dt, dt=dt, linear=False, Verbose=False)
    f = H5.File.files[fname]
    XD = np.asarray(f["Checkpoints"]["X_DATA"])
    sd = f["Scalar_Data"]
    out = dict(X_DATA=XD[[0, 5, 9]], saved_steps=np.array([1, 5001, 9001]), X_final=XN,
               Norm=np.asarray(sd["Norm"])[::10], KE=np.asarray(sd["KE"])[::10],
               NuT=np.asarray(sd["Nu_T"])[::10], NuS=np.asarray(sd["Nu_S"])[::10],
               params=np.array([N_r, N_fm, dt, d, Pr, Tau, Ra, Ra_s, 0.0, n_steps, 1234]))
    np.savez(os.path.join(HERE, "traj_c2.npz"), **out)
    print("wrote traj_c2", XD.shape, "|X_N| %.6e" % np.linalg.norm(XN))


def c2_operators_case():
    """The reference's own psi-solve blocks (Build_Matrix_Operators' L_inv_A4, Main.py:205, i.e. numpy's
    LAPACK inverses of A4_TSTEP_MATS, Matrix_Operators.py:1089-1112) for the N_r = 30, N_fm = 256,
    dt = 5e-4 configuration.  These blocks are ill-conditioned: another platform's LAPACK inverts them
    differently by up to ~1e-13 relative, and over 10^4 steps that alone moves the trajectory by ~5e-11, so
    the trajectory check builds its plan from the blocks the reference itself used."""
    d, Pr, Tau = PARAMS["d"], PARAMS["Pr"], PARAMS["Tau"]
    ops = Main.Build_Matrix_Operators(256, 30, d, 5e-4, Pr, Tau)
    np.savez(os.path.join(HERE, "traj_c2_linv_a4.npz"), Linv_A4=np.asarray(ops[5]))
    print("wrote traj_c2_linv_a4")


def layout_case():
    """Matrix_Operators.py:529-627 Vecs_to_X / X_to_Vecs on seeded fields, symmetric and not."""
    rng = np.random.default_rng(51)
    N_fm, nr = 10, 7
    PSI, T, C = (rng.standard_normal((nr, N_fm)) for _ in range(3))
    out = dict(PSI=PSI, T=T, C=C)
    for sym in (False, True):
        X = MO.Vecs_to_X(PSI, T, C, N_fm, nr, sym)
        out[f"X_{int(sym)}"] = X
        P2, T2, C2 = MO.X_to_Vecs(X, N_fm, nr, sym)
        out[f"PSI_{int(sym)}"], out[f"T_{int(sym)}"], out[f"C_{int(sym)}"] = P2, T2, C2
    Xr = rng.standard_normal(3 * N_fm * nr)
    out["X_raw"] = Xr
    for sym in (False, True):
        P2, T2, C2 = MO.X_to_Vecs(Xr, N_fm, nr, sym)
        out[f"PSI_raw_{int(sym)}"], out[f"T_raw_{int(sym)}"], out[f"C_raw_{int(sym)}"] = P2, T2, C2
    np.savez(os.path.join(HERE, "layout.npz"), **out)
    print("wrote layout")


def continuation_run_case(n_steps=11):
    """The reference's branch-following loop _Continuation (Main.py:958-1045) as written, from the
    steady convective state of cont_tau1.npz (N_r = 16, N_fm = 16, Tau = 1, Ra_T = 9000): it starts at
    ds = 0.01 with pseudo-arclength steps (_ContinC), doubling ds after each step that needs <= 4 corrector
    iterations, and switches to natural-parameter Newton steps (_NewtonC, ds doubling up to ds_max = 10) once
    ds > 1.  The record it writes every 5 iterations (Checkpoints/*, Bifurcation/*) comes back through the
    fake h5py File; n_steps = 11 so that the last write holds all 11 iterations."""
    Z = np.load(os.path.join(HERE, "cont_tau1.npz"))
    N_r, N_fm, _, d, Pr, Tau, Ra0, Ra_s, _ = Z["params"]
    kwargs = {"Ra": float(Ra0), "Ra_s": float(Ra_s), "Tau": float(Tau), "Pr": float(Pr), "d": float(d),
              "N_fm": int(N_fm), "N_r": int(N_r), "symmetric": False}
    Y = np.hstack((Z["X_steady"], float(Ra0)))
    fname = "golden_contrun.h5"
    Main._Continuation(fname, n_steps, 1.0, Y, **kwargs)
    f = H5.File.files[fname]
    bif, chk = f["Bifurcation"], f["Checkpoints"]
    out = {k: np.asarray(bif[k]) for k in ("Ra", "Ra_dot", "Norm", "KE", "NuT", "NuS")}
    out["n_folds"] = np.array(len(bif["Y_FOLD"]))
    out["X_DATA"] = np.asarray(chk["X_DATA"])
    out["Ra_DATA"] = np.asarray(chk["Ra_DATA"])
    out["Y0"] = Y
    out["params"] = Z["params"]
    out["n_steps"] = np.array(n_steps)
    np.savez(os.path.join(HERE, "contrun_tau1.npz"), **out)
    print("wrote contrun", "Ra:", np.array2string(out["Ra"], precision=6))


if __name__ == "__main__":
    if "--only-eigen" in OPTS:
        eigen_case()
        sys.exit(0)
    if "--only-interp" in OPTS:
        interp_case()
        sys.exit(0)
    if "--only-continuation" in OPTS:
        continuation_case("tau1", N_r=16, N_fm=16, Ra0=9000.0, Tau=1.0, ds=50.0, n_steps=40000, dt_ts=5e-3, seed=31)
        sys.exit(0)
    if "--only-continuation-run" in OPTS:
        continuation_run_case()
        sys.exit(0)
    if "--only-c2" in OPTS:
        trajectory_c2_case()
        sys.exit(0)
    if "--only-c2-operators" in OPTS:
        c2_operators_case()
        sys.exit(0)
    if "--only-layout" in OPTS:
        layout_case()
        sys.exit(0)
    # the reference's own known-answer tests must pass before anything is recorded (Transforms.py:132-374)
    for k in range(4):
        Tr.test_Cosine_Transform(k, 64)
        Tr.test_Sine_Transform(k + 1, 64)
        Tr.test_Cosine_Transform_deal(k, 64)
        Tr.test_Sine_Transform_deal(k + 1, 64)
    Tr.test_Cosine_Transform_NL(64)
    Tr.test_Sine_Transform_NL(64)
    transform_case()
    operator_case("tiny", N_r=6, N_fm=8, dt=1e-3, symmetric=False, seed=11, store_linv=True)
    operator_case("tiny_sym", N_r=6, N_fm=8, dt=1e-3, symmetric=True, seed=12, store_linv=True)
    operator_case("m10_sym", N_r=8, N_fm=10, dt=5e-3, symmetric=True, seed=13)
    operator_case("c1", N_r=20, N_fm=64, dt=1e-3, symmetric=False, seed=1234)
    operator_case("c1_sym", N_r=20, N_fm=64, dt=1e-3, symmetric=True, seed=1234)
    trajectory_case("c1", N_r=20, N_fm=64, dt=1e-3, n_steps=2000, symmetric=False, seed=1234)
    trajectory_case("tiny", N_r=6, N_fm=8, dt=1e-3, n_steps=200, symmetric=False, seed=21)
    trajectory_case("sym_lin", N_r=8, N_fm=10, dt=5e-3, n_steps=100, symmetric=True, seed=22, linear=True)
    continuation_case("tau1", N_r=16, N_fm=16, Ra0=9000.0, Tau=1.0, ds=50.0, n_steps=40000, dt_ts=5e-3, seed=31)
    interp_case()
    layout_case()
    continuation_run_case()
    trajectory_c2_case()
    c2_operators_case()
