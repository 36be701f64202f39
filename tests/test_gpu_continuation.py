"""Pseudo-arclength continuation (Main.py:742-955) on the GPU against the reference's own _ContinC step.

The golden (tests/golden/cont_tau1.npz, made by running the reference) starts from a nontrivial steady
convective state at Ra_T = 9000 (N_r=16, N_fm=16, Tau=1, Ra_S=500, d=2) and takes one arclength step with
ds=50, sign=+1.  The reference's corrector stops on a relative step of 1e-8; the GPU's on an absolute
residual of 1e-10, so the two branch points agree to the reference's own accuracy (checked at 1e-6)."""
import numpy as np
import pytest

from conftest import load_golden, rel
from oracle import sdd_oracle as O

pytestmark = pytest.mark.gpu


def _golden():
    Z = load_golden("cont_tau1.npz")
    N_r, N_fm, dt, d, Pr, Tau, Ra0, Ra_s, sym = Z["params"]
    return Z, int(N_r), int(N_fm), d, Pr, Tau, Ra0, Ra_s


def test_contin_step_matches_reference_contin(cuda):
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    Z, N_r, N_fm, d, Pr, Tau, Ra0, Ra_s = _golden()
    p = Plan(N_fm, N_r, d, 1.0, Pr, Tau)
    X = torch.from_numpy(Z["X_steady"].copy()).cuda().reshape(1, -1)
    Ra = torch.tensor([Ra0], dtype=torch.float64, device="cuda")
    Xd, res = p.contin_step(X, Ra, Ra_s, sign=1.0, ds=float(Z["ds"]), tol=1e-10, tangent_rtol=1e-12)
    r = res[0]
    assert r["converged"] and r["residual"] <= 1e-10 and r["arclength"] <= 1e-10, r
    Y = Z["Y"]
    assert abs(float(Ra.item()) - Y[-1]) <= 1e-6 * abs(Y[-1])
    assert rel(X.cpu().numpy().ravel(), Y[:-1]) <= 1e-6
    # new tangent: parameter component against the reference's; state component against the exact
    # direction y_X = y_mu xi, xi = -J^{-1} J_mu from a dense solve with the oracle (n = 720), with the tangent
    # solved to 1e-12.  The reference's own lgmres tangent misses that direction by 34% in its (small) state
    # part, so it is not the yardstick.
    Yd = Z["Y_dot"]
    assert abs(r["Ra_dot"] - Yd[-1]) <= 1e-6 * abs(Yd[-1])
    assert r["ds"] == pytest.approx(float(Z["ds_new"]))
    ops1 = O.Operators(N_fm, N_r, d, 1.0, Pr, Tau)
    Xg, mu = X.cpu().numpy().ravel(), float(Ra.item())
    n, N = Xg.size, Xg.size // 3
    Jd = np.stack([O.PDFX(ops1, e, Xg, mu, Ra_s, False) for e in np.eye(n)], axis=1)
    g = O._gr_apply(ops1, Xg[N:2 * N]) * Pr
    jmu = np.zeros(n)
    jmu[:N] = O.A4_BSub_TSTEP_V2(g, ops1.Linv_A4, ops1.D2_A4, ops1.IR4_A4, ops1.IR2_A4, N_fm, N_r - 1, Pr, False)
    xi = -np.linalg.solve(Jd, jmu)
    assert rel(Xd.cpu().numpy().ravel(), r["Ra_dot"] * xi) <= 1e-5
    # independent residual check with the oracle
    assert np.linalg.norm(O.PFX(ops1, Xg, mu, Ra_s, False)) <= 1.5e-10


def test_contin_step_on_the_conduction_branch(cuda):
    """On X = 0, F = 0 and DF_mu = 0 for every Ra: xi = 0, mu_dot = 1/sqrt(1 - delta) and the step lands
    exactly at Ra0 + ds/sqrt(1 - delta) with X = 0 and no corrector iteration."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 64, 20
    p = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    X = torch.zeros((2, p.n_state), dtype=torch.float64, device="cuda")
    Ra = torch.tensor([8000.0, 9000.0], dtype=torch.float64, device="cuda")
    Xd, res = p.contin_step(X, Ra, 500.0, sign=[1.0, -1.0], ds=[50.0, 20.0], tol=1e-10)
    delta = 1.0 / p.n_state
    assert all(r["converged"] and r["corrector_iters"] == 0 for r in res)
    assert float(X.abs().max()) == 0.0
    assert float(Ra[0]) == pytest.approx(8000.0 + 50.0 / np.sqrt(1 - delta), rel=1e-14)
    assert float(Ra[1]) == pytest.approx(9000.0 - 20.0 / np.sqrt(1 - delta), rel=1e-14)


def test_main_contin_and_continuation_dropins(cuda):
    from spectraldoublediffusiveconvection_gb300 import Main
    Z, N_r, N_fm, d, Pr, Tau, Ra0, Ra_s = _golden()
    kw = dict(Ra=Ra0, Ra_s=Ra_s, Tau=Tau, Pr=Pr, d=d, N_fm=N_fm, N_r=N_r, symmetric=False)
    Y0 = np.hstack((Z["X_steady"], Ra0))
    Y_dot, Y, sign, ds, Norm, KE, NuT, NuS, ok = Main._ContinC(0 * Y0, Y0, 1.0, 50.0, tol_newton=1e-10, **kw)
    assert ok and abs(Y[-1] - Z["Y"][-1]) <= 1e-6 * Z["Y"][-1]
    assert abs(Norm - float(Z["Norm"])) <= 1e-6 * float(Z["Norm"])
    assert abs(NuT - float(Z["NuT"])) <= 1e-6 * abs(float(Z["NuT"]))
    kw2 = {k: v for k, v in kw.items() if k != "Ra"}
    R = Main._Continuation(None, 3, 1.0, Y0, Ra=Ra0, **kw2)
    assert len(R.Ra) == 3 and R.Ra[-1] > Ra0


def test_continuation_run_matches_reference_run(cuda):
    """Main._Continuation (Main.py:958-1045) against 11 iterations of the reference's own loop from the same
    steady state (tests/golden/contrun_tau1.npz): 7 pseudo-arclength steps with ds doubling 0.01 -> 1.28, the
    switch to natural-parameter Newton steps once ds > 1, and ds doubling up to ds_max = 10.  The Ra
    sequence, the scalar records, the checkpointed states (iterations 0, 5, 10) and the tangent's parameter
    component carried through the natural steps all agree at the reference's own accuracy: its correctors and
    Newton stop on a relative step of 1e-8, this build's on an absolute residual of 1e-8, so states agree to
    about 1e-7 and the parameter to 1e-9 of its increments (checked at 1e-6 and 1e-6)."""
    from spectraldoublediffusiveconvection_gb300 import Main
    Z = load_golden("contrun_tau1.npz")
    N_r, N_fm, _, d, Pr, Tau, Ra0, Ra_s, _ = Z["params"]
    kw = dict(Ra=float(Ra0), Ra_s=float(Ra_s), Tau=float(Tau), Pr=float(Pr), d=float(d), N_fm=int(N_fm),
              N_r=int(N_r), symmetric=False)
    R = Main._Continuation(None, int(Z["n_steps"]), 1.0, Z["Y0"], **kw)
    Ra = np.array(R.Ra)
    assert Ra.shape == Z["Ra"].shape
    # arclength steps: Ra to 1e-6 of its distance from Ra0 (9000.01 .. 9001.27) and 1e-9 relative overall
    assert np.all(np.abs(Ra - Z["Ra"]) <= 1e-6 * np.abs(Z["Ra"] - Ra0) + 1e-9 * Ra0), (Ra, Z["Ra"])
    # then natural-parameter steps of ds = 1.28, 2.56, 5.12 and ds_max = 10
    assert np.allclose(np.diff(Ra)[-4:], [1.28, 2.56, 5.12, 10.0], rtol=0, atol=1e-9)
    assert np.allclose(R.Ra_dot, Z["Ra_dot"], rtol=1e-6, atol=0)
    for k in ("Norm", "KE", "NuT", "NuS"):
        assert np.allclose(getattr(R, k), Z[k], rtol=1e-6, atol=0), k
    assert len(R.Y_FOLD) == int(Z["n_folds"])
    assert len(R.X_DATA) == len(Z["X_DATA"])
    for a, b in zip(R.X_DATA, Z["X_DATA"]):
        assert rel(a, b) <= 1e-6
    assert np.allclose(R.Ra_DATA, Z["Ra_DATA"], rtol=1e-12, atol=1e-6)
    # the state stays on the device: the record's last branch point is a CUDA tensor
    assert R.X.is_cuda and rel(R.X.cpu().numpy(), R.X_DATA[-1]) == 0.0
