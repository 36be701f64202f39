"""Mixed precision: FP32 nonlinear term (transforms, products, radial contractions) with FP64 right-hand
sides, chains and Newton residual.  Every number is compared against the FP64 path / the oracle."""
import numpy as np
import pytest

from conftest import rel
from oracle import sdd_oracle as O

pytestmark = pytest.mark.gpu


def test_mixed_nlin_fx_error_is_fp32_level(cuda):
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 64, 20
    pm = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01, precision="mixed")
    pd = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01)
    X = torch.from_numpy(O.seeded_state(N_fm, N_r - 1, 1234)).cuda().reshape(1, -1)
    # one step: the FP32 error enters through dt * F
    e = rel(pm.step(X, 8000.0, 500.0).cpu().numpy(), pd.step(X, 8000.0, 500.0).cpu().numpy())
    assert 1e-12 < e < 1e-6, e


def test_mixed_trajectory_to_t5(cuda):
    """Config 'mixed precision, N_r=20, N_theta=64': 5000 steps of dt=1e-3 (t = 5); the error against the FP64
    path (which matches the oracle to 1e-11) is reported and bounded.  The FP32 nonlinear term enters each step
    through dt * F, so the drift stays near FP32 rounding times the step's nonlinear share (measured ~1e-8 on
    GB300, tensor-core contractions included); 5e-8 leaves room for rounding-order changes only."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 64, 20
    pm = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01, precision="mixed")
    pd = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01)
    X = torch.from_numpy(O.seeded_state(N_fm, N_r - 1, 1234)).cuda().reshape(1, -1)
    Xm = pm.step(X, 8000.0, 500.0, nsteps=5000)
    Xd = pd.step(X, 8000.0, 500.0, nsteps=5000)
    e = rel(Xm.cpu().numpy(), Xd.cpu().numpy())
    print(f"mixed vs FP64 relative error at t=5: {e:.3e}")
    assert e < 5e-8


def test_mixed_newton_reaches_fp64_residual(cuda):
    """Inexact Newton: FP32 nonlinear term inside the Jacobian products, FP64 residual; the residual is
    re-checked with the oracle."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 64, 20
    p = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01, precision="mixed")
    X0 = O.seeded_state(N_fm, N_r - 1, 1234)
    X = torch.from_numpy(X0).cuda().reshape(1, -1)
    r = p.newton(X, 8000.0, 500.0, tol=1e-10, mixed_matvec=True)[0]
    assert r["converged"] and r["residual"] <= 1e-10, r
    ops1 = O.Operators(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    assert np.linalg.norm(O.PFX(ops1, X.cpu().numpy().ravel(), 8000.0, 500.0, False)) <= 1.5e-10


@pytest.mark.parametrize("layout", [0, 2, 4, 5])
def test_fp32_rhs_newton_matches_mixed_newton(cuda, layout):
    """mixed_matvec=2: FP32 right-hand sides and h = Linv g matvecs inside the Jacobian products as well (the
    chains and the residual stay FP64).  A batch of shells (perturbed states, different Ra_T) reaches the
    FP64 residual, the oracle's residual agrees, and the steady states equal those of mixed_matvec=1."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r, B = 64, 20, 4
    p = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01, precision="mixed")
    p.set_chain_layout(layout)
    X0 = np.stack([O.seeded_state(N_fm, N_r - 1, 1234 + i) for i in range(B)])
    Ra = torch.tensor([7000.0, 8000.0, 9000.0, 10000.0], dtype=torch.float64, device="cuda")
    X1 = torch.from_numpy(X0).cuda()
    X2 = X1.clone()
    r1 = p.newton(X1, Ra, 500.0, tol=1e-10, mixed_matvec=1)
    r2 = p.newton(X2, Ra, 500.0, tol=1e-10, mixed_matvec=2)
    ops1 = O.Operators(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    for b in range(B):
        assert r2[b]["converged"] and r2[b]["residual"] <= 1e-10, (b, r2[b])
        assert np.linalg.norm(O.PFX(ops1, X2[b].cpu().numpy(), float(Ra[b]), 500.0, False)) <= 1.5e-10
        assert r2[b]["newton_iters"] <= r1[b]["newton_iters"] + 1, (r1[b], r2[b])
    # both converge to the same steady states (to the Newton tolerance)
    d = (X2 - X1).norm().item()
    assert d <= 1e-8 * max(1.0, X1.norm().item()), d
    assert r2[0]["matvecs"] <= 1.25 * r1[0]["matvecs"] + 2, (r1[0]["matvecs"], r2[0]["matvecs"])


def test_fp32_rhs_newton_requires_mixed_plan(cuda):
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    from spectraldoublediffusiveconvection_gb300 import _lib
    torch = cuda
    p = Plan(16, 8, 2.0, 1.0, 1.0, 0.01)
    X = torch.from_numpy(O.seeded_state(16, 7, 3)).cuda().reshape(1, -1)
    with pytest.raises(_lib.SDDError):
        p.newton(X, 8000.0, 500.0, mixed_matvec=2)
    with pytest.raises(_lib.SDDError):
        p.newton(X, 8000.0, 500.0, mixed_matvec=3)
    with pytest.raises(ValueError):
        p.newton(X, 8000.0, 500.0, mixed_matvec=4)


def _nontrivial_batch(N_r, N_fm, B, seed):
    from conftest import load_golden
    G = load_golden("cont_tau1.npz")
    _, _, _, d, Pr, Tau, Ra, Ra_s, _ = G["params"]
    X = O.INTERP_THETAS(N_fm, 16, O.INTERP_RADIAL(N_r, 16, G["X_steady"], d))
    rng = np.random.default_rng(seed)
    Xs = np.stack([X + 1e-3 * np.linalg.norm(X) / np.sqrt(X.size) * rng.standard_normal(X.size) for _ in range(B)])
    return Xs, d, Pr, Tau, Ra, Ra_s


@pytest.mark.parametrize("layout", [0, 4])
def test_fp32_basis_newton_reaches_fp64_residual(cuda, layout):
    """mixed_matvec=3: the GMRES basis stored and orthogonalised in FP32 on top of mode 2's FP32 products.
    From a nontrivial start (a convective steady state interpolated and perturbed, three Ra_T) every shell
    reaches the FP64 residual 1e-10, the oracle's residual of the result agrees, the steady states equal
    mode 2's to the Newton tolerance, and the products needed stay within a few of mode 2's."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_r, N_fm, B = 24, 32, 3
    Xs, d, Pr, Tau, Ra, Ra_s = _nontrivial_batch(N_r, N_fm, B, 11)
    p = Plan(N_fm, N_r, d, 1.0, Pr, Tau, precision="mixed")
    p.set_chain_layout(layout)
    Ra_t = torch.tensor([Ra - 100.0, Ra, Ra + 100.0], dtype=torch.float64, device="cuda")
    X2 = torch.from_numpy(Xs.copy()).cuda()
    X3 = X2.clone()
    r2 = p.newton(X2, Ra_t, Ra_s, tol=1e-10, mixed_matvec=2)
    r3 = p.newton(X3, Ra_t, Ra_s, tol=1e-10, mixed_matvec=3)
    ops1 = O.Operators(N_fm, N_r, d, 1.0, Pr, Tau)
    for b in range(B):
        assert r3[b]["converged"] and r3[b]["residual"] <= 1e-10, (b, r3[b])
        x = X3[b].cpu().numpy()
        assert np.linalg.norm(x) > 1.0                   # a convective state, not X = 0
        assert np.linalg.norm(O.PFX(ops1, x, float(Ra_t[b]), Ra_s, False)) <= 1.5e-10
        assert r3[b]["newton_iters"] <= r2[b]["newton_iters"] + 1, (r2[b], r3[b])
        assert rel(x, X2[b].cpu().numpy()) <= 1e-9
    print("products: mode 2 %d, mode 3 %d" % (r2[0]["matvecs"], r3[0]["matvecs"]))
    assert r3[0]["matvecs"] <= 1.25 * r2[0]["matvecs"] + 4, (r2[0]["matvecs"], r3[0]["matvecs"])


def test_fp32_basis_is_orthonormal_to_fp32_level(cuda):
    """The FP32 basis after 40-50-column cycles (tight inner tolerance) is orthonormal to FP32 rounding,
    |V^T V - I|_max <= 1e-5, read back through sdd_krylov_basis (widened to FP64)."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_r, N_fm, B = 24, 32, 2
    Xs, d, Pr, Tau, Ra, Ra_s = _nontrivial_batch(N_r, N_fm, B, 9)
    p = Plan(N_fm, N_r, d, 1.0, Pr, Tau, precision="mixed")
    Xt = torch.from_numpy(Xs).cuda()
    Ra_t = torch.tensor([Ra, Ra + 100.0], dtype=torch.float64, device="cuda")
    p.newton(Xt, Ra_t, Ra_s, tol=1e-12, restart=50, gmres_rtol=1e-13, max_newton=1, max_restarts=2, mixed_matvec=3)
    worst = 0.0
    for b in range(B):
        V = p.krylov_basis(b, 64)
        assert V.shape[0] >= 40, V.shape
        assert torch.equal(V, V.float().double())       # the stored vectors are FP32 values
        err = float((V @ V.T - torch.eye(V.shape[0], dtype=torch.float64, device="cuda")).abs().max())
        worst = max(worst, err)
    print(f"FP32 basis: max |V^T V - I| = {worst:.2e}")
    assert worst <= 1e-5


def test_fp32_basis_continuation_step(cuda):
    """One pseudo-arclength step (bordered system, n + 1 unknowns) with mixed_matvec=3 lands on mode 2's branch
    point: Ra to 1e-8 relative, the state to 1e-7, corrector residual <= 1e-10."""
    from conftest import load_golden
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    Z = load_golden("cont_tau1.npz")
    N_r, N_fm, dt, d, Pr, Tau, Ra0, Ra_s, sym = Z["params"]
    p = Plan(int(N_fm), int(N_r), d, 1.0, Pr, Tau, precision="mixed")
    out = []
    for mv in (2, 3):
        X = torch.from_numpy(Z["X_steady"].copy()).cuda().reshape(1, -1)
        Ra = torch.tensor([Ra0], dtype=torch.float64, device="cuda")
        Xd, res = p.contin_step(X, Ra, Ra_s, sign=1.0, ds=float(Z["ds"]), tol=1e-10, mixed_matvec=mv)
        assert res[0]["converged"] and res[0]["residual"] <= 1e-10, res[0]
        out.append((X.cpu().numpy().ravel(), float(Ra[0])))
    assert abs(out[1][1] - out[0][1]) <= 1e-8 * abs(out[0][1])
    assert rel(out[1][0], out[0][0]) <= 1e-7


def test_mixed_plan_at_the_largest_shape(cuda):
    """Mixed precision at the largest accepted shape (N_r = 65, N_theta = 540: tensor-core tiles with K = N =
    64, the widest accumulator): two steps against the FP64 plan at FP32 level, and Newton with the FP32
    basis (mixed_matvec=3) reaching the FP64 residual 1e-10."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_r, N_fm = 65, 540
    X = torch.from_numpy(O.seeded_state(N_fm, N_r - 1, 4)).cuda().reshape(1, -1)
    pm = Plan(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01, precision="mixed")
    pd = Plan(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01)
    e = rel(pm.step(X, 8000.0, 500.0, nsteps=2).cpu().numpy(), pd.step(X, 8000.0, 500.0, nsteps=2).cpu().numpy())
    assert e < 1e-6, e
    assert not pm.tensor_core_timed_out()
    pn = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01, precision="mixed")
    Xn = X.clone()
    r = pn.newton(Xn, 8000.0, 500.0, tol=1e-10, mixed_matvec=3)[0]
    assert r["converged"] and r["residual"] <= 1e-10, r
