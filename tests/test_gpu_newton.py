"""GPU Newton-GMRES and the Main.py drop-in drivers against the oracle.

The seeded states of the benchmark converge to the conduction state X = 0 (Ra_T = 8000 .. 30000), so
the convergence test is checked independently: the oracle's residual PFX evaluated at the GPU's solution
must also be <= 1e-10.
"""
import numpy as np
import pytest

from conftest import load_golden, rel
from oracle import sdd_oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N_r,N_fm", [(20, 64), (30, 256)])
def test_newton_converges_and_oracle_agrees(cuda, N_r, N_fm):
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    nr = N_r - 1
    d, Pr, Tau, Ra, Ra_s = 2.0, 1.0, 0.01, 8000.0, 500.0
    p = Plan(N_fm, N_r, d, 1.0, Pr, Tau)
    X0 = O.seeded_state(N_fm, nr, 1234)
    X = torch.from_numpy(X0).cuda().reshape(1, -1)
    res = p.newton(X, Ra, Ra_s, tol=1e-10, restart=50)[0]
    assert res["converged"] and res["residual"] <= 1e-10, res
    assert 2 <= res["newton_iters"] <= 8
    ops1 = O.Operators(N_fm, N_r, d, 1.0, Pr, Tau)
    Xg = X.cpu().numpy().ravel()
    assert np.linalg.norm(O.PFX(ops1, Xg, Ra, Ra_s, False)) <= 1.5e-10
    assert abs(res["residual0"] - np.linalg.norm(O.PFX(ops1, X0, Ra, Ra_s, False))) <= 1e-12 * res["residual0"]


def test_newton_batch_matches_single(cuda):
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 64, 20
    p = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    Xs = np.stack([O.seeded_state(N_fm, N_r - 1, s) for s in (1, 2, 3)])
    Ra = torch.tensor([6000.0, 9000.0, 12000.0], dtype=torch.float64, device="cuda")
    Xb = torch.from_numpy(Xs).cuda()
    rb = p.newton(Xb, Ra, 500.0, tol=1e-10)
    for i in range(3):
        Xi = torch.from_numpy(Xs[i:i + 1].copy()).cuda()
        ri = p.newton(Xi, float(Ra[i]), 500.0, tol=1e-10)[0]
        assert rb[i]["converged"] and ri["converged"]
        assert rb[i]["newton_iters"] == ri["newton_iters"]
        assert rel(Xb[i].cpu().numpy(), Xi[0].cpu().numpy()) <= 1e-13 or \
            np.linalg.norm(Xb[i].cpu().numpy() - Xi[0].cpu().numpy()) <= 1e-14


def test_newton_iteration_cap_reports_failure(cuda):
    """A forced cap of one Newton iteration cannot reach 1e-10: status not converged, no exception."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    p = Plan(64, 20, 2.0, 1.0, 1.0, 0.01)
    X = torch.from_numpy(O.seeded_state(64, 19, 7)).cuda().reshape(1, -1)
    r = p.newton(X, 8000.0, 500.0, tol=1e-10, max_newton=1)[0]
    assert not r["converged"] and r["newton_iters"] == 1 and r["residual"] > 1e-10


def test_jacobian_matches_finite_difference(cuda):
    """PDFX on the GPU against a central difference of PFX on the GPU (independent of the oracle)."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    p = Plan(64, 20, 2.0, 1.0, 1.0, 0.01)
    X = torch.from_numpy(O.seeded_state(64, 19, 5) * 50).cuda().reshape(1, -1)
    v = torch.from_numpy(O.seeded_state(64, 19, 6)).cuda().reshape(1, -1)
    eps = 1e-4
    fd = (p.pfx(X + eps * v, 8000.0, 500.0) - p.pfx(X - eps * v, 8000.0, 500.0)) / (2 * eps)
    J = p.pdfx(v, X, 8000.0, 500.0)
    assert rel(J.cpu().numpy(), fd.cpu().numpy()) < 1e-7


def test_main_time_step_dropin(cuda):
    from spectraldoublediffusiveconvection_gb300 import Main
    Z = load_golden("traj_tiny.npz")
    N_r, N_fm, dt, d, Pr, Tau, Ra, Ra_s, sym, ns = Z["params"]
    X = Main._Time_Step(Z["X0"].copy(), Ra, Ra_s, Tau, Pr, d, int(N_fm), int(N_r), bool(sym), save_filename=None,
                        start_time=0, Total_time=int(ns) * dt, dt=dt)
    assert isinstance(X, np.ndarray)
    assert rel(X, Z["X_final"]) < 1e-11


def test_main_newton_dropin(cuda):
    from spectraldoublediffusiveconvection_gb300 import Main
    X0 = O.seeded_state(64, 19, 1234)
    out = Main._Newton(X0, 8000.0, 500.0, 0.01, 1.0, 2.0, 64, 20, False, tol_newton=1e-10)
    X, Norm, KE, NuT, NuS, ok = out
    assert ok and Norm < 1e-8 and np.isfinite(KE)


def test_main_build_matrix_operators_matches_reference_tuple(cuda):
    from spectraldoublediffusiveconvection_gb300 import Main
    Z = load_golden("ops_tiny.npz")
    ops = Main.Build_Matrix_Operators(8, 6, 2.0, 1e-3, 1.0, 0.01)
    D, R, Rsq, DT0, gr_k, LA4, LT, LS, args_A4, args_FX = ops
    assert rel(np.array(LA4), Z["Linv_A4"]) < 1e-14
    assert rel(np.array(LT), Z["Linv_T"]) < 1e-14
    assert rel(args_A4[0], Z["D2_A4"]) < 1e-14
    assert Rsq.shape == (8 * 5, 8 * 5) and gr_k.shape == (8 * 5, 8 * 5)


def test_krylov_basis_stays_orthonormal(cuda):
    """The GMRES basis after 40-50-column cycles of a batched mixed-precision Newton solve (FP32 nonlinear term,
    right-hand sides and h in the products; FP64 basis) stays orthonormal, |V^T V - I|_max <= 1e-10, with the
    default conditional second Gram-Schmidt pass (|w'| < |w|/sqrt(2)).  A nontrivial start (a convective
    steady state interpolated and perturbed) and a tight inner tolerance keep the cycles long.  A threshold of
    1e-2 was measured to lose orthogonality entirely on this problem (|V^T V - I| = 1): classical Gram-Schmidt
    compounds each skipped pass's loss."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    G = load_golden("cont_tau1.npz")
    _, _, _, d, Pr, Tau, Ra, Ra_s, _ = G["params"]
    N_r, N_fm, B = 24, 32, 3
    X = O.INTERP_THETAS(N_fm, 16, O.INTERP_RADIAL(N_r, 16, G["X_steady"], d))
    rng = np.random.default_rng(9)
    Xs = np.stack([X + 1e-2 * np.linalg.norm(X) / np.sqrt(X.size) * rng.standard_normal(X.size) for _ in range(B)])
    p = Plan(N_fm, N_r, d, 1.0, Pr, Tau, precision="mixed")
    Xt = torch.from_numpy(Xs).cuda()
    Ra_t = torch.tensor([Ra - 100.0, Ra, Ra + 100.0], dtype=torch.float64, device="cuda")
    p.newton(Xt, Ra_t, Ra_s, tol=1e-12, restart=50, gmres_rtol=1e-13, max_newton=1, max_restarts=2, mixed_matvec=2)
    worst = 0.0
    for b in range(B):
        V = p.krylov_basis(b, 64)
        assert V.shape[0] >= 40, V.shape                 # a cycle stops early only once the target is met
        err = float((V @ V.T - torch.eye(V.shape[0], dtype=torch.float64, device="cuda")).abs().max())
        worst = max(worst, err)
    print(f"max |V^T V - I| over {B} shells, cycles of 40-50 columns: {worst:.2e}")
    assert worst <= 1e-10


def test_product_graphs_replay_and_match_direct_launches(cuda):
    """The GMRES products of Newton and of the pseudo-arclength step run as captured CUDA graphs (one capture
    per batch size and kind; every Arnoldi column reads the same fixed vector), with exactly the results of
    the same kernels launched one by one; a kernel-choice change recaptures."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    from conftest import load_golden
    torch = cuda
    N_fm, N_r = 64, 20
    X0 = np.stack([O.seeded_state(N_fm, N_r - 1, s) for s in (4, 5)])
    out = []
    for graphs in (True, False):
        p = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
        p.set_product_graphs(graphs)
        X = torch.from_numpy(X0.copy()).cuda()
        r = p.newton(X, 8000.0, 500.0, tol=1e-10)
        st = p.product_graph_stats()
        if graphs:
            assert st["direct"] == 0 and 1 <= st["captured"] <= 2 and st["replayed"] >= r[0]["matvecs"] - 2
            X2 = torch.from_numpy(X0.copy()).cuda()
            p.newton(X2, 8000.0, 500.0, tol=1e-10)
            assert p.product_graph_stats()["captured"] == st["captured"]      # the second solve replays
            assert torch.equal(X2, X)
            p.set_chain_layout(1)                                             # a kernel choice: recaptured
            X3 = torch.from_numpy(X0.copy()).cuda()
            p.newton(X3, 8000.0, 500.0, tol=1e-10)
            assert p.product_graph_stats()["captured"] > st["captured"]
        else:
            assert st["captured"] == 0 and st["replayed"] == 0 and st["direct"] >= r[0]["matvecs"]
        out.append((X.cpu().numpy(), [x["matvecs"] for x in r]))
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1] == out[1][1]
    # the bordered products of a continuation step
    Z = load_golden("cont_tau1.npz")
    N_r2, N_fm2, _, d, Pr, Tau, Ra0, Ra_s, _ = Z["params"]
    res = []
    for graphs in (True, False):
        p = Plan(int(N_fm2), int(N_r2), d, 1.0, Pr, Tau)
        p.set_product_graphs(graphs)
        X = torch.from_numpy(Z["X_steady"].copy()).cuda().reshape(1, -1)
        Ra = torch.tensor([Ra0], dtype=torch.float64, device="cuda")
        Xd, r = p.contin_step(X, Ra, Ra_s, sign=1.0, ds=50.0, tol=1e-10)
        assert r[0]["converged"]
        if graphs:
            assert p.product_graph_stats()["direct"] == 0
        res.append((X.cpu().numpy(), Ra.cpu().numpy(), Xd.cpu().numpy()))
    for a, b in zip(*res):
        assert np.array_equal(a, b)
