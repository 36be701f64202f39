"""Request server (continuous batching of integrations, batched continuation steps) on the GPU.

Each served result must equal the same request run alone through a plan with the same chain layout, bit
for bit: batching across requests may change which shells share a launch, never a shell's arithmetic.
The branch seed is the reference's steady state at Ra_T = 9000 (N_r=16, N_fm=16, Tau=1) from
tests/golden/cont_tau1.npz."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import sdd_oracle as O

pytestmark = pytest.mark.gpu

D, PR, TAU, RAS = 2.0, 1.0, 1.0, 500.0


@pytest.fixture(scope="module")
def branch(cuda):
    from spectraldoublediffusiveconvection_gb300 import serve
    Z = load_golden("cont_tau1.npz")
    N_r, N_fm = int(Z["params"][0]), int(Z["params"][1])
    return serve.branch_states([(16, 16), (20, 32)], Ra=9000.0, d=D, Pr=PR, Tau=TAU, Ra_s=RAS,
                               source=(Z["X_steady"], N_r, N_fm))


def test_branch_states_are_steady(branch):
    assert set(branch) == {(16, 16), (20, 32)}
    for (N_r, M), (X, res) in branch.items():
        assert res <= 1e-10
        ops1 = O.Operators(M, N_r, D, 1.0, PR, TAU)
        assert np.linalg.norm(O.PFX(ops1, X, 9000.0, RAS, False)) <= 1.5e-10
        assert np.linalg.norm(X) > 0.1          # a convective state, not the conduction branch


def _requests(serve, branch):
    reqs = []
    for (shape, Ra, n) in [((16, 16), 8700.0, 120), ((20, 32), 9100.0, 75), ((16, 16), 9300.0, 200)]:
        reqs.append(serve.Request("integrate", shape[0], shape[1], Ra, n_steps=n, seed=len(reqs) + 7))
    for (shape, sign) in [((16, 16), 1.0), ((20, 32), -1.0), ((16, 16), -1.0), ((20, 32), 1.0)]:
        reqs.append(serve.Request("continue", shape[0], shape[1], 9000.0, X=branch[shape][0], sign=sign, ds=50.0))
    return reqs


def test_served_results_equal_alone(cuda, branch):
    from spectraldoublediffusiveconvection_gb300 import serve
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    srv = serve.Server(d=D, Pr=PR, Tau=TAU, Ra_s=RAS, dt=1e-3, quantum=50).start()
    reqs = _requests(serve, branch)
    for r in reqs:
        srv.submit(r)
    assert srv.drain(timeout=300)
    srv.stop()
    assert all(r.error is None and r.result is not None for r in reqs), [r.error for r in reqs]
    assert srv.used == 0
    for r in reqs:
        if r.kind == "integrate":
            p = Plan(r.N_theta, r.N_r, D, 1e-3, PR, TAU, precision=srv.int_precision)
            p.set_chain_layout(srv.chain_layout)
            X = torch.from_numpy(serve._seeded(r.N_theta, r.N_r - 1, r.seed)).cuda().reshape(1, -1)
            Y = p.step(X, r.Ra, RAS, nsteps=r.n_steps)
            assert np.array_equal(Y.cpu().numpy().ravel(), r.result["X"]), r.id
        else:
            p = Plan(r.N_theta, r.N_r, D, 1.0, PR, TAU, precision="mixed")
            p.set_chain_layout(srv.chain_layout)
            X = torch.from_numpy(np.asarray(r.X).copy()).cuda().reshape(1, -1)
            Ra = torch.tensor([r.Ra], dtype=torch.float64, device="cuda")
            Xd, res = p.contin_step(X, Ra, RAS, r.sign, r.ds, tol=1e-10, restart=50, mixed_matvec=srv.con_mixed,
                                    tangent_rtol=srv.tangent_rtol)
            assert res[0]["converged"] and r.result["converged"]
            assert np.array_equal(X.cpu().numpy().ravel(), r.result["X"]), r.id
            assert float(Ra.item()) == r.result["Ra"]
            assert np.array_equal(Xd.cpu().numpy().ravel(), r.result["X_dot"]), r.id


def test_served_continuation_steps_reach_fp64_residual(cuda, branch):
    from spectraldoublediffusiveconvection_gb300 import serve
    srv = serve.Server(d=D, Pr=PR, Tau=TAU, Ra_s=RAS).start()
    reqs = [srv.submit(serve.Request("continue", 16, 16, 9000.0, X=branch[(16, 16)][0], sign=s, ds=50.0))
            for s in (1.0, -1.0)]
    assert srv.drain(timeout=300)
    srv.stop()
    ops1 = O.Operators(16, 16, D, 1.0, PR, TAU)
    Ras = []
    for r in reqs:
        res = r.result
        assert res["converged"] and res["residual"] <= 1e-10
        assert np.linalg.norm(O.PFX(ops1, res["X"], res["Ra"], RAS, False)) <= 1.5e-10
        Ras.append(res["Ra"])
    assert Ras[0] != Ras[1]                      # the two signs step to opposite sides along the branch
    lat = serve.latency_report(reqs)
    assert lat["n"] == 2 and lat["p99_ms"] >= lat["p50_ms"] > 0


def test_poisson_workload_runs_to_completion(cuda, branch):
    from spectraldoublediffusiveconvection_gb300 import serve
    srv = serve.Server(d=D, Pr=PR, Tau=TAU, Ra_s=RAS).start()
    wl = serve.poisson_workload(24, 400.0, [(16, 16), (20, 32)], branch, n_steps=100, seed=5)
    wall = serve.run_workload(srv, wl)
    srv.stop()
    reqs = [r for _, r in wl]
    assert all(r.done.is_set() and r.error is None for r in reqs)
    assert all(r.result["converged"] and r.result["residual"] <= 1e-10 for r in reqs if r.kind == "continue")
    assert wall > 0 and srv.stats["int_steps"] == sum(r.n_steps for r in reqs if r.kind == "integrate")
