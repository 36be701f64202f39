"""Failure paths, all injected on the host (no GPU fault, trap or hang is provoked):

* a NaN state into Newton-GMRES and into the pseudo-arclength step: that shell stops at once and is reported
  not converged (the reference returns its "could not converge" flag, Main.py:541-544, or raises,
  Main.py:888-899, 923), while the other shells of the same batched call converge as they do alone;
* a refused workspace allocation (sdd_debug_fail_allocations: the library's allocator refuses on the host
  before cudaMalloc is called): SDD_ERR_NOMEM reaches Python as a MemoryError, and the plan works again once
  allocations succeed;
* served requests with a NaN state complete with an error while the rest of the mix completes normally, and
  a cancelled in-flight integration is retired at its next quantum.
"""
import numpy as np
import pytest

from conftest import rel
from oracle import sdd_oracle as O

pytestmark = pytest.mark.gpu


def test_newton_nan_shell_stops_and_others_converge(cuda):
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 64, 20
    p = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    good = O.seeded_state(N_fm, N_r - 1, 3)
    bad = good.copy()
    bad[17] = np.nan
    Xb = torch.from_numpy(np.stack([good, bad, good])).cuda()
    res = p.newton(Xb, 8000.0, 500.0, tol=1e-10)
    assert not res[1]["converged"] and res[1]["newton_iters"] == 0 and not np.isfinite(res[1]["residual"])
    Xi = torch.from_numpy(good.copy()).cuda().reshape(1, -1)
    ri = p.newton(Xi, 8000.0, 500.0, tol=1e-10)[0]
    for b in (0, 2):
        assert res[b]["converged"] and res[b]["newton_iters"] == ri["newton_iters"]
        assert np.linalg.norm(Xb[b].cpu().numpy() - Xi[0].cpu().numpy()) <= 1e-14 + 1e-13 * Xi.norm().item()
    # the NaN shell costs no Jacobian products of its own: the batch needs no more than the good shell alone
    assert res[0]["matvecs"] <= ri["matvecs"]
    # an Inf state stops the same way
    Xinf = torch.from_numpy(good.copy()).cuda().reshape(1, -1)
    Xinf[0, 5] = float("inf")
    r = p.newton(Xinf, 8000.0, 500.0, tol=1e-10)[0]
    assert not r["converged"] and r["newton_iters"] == 0 and r["matvecs"] == 0


def test_contin_step_nan_shell_fails_without_iterating(cuda):
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    from conftest import load_golden
    torch = cuda
    Z = load_golden("cont_tau1.npz")
    N_r, N_fm, _, d, Pr, Tau, Ra0, Ra_s, _ = Z["params"]
    p = Plan(int(N_fm), int(N_r), d, 1.0, Pr, Tau)
    Xs = Z["X_steady"]
    bad = Xs.copy()
    bad[3] = np.nan
    X = torch.from_numpy(np.stack([Xs, bad])).cuda()
    Ra = torch.tensor([Ra0, Ra0], dtype=torch.float64, device="cuda")
    _, res = p.contin_step(X, Ra, Ra_s, sign=1.0, ds=50.0, tol=1e-10)
    assert res[0]["converged"] and not res[1]["converged"]
    assert res[1]["corrector_iters"] == 0 and res[1]["halvings"] == 0
    X1 = torch.from_numpy(Xs.copy()).cuda().reshape(1, -1)
    Ra1 = torch.tensor([Ra0], dtype=torch.float64, device="cuda")
    _, r1 = p.contin_step(X1, Ra1, Ra_s, sign=1.0, ds=50.0, tol=1e-10)
    assert rel(X[0].cpu().numpy(), X1[0].cpu().numpy()) <= 1e-12
    assert abs(float(Ra[0]) - float(Ra1[0])) <= 1e-12 * float(Ra1[0])


def test_refused_allocation_raises_memory_error_and_recovers(cuda):
    from spectraldoublediffusiveconvection_gb300 import _lib
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    L = _lib.lib()
    p = Plan(16, 8, 2.0, 1e-3, 1.0, 0.01)
    X = torch.from_numpy(O.seeded_state(16, 7, 2)).cuda().reshape(1, -1)
    try:
        L.sdd_debug_fail_allocations(0)
        with pytest.raises(MemoryError) as ei:
            p.reserve(8)
        assert isinstance(ei.value, _lib.SDDError) and ei.value.status == _lib.SDD_ERR_NOMEM
        with pytest.raises(MemoryError):
            p.step(X, 8000.0, 500.0)               # the first call reserves its workspace: refused too
        p1 = Plan(16, 8, 2.0, 1.0, 1.0, 0.01)
        L.sdd_debug_fail_allocations(-1)
        p1.reserve(1)
        L.sdd_debug_fail_allocations(3)            # the Krylov workspace fails part way through
        with pytest.raises(MemoryError):
            p1.newton(X.clone(), 8000.0, 500.0)
    finally:
        L.sdd_debug_fail_allocations(-1)
    ref = O.step(O.Operators(16, 8, 2.0, 1e-3, 1.0, 0.01), X.cpu().numpy().ravel(), 8000.0, 500.0, False)
    assert rel(p.step(X, 8000.0, 500.0).cpu().numpy().ravel(), ref) < 1e-12
    r = p1.newton(X.clone(), 8000.0, 500.0, tol=1e-10)[0]
    assert r["converged"]


def test_served_nan_requests_fail_and_the_mix_completes(cuda):
    from spectraldoublediffusiveconvection_gb300 import serve
    from conftest import load_golden
    Z = load_golden("cont_tau1.npz")
    srv = serve.Server(Tau=1.0, quantum=10, con_workers=2).start()
    try:
        Xn = O.seeded_state(16, 15, 1)
        Xn[4] = np.nan
        bad_int = serve.Request("integrate", 16, 16, 9000.0, X=Xn, n_steps=20)
        good_int = serve.Request("integrate", 16, 16, 9000.0, n_steps=20, seed=5)
        Xc = Z["X_steady"].copy()
        Xc[7] = np.nan
        bad_con = serve.Request("continue", 16, 16, 9000.0, X=Xc, ds=5.0)
        good_con = serve.Request("continue", 16, 16, 9000.0, X=Z["X_steady"].copy(), ds=5.0)
        for r in (bad_int, good_int, bad_con, good_con):
            srv.submit(r)
        assert srv.drain(timeout=120)
    finally:
        srv.stop()
    assert bad_int.error and "non-finite" in bad_int.error and bad_int.result is None
    assert bad_con.error and bad_con.result is None
    assert good_int.error is None and np.isfinite(good_int.result["X"]).all()
    assert good_con.error is None and good_con.result["converged"]
    assert srv.used == 0


def test_served_cancel_in_flight_integration(cuda):
    from spectraldoublediffusiveconvection_gb300 import serve
    srv = serve.Server(Tau=1.0, quantum=5, con_workers=1).start()
    try:
        long = serve.Request("integrate", 20, 64, 9000.0, n_steps=200000, seed=3)
        short = serve.Request("integrate", 20, 64, 9000.0, n_steps=50, seed=4)
        srv.submit(long)
        srv.submit(short)
        assert short.done.wait(60)
        assert srv.cancel(long) is True
        assert long.done.wait(60)
        assert srv.drain(timeout=60)
    finally:
        srv.stop()
    assert long.error == "cancelled" and long.t_start is not None
    assert short.error is None and short.result["steps"] == 50
    assert srv.used == 0 and srv._active == 0
