"""The opt-in Crank-Nicolson / Adams-Bashforth-2 step (sdd_step_cnab2, plan.CNAB2Stepper) against its oracle: a
composition of the reference's own NLIN_FX, DT0_theta, A2_SINE, kGR_RT, A4_BSub_TSTEP_V2 and NAB2_BSub_TSTEP_V2
with the operators of dt/2 (oracle.step_cnab2), at 1e-11 over whole trajectories; and its second-order
accuracy in time (the reference's IMEX Euler, which sdd_step reproduces, is first order)."""
import numpy as np
import pytest

from conftest import rel
from oracle import sdd_oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N_r,N_fm,dt,steps,sym,amp", [(20, 64, 1e-3, 300, False, 30.0),
                                                     (8, 10, 5e-3, 200, True, 30.0),
                                                     (30, 256, 5e-4, 100, False, 1.0)])
def test_cnab2_trajectory_matches_composed_oracle(cuda, N_r, N_fm, dt, steps, sym, amp):
    """(At N_theta = 256 the seeded state is not amplified: 30x it drives the explicit Adams-Bashforth term past
    its stability limit at dt = 5e-4, and the oracle's own trajectory overflows within 30 steps.)"""
    from spectraldoublediffusiveconvection_gb300.plan import CNAB2Stepper
    torch = cuda
    d, Pr, Tau, Ra, Ra_s = 2.0, 1.0, 0.01, 8000.0, 500.0
    nr = N_r - 1
    X0 = O.seeded_state(N_fm, nr, 77, sym) * amp
    oh = O.Operators(N_fm, N_r, d, 0.5 * dt, Pr, Tau)
    X, E = X0.copy(), None
    snaps = {}
    for it in range(steps):
        X, E = O.step_cnab2(oh, X, E, Ra, Ra_s, sym, dt)
        if it in (0, 1, steps // 2 - 1):
            snaps[it + 1] = X.copy()
    st = CNAB2Stepper(N_fm, N_r, d, dt, Pr, Tau, symmetric=sym)
    Xg = torch.from_numpy(X0.copy()).cuda().reshape(1, -1)
    done = 0
    for k in sorted(snaps):
        Xg = st.step(Xg, Ra, Ra_s, nsteps=k - done)
        done = k
        e = rel(Xg.cpu().numpy().ravel(), snaps[k])
        assert e <= 1e-11, (k, e)
    Xg = st.step(Xg, Ra, Ra_s, nsteps=steps - done)
    e = rel(Xg.cpu().numpy().ravel(), X)
    print(f"CNAB2 N_r={N_r} N_fm={N_fm}: {steps} steps, relative difference to the composed oracle {e:.2e}")
    assert e <= 1e-11


def test_cnab2_is_second_order_and_cnab1_first(cuda):
    """Errors at t = 0.02 against an 8x finer run of the same scheme: halving dt divides the CNAB2 error by ~4
    and the IMEX-Euler (reference scheme) error by ~2.  (At dt = 1e-3 the seeded high modes still ring under
    Crank-Nicolson, which is A- but not L-stable, so the steps start at 5e-4.)"""
    from spectraldoublediffusiveconvection_gb300.plan import CNAB2Stepper, Plan
    torch = cuda
    N_fm, N_r, d, Pr, Tau, Ra, Ra_s = 32, 16, 2.0, 1.0, 0.01, 8000.0, 500.0
    X0 = torch.from_numpy(O.seeded_state(N_fm, N_r - 1, 5) * 30).cuda().reshape(1, -1)
    T = 0.02
    dts = [5e-4, 2.5e-4, 1.25e-4]
    fine = 1.25e-4 / 8

    def cnab2(dt):
        return CNAB2Stepper(N_fm, N_r, d, dt, Pr, Tau).step(X0, Ra, Ra_s, nsteps=int(round(T / dt)))

    def cnab1(dt):
        return Plan(N_fm, N_r, d, dt, Pr, Tau).step(X0, Ra, Ra_s, nsteps=int(round(T / dt)))

    for scheme, order in ((cnab2, 2.0), (cnab1, 1.0)):
        ref = scheme(fine).cpu().numpy().ravel()
        errs = [rel(scheme(dt).cpu().numpy().ravel(), ref) for dt in dts]
        rates = [np.log2(errs[i] / errs[i + 1]) for i in range(len(errs) - 1)]
        print(scheme.__name__, ["%.2e" % e for e in errs], "observed orders", ["%.2f" % r for r in rates])
        assert all(abs(r - order) < 0.25 for r in rates), (scheme.__name__, errs, rates)
