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
    path (which matches the oracle to 1e-11) is reported and bounded."""
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
    assert e < 1e-5


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
