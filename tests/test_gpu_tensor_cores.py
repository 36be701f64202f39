"""The mixed form's radial contractions on the tensor cores (tcgen05 3xTF32, sdd_deriv_tc / k_deriv_tc).

Each FP32 operand is split into TF32 hi and lo parts and the product formed as a_lo b_hi + a_hi b_lo +
a_hi b_hi with FP32 accumulation: FP32-level accuracy.  Checked against FP64 products of the same operators
(Derivatives, Matrix_Operators.py:698-729) on FP32 inputs: the error is bounded by a few units of FP32
rounding of the row's magnitude, 2e-6 of the largest entry of each block (|x| max * |D| row sums ~ the
entries; observed errors are ~1e-7).  Then the effect on whole steps and Newton solves: the mixed form with
tensor cores against the FP64 path and against the CUDA-core FP32 contractions.
"""
import numpy as np
import pytest

from conftest import rel
from oracle import sdd_oracle as O

pytestmark = pytest.mark.gpu


def _ref_blocks(X, ops, N_fm, nr, sym):
    """FP64 Dr psi, (D^2/r^2) psi, Dr T, Dr S of the FP32-rounded state, as [4][nr][N_fm]."""
    V = X.astype(np.float32).astype(np.float64).reshape(3, N_fm, nr)
    Dr = ops.D[1:-1, 1:-1]
    D2r2 = (np.diag(1.0 / ops.R ** 2) @ (ops.D @ ops.D))[1:-1, 1:-1]
    out = np.stack([Dr @ V[0].T, D2r2 @ V[0].T, Dr @ V[1].T, Dr @ V[2].T])      # (4, nr, N_fm)
    if sym:
        out[0:2, :, 0::2] = 0.0
        out[2:4, :, 1::2] = 0.0
    return out


@pytest.mark.parametrize("N_r,N_fm,B,sym", [(20, 64, 3, False), (30, 256, 2, False), (48, 128, 2, False),
                                            (12, 16, 5, True), (9, 10, 4, False), (65, 32, 1, False)])
def test_deriv_tc_matches_fp64_products(cuda, N_r, N_fm, B, sym):
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    nr = N_r - 1
    ops = O.Operators(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01)
    Xs = [O.seeded_state(N_fm, nr, 7 + i, sym) * (1 + 100 * i) for i in range(B)]
    p = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01, symmetric=sym, precision="mixed")
    X32 = torch.from_numpy(np.stack(Xs).astype(np.float32)).cuda()
    for rep in range(2):                       # a second call gives the same bits
        out = p.deriv_tc(X32).cpu().numpy().astype(np.float64)
        if rep == 0:
            first = out.copy()
        else:
            assert np.array_equal(out, first)
    assert not p.tensor_core_timed_out()
    worst = 0.0
    for i, X in enumerate(Xs):
        ref = _ref_blocks(X, ops, N_fm, nr, sym)
        for op in range(4):
            scale = np.abs(ref[op]).max()
            err = np.abs(out[i, op] - ref[op]).max() / scale
            worst = max(worst, err)
            assert err <= 2e-6, (i, op, err)
        if sym:
            assert np.all(out[i, 0:2, :, 0::2] == 0.0) and np.all(out[i, 2:4, :, 1::2] == 0.0)
    print(f"N_r={N_r} N_fm={N_fm}: worst error of the 3xTF32 contractions vs FP64 products: {worst:.2e}")


def test_deriv_tc_is_three_pass_not_single_tf32(cuda):
    """A single TF32 product would lose ~3 decimal digits (2^-11 relative); the three-pass split keeps FP32
    accuracy.  The errors measured above are far below TF32's: here a state whose entries all carry
    information below the TF32 mantissa."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 32, 24
    nr = N_r - 1
    ops = O.Operators(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01)
    rng = np.random.default_rng(3)
    X = (1.0 + rng.random(3 * N_fm * nr) * 2.0 ** -12)        # 1 + tiny: lost entirely by one TF32 rounding
    p = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01, precision="mixed")
    out = p.deriv_tc(torch.from_numpy(X.astype(np.float32)).cuda().reshape(1, -1)).cpu().numpy()[0]
    ref = _ref_blocks(X, ops, N_fm, nr, False)
    e = max(np.abs(out[op] - ref[op]).max() / np.abs(ref[op]).max() for op in range(4))
    assert e <= 2e-6, e


def test_fp64_plan_has_no_tensor_core_path(cuda):
    from spectraldoublediffusiveconvection_gb300 import _lib
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    p = Plan(16, 8, 2.0, 1e-3, 1.0, 0.01)
    with pytest.raises(_lib.SDDError):
        p.deriv_tc(torch.zeros((1, p.n_state), dtype=torch.float32, device="cuda"))
    with pytest.raises(_lib.SDDError):
        p.set_tensor_cores(True)


@pytest.mark.parametrize("split", [1, 2])
def test_mixed_step_with_tensor_cores_against_fp64_and_cuda_cores(cuda, split):
    """One mixed step (fused row kernel or split path, both reading the tensor-core contractions) stays at
    FP32 level against the FP64 step, and within the same bound of the CUDA-core FP32 contractions."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 64, 20
    X = torch.from_numpy(np.stack([O.seeded_state(N_fm, N_r - 1, s) * 30 for s in (1, 2)])).cuda()
    pd = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01)
    ref = pd.step(X, 8000.0, 500.0).cpu().numpy()
    pm = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01, precision="mixed")
    pm.set_fx_split(split)
    tc = pm.step(X, 8000.0, 500.0).cpu().numpy()
    pm.set_tensor_cores(False)
    cc = pm.step(X, 8000.0, 500.0).cpu().numpy()
    e_tc, e_cc = rel(tc, ref), rel(cc, ref)
    print(f"split={split}: one mixed step vs FP64, tensor cores {e_tc:.2e}, CUDA cores {e_cc:.2e}")
    assert 0 < e_tc < 1e-6 and 0 < e_cc < 1e-6
    assert rel(tc, cc) < 1e-6
    assert not pm.tensor_core_timed_out()


def test_fused_and_split_mixed_paths_agree_bitwise_with_tensor_cores(cuda):
    """Both nonlinear-term forms read the same tensor-core contractions: the same bits."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 128, 24
    X = torch.from_numpy(np.stack([O.seeded_state(N_fm, N_r - 1, s) * 20 for s in (4, 5, 6)])).cuda()
    outs = []
    for mode in (1, 2):
        p = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01, precision="mixed")
        p.set_chain_layout(1)
        p.set_fx_split(mode)
        outs.append(p.step(X, 9000.0, 500.0, nsteps=3).cpu().numpy())
    assert np.array_equal(outs[0], outs[1])


def test_batched_newton_with_tensor_cores_reaches_fp64_residual(cuda):
    """mixed_matvec 2 Jacobian products (FP32 nonlinear term with tensor-core contractions, FP32 rhs and h) in
    a batched Newton: every shell at |F| <= 1e-10, the oracle's residual agrees, and the steady states equal
    those of the CUDA-core contractions to the Newton tolerance."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r, B = 64, 20, 6
    X0 = np.stack([O.seeded_state(N_fm, N_r - 1, 1234 + i) for i in range(B)])
    Ra = torch.linspace(7000.0, 10000.0, B, dtype=torch.float64, device="cuda")
    res, sols = [], []
    for tc in (True, False):
        p = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01, precision="mixed")
        p.set_tensor_cores(tc)
        X = torch.from_numpy(X0.copy()).cuda()
        res.append(p.newton(X, Ra, 500.0, tol=1e-10, mixed_matvec=2))
        sols.append(X.cpu().numpy())
    ops1 = O.Operators(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    for b in range(B):
        assert res[0][b]["converged"] and res[0][b]["residual"] <= 1e-10
        assert np.linalg.norm(O.PFX(ops1, sols[0][b], float(Ra[b]), 500.0, False)) <= 1.5e-10
    assert np.linalg.norm(sols[0] - sols[1]) <= 1e-9 * max(1.0, np.linalg.norm(sols[1]))
