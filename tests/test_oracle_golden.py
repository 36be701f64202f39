"""The oracle (numpy restatement) against the golden vectors produced by the reference itself."""
import numpy as np
import pytest

from conftest import load_golden, rel
from oracle import sdd_oracle as O

OPS_CASES = ["tiny", "tiny_sym", "m10_sym", "c1", "c1_sym"]


def test_transforms_match_reference():
    G = load_golden("transforms.npz")
    for M in (8, 10, 16, 64):
        P = 3 * M // 2
        a, g = G[f"IDCT_in_{M}"], G[f"DCT_in_{M}"]
        assert np.allclose(O.IDCT(a, n=P), G[f"IDCT_{M}"], rtol=0, atol=1e-13)
        assert np.allclose(O.IDST(a, n=P), G[f"IDST_{M}"], rtol=0, atol=1e-13)
        assert np.allclose(O.IDCT(a), G[f"IDCT_nonpad_{M}"], rtol=0, atol=1e-13)
        assert np.allclose(O.IDST(a), G[f"IDST_nonpad_{M}"], rtol=0, atol=1e-13)
        assert np.allclose(O.DCT(g), G[f"DCT_{M}"], rtol=0, atol=1e-13)
        assert np.allclose(O.DST(g), G[f"DST_{M}"], rtol=0, atol=1e-13)
        assert np.allclose(O.DCT(g, n=M), G[f"DCT_trunc_{M}"], rtol=0, atol=1e-13)
        assert np.allclose(O.DST(g, n=M), G[f"DST_trunc_{M}"], rtol=0, atol=1e-13)
        assert np.allclose(O.grid(P), G[f"grid_{M}"], rtol=0, atol=1e-15)


@pytest.mark.parametrize("tag", OPS_CASES)
def test_operators_match_reference(tag):
    Z = load_golden(f"ops_{tag}.npz")
    N_r, N_fm, dt, d, Pr, Tau, Ra, Ra_s, sym = Z["params"]
    N_r, N_fm, sym = int(N_r), int(N_fm), bool(sym)
    nr = N_r - 1
    N = nr * N_fm
    ops = O.Operators(N_fm, N_r, d, dt, Pr, Tau)
    X, dv = Z["X"], Z["dv"]
    psi = X[:N]
    tol = 1e-13
    assert rel(ops.D, Z["D"]) < tol
    assert rel(O.J_theta_RT(psi, nr, N_fm, sym), Z["J_theta_RT"]) < tol
    assert rel(O.A2_SINE_R2(psi, N_fm, nr, ops.D, ops.R, sym), Z["A2_SINE_R2"]) < tol
    assert rel(O.A2_SINE(psi, ops.D, ops.R, N_fm, nr, sym), Z["A2_SINE"]) < tol
    assert rel(O.DT0_theta(psi, ops.DT0, N_fm, nr, sym), Z["DT0_theta"]) < tol
    assert rel(O.NLIN_FX(X, ops.D, ops.R, N_fm, nr, sym), Z["NLIN_FX"]) < tol
    assert rel(O.NLIN_DFX(dv, X, ops.D, ops.R, N_fm, nr, sym), Z["NLIN_DFX"]) < tol
    g = Z["A4_g"]
    assert rel(O.A4_BSub_TSTEP_V2(g, ops.Linv_A4, ops.D2_A4, ops.IR4_A4, ops.IR2_A4, N_fm, nr, Pr * dt, sym),
               Z["A4_BSub"]) < tol
    assert rel(O.NAB2_BSub_TSTEP_V2(g, ops.Linv_T, N_fm, nr, dt, sym), Z["NAB2_T"]) < tol
    assert rel(O.NAB2_BSub_TSTEP_V2(g, ops.Linv_S, N_fm, nr, Tau * dt, sym), Z["NAB2_S"]) < tol
    assert rel(O.step(ops, X, Ra, Ra_s, sym), Z["step1"]) < 1e-12
    assert rel(O.step(ops, X, Ra, Ra_s, sym, linear=True), Z["step1_linear"]) < 1e-12
    ops1 = O.Operators(N_fm, N_r, d, 1.0, Pr, Tau)
    assert rel(O.PFX(ops1, X, Ra, Ra_s, sym), Z["PFX"]) < 1e-12
    assert rel(O.PDFX(ops1, dv, X, Ra, Ra_s, sym), Z["PDFX"]) < 1e-12
    assert abs(O.Kinetic_Energy(X, ops.R, ops.D, N_fm, nr, sym) - Z["KE"]) <= 1e-12 * abs(Z["KE"])
    assert abs(O.Nusselt(X[N:2 * N], d, ops.R, ops.D, N_fm, nr) - Z["NuT"]) <= 1e-12 * abs(Z["NuT"])
    if "Linv_A4" in Z:
        assert rel(ops.Linv_A4, Z["Linv_A4"]) < tol
        assert rel(ops.Linv_T, Z["Linv_T"]) < tol
        assert rel(ops.Linv_S, Z["Linv_S"]) < tol


@pytest.mark.parametrize("tag", ["tiny", "sym_lin", "c1"])
def test_trajectory_matches_reference(tag):
    Z = load_golden(f"traj_{tag}.npz")
    N_r, N_fm, dt, d, Pr, Tau, Ra, Ra_s, sym, ns = Z["params"]
    N_r, N_fm, sym, ns = int(N_r), int(N_fm), bool(sym), int(ns)
    ops = O.Operators(N_fm, N_r, d, dt, Pr, Tau)
    XN, snaps = O.time_step(ops, Z["X0"], Ra, Ra_s, sym, ns, linear=(tag == "sym_lin"), every=ns // 10)
    assert rel(XN, Z["X_final"]) < 1e-12
    for s, r in zip(snaps, Z["X_DATA"]):
        assert rel(s, r) < 1e-12


def test_interpolation_matches_reference():
    Z = load_golden("interp.npz")
    X = Z["X"]
    # The reference's radial interpolation is np.polyfit of degree N_o+1 through N_o+1 points: an
    # underdetermined, ill-conditioned Vandermonde least-squares problem whose minimum-norm answer
    # depends on the platform's LAPACK at ~1e-6 relative (x86-64 vs aarch64 OpenBLAS differ by 2e-6),
    # so the radial check carries that tolerance; the theta transforms are well conditioned.
    assert rel(O.INTERP_RADIAL(20, 12, X, 2.0), Z["rad_up"]) < 2e-5
    assert rel(O.INTERP_RADIAL(8, 12, X, 2.0), Z["rad_down"]) < 2e-5
    assert rel(O.INTERP_THETAS(32, 16, X), Z["th_up"]) < 1e-13
    assert rel(O.INTERP_THETAS(8, 16, X), Z["th_down"]) < 1e-13


def test_package_seeded_state_matches_oracle():
    """The synthetic inputs the library, the batch/serving code and the bench generate are the oracle's."""
    import numpy as np
    from spectraldoublediffusiveconvection_gb300.seeds import seeded_state
    for (M, nr, seed, sym) in [(64, 19, 1234, False), (16, 11, 7, True), (256, 29, 1, False)]:
        assert np.array_equal(seeded_state(M, nr, seed, sym), O.seeded_state(M, nr, seed, sym))


def test_linear_problem_matches_reference():
    """Linear_Matrix_Operators.py ML_0/Ll_0 and Linear_Problem.py Eig_Vals/Eig_Vec (host dense eigenproblem,
    the library's own host code) and the oracle's Full_Eig_Vec against the reference's outputs.  The
    eigenvectors are LAPACK's up to sign; M^-1 L is formed by a solve instead of an inverse (1e-13)."""
    import numpy as np
    from spectraldoublediffusiveconvection_gb300 import Linear_Matrix_Operators as LMO
    from spectraldoublediffusiveconvection_gb300 import Linear_Problem as LP
    Z = load_golden("eigen.npz")
    for tag in ("a", "b"):
        Ra, l, d, Ras, Pr, Tau, Nr = Z[f"params_{tag}"]
        Nr = int(Nr)
        D, R = LMO.cheb_radial(Nr, d)
        assert rel(D, Z[f"D_{tag}"]) < 1e-14 and rel(R, Z[f"R_{tag}"]) < 1e-15
        assert rel(LMO.ML_0(D, R, l), Z[f"ML0_{tag}"]) < 1e-14
        assert rel(LMO.Ll_0(D, R, d, l, Ra, Ras, Pr, Tau), Z[f"Ll0_{tag}"]) < 1e-14
        vals, ref = LP.Eig_Vals(Ra, l, d, 5, Ras, Pr, Tau, Nr), Z[f"vals_{tag}"]     # complex
        assert np.abs(vals - ref).max() < 1e-11 * np.abs(ref).max()
        assert abs(LP.Eig_Vals(Ra, l, d, 1, Ras, Pr, Tau, Nr) - Z[f"val1_{tag}"]) < 1e-10 * (1 + abs(Z[f"val1_{tag}"]))
        for k in (0, 1):
            e, g = LP.Eig_Vec(Ra, l, d, k, Ras, Pr, Tau, Nr).ravel(), Z[f"vec{k}_{tag}"].ravel()
            assert rel(np.sign(e @ g) * e, g) < 1e-10
    f = Z["vec0_a"]
    for N_fm in (16, 32):
        assert rel(O.Full_Eig_Vec(f, 2.0, N_fm, 19), Z[f"full_{N_fm}"]) < 1e-13
    assert rel(O.Full_Eig_Vec(f, 2.0, 16, 19, symmetric=True), Z["full_sym_16"]) < 1e-13


def test_oracle_on_continuation_golden():
    """The reference's steady convective state (Ra_T = 9000, N_r = N_fm = 16, Tau = 1) and the point its
    _ContinC step reached (tests/golden/cont_tau1.npz) are zeros of the oracle's PFX, and the oracle's
    diagnostics of both equal the Norm / Kinetic_Energy / Nusselt values the reference reported."""
    import numpy as np
    Z = load_golden("cont_tau1.npz")
    N_r, N_fm, dt, d, Pr, Tau, Ra0, Ra_s, sym = Z["params"]
    N_r, N_fm = int(N_r), int(N_fm)
    nr, N = N_r - 1, N_fm * (N_r - 1)
    ops1 = O.Operators(N_fm, N_r, d, 1.0, Pr, Tau)
    D, R = O.cheb_radial(N_r, d)
    X, Y = Z["X_steady"], Z["Y"]
    assert np.linalg.norm(O.PFX(ops1, X, Ra0, Ra_s, False)) <= 1e-12
    assert np.linalg.norm(O.PFX(ops1, Y[:-1], Y[-1], Ra_s, False)) <= 1e-12

    def diag(v):
        return np.array([np.linalg.norm(v), O.Kinetic_Energy(v, R, D, N_fm, nr, False),
                         O.Nusselt(v[N:2 * N], d, R, D, N_fm, nr), O.Nusselt(v[2 * N:], d, R, D, N_fm, nr)])
    assert np.allclose(diag(X), Z["steady_diag"], rtol=1e-12, atol=0)
    assert np.allclose(diag(Y[:-1]), [Z["Norm"], Z["KE"], Z["NuT"], Z["NuS"]], rtol=1e-12, atol=0)
