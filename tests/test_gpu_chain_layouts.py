"""Every chain layout of the implicit solves (1 one lane per row, 2 chunked with a sequential carry, 3
chunked with a parallel carry, 4 rows split over 4 lanes, 5 over 2 lanes, 6 and 7 the reference's own order
of operations with rows over 2 or 4 lanes, 8 that order with the three chains of a (parity, shell) in one
CTA, 9 the h pre-pass form with the three chains of a (parity, shell) in one CTA, 10 / 11 the chunks of 2 / 3
in the reference's order) against the oracle's A4_BSub_TSTEP_V2 / NAB2_BSub_TSTEP_V2
chains (Matrix_Operators.py:1033-1194), alone and inside the step, the Newton residual and its Jacobian.
The chunked layouts reorder the arithmetic (carried states through precomputed chunk maps or their
products), so they agree with the sequential chain to rounding, not bitwise."""
import numpy as np
import pytest

from conftest import rel
from oracle import sdd_oracle as O

pytestmark = pytest.mark.gpu

SHAPES = [(16, 16, False), (20, 64, False), (30, 256, False), (48, 512, False), (36, 384, True), (12, 10, True),
          (3, 2, False), (2, 4, False)]


@pytest.mark.parametrize("N_r,N_fm,sym", SHAPES)
@pytest.mark.parametrize("layout", [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11])
def test_chain_solves_against_oracle(cuda, N_r, N_fm, sym, layout):
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    nr = N_r - 1
    dt = 5e-4
    ops = O.Operators(N_fm, N_r, 2.0, dt, 1.0, 0.01)
    p = Plan(N_fm, N_r, 2.0, dt, 1.0, 0.01, symmetric=sym)
    p.set_chain_layout(layout)
    rng = np.random.default_rng(N_fm + nr)
    G = rng.standard_normal((2, N_fm * nr)) * np.repeat(np.exp(-np.arange(N_fm) / 40.0), nr)
    Gt = torch.from_numpy(G).cuda()
    fa = p.a4_bsub(Gt).cpu().numpy()
    ft = p.nab2_bsub(1, Gt).cpu().numpy()
    fs = p.nab2_bsub(2, Gt).cpu().numpy()
    for k in range(2):
        ra = O.A4_BSub_TSTEP_V2(G[k], ops.Linv_A4, ops.D2_A4, ops.IR4_A4, ops.IR2_A4, N_fm, nr, dt, sym)
        rt = O.NAB2_BSub_TSTEP_V2(G[k], ops.Linv_T, N_fm, nr, dt, sym)
        rs = O.NAB2_BSub_TSTEP_V2(G[k], ops.Linv_S, N_fm, nr, 0.01 * dt, sym)
        assert rel(fa[k], ra) < 1e-13
        assert rel(ft[k], rt) < 1e-13
        assert rel(fs[k], rs) < 1e-13


@pytest.mark.parametrize("layout", [2, 3, 10, 11])
@pytest.mark.parametrize("N_r,N_fm", [(20, 64), (30, 256), (48, 512)])
def test_chunked_step_newton_operators_against_oracle(cuda, N_r, N_fm, layout):
    """Chunked chains: 2 / 3 (h pre-pass, sequential / parallel carry) and 10 / 11 (each chunk in the
    reference's order, no pre-pass), the latter under the fused row kernel (full right-hand sides) and under
    the split nonlinear term (the chunks form their right-hand side themselves): the same bits."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    nr = N_r - 1
    X = O.seeded_state(N_fm, nr, 1234)
    dv = O.seeded_state(N_fm, nr, 77)
    Xt = torch.from_numpy(np.stack([X, 2 * X])).cuda()
    dvt = torch.from_numpy(np.stack([dv, dv])).cuda()
    ops = O.Operators(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01)
    p = Plan(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01)
    p.set_chain_layout(layout)
    if layout >= 10:
        p.set_fx_split(2)
        assert p.chain_choice(2)[0] == layout
        Y2 = p.step(Xt, 8000.0, 500.0, nsteps=3).cpu().numpy()
        p.set_fx_split(1)
        assert p.chain_choice(2)[0] == layout
    Y = p.step(Xt, 8000.0, 500.0, nsteps=3).cpu().numpy()
    if layout >= 10:
        assert np.array_equal(Y, Y2)
    for k, x in enumerate([X, 2 * X]):
        r = x
        for _ in range(3):
            r = O.step(ops, r, 8000.0, 500.0, False)
        assert rel(Y[k], r) < 1e-12
    ops1 = O.Operators(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    p1 = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    p1.set_chain_layout(layout)
    if layout >= 10:
        p1.set_fx_split(1)
    F = p1.pfx(Xt, 8000.0, 500.0).cpu().numpy()
    J = p1.pdfx(dvt, Xt, 8000.0, 500.0).cpu().numpy()
    for k, x in enumerate([X, 2 * X]):
        assert rel(F[k], O.PFX(ops1, x, 8000.0, 500.0, False)) < 1e-12
        assert rel(J[k], O.PDFX(ops1, dv, x, 8000.0, 500.0, False)) < 1e-12


@pytest.mark.parametrize("layout", [6, 7, 8])
@pytest.mark.parametrize("N_r,N_fm,prec", [(20, 64, "fp64"), (30, 256, "fp64"), (48, 512, "fp64"), (30, 256, "mixed"),
                                           (12, 16, "fp64"), (65, 32, "fp64")])
def test_reference_order_chains_in_steps_and_newton_operators(cuda, N_r, N_fm, prec, layout):
    """Layouts 6/7/8 (no h pre-pass; they need the full right-hand side, so the fused row kernel): steps, the
    Newton residual and its Jacobian against the oracle, and a batch equal to its shells alone.  The shapes
    cover one warp per chain (nr = 11: psi on one warp), several warps per T/S chain (nr = 47, 64) and the
    largest shared-memory footprint of layout 8 (N_r = 48, N_theta = 512: three rings in one CTA)."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    nr = N_r - 1
    X = O.seeded_state(N_fm, nr, 1234)
    dv = O.seeded_state(N_fm, nr, 77)
    Xt = torch.from_numpy(np.stack([X, 2 * X, 0.5 * X])).cuda()
    ops = O.Operators(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01)
    p = Plan(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01, precision=prec)
    p.set_chain_layout(layout)
    p.set_fx_split(1)
    # nr = 64: layout 8's three rings (333 KB) exceed a CTA's shared memory, and it runs layout 6
    assert p.chain_choice(3)[0] == (6 if (layout == 8 and N_r == 65) else layout)
    Y = p.step(Xt, 8000.0, 500.0, nsteps=3).cpu().numpy()
    for k, x in enumerate([X, 2 * X, 0.5 * X]):
        r = x
        for _ in range(3):
            r = O.step(ops, r, 8000.0, 500.0, False)
        assert rel(Y[k], r) < (1e-12 if prec == "fp64" else 1e-6)
        Yk = p.step(Xt[k:k + 1].clone(), 8000.0, 500.0, nsteps=3).cpu().numpy()
        assert np.array_equal(Yk[0], Y[k])
    if prec != "fp64":
        return
    ops1 = O.Operators(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    p1 = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    p1.set_chain_layout(layout)
    p1.set_fx_split(1)
    dvt = torch.from_numpy(np.stack([dv, dv, dv])).cuda()
    F = p1.pfx(Xt, 8000.0, 500.0).cpu().numpy()
    J = p1.pdfx(dvt, Xt, 8000.0, 500.0).cpu().numpy()
    for k, x in enumerate([X, 2 * X, 0.5 * X]):
        assert rel(F[k], O.PFX(ops1, x, 8000.0, 500.0, False)) < 1e-12
        assert rel(J[k], O.PDFX(ops1, dv, x, 8000.0, 500.0, False)) < 1e-12


@pytest.mark.parametrize("layout", [2, 3, 10, 11])
def test_chunked_batch_equals_alone(cuda, layout):
    """No arithmetic crosses shells in the chunked layouts either: a batch equals its shells alone."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 128, 24
    p = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01)
    p.set_chain_layout(layout)
    if layout >= 10:
        p.set_fx_split(1)
    Xs = np.stack([O.seeded_state(N_fm, N_r - 1, s) for s in range(4)])
    Ra = torch.tensor([6000.0, 8000.0, 10000.0, 12000.0], dtype=torch.float64, device="cuda")
    Xb = p.step(torch.from_numpy(Xs).cuda(), Ra, 500.0, nsteps=4)
    for i in range(4):
        Xi = p.step(torch.from_numpy(Xs[i:i + 1]).cuda(), float(Ra[i]), 500.0, nsteps=4)
        assert torch.equal(Xb[i:i + 1], Xi)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_split_nonlinear_term_equals_fused(cuda, precision):
    """Small batches run the nonlinear term split over 7 CTAs per radial row, large ones the fused row
    kernel; per element the arithmetic is the same, so a shell gives identical bits either way."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 256, 30        # split while 2 * 29 * batch <= #SMs: batch 1 split, batch 4 fused
    p = Plan(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01, precision=precision)
    p.set_chain_layout(1)
    Xs = torch.from_numpy(np.stack([O.seeded_state(N_fm, N_r - 1, s) for s in range(4)])).cuda()
    dvs = torch.from_numpy(np.stack([O.seeded_state(N_fm, N_r - 1, 50 + s) for s in range(4)])).cuda()
    Fb = p.nlin_fx(Xs)
    Db = p.nlin_dfx(dvs, Xs)
    Sb = p.step(Xs, 8000.0, 500.0, nsteps=2)
    for i in range(4):
        assert torch.equal(p.nlin_fx(Xs[i:i + 1]), Fb[i:i + 1])
        assert torch.equal(p.nlin_dfx(dvs[i:i + 1], Xs[i:i + 1]), Db[i:i + 1])
        assert torch.equal(p.step(Xs[i:i + 1], 8000.0, 500.0, nsteps=2), Sb[i:i + 1])


def test_forced_nonlinear_term_paths_agree(cuda):
    """sdd_plan_set_fx_split: the forced fused and forced split kernels give the same bits on one batch (under
    one chain layout: the automatic choice runs chunks in the reference's order where the right-hand side is
    not fused into the split nonlinear term, and the pre-pass chunks where it is).  Layouts 3 and 11 (the
    parallel-carry chunks whose correction the split form's steps leave to the next step's nonlinear term)."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 128, 24
    Xs = torch.from_numpy(np.stack([O.seeded_state(N_fm, N_r - 1, s) for s in range(5)])).cuda()
    dvs = torch.from_numpy(np.stack([O.seeded_state(N_fm, N_r - 1, 20 + s) for s in range(5)])).cuda()
    for layout in (3, 11):
        p = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
        p.set_chain_layout(layout)
        q = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01)
        q.set_chain_layout(layout)
        out = []
        for mode in (1, 2):
            p.set_fx_split(mode)
            q.set_fx_split(mode)
            out.append((p.nlin_fx(Xs), p.nlin_dfx(dvs, Xs), p.pfx(Xs, 9000.0, 500.0),
                        p.pdfx(dvs, Xs, 9000.0, 500.0), q.step(Xs, 9000.0, 500.0, nsteps=5)))
        for a, b in zip(*out):
            assert torch.equal(a, b)
    with pytest.raises(Exception):
        p.set_fx_split(3)


@pytest.mark.parametrize("layout", [1, 2, 3, 4, 5])
def test_matvec_variants_agree_across_batch_sizes(cuda, layout):
    """The per-mode h = Linv g (and chunk correction) kernels switch from one matvec per CTA to one per
    warp as the batch grows (3 fields x 256 modes x 4 shells crosses the switch); both sum in the same
    order, so a shell gives the same bits in a batch of 4 as alone."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 256, 30
    p = Plan(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01)
    p.set_chain_layout(layout)
    Xs = torch.from_numpy(np.stack([O.seeded_state(N_fm, N_r - 1, 30 + s) for s in range(4)])).cuda()
    Xb = p.step(Xs, 8000.0, 500.0, nsteps=3)
    for i in range(4):
        assert torch.equal(p.step(Xs[i:i + 1], 8000.0, 500.0, nsteps=3), Xb[i:i + 1])


def test_automatic_layout_choice(cuda):
    """sdd_plan_chain_choice (as the step launches: the right-hand side fused into the split nonlinear term
    for one shell): one production shell runs the parallel-carry chunks (layout 3, kc ~ sqrt(S/2)), a batch
    too large for its CTAs falls back to whole chains in the reference's order, three per CTA (layout 8);
    forced layouts are reported as they run."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    p = Plan(256, 30, 2.0, 5e-4, 1.0, 0.01)
    assert p.chain_choice(1) == (3, 8, 16)
    lay, kc, nch = p.chain_choice(64)
    assert lay == 8 and (kc, nch) == (0, 1)
    p.set_chain_layout(2)
    assert p.chain_choice(1) == (2, 16, 8)
    p.set_chain_layout(3)
    assert p.chain_choice(64) == (3, 8, 16)
    p.set_chain_layout(8)
    assert p.chain_choice(64)[0] == 8
    p.set_chain_layout(9)
    assert p.chain_choice(64)[0] == 9
    p.set_chain_layout(10)                 # 64 shells: the fused row kernel, full right-hand sides
    assert p.chain_choice(64) == (10, 16, 8)
    assert p.chain_choice(1) == (10, 16, 8)   # one shell: the split nonlinear term, the chunks form g
    p.set_chain_layout(11)
    assert p.chain_choice(64) == (11, 8, 16)
    assert p.chain_choice(1) == (11, 8, 16)
    with pytest.raises(Exception):
        p.set_chain_layout(12)


@pytest.mark.parametrize("N_r,N_fm,split", [(20, 64, 1), (30, 256, 2), (48, 512, 1), (12, 16, 2), (65, 32, 1)])
def test_prepass_three_chain_layout_in_steps_and_newton(cuda, N_r, N_fm, split):
    """Layout 9 (h pre-pass, the three chains of a (parity, shell) per CTA; with the fused right-hand side of
    the split nonlinear term too): steps, the Newton residual and Jacobian against the oracle, a batch equal
    to its shells alone, and mixed Jacobian products with FP32 right-hand sides (mixed_matvec 2) reaching the
    FP64 residual.  N_r = 48 with N_theta = 512 and nr = 64 do not fit their three rings in a CTA: layout 5 runs,
    rows over 4 warps for nr > 32 (layout 4)."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    nr = N_r - 1
    X = O.seeded_state(N_fm, nr, 1234)
    dv = O.seeded_state(N_fm, nr, 77)
    Xt = torch.from_numpy(np.stack([X, 2 * X, 0.5 * X])).cuda()
    ops = O.Operators(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01)
    p = Plan(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01)
    p.set_chain_layout(9)
    p.set_fx_split(split)
    assert p.chain_choice(3)[0] == (4 if (N_r, N_fm) in ((48, 512), (65, 32)) else 9)
    Y = p.step(Xt, 8000.0, 500.0, nsteps=3).cpu().numpy()
    for k, x in enumerate([X, 2 * X, 0.5 * X]):
        r = x
        for _ in range(3):
            r = O.step(ops, r, 8000.0, 500.0, False)
        assert rel(Y[k], r) < 1e-12
        Yk = p.step(Xt[k:k + 1].clone(), 8000.0, 500.0, nsteps=3).cpu().numpy()
        assert np.array_equal(Yk[0], Y[k])
    ops1 = O.Operators(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    p1 = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    p1.set_chain_layout(9)
    p1.set_fx_split(split)
    dvt = torch.from_numpy(np.stack([dv, dv, dv])).cuda()
    F = p1.pfx(Xt, 8000.0, 500.0).cpu().numpy()
    J = p1.pdfx(dvt, Xt, 8000.0, 500.0).cpu().numpy()
    for k, x in enumerate([X, 2 * X, 0.5 * X]):
        assert rel(F[k], O.PFX(ops1, x, 8000.0, 500.0, False)) < 1e-12
        assert rel(J[k], O.PDFX(ops1, dv, x, 8000.0, 500.0, False)) < 1e-12
    if N_fm > 256:
        return
    pm = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01, precision="mixed")
    pm.set_chain_layout(9)
    X0 = np.stack([O.seeded_state(N_fm, nr, 40 + s) for s in range(4)])
    Xm = torch.from_numpy(X0.copy()).cuda()
    res = pm.newton(Xm, torch.linspace(7000.0, 9000.0, 4, dtype=torch.float64, device="cuda"), 500.0, tol=1e-10,
                    mixed_matvec=2)
    for b in range(4):
        assert res[b]["converged"] and res[b]["residual"] <= 1e-10
        assert np.linalg.norm(O.PFX(ops1, Xm[b].cpu().numpy(), 7000.0 + 2000.0 * b / 3, 500.0, False)) <= 1.5e-10


@pytest.mark.parametrize("layout", [8, 9, 10, 11])
@pytest.mark.parametrize("N_r,N_fm", [(16, 16), (36, 384)])
def test_three_chain_layouts_symmetric(cuda, N_r, N_fm, layout):
    """Symmetric plans under layouts 8 and 9 (in each (parity, shell) CTA one or two of the three chains are
    inactive, their rows are zero, and leave at once while the others run on their own barriers) and under
    the reference-order chunks of layouts 10 and 11 (inactive chains' chunks write zeros; with the split
    nonlinear term the active chunks form their own right-hand sides, the same bits as the full form): steps
    and the Newton residual against the oracle's symmetric solves, a batch equal to its shells alone."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    nr = N_r - 1
    Xs = [O.seeded_state(N_fm, nr, 60 + s, True) for s in range(3)]
    ops = O.Operators(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01)
    p = Plan(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01, symmetric=True)
    p.set_chain_layout(layout)
    p.set_fx_split(1)
    Xt = torch.from_numpy(np.stack(Xs)).cuda()
    Y = p.step(Xt, 8000.0, 500.0, nsteps=2).cpu().numpy()
    if layout >= 10:
        p.set_fx_split(2)
        assert p.chain_choice(3)[0] == layout
        assert np.array_equal(p.step(Xt, 8000.0, 500.0, nsteps=2).cpu().numpy(), Y)
        p.set_fx_split(1)
    for k, x in enumerate(Xs):
        r = x
        for _ in range(2):
            r = O.step(ops, r, 8000.0, 500.0, True)
        assert rel(Y[k], r) < 1e-12
        assert np.array_equal(p.step(Xt[k:k + 1].clone(), 8000.0, 500.0, nsteps=2).cpu().numpy()[0], Y[k])
    ops1 = O.Operators(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    p1 = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01, symmetric=True)
    p1.set_chain_layout(layout)
    F = p1.pfx(Xt, 8000.0, 500.0).cpu().numpy()
    for k, x in enumerate(Xs):
        assert rel(F[k], O.PFX(ops1, x, 8000.0, 500.0, True)) < 1e-12


@pytest.mark.parametrize("layout,cset,kc", [(2, 0, 6), (10, 0, 40), (3, 1, 4), (11, 1, 13)])
def test_chunk_lengths_against_oracle(cuda, layout, cset, kc):
    """sdd_plan_set_chunk_length: chunk sets rebuilt for a chunk length other than the rule (shorter: more
    chunks, the carry workspace regrown; longer: fewer) give the oracle's steps and Newton operators, through
    captured step graphs (dropped and recaptured with the new tables) and one by one; 0 restores the rule;
    lengths outside 2..S or with too many chunks are refused."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    from spectraldoublediffusiveconvection_gb300 import _lib
    torch = cuda
    N_fm, N_r = 256, 30
    nr = N_r - 1
    ops = O.Operators(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01)
    X = O.seeded_state(N_fm, nr, 321)
    Xt = torch.from_numpy(np.stack([X, 0.5 * X])).cuda()
    p = Plan(N_fm, N_r, 2.0, 5e-4, 1.0, 0.01)
    p.set_chain_layout(layout)
    rule = p.chain_choice(2)
    Y0 = p.step(Xt, 8000.0, 500.0, nsteps=10).cpu().numpy()     # graphs captured with the rule's tables
    p.set_chunk_length(cset, kc)
    lay, kc2, nch = p.chain_choice(2)
    assert lay == layout and kc2 == kc and nch == (N_fm // 2 + kc - 1) // kc
    Y = p.step(Xt, 8000.0, 500.0, nsteps=10).cpu().numpy()
    Y1 = p.step(Xt, 8000.0, 500.0, nsteps=1).cpu().numpy()
    for k, x in enumerate([X, 0.5 * X]):
        r = x
        r1 = O.step(ops, x, 8000.0, 500.0, False)
        for _ in range(10):
            r = O.step(ops, r, 8000.0, 500.0, False)
        assert rel(Y[k], r) < 1e-12 and rel(Y0[k], r) < 1e-12
        assert rel(Y1[k], r1) < 1e-12
    p.set_chunk_length(cset, 0)
    assert p.chain_choice(2) == rule
    for bad in (1, N_fm, 3 if cset == 1 else 1):
        with pytest.raises(_lib.SDDError):
            p.set_chunk_length(cset, bad)
    p1 = Plan(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    p1.set_chain_layout(layout)
    p1.set_chunk_length(cset, kc)
    dv = O.seeded_state(N_fm, nr, 77)
    ops1 = O.Operators(N_fm, N_r, 2.0, 1.0, 1.0, 0.01)
    J = p1.pdfx(torch.from_numpy(dv).cuda().reshape(1, -1), Xt[:1], 8000.0, 500.0).cpu().numpy().ravel()
    assert rel(J, O.PDFX(ops1, dv, X, 8000.0, 500.0, False)) < 1e-12
