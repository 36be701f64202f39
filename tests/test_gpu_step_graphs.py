"""sdd_step replays captured CUDA graphs of step pairs for long step counts.  The graphs launch the same
kernels on the same buffers, so the result equals stepping one call at a time bit for bit, for every
parity of the step count, in place or not, and after the plan's kernel choices change (which drops the
captured graphs).  Inside one call the parallel-carry chains (layout 3) leave each step's correction to
the next step's first kernel and mixed plans feed FP32 copies of the state forward; one step per call does
neither, so these tests also hold those paths to the same bits."""
import numpy as np
import pytest

from oracle import sdd_oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("nsteps", [8, 9, 10, 20, 37])
@pytest.mark.parametrize("inplace", [False, True])
def test_graph_steps_equal_single_steps(cuda, nsteps, inplace, precision):
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 64, 20
    p = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01, precision=precision)
    assert p.chain_choice(2)[0] == 3
    X0 = torch.from_numpy(np.stack([O.seeded_state(N_fm, N_r - 1, s) for s in (3, 4)])).cuda()
    Ra = torch.tensor([8000.0, 9000.0], dtype=torch.float64, device="cuda")
    ref = X0.clone()
    for _ in range(nsteps):
        ref = p.step(ref, Ra, 500.0, nsteps=1)
    for _ in range(2):                     # second call replays the cached graphs
        if inplace:
            X = X0.clone()
            p.step(X, Ra, 500.0, nsteps=nsteps, out=X)
        else:
            X = p.step(X0, Ra, 500.0, nsteps=nsteps)
        assert torch.equal(X, ref)


def test_graph_cache_follows_kernel_choices(cuda):
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 128, 24
    p = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01)
    X0 = torch.from_numpy(O.seeded_state(N_fm, N_r - 1, 8)).cuda().reshape(1, -1)
    for layout in (1, 2, 3, 4, 5, 1):
        p.set_chain_layout(layout)
        ref = X0.clone()
        for _ in range(12):
            ref = p.step(ref, 8000.0, 500.0, nsteps=1)
        assert torch.equal(p.step(X0, 8000.0, 500.0, nsteps=12), ref)
    lin_ref = X0.clone()
    for _ in range(10):
        lin_ref = p.step(lin_ref, 8000.0, 500.0, nsteps=1, linear=True)
    assert torch.equal(p.step(X0, 8000.0, 500.0, nsteps=10, linear=True), lin_ref)


def test_batch_step_groups_equal_their_steps_alone(cuda):
    """sdd_batch_step: three plans of different shapes advanced in one call (their groups on branch streams
    forked from and joined into the caller's stream) give each group exactly its sdd_step alone, for a
    graph-replayed count of steps and for a single step; the same call captured into a CUDA graph on the
    caller's stream replays to the same bits; a plan listed twice is refused."""
    from spectraldoublediffusiveconvection_gb300.plan import Plan, batch_step
    from spectraldoublediffusiveconvection_gb300 import _lib
    torch = cuda
    shapes = [(64, 20, 3), (128, 24, 2), (256, 30, 1)]
    plans, Xs, Ras = [], [], []
    for k, (N_fm, N_r, B) in enumerate(shapes):
        plans.append(Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01))
        Xs.append(torch.from_numpy(np.stack([O.seeded_state(N_fm, N_r - 1, 40 + 3 * k + i) for i in range(B)])).cuda())
        Ras.append(torch.linspace(7000.0, 9000.0, B, dtype=torch.float64, device="cuda"))
    for nsteps in (20, 1):
        outs = batch_step([(p, X, Ra, 500.0) for p, X, Ra in zip(plans, Xs, Ras)], nsteps=nsteps)
        torch.cuda.synchronize()
        for p, X, Ra, Y in zip(plans, Xs, Ras, outs):
            assert torch.equal(Y, p.step(X, Ra, 500.0, nsteps=nsteps))
    # captured on the caller's stream: one graph with a branch per group
    outs = [torch.empty_like(X) for X in Xs]
    ras = [Ra.clone() for Ra in Ras]
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        batch_step([(p, X, Ra, 500.0, o) for p, X, Ra, o in zip(plans, Xs, ras, outs)], nsteps=3)  # warm-up
        torch.cuda.synchronize()
        with torch.cuda.graph(g, stream=s):
            batch_step([(p, X, Ra, 500.0, o) for p, X, Ra, o in zip(plans, Xs, ras, outs)], nsteps=3)
    torch.cuda.current_stream().wait_stream(s)
    for o in outs:
        o.zero_()
    g.replay()
    torch.cuda.synchronize()
    for p, X, Ra, o in zip(plans, Xs, Ras, outs):
        assert torch.equal(o, p.step(X, Ra, 500.0, nsteps=3))
    with pytest.raises(_lib.SDDError):
        batch_step([(plans[0], Xs[0], Ras[0], 500.0), (plans[0], Xs[0], Ras[0], 500.0)])
