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
