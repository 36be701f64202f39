"""Ragged batches: shells of different (N_r, N_theta, Ra_T) advanced together (eagerly and through one
captured CUDA graph) give the same states as each shell advanced alone."""
import numpy as np
import pytest

from conftest import rel
from oracle import sdd_oracle as O

pytestmark = pytest.mark.gpu

SHELLS = [dict(N_r=12, N_theta=16, Ra=7000.0), dict(N_r=20, N_theta=64, Ra=8000.0),
          dict(N_r=12, N_theta=16, Ra=11000.0), dict(N_r=10, N_theta=24, Ra=6500.0),
          dict(N_r=20, N_theta=64, Ra=9500.0), dict(N_r=36, N_theta=128, Ra=12000.0)]


def _alone(shell, X0, nsteps, precision, layout):
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    import torch
    p = Plan(shell["N_theta"], shell["N_r"], 2.0, 1e-3, 1.0, 0.01, precision=precision)
    p.set_chain_layout(layout)
    X = torch.from_numpy(X0).cuda().reshape(1, -1)
    return p.step(X, shell["Ra"], 500.0, nsteps=nsteps).cpu().numpy().ravel()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_batch_equals_alone(cuda, precision):
    from spectraldoublediffusiveconvection_gb300.batch import ShellBatch
    sh = [dict(s, X=O.seeded_state(s["N_theta"], s["N_r"] - 1, 10 + i)) for i, s in enumerate(SHELLS)]
    b = ShellBatch(sh, precision=precision)
    for g in b.groups:
        g.plan.set_chain_layout(1)
    b.capture(steps_per_launch=4)
    b.replay(3)                       # 12 steps
    got = b.states()
    for i, s in enumerate(sh):
        ref = _alone(s, s["X"], 12, precision, 1)
        assert rel(got[i], ref) <= 1e-14, (i, rel(got[i], ref))


def test_batch_fp64_matches_oracle_and_layouts_agree(cuda):
    from spectraldoublediffusiveconvection_gb300.batch import ShellBatch
    sh = [dict(s, X=O.seeded_state(s["N_theta"], s["N_r"] - 1, 20 + i)) for i, s in enumerate(SHELLS)]
    b = ShellBatch(sh, precision="fp64")
    b.step(3)
    got = b.states()
    for i, s in enumerate(sh):
        ops = O.Operators(s["N_theta"], s["N_r"], 2.0, 1e-3, 1.0, 0.01)
        X = s["X"]
        for _ in range(3):
            X = O.step(ops, X, s["Ra"], 500.0, False)
        assert rel(got[i], X) < 1e-12
        # the split-row chain layout gives the same result to rounding
        assert rel(_alone(s, s["X"], 3, "fp64", 4), X) < 1e-12


def test_autotune_records_choices(cuda):
    from spectraldoublediffusiveconvection_gb300.batch import ShellBatch
    b = ShellBatch(SHELLS, precision="mixed")
    t = b.autotune(steps_per_launch=2, reps=1)
    assert set(k for k in t if k.startswith("N_r")) == {"N_r=%d,N_theta=%d" % g.shape for g in b.groups}
    assert all(v["chain_layout"] in tuple(range(12)) for k, v in t.items() if k.startswith("N_r"))
    b.replay(1)
    assert all(np.isfinite(x).all() for x in b.states())
    # a fresh batch built with the tuned choices runs the same kernels: the same states after a launch
    b2 = ShellBatch(SHELLS, precision="mixed", tuning=t)
    assert all(b2.tuning[k] == {"chain_layout": v["chain_layout"], "fx_split": v["fx_split"],
                                "chunk_length": v["chunk_length"]}
               for k, v in t.items() if k.startswith("N_r"))
    assert all(b2.groups[i].plan.chunk_length == b.groups[i].plan.chunk_length for i in range(len(b.groups)))
    b2.capture(2)
    b2.replay(1)
    for x, y in zip(b2.states(), b.states()):
        assert np.array_equal(x, y)


def test_autotune_does_not_advance_states(cuda):
    from spectraldoublediffusiveconvection_gb300.batch import ShellBatch
    sh = [dict(s, X=O.seeded_state(s["N_theta"], s["N_r"] - 1, 30 + i)) for i, s in enumerate(SHELLS)]
    b = ShellBatch(sh, precision="mixed")
    b.autotune(steps_per_launch=2, reps=1)
    for x, s in zip(b.states(), sh):
        assert np.array_equal(x, s["X"])
