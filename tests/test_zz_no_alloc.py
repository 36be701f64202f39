"""The entry point that allocates nothing: sdd_nlin_fx_noalloc (C ABI) against sdd_nlin_fx.

sdd_nlin_fx_noalloc serves callers that must not allocate device memory when they call the library --
code whose device memory belongs to another allocator, or latency-critical paths where a cudaMalloc's
implicit device synchronisation is not allowed.  Its scratch is a fixed library-owned array, shared by
every call, so two calls in a row must both give the allocating entry point's result.  This file is
collected last so that a failure here stops a -x run only after every other test has run.
"""
import ctypes

import numpy as np
import pytest

from oracle import sdd_oracle as O

pytestmark = pytest.mark.gpu


def _noalloc(plan, X, F):
    from spectraldoublediffusiveconvection_gb300 import _lib
    import torch
    st = _lib.lib().sdd_nlin_fx_noalloc(plan._h, X.shape[0], ctypes.c_void_p(X.data_ptr()),
                                        ctypes.c_void_p(F.data_ptr()),
                                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return st


def test_noalloc_nlin_fx_matches_allocating_entry_point(cuda):
    from spectraldoublediffusiveconvection_gb300 import _lib
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 64, 20
    p = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01)
    for call, seeds in enumerate(((1, 2), (3, 4))):      # two calls in a row, different inputs
        X = torch.from_numpy(np.stack([O.seeded_state(N_fm, N_r - 1, s) for s in seeds])).cuda()
        ref = p.nlin_fx(X)
        F = torch.full_like(X, float("nan"))
        assert _noalloc(p, X, F) == _lib.SDD_OK
        torch.cuda.synchronize()
        err = float(torch.linalg.norm(F - ref) / torch.linalg.norm(ref))
        assert err <= 1e-12, (call, err)


def test_noalloc_rejects_batches_beyond_its_scratch(cuda):
    from spectraldoublediffusiveconvection_gb300 import _lib
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 64, 20
    p = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01)
    per_shell = 4 * N_fm * (N_r - 1)
    too_many = _lib.SDD_NOALLOC_SCRATCH_DOUBLES // per_shell + 1
    X = torch.zeros((too_many, 3 * N_fm * (N_r - 1)), dtype=torch.float64, device="cuda")
    F = torch.empty_like(X)
    assert _noalloc(p, X, F) == _lib.SDD_ERR_UNSUPPORTED


@pytest.mark.parametrize("sym", [False, True])
def test_noalloc_at_the_largest_accepted_batch(cuda, sym):
    """batch * 4 * N_fm * nr equal to (at most one shell below) the scratch size: the last shell's outputs
    sit at the end of the fixed array, where a wrong stride would run past it."""
    from spectraldoublediffusiveconvection_gb300 import _lib
    from spectraldoublediffusiveconvection_gb300.plan import Plan
    torch = cuda
    N_fm, N_r = 64, 20
    nr = N_r - 1
    p = Plan(N_fm, N_r, 2.0, 1e-3, 1.0, 0.01, symmetric=sym)
    B = _lib.SDD_NOALLOC_SCRATCH_DOUBLES // (4 * N_fm * nr)            # 215 shells
    assert (B + 1) * 4 * N_fm * nr > _lib.SDD_NOALLOC_SCRATCH_DOUBLES
    seeds = [O.seeded_state(N_fm, nr, s, sym) for s in range(4)]
    X = torch.from_numpy(np.stack([seeds[b % 4] * (1.0 + 0.01 * b) for b in range(B)])).cuda()
    ref = p.nlin_fx(X)
    for _ in range(2):
        F = torch.full_like(X, float("nan"))
        assert _noalloc(p, X, F) == _lib.SDD_OK
        torch.cuda.synchronize()
        for b in (0, B // 2, B - 1):
            err = float(torch.linalg.norm(F[b] - ref[b]) / torch.linalg.norm(ref[b]))
            assert err <= 1e-12, (b, err)
        assert bool(torch.isfinite(F).all())
