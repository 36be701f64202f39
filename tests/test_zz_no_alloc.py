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
