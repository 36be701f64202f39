"""Vecs_to_X / X_to_Vecs drop-ins (Matrix_Operators.py:529-627) against the reference's own outputs
(tests/golden/layout.npz), through the numpy branch and the torch branch (CPU tensors), symmetric and not.
Layout only: no GPU is needed."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import sdd_oracle as O


@pytest.mark.parametrize("sym", [False, True])
def test_vecs_to_x_numpy_matches_reference(sym):
    from spectraldoublediffusiveconvection_gb300 import Matrix_Operators as MO
    Z = load_golden("layout.npz")
    N_fm, nr = Z["PSI"].shape[1], Z["PSI"].shape[0]
    X = MO.Vecs_to_X(Z["PSI"], Z["T"], Z["C"], N_fm, nr, sym)
    assert np.array_equal(X, Z[f"X_{int(sym)}"])
    assert np.array_equal(O.Vecs_to_X(Z["PSI"], Z["T"], Z["C"], N_fm, nr, sym), Z[f"X_{int(sym)}"])
    for tag, src in (("", Z[f"X_{int(sym)}"]), ("raw_", Z["X_raw"])):
        got = MO.X_to_Vecs(src, N_fm, nr, sym)
        for name, g in zip(("PSI", "T", "C"), got):
            assert np.array_equal(g, Z[f"{name}_{tag}{int(sym)}"]), (name, tag)


@pytest.mark.parametrize("sym", [False, True])
def test_vecs_to_x_torch_matches_reference(sym):
    torch = pytest.importorskip("torch")
    from spectraldoublediffusiveconvection_gb300 import Matrix_Operators as MO
    Z = load_golden("layout.npz")
    N_fm, nr = Z["PSI"].shape[1], Z["PSI"].shape[0]
    t = {k: torch.from_numpy(np.ascontiguousarray(Z[k])) for k in ("PSI", "T", "C", "X_raw")}
    X = MO.Vecs_to_X(t["PSI"], t["T"], t["C"], N_fm, nr, sym)
    assert isinstance(X, torch.Tensor) and X.shape == (3 * N_fm * nr,)
    assert np.array_equal(X.numpy(), Z[f"X_{int(sym)}"])
    got = MO.X_to_Vecs(t["X_raw"], N_fm, nr, sym)
    for name, g in zip(("PSI", "T", "C"), got):
        assert isinstance(g, torch.Tensor)
        assert np.array_equal(g.numpy(), Z[f"{name}_raw_{int(sym)}"]), name
    # the inputs are not mutated (the reference returns fresh arrays)
    assert np.array_equal(t["X_raw"].numpy(), Z["X_raw"])
