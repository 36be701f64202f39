"""The HDF5 records of _Time_Step and _Continuation against the reference writers' layout.

h5py is not installed here or on the GPU machine, so the writers are run against a recording stand-in for
the h5py module (File / create_group / item assignment / create_dataset, the calls the reference's writers
make) and the recorded tree is compared with the reference's: _Time_Step, Main.py:305-319 (groups
Checkpoints/X_DATA, Scalar_Data/{Norm, KE, Nu_T, Nu_S, Time}, Parameters/{Ra, Ra_s, Tau, Pr, d, N_r, N_fm,
dt, start_time, symmetric}); _Continuation, Main.py:1026-1040 (Checkpoints/{X_DATA, Ra_DATA}, Parameters =
the keyword arguments, Bifurcation = every attribute of the result record, Main.py:677-714).  That the
real h5py stores these trees byte-compatibly is not checked (no h5py)."""
import sys
import types

import numpy as np
import pytest


class _Group(dict):
    def create_group(self, name):
        g = _Group()
        dict.__setitem__(self, name, g)
        return g

    def create_dataset(self, name, data):
        dict.__setitem__(self, name, np.asarray(data))
        return self[name]

    def __setitem__(self, key, value):
        dict.__setitem__(self, key, value if isinstance(value, _Group) else np.asarray(value))


class _File(_Group):
    opened = {}

    def __init__(self, name, mode="r"):
        super().__init__()
        assert mode == "w"
        _File.opened[name] = self

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        return False

    def close(self):
        pass


@pytest.fixture
def fake_h5py(monkeypatch):
    mod = types.ModuleType("h5py")
    mod.File = _File
    _File.opened = {}
    monkeypatch.setitem(sys.modules, "h5py", mod)
    return _File.opened


def _tree(g):
    return {k: (_tree(v) if isinstance(v, _Group) else None) for k, v in g.items()}


TIME_STEP_TREE = {"Checkpoints": {"X_DATA": None},
                  "Scalar_Data": {k: None for k in ("Norm", "KE", "Nu_T", "Nu_S", "Time")},
                  "Parameters": {k: None for k in ("Ra", "Ra_s", "Tau", "Pr", "d", "N_r", "N_fm", "dt", "start_time",
                                                   "symmetric")}}


def test_time_step_writer_layout(fake_h5py):
    from spectraldoublediffusiveconvection_gb300 import Main
    rng = np.random.default_rng(0)
    rec = {"X_DATA": [rng.standard_normal(12) for _ in range(3)]}
    for k in ("Norm", "KE", "Nu_T", "Nu_S", "Time"):
        rec[k] = rng.standard_normal(3)
    params = dict(Ra=8000.0, Ra_s=500.0, Tau=0.01, Pr=1.0, d=2.0, N_r=6, N_fm=2, dt=1e-3, start_time=0,
                  symmetric=False)
    Main._write_h5("ts.h5", rec, params)
    f = fake_h5py["ts.h5"]
    assert _tree(f) == TIME_STEP_TREE
    assert f["Checkpoints"]["X_DATA"].shape == (3, 12)
    assert np.array_equal(f["Checkpoints"]["X_DATA"], np.stack(rec["X_DATA"]))
    for k in ("Norm", "KE", "Nu_T", "Nu_S", "Time"):
        assert np.array_equal(f["Scalar_Data"][k], rec[k])
    for k, v in params.items():
        assert f["Parameters"][k][()] == v


def test_continuation_writer_layout(fake_h5py):
    from spectraldoublediffusiveconvection_gb300 import Main
    R = Main.result()
    for i in range(6):
        for k in ("NuT", "NuS", "KE", "Norm", "Ra", "Ra_dot"):
            getattr(R, k).append(float(i))
    R.X_DATA = [np.arange(12.0), np.arange(12.0) + 1]
    R.Ra_DATA = [9000.0, 9005.0]
    R.Iterations = 5
    kw = dict(Ra=9000.0, Ra_s=500.0, Tau=1.0, Pr=1.0, d=2.0, N_fm=2, N_r=6, symmetric=False)
    Main._write_continuation_h5("cont.h5", R, kw)
    f = fake_h5py["cont.h5"]
    ref_attrs = ("NuT", "NuS", "KE", "Norm", "Ra", "Ra_dot", "Y_FOLD", "X_DATA", "Ra_DATA", "Iterations")
    assert _tree(f) == {"Checkpoints": {"X_DATA": None, "Ra_DATA": None},
                        "Parameters": {k: None for k in kw},
                        "Bifurcation": {k: None for k in ref_attrs}}
    assert np.array_equal(f["Checkpoints"]["Ra_DATA"], R.Ra_DATA)
    assert np.array_equal(f["Bifurcation"]["X_DATA"], np.stack(R.X_DATA))
    assert f["Bifurcation"]["Iterations"][()] == 5


@pytest.mark.gpu
def test_time_step_writes_its_record(cuda, fake_h5py):
    """_Time_Step with a save file: the recorded checkpoints and scalar series are the run's own record."""
    from spectraldoublediffusiveconvection_gb300 import Main
    from oracle import sdd_oracle as O
    X0 = O.seeded_state(16, 9, 3)
    XN = Main._Time_Step(X0, 8000.0, 500.0, 0.01, 1.0, 2.0, 16, 10, False, save_filename="run.h5",
                         Total_time=40 * 1e-3, dt=1e-3)
    f = fake_h5py["run.h5"]
    assert _tree(f) == TIME_STEP_TREE
    rec = Main._Time_Step.last_record
    assert np.array_equal(f["Checkpoints"]["X_DATA"], np.stack(rec["X_DATA"]))
    assert f["Checkpoints"]["X_DATA"].shape[1] == XN.size
    for k in ("Norm", "KE", "Nu_T", "Nu_S", "Time"):
        assert np.array_equal(f["Scalar_Data"][k], rec[k])
    assert f["Parameters"]["dt"][()] == 1e-3 and f["Parameters"]["N_fm"][()] == 16
