"""The phase-boundary probe (sdd_probe_phase_boundaries): a captured graph of kernel launches against one
cooperative kernel with bounded grid barriers, on a small grid; both finish, no barrier runs out, and the
persistent form's work is the graph form's (the same element updates)."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_probe_runs_and_barriers_complete(cuda):
    from spectraldoublediffusiveconvection_gb300 import _lib
    torch = cuda
    L = _lib.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for ctas, nph, work in ((4, 8, 16), (64, 16, 0)):
        g, pz, to = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_int(0)
        _lib.check(L.sdd_probe_phase_boundaries(ctas, 128, nph, work, 2, ctypes.byref(g), ctypes.byref(pz),
                                                ctypes.byref(to), stream), "sdd_probe_phase_boundaries")
        assert to.value == 0
        assert 0.0 < g.value < 1e6 and 0.0 < pz.value < 1e6
    g, pz, to = ctypes.c_double(0), ctypes.c_double(0), ctypes.c_int(0)
    st = L.sdd_probe_phase_boundaries(0, 128, 4, 0, 1, ctypes.byref(g), ctypes.byref(pz), ctypes.byref(to), stream)
    assert st == _lib.SDD_ERR_ARG
