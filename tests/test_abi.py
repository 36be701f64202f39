"""C ABI: the library builds for sm_103a, loads without a GPU, and exports every declared symbol."""
import ctypes
import os
import re

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "sdd_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(sdd_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_bound_symbols():
    from spectraldoublediffusiveconvection_gb300 import _lib
    bound = sorted(n for n, _, _ in _lib.SIGNATURES)
    assert bound == _declared()


def test_library_loads_and_exports(built_lib):
    L = ctypes.CDLL(built_lib)
    for name in _declared():
        assert hasattr(L, name), name
    from spectraldoublediffusiveconvection_gb300 import _lib
    lib = _lib.load(built_lib)
    assert lib.sdd_version() >= 100
    assert lib.sdd_error_string(-2).decode().startswith("The number of Fourier modes")


def test_argument_errors_need_no_gpu(built_lib):
    """Argument checks run before any CUDA call, so they are testable on a CPU-only host."""
    from spectraldoublediffusiveconvection_gb300 import _lib
    lib = _lib.load(built_lib)
    assert lib.sdd_transform(9, 1, 4, 6, None, None, None) == _lib.SDD_ERR_ARG
    assert lib.sdd_plan_create(None, None) == _lib.SDD_ERR_ARG
    d = _lib.PlanDesc()
    d.N_fm, d.nr = 7, 4
    h = ctypes.c_void_p()
    assert lib.sdd_plan_create(ctypes.byref(d), ctypes.byref(h)) == _lib.SDD_ERR_ODD_NFM
    assert lib.sdd_step(None, 1, None, None, None, None, 1, 0, None) == _lib.SDD_ERR_ARG
    assert lib.sdd_batch_step(None, 1, 1, 0, None) == _lib.SDD_ERR_ARG
    g = (_lib.BatchGroup * 1)()
    assert lib.sdd_batch_step(g, 1, 1, 0, None) == _lib.SDD_ERR_ARG      # no plan
    assert lib.sdd_batch_step(g, 0, 1, 0, None) == _lib.SDD_ERR_ARG


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of the option/result structs have the C header's field offsets and sizes (a C
    program compiled against include/sdd_gb300.h prints them)."""
    import shutil
    import subprocess
    import pytest
    from spectraldoublediffusiveconvection_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"sdd_plan_desc": _lib.PlanDesc, "sdd_newton_opts": _lib.NewtonOpts,
               "sdd_newton_result": _lib.NewtonResult, "sdd_contin_opts": _lib.ContinOpts,
               "sdd_contin_result": _lib.ContinResult, "sdd_batch_group": _lib.BatchGroup}
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "sdd_gb300.h"', "int main(void) {"]
    for cname, cls in mirrors.items():
        lines.append('  printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for fname, _ in cls._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, fname, cname, fname))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, cls in mirrors.items():
        assert got[(cname, "sizeof")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, (cname, fname)
