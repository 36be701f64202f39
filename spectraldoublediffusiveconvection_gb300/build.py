"""Build ``libsdd_gb300.so`` in-tree with nvcc for sm_103a (GB300).

Each ``csrc/*.cu`` is compiled to an object in parallel and the objects are linked into a shared
library next to this file.  ``python -m spectraldoublediffusiveconvection_gb300.build`` runs it.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsdd_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"]
# The nonlinear-term kernels write every multiply-add as an explicit fma and are compiled without
# automatic contraction, so the fused and the split kernels (and every batch size) round identically.
FILE_FLAGS = {"sdd_fx.cu": ["-fmad=false"]}


def _nvcc():
    nv = shutil.which("nvcc")
    if nv is None:
        for cand in ("/usr/local/cuda/bin/nvcc",):
            if os.path.exists(cand):
                nv = cand
    if nv is None:
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsdd_gb300")
    return nv


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, extra_flags=()):
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(HERE, "..", "include", "sdd_gb300.h"))
    headers.append(os.path.abspath(__file__))     # flag changes rebuild
    srcs = sources()
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        if not force and not _stale(obj, [src] + headers):
            return None
        cmd = [nvcc, *ARCH, *FLAGS, *FILE_FLAGS.get(os.path.basename(src), []), *extra_flags, "-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            print(r.stderr, flush=True)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    if force or _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv,
          extra_flags=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else ())
