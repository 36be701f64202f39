"""Drop-in for the reference's ``Transforms.py``: the theta transforms on the GPU.

Same call surface and scaling conventions as Transforms.py:8-129 (``grid``, ``DCT``, ``IDCT``, ``DST``,
``IDST``); the transforms run as batched rows in ``sdd_transform`` (FP64 FFT-based DCT-II/III and
DST-II/III in shared memory).  numpy in -> numpy out; CUDA tensors stay on the device.
"""
import ctypes

import numpy as np

from . import _lib
from ._dev import back, to_dev, torch

L = np.pi


def grid(N):
    """Transforms.py:8-13: theta_i = pi(2i+1)/(2N)."""
    dx = L / N
    return dx * (2.0 * np.arange(N) + 1.0) / 2.0


def _run(kind, x, n_out_fn, axis):
    t = torch()
    xt, was_np = to_dev(x)
    xt = t.movedim(xt, axis, -1).contiguous()
    n_in = xt.shape[-1]
    n_out = n_out_fn(n_in)
    rows = int(np.prod(xt.shape[:-1])) if xt.dim() > 1 else 1
    out = t.empty(xt.shape[:-1] + (n_out,), dtype=t.float64, device=xt.device)
    stream = ctypes.c_void_p(t.cuda.current_stream(xt.device).cuda_stream)
    _lib.check(_lib.lib().sdd_transform(kind, rows, n_in, n_out, ctypes.c_void_p(xt.data_ptr()),
                                        ctypes.c_void_p(out.data_ptr()), stream), "sdd_transform")
    out = t.movedim(out, -1, axis)
    return back(out, was_np)


def DST(g, n=None, axis=-1):
    """Transforms.py:73-85: sinusoid amplitudes b_w = (2/N) sum_i g_i sin(w theta_i), [0] = 0, first n."""
    return _run(_lib.SDD_DST, g, lambda m: m if n is None else min(int(n), m), axis)


def IDST(g_hat, n=None, axis=-1):
    """Transforms.py:87-100: g(theta_i) = sum_{w=1}^{N-1} b_w sin(w theta_i) on grid(n)."""
    return _run(_lib.SDD_IDST, g_hat, lambda m: m if n is None else int(n), axis)


def DCT(f, n=None, axis=-1):
    """Transforms.py:102-114: a_k = (2/N) sum_i f_i cos(k theta_i), a_0 halved, first n."""
    return _run(_lib.SDD_DCT, f, lambda m: m if n is None else min(int(n), m), axis)


def IDCT(f_hat, n=None, axis=-1):
    """Transforms.py:116-129: f(theta_i) = a_0 + sum_{k>=1} a_k cos(k theta_i) on grid(n)."""
    return _run(_lib.SDD_IDCT, f_hat, lambda m: m if n is None else int(n), axis)
