"""numpy <-> device helpers shared by the drop-in modules.

The drop-ins accept numpy arrays (copied to the GPU and back: the reference's numpy-in/numpy-out
contract) or CUDA float64 torch tensors (used in place, results stay on the device).
"""
import numpy as np


def torch():
    import torch as _t
    return _t


def is_tensor(x):
    try:
        import torch as _t
    except ImportError:
        return False
    return isinstance(x, _t.Tensor)


def to_dev(x, device=None):
    """Returns (contiguous float64 CUDA tensor, came_from_numpy)."""
    t = torch()
    if is_tensor(x):
        if x.device.type != "cuda":
            return x.to(device=device or "cuda", dtype=t.float64).contiguous(), True
        return x.to(dtype=t.float64).contiguous(), False
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    return t.from_numpy(a).to(device=device or "cuda", non_blocking=False), True


def back(t, was_numpy):
    return t.cpu().numpy() if was_numpy else t
