"""Array plumbing shared by the 2D/3D front ends: type/shape rules and device transfer."""
import numpy as np
import torch


def is_cuda_tensor(x):
    return isinstance(x, torch.Tensor) and x.is_cuda


def shape_of(x):
    if isinstance(x, torch.Tensor):
        return tuple(x.shape)
    return tuple(np.shape(x))


def is_scalar(x):
    """jnp.isscalar on a traced argument: a Python scalar or a 0-d array."""
    return len(shape_of(x)) == 0


def is_float64(x):
    """dtype rule of the reference (solver_2d.py:449): every argument must be float64.

    A Python float is float64; a Python int or bool is not (the reference traces them
    as integer/bool arrays and raises)."""
    if isinstance(x, torch.Tensor):
        return x.dtype == torch.float64
    if isinstance(x, bool):
        return False
    if isinstance(x, float):
        return True
    if isinstance(x, int):
        return False
    return np.asarray(x).dtype == np.float64


def scalar_value(x):
    if isinstance(x, torch.Tensor):
        return float(x.item())
    return float(np.asarray(x))


def to_device(x, device, pin=False):
    """float64 contiguous CUDA tensor view of an array argument."""
    if isinstance(x, torch.Tensor):
        t = x.to(device=device, dtype=torch.float64)
        return t.contiguous()
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    t = torch.from_numpy(a)
    if pin:
        t = t.pin_memory()
    return t.to(device, non_blocking=pin)


def pick_device(*args):
    for a in args:
        if is_cuda_tensor(a):
            return a.device
    if not torch.cuda.is_available():
        raise RuntimeError("jsolver_gb300 runs on a CUDA GPU (sm_103a); no CUDA device is available")
    return torch.device("cuda", torch.cuda.current_device())
