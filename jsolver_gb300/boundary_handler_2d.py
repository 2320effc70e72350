"""do_BCs for 2D arrays (jsolver/boundary_handler_2d.py:3-30).

Sets the first/last ``rim + 1`` columns (direction 0 or -1) and then rows (direction 1
or -1) to zero or to the given value vectors; returns a new array. NumPy arrays are
handled on the host; CUDA tensors on the device (the default zero frame through the
library's ``jmg_do_bcs`` kernel).
"""
import ctypes

import numpy as np
import torch


def do_BCs(arr, rim=1, direction=-1, vals_xb=None, vals_xe=None, vals_yb=None, vals_ye=None):  # noqa: N802
    upper = rim + 1
    if isinstance(arr, torch.Tensor):
        out = arr.clone()
        if (arr.is_cuda and rim == 1 and direction == -1 and arr.dtype == torch.float64
                and all(v is None for v in (vals_xb, vals_xe, vals_yb, vals_ye))):
            from . import _lib
            out = out.contiguous()
            shape = (ctypes.c_int32 * 2)(*out.shape)
            _lib.check(_lib.load().jmg_do_bcs(2, shape, ctypes.c_void_p(out.data_ptr()),
                                               ctypes.c_void_p(torch.cuda.current_stream(out.device).cuda_stream)))
            return out
        conv = (lambda v: torch.as_tensor(v, dtype=out.dtype, device=out.device))
    else:
        out = np.array(arr, copy=True)
        conv = np.asarray
    if direction in (-1, 0):
        out[:, :upper] = 0 if vals_xb is None else conv(vals_xb)[:, None]
        out[:, -upper:] = 0 if vals_xe is None else conv(vals_xe)[:, None]
    if direction in (-1, 1):
        out[:upper] = 0 if vals_yb is None else conv(vals_yb)[None, :]
        out[-upper:] = 0 if vals_ye is None else conv(vals_ye)[None, :]
    return out
