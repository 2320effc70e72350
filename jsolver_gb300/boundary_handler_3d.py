"""do_BCs for 3D arrays (jsolver/boundary_handler_3d.py:3-35).

Same behaviour as the reference, including its use of ``vals_yb`` / ``vals_ye`` for the
z faces (boundary_handler_3d.py:32-33; ``vals_zb`` / ``vals_ze`` are accepted and unused).
"""
import ctypes

import numpy as np
import torch


def do_BCs(arr, rim=1, direction=-1, vals_xb=None, vals_xe=None, vals_yb=None, vals_ye=None, vals_zb=None,  # noqa: N802
           vals_ze=None):
    upper = rim + 1
    if isinstance(arr, torch.Tensor):
        out = arr.clone()
        if (arr.is_cuda and rim == 1 and direction == -1 and arr.dtype == torch.float64
                and all(v is None for v in (vals_xb, vals_xe, vals_yb, vals_ye))):
            from . import _lib
            out = out.contiguous()
            shape = (ctypes.c_int32 * 3)(*out.shape)
            _lib.check(_lib.load().jmg_do_bcs(3, shape, ctypes.c_void_p(out.data_ptr()),
                                               ctypes.c_void_p(torch.cuda.current_stream(out.device).cuda_stream)))
            return out
        conv = (lambda v: torch.as_tensor(v, dtype=out.dtype, device=out.device))
    else:
        out = np.array(arr, copy=True)
        conv = np.asarray
    if direction in (-1, 0):
        out[:, :, :upper] = 0 if vals_xb is None else conv(vals_xb)[:, :, None]
        out[:, :, -upper:] = 0 if vals_xe is None else conv(vals_xe)[:, :, None]
    if direction in (-1, 1):
        out[:, :upper, :] = 0 if vals_yb is None else conv(vals_yb)[:, None, :]
        out[:, -upper:, :] = 0 if vals_ye is None else conv(vals_ye)[:, None, :]
    if direction in (-1, 2):
        out[:upper, :, :] = 0 if vals_yb is None else conv(vals_yb)[None, :, :]
        out[-upper:, :, :] = 0 if vals_ye is None else conv(vals_ye)[None, :, :]
    return out
