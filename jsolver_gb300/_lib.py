"""ctypes binding of libjmg.so (declarations in include/jmg.h).

The library is the only compute path of this package: there is no CPU fallback. If
``libjmg.so`` is missing, or no CUDA device is present when a solve is requested, the
calls raise instead of computing anything elsewhere.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libjmg.so")

JMG_OK, JMG_ERR_VALUE, JMG_ERR_CUDA, JMG_ERR_WORKSPACE, JMG_ERR_TIMEOUT = 0, 1, 2, 3, 4
STOP_DISTANCE, STOP_RESIDUAL = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
OUTER_RICHARDSON, OUTER_FCG = 0, 1


class JmgGrid(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int32), ("m", ctypes.c_int32 * 3), ("idel", ctypes.c_double * 3),
                ("is_linear", ctypes.c_int32 * 3)]


class JmgConfig(ctypes.Structure):
    _fields_ = [("fixed", ctypes.c_int32), ("gamma", ctypes.c_int32), ("fcycle", ctypes.c_int32),
                ("skip_pre", ctypes.c_int32), ("nu1", ctypes.c_int32), ("nu2", ctypes.c_int32),
                ("max_iters_outer", ctypes.c_int64), ("max_iters_inner", ctypes.c_int64),
                ("epsilon", ctypes.c_double), ("stop", ctypes.c_int32), ("rtol", ctypes.c_double),
                ("precision", ctypes.c_int32), ("inner_cycles", ctypes.c_int32), ("outer", ctypes.c_int32),
                ("off_diag", ctypes.c_int32)]


class JmgCoeffs(ctypes.Structure):
    _fields_ = [("lam", ctypes.c_void_p), ("lam_scalar", ctypes.c_double),
                ("D", ctypes.c_void_p * 3), ("D_scalar", ctypes.c_double * 3), ("D_xy", ctypes.c_void_p)]


class JmgBatchStrides(ctypes.Structure):
    _fields_ = [("lam", ctypes.c_int64), ("D", ctypes.c_int64 * 3), ("D_xy", ctypes.c_int64)]


# every symbol of include/jmg.h with its ctypes signature
_P = ctypes.c_void_p
_SIGS = {
    "jmg_config_default": (None, [ctypes.POINTER(JmgConfig)]),
    "jmg_plan_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.POINTER(JmgGrid), ctypes.POINTER(JmgConfig)]),
    "jmg_plan_destroy": (ctypes.c_int, [_P]),
    "jmg_plan_workspace_bytes": (ctypes.c_size_t, [_P]),
    "jmg_plan_levels": (ctypes.c_int, [_P]),
    "jmg_solve": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(JmgCoeffs), _P, _P, _P, ctypes.c_size_t, _P]),
    "jmg_batched_workspace_bytes": (ctypes.c_size_t, [_P, ctypes.c_int32]),
    "jmg_plan_sweep_launches": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
    "jmg_solve_batched": (ctypes.c_int, [_P, ctypes.c_int32, _P, _P, ctypes.POINTER(JmgCoeffs),
                                         ctypes.POINTER(JmgBatchStrides), _P, _P, _P, ctypes.c_size_t, _P]),
    "jmg_solve2d_f64": (ctypes.c_int, [ctypes.POINTER(JmgGrid), ctypes.POINTER(JmgConfig), _P, _P,
                                       ctypes.POINTER(JmgCoeffs), _P, _P, _P, ctypes.c_size_t, _P]),
    "jmg_solve3d_f64": (ctypes.c_int, [ctypes.POINTER(JmgGrid), ctypes.POINTER(JmgConfig), _P, _P,
                                       ctypes.POINTER(JmgCoeffs), _P, _P, _P, ctypes.c_size_t, _P]),
    "jmg_build_hierarchy": (ctypes.c_int, [_P, ctypes.POINTER(JmgCoeffs), _P, ctypes.c_size_t, _P]),
    "jmg_op_sweep": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, ctypes.c_size_t, _P]),
    "jmg_op_restrict": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "jmg_op_prolong": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, ctypes.c_size_t, _P]),
    "jmg_op_residual": (ctypes.c_int, [_P, ctypes.c_int, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "jmg_op_coeff": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _P, _P, ctypes.c_size_t, _P]),
    "jmg_rel_residual": (ctypes.c_int, [_P, _P, _P, _P, _P, ctypes.c_size_t, _P]),
    "jmg_do_bcs": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int32), _P, _P]),
    "jmg_op_smooth_ws": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _P, ctypes.c_size_t, _P]),
    "jmg_op_smooth32_ws": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _P, ctypes.c_size_t, _P]),
    "jmg_op_coarse_ws": (ctypes.c_int, [_P, ctypes.c_int, _P, ctypes.c_size_t, _P]),
    "jmg_op_fcg_residual_ws": (ctypes.c_int, [_P, _P, ctypes.c_size_t, _P]),
    "jmg_plan_coarse_start": (ctypes.c_int, [_P]),
    "jmg_plan_mid_start": (ctypes.c_int, [_P]),
    "jmg_plan_level_fused": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int]),
    "jmg_op_smooth_restrict_ws": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int, _P, ctypes.c_size_t, _P]),
    "jmg_plan_launch_counts": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "jmg_solve_check": (ctypes.c_int, [_P, _P, ctypes.c_size_t, _P]),
    "jmg_rel_residual_noalloc": (ctypes.c_int, [ctypes.POINTER(JmgGrid), _P, _P, ctypes.POINTER(JmgCoeffs), _P, _P]),
    "jmg_adjoint_workspace_bytes": (ctypes.c_size_t, [_P]),
    "jmg_tangent_workspace_bytes": (ctypes.c_size_t, [_P]),
    "jmg_solve_fixed_jvp": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(JmgCoeffs), _P, _P, ctypes.POINTER(JmgCoeffs), _P,
                                           _P, _P, ctypes.c_size_t, _P, ctypes.c_size_t, _P]),
    "jmg_solve_jvp": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(JmgCoeffs), _P, _P, ctypes.POINTER(JmgCoeffs), _P, _P,
                                     _P, _P, ctypes.c_size_t, _P, ctypes.c_size_t, _P]),
    "jmg_solve_fixed_vjp": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(JmgCoeffs), _P, _P, _P, _P, _P, _P, _P,
                                           ctypes.c_size_t, _P, ctypes.c_size_t, _P]),
    "jmg_solve_fixed_vjp_nd": (ctypes.c_int, [_P, _P, _P, ctypes.POINTER(JmgCoeffs), _P, _P, _P, _P,
                                              ctypes.POINTER(_P), _P, _P, ctypes.c_size_t, _P, ctypes.c_size_t, _P]),
    "jmg_net_num_params": (ctypes.c_int64, []),
    "jmg_net_create": (ctypes.c_int, [ctypes.POINTER(_P), ctypes.c_int, ctypes.c_int]),
    "jmg_net_destroy": (None, [_P]),
    "jmg_net_set_params": (ctypes.c_int, [_P, _P, _P]),
    "jmg_net_get_params": (ctypes.c_int, [_P, _P, _P]),
    "jmg_net_forward": (ctypes.c_int, [_P, _P, ctypes.c_int, _P, _P]),
    "jmg_net_loss_grad": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, _P, _P, _P]),
    "jmg_net_train_step": (ctypes.c_int, [_P, _P, _P, ctypes.c_int, ctypes.c_float, _P, _P]),
    "jmg_net_inputs_2d": (ctypes.c_int, [_P, ctypes.POINTER(JmgGrid), ctypes.POINTER(JmgCoeffs), _P, _P, _P, _P]),
    "jmg_net_target_2d": (ctypes.c_int, [_P, ctypes.POINTER(JmgGrid), _P, _P, ctypes.c_float, _P, _P]),
    "jmg_net_guess_2d": (ctypes.c_int, [_P, ctypes.POINTER(JmgGrid), ctypes.POINTER(JmgCoeffs), _P, ctypes.c_float,
                                        _P, _P]),
    "jmg_last_error": (ctypes.c_char_p, []),
}

_lib = None


def load():
    """Load libjmg.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
                          "or `python -m jsolver_gb300._build` (CUDA toolkit required)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc):
    """Translate a status code into the exception the reference would raise."""
    if rc == JMG_OK:
        return
    msg = load().jmg_last_error().decode()
    if rc == JMG_ERR_VALUE:
        raise ValueError(msg)
    raise RuntimeError(f"jmg error {rc}: {msg}")


def default_config():
    c = JmgConfig()
    load().jmg_config_default(ctypes.byref(c))
    return c


class Plan:
    """Owns a JmgPlan (validated level layout + cached CUDA graph)."""

    def __init__(self, grid, config):
        lib = load()
        self._h = ctypes.c_void_p()
        check(lib.jmg_plan_create(ctypes.byref(self._h), ctypes.byref(grid), ctypes.byref(config)))
        self.grid, self.config = grid, config
        self.workspace_bytes = lib.jmg_plan_workspace_bytes(self._h)
        self.levels = lib.jmg_plan_levels(self._h)

    @property
    def handle(self):
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib is not None:
            _lib.jmg_plan_destroy(h)
            self._h = None
