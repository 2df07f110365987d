"""ctypes binding of ``libfdlbm.so`` (the C ABI declared in include/fdlbm.h).

There is no fallback: if the shared library is missing or fails to load,
:func:`lib` raises.  Build it with ``python -m fingering_dynamics_gb300.build``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

PKG = os.path.dirname(os.path.abspath(__file__))
# the in-tree build; FDLBM_LIBRARY names another build of the same sources (built with other
# compile-time tile options: python -m fingering_dynamics_gb300.build --out DIR --define ...)
LIB_PATH = os.environ.get("FDLBM_LIBRARY") or os.path.join(PKG, "_lib", "libfdlbm.so")

FD_OK = 0
FD_F64, FD_F32, FD_F16, FD_BF16 = 0, 1, 2, 3
FD_VARIANT_PERIODIC, FD_VARIANT_WALLS, FD_VARIANT_PERIODIC_XY = 0, 1, 2
FD_INIT_MU, FD_INIT_UY, FD_INIT_VELOCITY, FD_OUTLET_PRESSURE = 1, 2, 4, 8
FD_ROUND_NEAREST, FD_ROUND_STOCHASTIC = 0, 1
ROUNDING = {"nearest": FD_ROUND_NEAREST, "stochastic": FD_ROUND_STOCHASTIC}
TERMS = {"large_F": 0, "feq": 1, "geq": 2, "F": 3, "G": 4}
FIELDS = {"rho": 0, "npx": 1, "npy": 2, "np2": 3, "mu": 4, "mu_plain": 5, "ux": 6, "uy": 7, "p": 8, "mix_tau": 9, "psi": 10}
ERRORS = {-1: "FD_ERR_ARG", -2: "FD_ERR_SHAPE", -3: "FD_ERR_CUDA", -4: "FD_ERR_DTYPE", -5: "FD_ERR_SCRATCH",
          -6: "FD_ERR_NONFINITE"}
FD_ERR_NONFINITE = -6
FD_STATUS_WAIT_TIMEOUT, FD_STATUS_NONFINITE = 1, 2


class FDError(RuntimeError):
    """A libfdlbm call returned a negative status."""

    def __init__(self, code, fn, msg):
        super().__init__(f"{fn}: {ERRORS.get(code, code)}: {msg}")
        self.code = code


class fd_params(C.Structure):
    _fields_ = [("H", C.c_int32), ("W", C.c_int32), ("variant", C.c_int32), ("flags", C.c_uint32),
                ("tau", C.c_double), ("eta_n", C.c_double), ("M", C.c_double), ("a", C.c_double),
                ("kappa", C.c_double), ("gamma", C.c_double), ("psi_wall", C.c_double),
                ("outlet_coef", C.c_double), ("force_x", C.c_double), ("force_y", C.c_double)]


class fd_storage(C.Structure):
    _fields_ = [("dtype", C.c_int32), ("f_scale_log2", C.c_int32), ("g_scale_log2", C.c_int32),
                ("rounding", C.c_int32), ("seed", C.c_uint32)]


class fd_diag(C.Structure):
    _fields_ = [("mass_r", C.c_double), ("mass_b", C.c_double), ("saturation", C.c_double),
                ("invaded", C.c_int64), ("fluid", C.c_int64), ("tip_x", C.c_int32), ("breakthrough", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class fd_instance(C.Structure):
    _fields_ = [("prm", fd_params), ("mask", C.c_void_p), ("inlet_ux", C.c_void_p), ("pop_a", C.c_void_p),
                ("pop_b", C.c_void_p), ("side_a", C.c_void_p), ("side_b", C.c_void_p), ("seed", C.c_uint32)]


class fd_fields(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("f", "g", "psi", "npx", "npy", "np2", "rho", "ux", "uy", "p", "mu",
                                          "mix_tau")]


_VP, _I, _PD, _SZ, _FL = C.c_void_p, C.c_int, C.c_ssize_t, C.c_size_t, C.c_float
_P = C.POINTER(fd_params)
_S = C.POINTER(fd_storage)
_F = C.POINTER(fd_fields)

# name -> argtypes (all return int status unless listed in _RET)
SIGNATURES = {
    "fd_abi_version": [],
    "fd_last_error": [],
    "fd_compute_init": [_P, _I, _VP, _VP, _VP, _F, _VP],
    "fd_collide": [_P, _I, _VP, _F, _VP],
    "fd_add_nonequilibrium": [_P, _I, _VP, _F, _VP],
    "fd_collision_term": [_P, _I, _I, _I, _VP, _F, _VP, _VP],
    "fd_stream": [_P, _I, _VP, _VP, _VP, _VP, _VP],
    "fd_bounce_back": [_P, _I, _VP, _VP, _VP, _VP, _VP, _VP],
    "fd_bottom_top_wall": [_I, _I, _I, _PD, _PD, _VP, _VP, _VP, _VP, _VP],
    "fd_boundary_fields": [_P, _I, _VP, _VP, _VP, _VP, _VP],
    "fd_zou_he_inlet": [_P, _I, _VP, _VP, _VP, _VP, _VP],
    "fd_zou_he_outlet": [_P, _I, _VP, _VP, _VP, _VP, _VP],
    "fd_update_rho_psi": [_P, _I, _VP, _F, _VP],
    "fd_update_macros": [_P, _I, _VP, _F, _VP],
    "fd_field": [_P, _I, _I, _VP, _F, _VP, _VP],
    "fd_fused_step": [_P, _I, _VP, _VP, _VP, _VP, _VP, _VP, _I, _I, _VP],
    "fd_packed_bytes": [_I, _I, _S],
    "fd_pack": [_P, _I, _VP, _S, _VP, _VP],
    "fd_unpack": [_P, _S, _VP, _I, _VP, _VP],
    "fd_fused_step_packed": [_P, _S, _VP, _VP, _VP, _VP, _VP, _VP, _I, _I, _VP],
    "fd_device_status": [C.POINTER(C.c_uint), _I],
    "fd_selftest_wait_timeout": [C.c_uint, _I, _VP],
    "fd_fused_step_packed_noalloc": [_P, _S, _VP, _VP, _VP, _VP, _VP, _I, _I, _VP],
    "fd_fused_step_packed_host": [_P, _S, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _VP, _I, _I, _VP],
    "fd_diag_scratch_bytes": [],
    "fd_batch_create": [C.POINTER(fd_instance), _I, _S, _I, _I, C.POINTER(C.c_void_p)],
    "fd_batch_configure": [_VP, _I, _I],
    "fd_batch_step": [_VP, _I, _I, _VP],
    "fd_batch_parity": [_VP],
    "fd_batch_member_status": [_VP, C.POINTER(C.c_uint32), _I],
    "fd_batch_tiles": [_VP],
    "fd_batch_grid": [_VP],
    "fd_batch_destroy": [_VP],
    "fd_diagnostics": [_P, _I, _S, _VP, _VP, _VP, _VP, _VP],
    # learned surrogate (include/fdsurrogate.h)
    "sg_conv3x3": [_VP, _I, _I, _I, _I, _VP, _VP, _I, _I, _VP, _VP, _VP],
    "sg_flip_weights": [_VP, _I, _I, _VP, _VP],
    "sg_conv3x3_tc": [_VP, _I, _I, _I, _I, _VP, _VP, _I, _I, _VP, _VP, _VP],
    "sg_tc_status": [C.POINTER(C.c_uint), _I],
    "sg_conv3x3_tma": [_VP, _I, _I, _I, _I, _VP, _VP, _I, _I, _VP, _VP, _VP],
    "sg_conv3x3_tma_ws": [_VP, _I, _I, _I, _I, _VP, _VP, _I, _I, _VP, _VP, _VP],
    "sg_conv3x3_wgrad": [_VP, _VP, _I, _I, _I, _I, _I, _VP, _VP, _SZ, _I, _VP],
    "sg_conv3x3_wgrad_tc": [_VP, _VP, _I, _I, _I, _I, _I, _VP, _VP, _SZ, _I, _VP],
    "sg_wgrad_partial_floats": [_I, _I, _I, _I, _I],
    "sg_bias_grad": [_VP, _SZ, _I, _VP, _VP, _VP],
    "sg_bias_partial_floats": [_I],
    "sg_gelu_bwd": [_VP, _VP, _SZ, _VP, _VP],
    "sg_pool2": [_VP, _I, _I, _I, _I, _VP, _VP],
    "sg_pool2_bwd": [_VP, _I, _I, _I, _I, _VP, _VP],
    "sg_up2": [_VP, _I, _I, _I, _I, _VP, _I, _I, _VP],
    "sg_up2_bwd": [_VP, _I, _I, _I, _I, _I, _I, _VP, _VP],
    "sg_copy_channels": [_VP, _SZ, _I, _VP, _I, _I, _VP],
    "sg_add_channels": [_VP, _SZ, _I, _I, _I, _VP, _VP],
    "sg_masked_mse": [_VP, _VP, _VP, _SZ, _I, _VP, _VP, _FL, _VP],
    "sg_loss_blocks": [],
    "sg_adamw": [_VP, _VP, _VP, _VP, _VP, _SZ, _FL, _FL, _FL, _FL, _FL, _I, _VP],
    "sg_to_bf16": [_VP, _SZ, _VP, _VP],
}
_RET = {"fd_last_error": C.c_char_p, "fd_packed_bytes": C.c_size_t, "fd_diag_scratch_bytes": C.c_size_t,
        "sg_wgrad_partial_floats": C.c_size_t, "sg_bias_partial_floats": C.c_size_t}

_lock = threading.Lock()
_handle = None


def lib():
    """Load (once) and return the bound library.  Raises if it is missing."""
    global _handle
    with _lock:
        if _handle is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"libfdlbm.so not built ({LIB_PATH}); run python -m fingering_dynamics_gb300.build")
            h = C.CDLL(LIB_PATH)
            for name, args in SIGNATURES.items():
                fn = getattr(h, name)
                fn.argtypes = args
                fn.restype = _RET.get(name, C.c_int)
            _handle = h
        return _handle


def call(name, *args):
    """Call an entry point and raise FDError on a negative status."""
    h = lib()
    r = getattr(h, name)(*args)
    if r != FD_OK:
        raise FDError(r, name, h.fd_last_error().decode(errors="replace"))
    return r
