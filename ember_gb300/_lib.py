"""ctypes binding of libember_gpu.so (the C ABI declared in include/ember_gpu.h).

The product path has no CPU fallback: if the shared library is missing or
fails to load, every call raises ``EmberGpuError``.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import _build

OK, EINVAL, ECUDA, ENOMEM, EFAIL = 0, -1, -2, -3, -4
MEM_HOST, MEM_DEVICE = 0, 1

BC_FIXED_VALUE, BC_ZERO_GRADIENT, BC_CONTROL_VOLUME, BC_WALL_FLUX, BC_FLOATING = 0, 1, 2, 3, 4

dp = C.POINTER(C.c_double)
ip = C.POINTER(C.c_int)
i64p = C.POINTER(C.c_int64)


class EmberGpuError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


class DiffusionGrid(C.Structure):
    _fields_ = [("n_points", C.c_int), ("left_bc", C.c_int), ("right_bc", C.c_int), ("alpha", C.c_int)]


class DiffusionOptions(C.Structure):
    _fields_ = [("t_start", C.c_double), ("t_end", C.c_double), ("dt_multiplier", C.c_double),
                ("global_timestep", C.c_double), ("h", C.c_void_p), ("wall_const", C.c_void_p),
                ("y_inf", C.c_void_p), ("algorithm", C.c_int)]

DIFFUSION_PARALLEL, DIFFUSION_SERIAL = 0, 1


_lock = threading.Lock()
_lib = None


def _declare(lib):
    vp = C.c_void_p
    sig = {
        "ember_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
        "ember_version": (C.c_int, []),
        "ember_device_count": (C.c_int, []),
        "ember_tridiag_create": (C.c_int, [C.c_int, i64p, C.POINTER(vp)]),
        "ember_tridiag_destroy": (C.c_int, [vp]),
        "ember_tridiag_set_coefficients": (C.c_int, [vp, vp, vp, vp, vp, C.c_int, vp]),
        "ember_tridiag_set_y0": (C.c_int, [vp, vp, C.c_int, vp]),
        "ember_tridiag_initialize": (C.c_int, [vp, vp, vp, C.c_int, vp]),
        "ember_tridiag_step": (C.c_int, [vp, vp]),
        "ember_tridiag_integrate_to_time": (C.c_int, [vp, vp, C.c_int, vp]),
        "ember_tridiag_get_state": (C.c_int, [vp, vp, vp, vp, C.c_int, vp]),
        "ember_tridiag_get_ydot": (C.c_int, [vp, vp, C.c_int, vp]),
        "ember_diffusion_integrate": (C.c_int, [C.c_int, C.POINTER(DiffusionGrid), C.c_int, vp, vp, vp, vp, vp,
                                                C.POINTER(DiffusionOptions), vp, C.c_int, vp]),
        "ember_diffusion_integrate_noalloc": (C.c_int, [C.c_int, C.POINTER(DiffusionGrid), C.c_int, vp, vp, vp,
                                                        vp, vp, C.POINTER(DiffusionOptions), vp, vp]),
        "ember_diffusion_adjoint": (C.c_int, [C.c_int, C.POINTER(DiffusionGrid), C.c_int, vp, vp, vp, vp,
                                              C.POINTER(DiffusionOptions), vp, C.c_int, vp]),
        "ember_probe_fp64_rate": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
        "ember_probe_fp64_issue": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]),
        "ember_math_eval": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_int64]),
        "ember_mech_create": (C.c_int, [vp, C.POINTER(vp)]),
        "ember_mech_destroy": (C.c_int, [vp]),
        "ember_mech_set_multipliers": (C.c_int, [vp, vp, C.c_int, vp]),
        "ember_gas_eval": (C.c_int, [vp, C.c_int, C.c_double, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp,
                                     C.c_int, vp]),
        "ember_source_options_default": (C.c_int, [vp]),
        "ember_selftest_qss_cesium": (C.c_int, [C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                                C.c_int, C.c_int, C.c_double, C.c_int, vp, vp]),
        "ember_source_integrate": (C.c_int, [vp, C.c_int, C.c_int, vp, vp, vp, C.c_double, vp, vp, vp, vp, vp,
                                             C.c_int, vp]),
        "ember_source_adjoint": (C.c_int, [vp, C.c_int, vp, vp, vp, C.c_double, vp, vp, vp, C.c_int, vp, vp, vp, vp,
                                           C.c_int, vp]),
        "ember_source_adjoint_qss": (C.c_int, [vp, C.c_int, vp, vp, vp, C.c_double, vp, vp, vp, C.c_int, vp, vp, vp,
                                               vp, C.c_int, vp]),
        "ember_source_autotune": (C.c_int, [vp, C.c_int, C.c_int, vp, vp, vp, C.c_double, vp, vp, vp, vp, C.c_int,
                                            vp]),
        "ember_transport_create": (C.c_int, [vp, vp, vp]),
        "ember_transport_destroy": (C.c_int, [vp]),
        "ember_transport_eval": (C.c_int, [vp, C.c_int, C.c_double, C.c_double, vp, vp, vp, C.c_int, vp]),
        "ember_split_set_transport_model": (C.c_int, [vp, vp, C.c_double, C.c_int]),
        "ember_split_load_state": (C.c_int, [vp, vp, C.c_int, vp]),
        "ember_mech_get_tuning": (C.c_int, [vp, vp, vp, vp, vp, vp, vp]),
        "ember_convection_integrate": (C.c_int, [C.c_int, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp,
                                                 C.c_int, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def library_path() -> str:
    return _build.LIB


def lib():
    """Load libember_gpu.so (building it first if the sources are newer)."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if not os.path.exists(path) or _build._stale():
                try:
                    _build.build()
                except Exception as e:  # no nvcc, or a compile error
                    if not os.path.exists(path):
                        raise EmberGpuError(ECUDA, f"libember_gpu.so is not built and cannot be built: {e}")
            try:
                _lib = _declare(C.CDLL(path))
            except OSError as e:
                raise EmberGpuError(ECUDA, f"cannot load {path}: {e}")
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(2048)
    lib().ember_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, what: str = "") -> None:
    if rc != OK:
        raise EmberGpuError(rc, f"{what}: {last_error()}" if what else last_error())


def ptr(a) -> int | None:
    """Address of a contiguous float64/int array: numpy (host) or torch (host or device)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return a.data_ptr()
    raise TypeError(f"unsupported array type {type(a)!r}")


def mem_of(a) -> int:
    if hasattr(a, "is_cuda") and a.is_cuda:
        return MEM_DEVICE
    return MEM_HOST


def stream_ptr(stream) -> int | None:
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)
