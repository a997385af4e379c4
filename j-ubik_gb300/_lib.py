"""ctypes binding of ``libjubik_gb300.so`` (the C ABI of ``include/jubik_gb300.h``).

Only plain pointers, sizes and a stream handle cross this boundary; device
memory and streams come from PyTorch.  There is no CPU fallback: if the
library is missing, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libjubik_gb300.so")
HEADER = os.path.join(os.path.dirname(_HERE), "include", "jubik_gb300.h")

OK = 0
ERR_INVALID_ARGUMENT = -1
ERR_UNSUPPORTED = -2
ERR_CUDA = -3
ERR_ALLOC = -4
ERR_STATE = -5

F32, F64 = 0, 1
PATH_AUTO, PATH_FUSED, PATH_PLAIN, PATH_FUSED_UNIT = 0, 1, 2, 3
PSF_PRECUT, PSF_FULL = 0, 1


class PlanDesc(C.Structure):
    _fields_ = [("n_modules", C.c_int32), ("n_energies", C.c_int32),
                ("nx", C.c_int32), ("ny", C.c_int32),
                ("n_patches", C.c_int32), ("margin", C.c_int32),
                ("dtype", C.c_int32), ("path", C.c_int32),
                ("pixel_area", C.c_double)]


class JubikError(RuntimeError):
    """A CUDA-side failure reported by the library."""


class JubikUnsupported(NotImplementedError):
    """The shape is outside what the GB300 kernels cover."""


class JubikStateError(RuntimeError):
    """A plan was used before its PSF / exposure / data were set."""


_vp, _i32, _i64, _dbl = C.c_void_p, C.c_int32, C.c_int64, C.c_double
_SIGS = {
    "jubik_abi_version": ([], C.c_int),
    "jubik_last_error": ([], C.c_char_p),
    "jubik_fused_supported": ([_i32, _i32], C.c_int),
    "jubik_fft_length_supported": ([_i32], C.c_int),
    "jubik_plan_create": ([C.POINTER(PlanDesc), C.POINTER(_vp)], C.c_int),
    "jubik_plan_destroy": ([_vp], C.c_int),
    "jubik_plan_workspace_bytes": ([_vp, C.POINTER(_i64)], C.c_int),
    "jubik_plan_path": ([_vp, C.POINTER(_i32)], C.c_int),
    "jubik_plan_set_profiling": ([_vp, _i32], C.c_int),
    "jubik_plan_profile": ([_vp, C.POINTER(C.c_double), C.POINTER(_i64)], C.c_int),
    "jubik_plan_set_psf": ([_vp, _vp, _i32, _i32, _vp], C.c_int),
    "jubik_plan_set_exposure": ([_vp, _vp, _vp, _vp], C.c_int),
    "jubik_plan_readout_sizes": ([_vp, C.POINTER(_i64), C.POINTER(_i64)], C.c_int),
    "jubik_plan_readout_index": ([_vp, C.POINTER(_vp)], C.c_int),
    "jubik_plan_set_data": ([_vp, _vp, _vp], C.c_int),
    "jubik_psf_forward": ([_vp, _vp, _vp, _vp], C.c_int),
    "jubik_psf_adjoint": ([_vp, _vp, _vp, _vp], C.c_int),
    "jubik_response_forward": ([_vp, _vp, _vp, _vp], C.c_int),
    "jubik_response_jvp": ([_vp, _vp, _vp, _vp], C.c_int),
    "jubik_response_vjp": ([_vp, _vp, _vp, _vp], C.c_int),
    "jubik_poisson_energy_grad": ([_vp, _vp, _vp, _vp, _vp], C.c_int),
    "jubik_metric_apply": ([_vp, _vp, _vp, _vp, _vp], C.c_int),
    "jubik_poisson_energy": ([_vp, _vp, _i64, _i32, _vp, _vp, _vp], C.c_int),
    "jubik_elementwise": ([_i32, _vp, _vp, _vp, _i64, _i32, _vp, _vp], C.c_int),
    "jubik_readout_gather": ([_vp, _vp, _vp, _i64, _i32, _vp, _vp], C.c_int),
    "jubik_readout_scatter": ([_vp, _vp, _vp, _i64, _i32, _vp, _vp], C.c_int),
    "jubik_slice_patches": ([_vp, _i64, _i32, _i32, _i32, _i32, _i32, _vp, _vp], C.c_int),
    "jubik_slice_patches_adjoint": ([_vp, _i64, _i32, _i32, _i32, _i32, _i32, _vp, _vp],
                                    C.c_int),
    "jubik_convolve2d": ([_vp, _i64, _vp, _i64, _i32, _i32, _dbl, _i32, _vp, _vp], C.c_int),
    "jubik_convolve2d_noalloc": ([_vp, _i64, _vp, _i64, _i32, _i32, _dbl, _i32, _vp, _vp],
                                 C.c_int),
    "jubik_philox4x32_10": ([_vp, _vp, _vp], C.c_int),
    "jubik_random_normal": ([_vp, _i64, _i32, C.c_uint64, C.c_uint64, _vp], C.c_int),
    "jubik_random_poisson": ([_vp, _i64, _i32, C.c_uint64, C.c_uint32, _vp, _vp], C.c_int),
    "jubik_dot": ([_vp, _vp, _i64, _i32, _vp, _vp], C.c_int),
    "jubik_plan_set_dependent_launch": ([_vp, _i32], C.c_int),
    "jubik_plan_set_forward_run": ([_vp, _i32], C.c_int),
    "jubik_plan_set_metric_lambda": ([_vp, _vp, _i32, _vp], C.c_int),
    "jubik_plan_forward_run": ([_vp, _vp], C.c_int),
    "jubik_group_create": ([_vp, _i32, _vp], C.c_int),
    "jubik_group_set_io": ([_vp, _vp, _vp, _vp], C.c_int),
    "jubik_group_energy_grad": ([_vp, _vp], C.c_int),
    "jubik_group_launches": ([_vp, _vp], C.c_int),
    "jubik_group_destroy": ([_vp], C.c_int),
    "jubik_poisson_energy_grad_logsky": ([_vp, _vp, _i32, _i32, _i32, _vp, _vp, _vp], C.c_int),
    "jubik_psf_interpolate": ([_vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _i32, _i32, _i32,
                               _dbl, _dbl, _i32, _i32, _i32, _vp, _vp], C.c_int),
    "jubik_cf_create": ([_i32, _i32, _i32, _vp, _i32, _i32, _vp], C.c_int),
    "jubik_cf_apply": ([_vp, _vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp], C.c_int),
    "jubik_cf_vjp": ([_vp, _vp, _vp, _vp, _vp, _i32, _i32, _i32, _vp, _vp, _vp, _vp, _vp],
                     C.c_int),
    "jubik_cf_destroy": ([_vp], C.c_int),
}

_lib = None


def header_symbols(path: str = HEADER):
    """Every function the public header declares."""
    with open(path) as f:
        text = f.read()
    return sorted(set(re.findall(r"JUBIK_API\s+(?:const\s+)?\w+\*?\s+(jubik_\w+)\s*\(", text)))


def load(path: str = LIB_PATH):
    """Load the library (no CUDA call is made)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise JubikError(
            f"{os.path.basename(path)} is not built; run "
            "`python -c 'import __graft_entry__ as g; g.build()'` first")
    lib = C.CDLL(path)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _lib = lib
    return lib


def last_error() -> str:
    msg = load().jubik_last_error()
    return msg.decode(errors="replace") if msg else ""


def check(status: int, what: str = "") -> None:
    if status == OK:
        return
    msg = last_error()
    text = f"{what}: {msg}" if what else msg
    if status == ERR_INVALID_ARGUMENT:
        raise ValueError(text)
    if status == ERR_UNSUPPORTED:
        raise JubikUnsupported(text)
    if status == ERR_ALLOC:
        raise MemoryError(text)
    if status == ERR_STATE:
        raise JubikStateError(text)
    raise JubikError(text)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)
