"""ctypes binding of include/bricklib_gb300.h (libbrick_gb300.so).

Loading fails loudly when the library has not been built: there is no fallback.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libbrick_gb300.so")

BK_MAX_TAPS = 343
BK_MAX_TAPS4 = 81

BK_OK, BK_ERR_ARG, BK_ERR_CUDA, BK_ERR_NOMEM, BK_ERR_UNSUPPORTED, BK_ERR_BOUNDS, BK_ERR_BUDGET, \
    BK_ERR_STATE, BK_ERR_TIMEOUT = range(9)
STATUS_NAMES = ["BK_OK", "BK_ERR_ARG", "BK_ERR_CUDA", "BK_ERR_NOMEM", "BK_ERR_UNSUPPORTED",
                "BK_ERR_BOUNDS", "BK_ERR_BUDGET", "BK_ERR_STATE", "BK_ERR_TIMEOUT"]

BK_F64, BK_F32, BK_BF16 = 0, 1, 2
BK_ACC_NATIVE, BK_ACC_COMPENSATED, BK_ACC_FLOATFLOAT = 0, 1, 2


class BkError(RuntimeError):
    def __init__(self, status: int, msg: str):
        name = STATUS_NAMES[status] if 0 <= status < len(STATUS_NAMES) else str(status)
        super().__init__(f"{name}: {msg}")
        self.status = status


class bk_layout(C.Structure):
    _fields_ = [("bdim", C.c_int * 3), ("fold", C.c_int * 3)]


class bk_field(C.Structure):
    _fields_ = [("dat", C.c_void_p), ("chunks", C.c_long), ("step", C.c_size_t),
                ("offset", C.c_size_t), ("dtype", C.c_int)]


class bk_stencil(C.Structure):
    _fields_ = [("npoints", C.c_int), ("offsets", (C.c_int * 3) * BK_MAX_TAPS),
                ("coeff", C.c_double * BK_MAX_TAPS), ("pre_op", C.c_int), ("post_op", C.c_int)]


BK_OP_NONE, BK_OP_RELU, BK_OP_ABS = 0, 1, 2


class bk_batch_domain(C.Structure):
    _fields_ = [("adj", C.c_void_p), ("nbricks", C.c_uint), ("dat", C.c_void_p), ("chunks", C.c_long),
                ("step", C.c_size_t), ("off0", C.c_size_t), ("off1", C.c_size_t), ("blist", C.c_void_p),
                ("nlist", C.c_uint), ("pairs", C.c_void_p), ("npairs", C.c_uint), ("stencil", C.c_int),
                ("n", C.c_long * 3), ("gdims", C.c_long * 3), ("grid", C.c_void_p)]


class bk_layout4(C.Structure):
    _fields_ = [("bdim", C.c_int * 4), ("fold", C.c_int * 4)]


class bk_stencil4(C.Structure):
    _fields_ = [("npoints", C.c_int), ("offsets", (C.c_int * 4) * BK_MAX_TAPS4), ("coeff", C.c_double * BK_MAX_TAPS4)]


class bk_decomp_region(C.Structure):
    _fields_ = [("neighbor", C.c_uint64), ("skin_st", C.c_uint), ("skin_ed", C.c_uint), ("pos", C.c_uint),
                ("len", C.c_uint), ("first_pad", C.c_uint), ("last_pad", C.c_uint)]


class bk_job_desc(C.Structure):
    _fields_ = [("n", C.c_long * 3), ("stencil", C.POINTER(bk_stencil)), ("steps", C.c_int), ("dtype", C.c_int),
                ("acc", C.c_int), ("input", C.c_void_p), ("output", C.c_void_p)]


class bk_server_report(C.Structure):
    _fields_ = [("submitted", C.c_ulonglong), ("admitted", C.c_ulonglong), ("completed", C.c_ulonglong),
                ("rejected", C.c_ulonglong), ("ticks", C.c_ulonglong), ("p50_s", C.c_double), ("p99_s", C.c_double),
                ("mean_s", C.c_double), ("max_s", C.c_double), ("gstencil_s", C.c_double), ("span_s", C.c_double),
                ("hbm_budget", C.c_size_t), ("hbm_peak", C.c_size_t)]


_vp = C.c_void_p
_P = C.POINTER

# name: (restype, argtypes); every int-returning call is a bk_status
SIGNATURES = {
    "bk_abi_version": (C.c_int, []),
    "bk_last_error": (C.c_char_p, []),
    "bk_set_device": (C.c_int, [C.c_int]),
    "bk_device_synchronize": (C.c_int, []),
    "bk_stream_synchronize": (C.c_int, [_vp]),
    "bk_device_malloc": (C.c_int, [_P(_vp), C.c_size_t]),
    "bk_device_free": (C.c_int, [_vp]),
    "bk_host_malloc": (C.c_int, [_P(_vp), C.c_size_t]),
    "bk_host_free": (C.c_int, [_vp]),
    "bk_memcpy": (C.c_int, [_vp, _vp, C.c_size_t, C.c_int, _vp]),
    "bk_memset": (C.c_int, [_vp, C.c_int, C.c_size_t, _vp]),
    "bk_info_to_device": (C.c_int, [_vp, C.c_uint, _P(_vp)]),
    "bk_storage_to_device": (C.c_int, [_vp, C.c_long, C.c_size_t, C.c_int, _P(_vp)]),
    "bk_storage_to_host": (C.c_int, [_vp, C.c_long, C.c_size_t, C.c_int, _vp]),
    "bk_measure_fma_rate": (C.c_int, [C.c_int, _vp, _P(C.c_double)]),
    "bk_fill_uniform": (C.c_int, [_vp, C.c_size_t, C.c_int, C.c_uint64, C.c_double, C.c_double, _vp]),
    "bk_stencil_check": (C.c_int, [_P(bk_stencil), _P(bk_layout), _P(C.c_int), _P(C.c_int)]),
    "bk_sweep": (C.c_int, [_vp, C.c_uint, _P(bk_field), _P(bk_field), _vp, C.c_uint,
                           _P(bk_stencil), _P(bk_layout), C.c_int, _vp]),
    "bk_sweep_kernel": (C.c_int, [_P(bk_field), _P(bk_field), _P(bk_stencil), _P(bk_layout), C.c_int,
                                  _P(C.c_char_p)]),
    "bk_error_flags": (C.c_int, [_vp, _P(C.c_int)]),
    "bk_sweep4": (C.c_int, [_vp, C.c_uint, _P(bk_field), _P(bk_field), _vp, C.c_uint, _P(bk_stencil4),
                            _P(bk_layout4), _vp]),
    "bk_decomp_create": (C.c_int, [C.c_int, _P(C.c_uint), _P(C.c_uint), C.c_uint, C.c_uint, C.c_size_t, C.c_long,
                                   _P(C.c_uint64), C.c_uint, _P(_vp)]),
    "bk_decomp_info": (C.c_int, [_vp, _P(C.c_uint), _P(C.c_size_t), _P(C.c_uint), _P(C.c_uint)]),
    "bk_decomp_grid": (C.c_int, [_vp, _P(C.c_uint)]),
    "bk_decomp_adjacency": (C.c_int, [_vp, _P(C.c_uint)]),
    "bk_decomp_regions": (C.c_int, [_vp, _P(bk_decomp_region), _P(bk_decomp_region), _P(C.c_long)]),
    "bk_decomp_exchange_links": (C.c_int, [_vp, _vp, C.c_size_t, _P(C.c_uint64)]),
    "bk_decomp_destroy": (None, [_vp]),
    "bk_ghost_fill": (C.c_int, [_vp, C.c_uint, _P(bk_field), _P(bk_layout), _vp]),
    "bk_periodic_plan": (C.c_int, [_vp, _P(C.c_long), _P(C.c_long), _vp, C.c_long, _P(C.c_long)]),
    "bk_region_copy": (C.c_int, [_vp, C.c_uint, _vp]),
    "bk_convert": (C.c_int, [_P(bk_field), _P(bk_field), _vp, C.c_uint, _P(bk_layout), _vp]),
    "bk_field_norms": (C.c_int, [_P(bk_field), _P(bk_field), _vp, C.c_uint, _P(bk_layout), _vp,
                                 _P(C.c_double)]),
    "bk_field_norms_noalloc": (C.c_int, [_P(bk_field), _P(bk_field), _vp, C.c_uint, _P(bk_layout), _vp,
                                         _P(C.c_double)]),
    "bk_fill_sines": (C.c_int, [_P(bk_field), _P(bk_layout), _P(C.c_long), _P(C.c_long), C.c_int, C.c_uint64,
                                C.c_double, _vp]),
    "bk_batch_create": (C.c_int, [_P(_vp), _P(bk_batch_domain), C.c_uint, _P(bk_stencil), C.c_uint,
                                  _P(bk_layout), C.c_int, C.c_int]),
    "bk_batch_set_grid": (C.c_int, [_vp, C.c_int]),
    "bk_batch_run": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp]),
    "bk_batch_set_concurrent": (C.c_int, [_vp, C.c_int]),
    "bk_batch_set_stages": (C.c_int, [_vp, C.c_int]),
    "bk_set_pipeline_depth": (C.c_int, [C.c_int]),
    "bk_get_pipeline_depth": (C.c_int, []),
    "bk_batch_parity": (C.c_int, [_vp]),
    "bk_batch_is_arena": (C.c_int, [_vp]),
    "bk_batch_destroy": (C.c_int, [_vp]),
    "bk_copy_to_bricks": (C.c_int, [_vp, _P(C.c_long), _P(C.c_long), _P(C.c_long), _vp, _P(bk_field),
                                    _P(bk_layout), _vp]),
    "bk_copy_from_bricks": (C.c_int, [_vp, _P(C.c_long), _P(C.c_long), _P(C.c_long), _vp, _P(bk_field),
                                      _P(bk_layout), _vp]),
    "bk_server_create": (C.c_int, [_P(_vp), C.c_size_t, _P(bk_layout), C.c_int]),
    "bk_server_submit": (C.c_int, [_vp, _P(bk_job_desc), _P(C.c_ulonglong)]),
    "bk_server_wait": (C.c_int, [_vp, C.c_ulonglong, C.c_double, _P(C.c_double)]),
    "bk_server_drain": (C.c_int, [_vp, C.c_double]),
    "bk_server_stats": (C.c_int, [_vp, _P(bk_server_report)]),
    "bk_server_destroy": (C.c_int, [_vp]),
    "bk_steps": (C.c_int, [_vp, C.c_uint, _P(bk_field), _P(bk_field), _vp, C.c_uint, _vp, C.c_uint,
                           _P(bk_stencil), _P(bk_layout), C.c_int, C.c_int, C.c_int, C.c_int, _vp]),
}

_lib = None


def lib() -> C.CDLL:
    """The loaded library; raises if it was not built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: build it with "
                               "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != BK_OK:
        raise BkError(status, lib().bk_last_error().decode(errors="replace"))


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))
