"""ctypes binding of libjyulb_gb300.so (C ABI declared in include/jyulb_gb300.h).

The library is built in-tree by ``jyulb.build.build()`` (``__graft_entry__.build``)
into this package directory.  Loading fails loudly: there is no CPU fallback
for the time step.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libjyulb_gb300.so")

JLB_OK = 0
JLB_ERR_INVALID_ARG = -1
JLB_ERR_STATE = -2
JLB_ERR_CUDA = -3
JLB_ERR_NOMEM = -4
JLB_ERR_UNSUPPORTED = -5
JLB_ERR_NUMERIC = -6

# every symbol include/jyulb_gb300.h declares
EXPORTED_SYMBOLS = (
    "jlb_check_config", "jlb_create", "jlb_destroy", "jlb_finalize_init", "jlb_set_acc", "jlb_set_static_halo", "jlb_evolve",
    "jlb_step", "jlb_download_moments", "jlb_get_populations", "jlb_set_populations", "jlb_bc_data",
    "jlb_reduce", "jlb_residual", "jlb_flow_info", "jlb_reduce_moments_noalloc", "jlb_tot_tsteps", "jlb_rlx_prm", "jlb_kernel_launches",
    "jlb_transfer_bytes", "jlb_host_timers",
    "jlb_last_error", "jlb_batch_create", "jlb_batch_destroy", "jlb_batch_step", "jlb_batch_moments", "jlb_batch_set_bc",
    "jlb_batch_populations", "jlb_batch_info", "jlb_batch_domain_fluid", "jlb_batch_last_error",
    "jlb_adj_create", "jlb_adj_destroy", "jlb_adj_forward", "jlb_adj_backward", "jlb_adj_timers", "jlb_adj_last_error",
    "jlb_adj_create_moving", "jlb_adj_forward_fields", "jlb_adj_backward_fields",
    "jlb_build_info",
)


class jlb_config(ctypes.Structure):
    _fields_ = [
        ("lat_size", ctypes.c_int32 * 3),
        ("rlx_scheme", ctypes.c_int32),
        ("kvisc", ctypes.c_double),
        ("g", ctypes.c_double * 3),
        ("bc", ctypes.c_int32 * 6),
        ("precision", ctypes.c_int32),
        ("trt_magic", ctypes.c_double),
        ("kernel", ctypes.c_int32),
        ("kernel_opts", ctypes.c_int32),
        ("stream", ctypes.c_void_p),
    ]


JLB_KERNEL_JYULB = 0
JLB_KERNEL_CXX = 1
JLB_CXX_LINEAR_EQ = 1
JLB_CXX_FORCE2 = 2


class jlb_domain(ctypes.Structure):
    _fields_ = [
        ("lat_size", ctypes.c_int32 * 3),
        ("kvisc", ctypes.c_double),
        ("g", ctypes.c_double * 3),
        ("bc", ctypes.c_int32 * 6),
        ("trt_magic", ctypes.c_double),
        ("phase", ctypes.POINTER(ctypes.c_uint8)),
        ("den", ctypes.POINTER(ctypes.c_double)),
        ("vel", ctypes.POINTER(ctypes.c_double)),
    ]


class EngineUnavailable(RuntimeError):
    """The CUDA engine library is missing or cannot run here."""


_lib = None


def load() -> ctypes.CDLL:
    """Load the engine library (raises EngineUnavailable if it is not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise EngineUnavailable(
            f"{LIB_PATH} is not built; run __graft_entry__.build() (nvcc, sm_103a)")
    lib = ctypes.CDLL(LIB_PATH)
    vp, dp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)
    u8p = ctypes.POINTER(ctypes.c_uint8)
    cfgp = ctypes.POINTER(jlb_config)
    sig = {
        "jlb_check_config": (ctypes.c_int, [cfgp, ctypes.c_char_p, ctypes.c_size_t]),
        "jlb_create": (ctypes.c_int, [cfgp, ctypes.POINTER(vp)]),
        "jlb_destroy": (None, [vp]),
        "jlb_finalize_init": (ctypes.c_int, [vp, u8p, dp, dp, ctypes.POINTER(ctypes.c_uint64)]),
        "jlb_set_acc": (ctypes.c_int, [vp, dp]),
        "jlb_set_static_halo": (ctypes.c_int, [vp, ctypes.c_int]),
        "jlb_evolve": (ctypes.c_int, [vp, ctypes.c_uint32, dp, dp, dp, dp, ctypes.POINTER(ctypes.c_uint32)]),
        "jlb_step": (ctypes.c_int, [vp, ctypes.c_uint32, ctypes.c_int]),
        "jlb_download_moments": (ctypes.c_int, [vp, dp, dp]),
        "jlb_get_populations": (ctypes.c_int, [vp, dp]),
        "jlb_set_populations": (ctypes.c_int, [vp, dp]),
        "jlb_bc_data": (ctypes.c_int, [vp, ctypes.c_int32, dp, dp]),
        "jlb_reduce": (ctypes.c_int, [vp, dp]),
        "jlb_residual": (ctypes.c_int, [vp, dp]),
        "jlb_flow_info": (ctypes.c_int, [vp, ctypes.c_double, dp]),
        "jlb_reduce_moments_noalloc": (ctypes.c_int, [vp, vp, vp, vp, vp, ctypes.c_int64, ctypes.c_int32,
                                                      vp, vp]),
        "jlb_tot_tsteps": (ctypes.c_uint32, [vp]),
        "jlb_rlx_prm": (None, [vp, dp]),
        "jlb_kernel_launches": (ctypes.c_uint64, [vp]),
        "jlb_transfer_bytes": (None, [vp, ctypes.POINTER(ctypes.c_uint64)]),
        "jlb_host_timers": (None, [vp, dp]),
        "jlb_last_error": (ctypes.c_char_p, [vp]),
        "jlb_batch_create": (ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(jlb_domain), ctypes.c_int32, vp,
                                            ctypes.POINTER(vp)]),
        "jlb_batch_destroy": (None, [vp]),
        "jlb_batch_step": (ctypes.c_int, [vp, ctypes.c_uint32]),
        "jlb_batch_moments": (ctypes.c_int, [vp, ctypes.c_int32, dp, dp]),
        "jlb_batch_set_bc": (ctypes.c_int, [vp, ctypes.c_int32, dp, dp]),
        "jlb_batch_populations": (ctypes.c_int, [vp, ctypes.c_int32, dp]),
        "jlb_batch_info": (ctypes.c_int, [vp, ctypes.POINTER(ctypes.c_int64)]),
        "jlb_batch_domain_fluid": (ctypes.c_int32, [vp, ctypes.c_int32]),
        "jlb_batch_last_error": (ctypes.c_char_p, [vp]),
        "jlb_adj_create": (ctypes.c_int, [cfgp, u8p, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(vp)]),
        "jlb_adj_destroy": (None, [vp]),
        "jlb_adj_forward": (ctypes.c_int, [vp, ctypes.c_double, dp, dp, ctypes.c_double, ctypes.c_uint32, dp, dp,
                                           dp]),
        "jlb_adj_backward": (ctypes.c_int, [vp, dp, dp, dp]),
        "jlb_adj_create_moving": (ctypes.c_int, [cfgp, u8p, dp, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(vp)]),
        "jlb_adj_forward_fields": (ctypes.c_int, [vp, ctypes.c_double, dp, dp, dp, ctypes.c_uint32, dp, dp, dp]),
        "jlb_adj_backward_fields": (ctypes.c_int, [vp, dp, dp, dp, dp]),
        "jlb_adj_timers": (ctypes.c_int, [vp, dp]),
        "jlb_adj_last_error": (ctypes.c_char_p, [vp]),
        "jlb_build_info": (ctypes.c_char_p, []),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def u8ptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
