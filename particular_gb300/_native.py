"""Loads libparticular_cuda.so (the C ABI of include/particular_cuda.h) with ctypes.

There is no fallback: if the library is missing or a call fails, a CudaError is
raised, as particular's gpu method panics on a failed device call
(particular/src/gpu/resources.rs:345, gpu/mod.rs:200).
"""
import ctypes
import os
import re

from . import build_native

PT_OK = 0
PT_ERR_INVALID = -1
PT_ERR_CUDA = -2
PT_ERR_OOM = -3
PT_ERR_CAPACITY = -4
PT_ERR_TIMEOUT = -5
PT_ERR_DEPTH = -6

PT_BF_EXACT = 0x1
PT_BF_VEC3A = 0x2
PT_BH_QUADRUPOLE = 0x1
PT_BH_GROUP = 0x2
PT_BH_LEARNED = 0x4
PT_BH_LOCAL = 0x8
PT_BH_RELATIVE = 0x10
PT_MLP_NPARAM = 5188
PT_METHOD_BRUTE_FORCE = 0
PT_METHOD_BARNES_HUT = 1


class Timing(ctypes.Structure):
    _fields_ = [("build_ms", ctypes.c_float), ("walk_ms", ctypes.c_float)]


class BhStats(ctypes.Structure):
    _fields_ = [("nodes", ctypes.c_uint64), ("cells", ctypes.c_uint64),
                ("leaves", ctypes.c_uint64), ("interactions", ctypes.c_uint64),
                ("visits", ctypes.c_uint64), ("warps", ctypes.c_uint64),
                ("max_stack", ctypes.c_uint64), ("overflow", ctypes.c_uint64),
                ("learned", ctypes.c_uint64), ("cell_interactions", ctypes.c_uint64),
                ("local_nodes", ctypes.c_uint64), ("local_quad_nodes", ctypes.c_uint64)]

_NAMES = {PT_ERR_INVALID: "PT_ERR_INVALID", PT_ERR_CUDA: "PT_ERR_CUDA", PT_ERR_OOM: "PT_ERR_OOM",
          PT_ERR_CAPACITY: "PT_ERR_CAPACITY", PT_ERR_TIMEOUT: "PT_ERR_TIMEOUT",
          PT_ERR_DEPTH: "PT_ERR_DEPTH"}

HEADER = os.path.join(build_native.ROOT, "include", "particular_cuda.h")


class CudaError(RuntimeError):
    """A failed call into libparticular_cuda.so (status code + message)."""

    def __init__(self, code, message):
        self.code = code
        super().__init__(f"{_NAMES.get(code, code)}: {message}")


_lib = None

c_size = ctypes.c_size_t
c_ptr = ctypes.c_void_p


def _declare(L):
    sig = {
        "pt_ctx_create": (ctypes.c_int, [ctypes.POINTER(c_ptr), ctypes.c_int]),
        "pt_ctx_destroy": (None, [c_ptr]),
        "pt_last_error": (ctypes.c_char_p, []),
        "pt_ctx_set_stream": (ctypes.c_int, [c_ptr, c_ptr]),
        "pt_ctx_set_capacity_limit": (ctypes.c_int, [c_ptr, c_size]),
        "pt_ctx_device_bytes": (c_size, [c_ptr]),
        "pt_ctx_launch_count": (ctypes.c_uint64, [c_ptr]),
        "pt_ctx_sm_count": (ctypes.c_int, [c_ptr]),
        "pt_ctx_synchronize": (ctypes.c_int, [c_ptr]),
        "pt_bf_accel_f32": (ctypes.c_int, [c_ptr, c_ptr, c_size, c_ptr, c_size, ctypes.c_float,
                                           ctypes.c_int, ctypes.c_uint32, c_ptr]),
        "pt_bf_accel_f32_device": (ctypes.c_int, [c_ptr, c_ptr, c_size, c_ptr, c_size,
                                                  ctypes.c_float, ctypes.c_int, ctypes.c_uint32,
                                                  c_ptr]),
        "pt_bf_accel_dvec3": (ctypes.c_int, [c_ptr, c_ptr, ctypes.c_size_t, c_ptr, ctypes.c_size_t,
                                             ctypes.c_double, ctypes.c_int, c_ptr]),
        "pt_bf_accel_dvec3_device": (ctypes.c_int, [c_ptr, c_ptr, ctypes.c_size_t, c_ptr, ctypes.c_size_t,
                                                    ctypes.c_double, ctypes.c_int, c_ptr]),
        "pt_bf_accel_f64_device": (ctypes.c_int, [c_ptr, c_ptr, c_size, c_ptr, c_size,
                                                  ctypes.c_double, ctypes.c_int, c_ptr]),
        "pt_bf_set_plan": (ctypes.c_int, [c_ptr, ctypes.c_int, ctypes.c_int]),
        "pt_measure_fp32_peak": (ctypes.c_int, [c_ptr, ctypes.POINTER(ctypes.c_double)]),
        "pt_bf_accel_f32_noalloc": (ctypes.c_int, [c_ptr, c_size, c_ptr, c_size, ctypes.c_float,
                                                   ctypes.c_int, c_ptr, c_ptr]),
        "pt_bh_accel_f32": (ctypes.c_int, [c_ptr, c_ptr, c_size, c_ptr, c_size, ctypes.c_float,
                                           ctypes.c_float, ctypes.c_uint32, c_ptr]),
        "pt_bh_accel_f32_device": (ctypes.c_int, [c_ptr, c_ptr, c_size, c_ptr, c_size,
                                                  ctypes.c_float, ctypes.c_float, ctypes.c_uint32,
                                                  c_ptr]),
        "pt_bh_last_stats": (ctypes.c_int, [c_ptr, ctypes.POINTER(BhStats)]),
        "pt_bh_set_stack_limit": (ctypes.c_int, [c_ptr, ctypes.c_int]),
        "pt_bh_set_learned_capacity": (ctypes.c_int, [c_ptr, ctypes.c_int]),
        "pt_bh_set_local_ratio": (ctypes.c_int, [c_ptr, ctypes.c_float]),
        "pt_bh_set_relative_alpha": (ctypes.c_int, [c_ptr, ctypes.c_float]),
        "pt_bh_set_relative_monopole": (ctypes.c_int, [c_ptr, ctypes.c_float]),
        "pt_bh_accel_dvec3": (ctypes.c_int, [c_ptr, c_ptr, ctypes.c_size_t, c_ptr, ctypes.c_size_t,
                                             ctypes.c_double, ctypes.c_double, ctypes.c_uint32, c_ptr]),
        "pt_bh_accel_dvec3_device": (ctypes.c_int, [c_ptr, c_ptr, ctypes.c_size_t, c_ptr, ctypes.c_size_t,
                                                    ctypes.c_double, ctypes.c_double, ctypes.c_uint32,
                                                    c_ptr]),
        "pt_bh_export_tree_dvec3": (ctypes.c_int, [c_ptr, c_ptr, c_ptr, c_ptr, ctypes.c_size_t]),
        "pt_bh_build_device": (ctypes.c_int, [c_ptr, c_ptr, ctypes.c_size_t, c_ptr]),
        "pt_bh_walk_device": (ctypes.c_int, [c_ptr, c_ptr, ctypes.c_size_t, ctypes.c_float, ctypes.c_float,
                                             ctypes.c_uint32, c_ptr]),
        "pt_bh_tree_generation": (ctypes.c_int, [c_ptr, c_ptr]),
        "pt_bh_load_tree": (ctypes.c_int, [c_ptr, c_ptr, c_ptr, c_ptr, c_ptr, ctypes.c_size_t, ctypes.c_int64,
                                           c_ptr]),
        "pt_bh_build": (ctypes.c_int, [c_ptr, c_ptr, ctypes.c_size_t, c_ptr]),
        "pt_bh_walk": (ctypes.c_int, [c_ptr, c_ptr, ctypes.c_size_t, ctypes.c_float, ctypes.c_float,
                                      ctypes.c_uint32, c_ptr]),
        "pt_bh_export_tree": (ctypes.c_int, [c_ptr, c_ptr, c_ptr, c_ptr, c_size]),
        "pt_ctx_set_timing": (ctypes.c_int, [c_ptr, ctypes.c_int]),
        "pt_mlp_init": (ctypes.c_int, [c_ptr, ctypes.c_uint64]),
        "pt_mlp_set_params": (ctypes.c_int, [c_ptr, c_ptr, c_size, ctypes.c_float]),
        "pt_mlp_get_params": (ctypes.c_int, [c_ptr, c_ptr, c_size]),
        "pt_mlp_generate": (ctypes.c_int, [c_ptr, c_ptr, c_size, ctypes.c_int, ctypes.c_float,
                                           ctypes.c_float, ctypes.c_float, c_size,
                                           ctypes.POINTER(c_size)]),
        "pt_mlp_reset_dataset": (ctypes.c_int, [c_ptr]),
        "pt_mlp_export_dataset": (ctypes.c_int, [c_ptr, c_ptr, c_ptr, c_size]),
        "pt_mlp_train": (ctypes.c_int, [c_ptr, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                        ctypes.c_uint64, ctypes.POINTER(ctypes.c_float)]),
        "pt_mlp_loss_grad": (ctypes.c_int, [c_ptr, c_ptr, c_ptr, ctypes.c_int, c_ptr,
                                            ctypes.POINTER(ctypes.c_double)]),
        "pt_mlp_predict": (ctypes.c_int, [c_ptr, c_ptr, ctypes.c_int, c_ptr]),
        "pt_mlp_predict_tc": (ctypes.c_int, [c_ptr, c_ptr, ctypes.c_int, c_ptr]),
        "pt_ensemble_run": (ctypes.c_int, [c_ptr, c_ptr, ctypes.c_uint32, c_ptr, c_ptr,
                                           ctypes.c_float, ctypes.c_int, ctypes.c_float,
                                           ctypes.c_int]),
        "pt_ensemble_tune": (ctypes.c_int, [c_ptr, c_ptr, ctypes.c_uint32, c_ptr, ctypes.c_float,
                                            c_ptr]),
        "pt_ensemble_set_table": (ctypes.c_int, [c_ptr, c_ptr]),
        "pt_ensemble_set_tiles": (ctypes.c_int, [c_ptr, c_ptr]),
        "pt_ensemble_get_shape": (ctypes.c_int, [c_ptr, c_ptr, c_ptr]),
        "pt_ensemble_set_barrier": (ctypes.c_int, [c_ptr, ctypes.c_longlong, ctypes.c_int]),
        "pt_leapfrog": (ctypes.c_int, [c_ptr, c_ptr, c_ptr, c_size, ctypes.c_float, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                       ctypes.c_uint32]),
        "pt_leapfrog_device": (ctypes.c_int, [c_ptr, c_ptr, c_ptr, c_ptr, c_size, ctypes.c_float,
                                              ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                              ctypes.c_float, ctypes.c_uint32, ctypes.c_int]),
        "pt_last_timing": (ctypes.c_int, [c_ptr, ctypes.POINTER(Timing)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args


def lib_path():
    return build_native.LIB


def lib():
    """The loaded native library; raises if it has not been built."""
    global _lib
    if _lib is None:
        path = build_native.LIB
        if not os.path.exists(path):
            raise CudaError(PT_ERR_CUDA, f"{path} is not built: run "
                            "`python -c 'import __graft_entry__ as g; g.build()'` first")
        L = ctypes.CDLL(path)
        _declare(L)
        _lib = L
    return _lib


def last_error():
    msg = lib().pt_last_error()
    return msg.decode() if msg else ""


def check(rc):
    if rc != PT_OK:
        raise CudaError(rc, last_error())
    return rc


def header_functions():
    """Names of every function the C header declares."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pt_[a-z0-9_]+)\s*\(", text)))
