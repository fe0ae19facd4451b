"""ctypes binding of libporelb_gpu.so (declarations in include/porelb_gpu.h).

The library is built in-tree by ``__graft_entry__.build()`` (or ``make -C
porelb_gb300/csrc``).  Loading fails loudly when it is missing: there is no
CPU fallback for the solver.
"""
import ctypes
import os

import numpy as np

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib",
                        "libporelb_gpu.so")

Q = 19

# NEIGHBOR_INFO (porelb.h:58-62) and NODE_INFO (porelb.h:73-76) layouts.
NB_DTYPE = np.dtype([("node_type", "u1"), ("pad_", "u1"),
                     ("node_pid", "<u2"), ("node_id", "<u4")])
NODE_DTYPE = np.dtype([("x", "<u2"), ("y", "<u2"), ("z", "<u2"),
                       ("pad_", "<u2"), ("nb_info", NB_DTYPE, (Q - 1,))])
assert NB_DTYPE.itemsize == 8 and NODE_DTYPE.itemsize == 152

TYPE_FLUID, TYPE_SOLID, TYPE_EXTERN = 0, 1, 2

OK = 0
ERR_ARG, ERR_IO, ERR_TABLE, ERR_CUDA = -1, -2, -3, -4
ERR_NOMEM, ERR_DENSITY, ERR_NUMP, ERR_STATE = -5, -6, -7, -8

FP64_EXACT, FP64, FP32, FP16DEV, BF16DEV, FP64_FMA = 0, 1, 2, 3, 4, 5
ORDER_MORTON, ORDER_REFERENCE, ORDER_AUTO = 0, 1, 2
HALO_AUTO, HALO_SINGLE, HALO_REMOTE_WINS = -1, 0, 1
REDUCE_NOALLOC_MAX_NODES = 67108864
BOUNDARY_REFERENCE, BOUNDARY_HALFWAY = 0, 1


class Params(ctypes.Structure):
    _fields_ = [("tau", ctypes.c_double), ("force_x", ctypes.c_double),
                ("precision", ctypes.c_int), ("ordering", ctypes.c_int),
                ("halo", ctypes.c_int), ("block_size", ctypes.c_int),
                ("device", ctypes.c_int), ("boundary", ctypes.c_int),
                ("kernel_variant", ctypes.c_int), ("l2_prefetch", ctypes.c_int),
                ("reserved", ctypes.c_int * 4)]


class SampleParams(ctypes.Structure):
    _fields_ = [("tau", ctypes.c_double), ("force_x", ctypes.c_double),
                ("tol", ctypes.c_double), ("max_steps", ctypes.c_longlong),
                ("handoff_tol", ctypes.c_double), ("reserved", ctypes.c_int * 2)]


class BatchParams(ctypes.Structure):
    _fields_ = [("capacity_nodes", ctypes.c_size_t), ("max_samples", ctypes.c_int),
                ("precision", ctypes.c_int), ("check_every", ctypes.c_int),
                ("keep_macros", ctypes.c_int), ("device", ctypes.c_int),
                ("cta_threads", ctypes.c_int), ("l2_prefetch", ctypes.c_int),
                ("ordering", ctypes.c_int), ("l2_group_kb", ctypes.c_int),
                ("reserved", ctypes.c_int * 4)]


_P = ctypes.c_void_p
_I = ctypes.c_int
_D = ctypes.c_double
_IP = ctypes.POINTER(ctypes.c_int)
_DP = ctypes.POINTER(ctypes.c_double)

_SIGS = {
    "plb_default_params": (None, [ctypes.POINTER(Params)]),
    "plb_build_table": (_I, [_P, _I, _I, _I, _I, _P, _IP, _IP]),
    "plb_write_vbin": (_I, [ctypes.c_char_p, _P, _I, _I, _I, _I, _I, _IP]),
    "plb_read_vbin_header": (_I, [ctypes.c_char_p, _IP, _IP, _IP, _IP, _IP]),
    "plb_read_vbin": (_I, [ctypes.c_char_p, _P, _IP]),
    "plb_check_table": (_I, [_P, _I, _I, _I, _I, _I, _IP]),
    "plb_sphere_pack": (_I, [ctypes.c_uint64, _I, _I, _I, _D, _D, _D, _P,
                              _IP, _DP]),
    "plb_create": (_I, [_P, _I, _I, _I, _I, _I, _IP, ctypes.POINTER(Params),
                        ctypes.POINTER(_P)]),
    "plb_destroy": (None, [_P]),
    "plb_create_from_flag": (_I, [_P, _I, _I, _I, _I, ctypes.POINTER(Params),
                                  ctypes.POINTER(_P)]),
    "plb_sphere_pack_device": (_I, [ctypes.c_uint64, _I, _I, _I, _D, _D, _D,
                                    _I, _P, _IP, _DP]),
    "plb_create_packed": (_I, [ctypes.c_uint64, _I, _I, _I, _D, _D, _D, _I,
                               ctypes.POINTER(Params), ctypes.POINTER(_P),
                               _IP, _DP]),
    "plb_init_equilibrium": (_I, [_P]),
    "plb_step": (_I, [_P, _I, _I]),
    "plb_step_async": (_I, [_P, _I, _I]),
    "plb_sync": (_I, [_P]),
    "plb_get_macros": (_I, [_P, _P, _P, _P, _P]),
    "plb_save_parts": (_I, [_P, ctypes.c_char_p, _I]),
    "plb_get_f": (_I, [_P, _P]),
    "plb_set_f": (_I, [_P, _P]),
    "plb_reduce": (_I, [_P, _DP, _DP]),
    "plb_permeability": (_I, [_P, _DP, _DP]),
    "plb_last_error": (_I, [_P, _IP, _IP, _IP, _IP, _IP, _DP]),
    "plb_info": (_I, [_P, _IP, _IP, _IP, ctypes.POINTER(ctypes.c_size_t)]),
    "plb_stream": (_P, [_P]),
    "plb_status_string": (ctypes.c_char_p, [_I]),
    "plb_batch_bytes_per_node": (ctypes.c_size_t, [_I, _I]),
    "plb_batch_create": (_I, [ctypes.c_size_t, _I, _I, _I, _I, _I,
                              ctypes.POINTER(_P)]),
    "plb_batch_destroy": (None, [_P]),
    "plb_batch_add_flag": (_I, [_P, _P, _I, _I, _I,
                                ctypes.POINTER(SampleParams), _IP]),
    "plb_batch_add_packed": (_I, [_P, ctypes.c_uint64, _I, _I, _I, _D, _D, _D,
                                  ctypes.POINTER(SampleParams), _IP, _IP,
                                  _DP]),
    "plb_batch_create_ex": (_I, [ctypes.POINTER(BatchParams), ctypes.POINTER(_P)]),
    "plb_batch_run": (_I, [_P, _I, _IP]),
    "plb_batch_launch": (_I, [_P, _IP]),
    "plb_batch_finish": (_I, [_P]),
    "plb_batch_transfer": (_I, [_P, _I, _P, _IP]),
    "plb_batch_interval_ms": (_I, [_P, ctypes.POINTER(ctypes.c_float)]),
    "plb_batch_poll": (_I, [_P, _IP, _I, _IP]),
    "plb_batch_result": (_I, [_P, _I, _DP, _DP,
                              ctypes.POINTER(ctypes.c_longlong), _IP]),
    "plb_batch_release": (_I, [_P, _I]),
    "plb_batch_get_f": (_I, [_P, _I, _P]),
    "plb_batch_get_macros": (_I, [_P, _I, _P, _P, _P, _P]),
    "plb_batch_info": (_I, [_P, ctypes.POINTER(ctypes.c_longlong), _IP,
                            ctypes.POINTER(ctypes.c_longlong),
                            ctypes.POINTER(ctypes.c_longlong),
                            ctypes.POINTER(ctypes.c_size_t)]),
    "plb_kernel_flags": (_I, [_P, ctypes.POINTER(ctypes.c_uint)]),
    "plb_get_f_streamed": (_I, [_P, _P]),
    "plb_batch_sample_nodes": (_I, [_P, _I, _IP]),
    "plb_batch_free_nodes": (_I, [_P, ctypes.POINTER(ctypes.c_longlong),
                                  ctypes.POINTER(ctypes.c_longlong)]),
    "plb_batch_stream": (_P, [_P]),
    "plb_reduce_noalloc": (_I, [_P, _P, ctypes.c_longlong, _P, _P]),
    "plb_fault_inject_alloc": (_I, [ctypes.c_longlong]),
    "plb_auto_ordering": (_I, [ctypes.c_longlong, _I, _I, _I]),
    "plb_alloc_count": (ctypes.c_longlong, []),
}

_lib = None


def load():
    """Load libporelb_gpu.so and declare every exported symbol."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is not built; run __graft_entry__.build() "
            "(the solver has no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(_SIGS)
