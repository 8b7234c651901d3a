"""ctypes binding of libbsfh.so (the C ABI declared in include/bsfh.h).

The library must exist (build it with bs45_quantum_explorer_gb300.build.build_library());
loading fails loudly otherwise. There is no CPU fallback.
"""
import ctypes as C
import os

from .build import LIB

BS_OK = 0
BS_STOPPED, BS_WALLED = 1, 2  # partial results: the stop flag / the stream's wall limit
ERRORS = {
    1: "stopped by the context's stop flag", 2: "stream stopped by its wall limit",
    -1: "bad argument", -2: "CUDA runtime error", -3: "out of memory",
    -4: "device wait limit reached", -5: "internal consistency check failed",
    -6: "output capacity exceeded", -7: "no sm_103 CUDA device",
}

HALL_FP64, HALL_TC_FP16, HALL_TC_BF16X2 = 0, 1, 2


class BsError(RuntimeError):
    def __init__(self, code, what=""):
        super().__init__(f"{what}: {ERRORS.get(code, 'error')} ({code})")
        self.code = code


class HallStats(C.Structure):
    _fields_ = [("pairs", C.c_longlong), ("passed", C.c_longlong), ("rechecked", C.c_longlong),
                ("fp64_rechecked", C.c_longlong),
                ("pass_below", C.c_double), ("reject_above", C.c_double),
                ("quant_err", C.c_double), ("mode", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Cell(C.Structure):
    _fields_ = [("tx", C.c_int8 * 8), ("ty", C.c_int8 * 8), ("pinX", C.c_int32), ("pinY", C.c_int32)]


class StreamOpts(C.Structure):
    _fields_ = [("m", C.c_int32), ("rev", C.c_int32), ("endpos", C.c_int32),
                ("cd_prune", C.c_int32), ("hall_mode", C.c_int32), ("ab_side", C.c_int32),
                ("target_prefixes", C.c_longlong), ("leaf_chunk", C.c_longlong),
                ("survivor_cap", C.c_longlong), ("limit", C.c_longlong),
                ("round_us", C.c_longlong), ("wall_sec", C.c_double),
                ("fine_nodes", C.c_double), ("wave_nodes", C.c_double),
                ("dfs_blocks", C.c_int32), ("reserved", C.c_int32)]


class CellStats(C.Structure):
    _fields_ = [("nodes", C.c_longlong), ("leaves", C.c_longlong), ("ok", C.c_longlong)]


class ListOpts(C.Structure):
    _fields_ = [(f, C.c_int32) for f in ("m6", "thm211b", "thm212", "endpos", "orbit_canon",
                                         "orbit_q", "qprune", "prof_order", "nshard", "reserved")]


class AbCand(C.Structure):
    _fields_ = [("c", C.c_uint64), ("d", C.c_uint64), ("row_off", C.c_longlong),
                ("nrows", C.c_int32), ("reserved", C.c_int32)]


class AbOpts(C.Structure):
    _fields_ = [("budget", C.c_longlong), ("outer_k", C.c_int32), ("early", C.c_int32),
                ("canon", C.c_int32), ("m", C.c_int32), ("first_hit", C.c_int32),
                ("a2", C.c_int32), ("max_seconds", C.c_double),
                ("blocks_per_sm", C.c_int32), ("reserved", C.c_int32)]


_lib = None

# (name, restype, argtypes) for every entry point of include/bsfh.h
SIGNATURES = {
    "bs_version": (C.c_int, []),
    "bs_strerror": (C.c_char_p, [C.c_int]),
    "bs_ctx_create": (C.c_int, [C.c_int] * 6 + [C.POINTER(C.c_void_p)]),
    "bs_ctx_destroy": (None, [C.c_void_p]),
    "bs_ctx_retarget": (C.c_int, [C.c_void_p] + [C.c_int] * 5),
    "bs_ctx_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "bs_ctx_device_status": (C.c_int, [C.c_void_p]),
    "bs_ctx_stop_flag": (C.POINTER(C.c_int32), [C.c_void_p]),
    "bs_hall_filter_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_void_p,
                                       C.POINTER(HallStats)]),
    "bs_hall_filter_packed": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_void_p,
                                        C.POINTER(HallStats)]),
    "bs_hall_filter_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_void_p,
                                     C.POINTER(HallStats)]),
    "bs_hall_tc_dump_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.c_int, C.c_void_p]),
    "bs_hall_filter_noalloc": (C.c_int, [C.c_int, C.c_void_p, C.c_longlong, C.c_void_p,
                                         C.c_void_p]),
    "bs_pack_rows": (C.c_int, [C.c_void_p, C.c_longlong, C.c_int, C.c_void_p]),
    "bs_gen_hall_pairs_dev": (C.c_int, [C.c_void_p, C.c_longlong, C.c_uint64, C.c_void_p]),
    "bs_cd_stream": (C.c_int, [C.c_void_p, C.POINTER(Cell), C.c_int, C.POINTER(StreamOpts),
                               C.c_void_p, C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong),
                               C.POINTER(CellStats)]),
    "bs_cell_list": (C.c_int, [C.c_int] * 5 + [C.POINTER(ListOpts), C.POINTER(Cell), C.c_void_p,
                               C.c_longlong, C.POINTER(C.c_longlong), C.c_char_p]),
    "bs_ab_rows": (C.c_int, [C.c_int] * 4 + [C.POINTER(Cell), C.c_longlong, C.c_void_p, C.c_longlong,
                             C.c_void_p, C.c_void_p, C.POINTER(C.c_longlong)]),
    "bs_flat_topk": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.c_longlong, C.c_longlong,
                               C.c_void_p, C.c_void_p, C.POINTER(C.c_longlong)]),
    "bs_flat_topk_dev": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.c_longlong,
                                   C.c_longlong, C.c_void_p, C.c_void_p, C.c_void_p]),
    "bs_complete_ab_batch": (C.c_int, [C.c_void_p, C.POINTER(AbCand), C.c_longlong, C.c_void_p,
                                       C.c_longlong, C.POINTER(AbOpts), C.c_void_p, C.c_void_p,
                                       C.c_void_p, C.c_void_p]),
    "bs_npaf_verify_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p]),
    "bs_join_quads": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p, C.c_longlong,
                                C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong),
                                C.POINTER(C.c_longlong)]),
    "bs_ctx_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "bs_ctx_timing_read": (C.c_int, [C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_longlong),
                                     C.POINTER(C.c_longlong)]),
}


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"{LIB} is missing: build it first (bs45_quantum_explorer_gb300.build)")
        L = C.CDLL(LIB)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code, what):
    if code != BS_OK:
        raise BsError(code, what)
    return code
