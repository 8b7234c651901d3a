"""ctypes binding of the CPU oracle (oracle/liboracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg to check or time against the product. The product never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
_lib = None

i8p = np.ctypeslib.ndpointer(dtype=np.int8, flags="C_CONTIGUOUS")
u8p = np.ctypeslib.ndpointer(dtype=np.uint8, flags="C_CONTIGUOUS")
i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


class StreamStats(C.Structure):
    _fields_ = [("nodes", C.c_longlong), ("leaves", C.c_longlong), ("ok", C.c_longlong)]


def build():
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.or_hall_tables.argtypes = [C.c_int, f64p, f64p]
        L.or_hall_pair.argtypes = [C.c_int, i8p, i8p, C.c_int, f64p, f64p,
                                   C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.or_hall_pair.restype = C.c_int
        L.or_hall_batch.argtypes = [C.c_int, C.c_int, i8p, C.c_longlong, u8p, C.c_int]
        L.or_hall_batch.restype = C.c_double
        L.or_npaf_at.argtypes = [i8p, i8p, C.c_int, i8p, i8p, C.c_int, C.c_int]
        L.or_npaf_at.restype = C.c_int
        L.or_flat_score.argtypes = [i8p, i8p, C.c_int]
        L.or_flat_score.restype = C.c_longlong
        L.or_autocorr_key.argtypes = [i8p, i8p, C.c_int, C.c_int, C.c_int]
        L.or_autocorr_key.restype = C.c_uint64
        L.or_cd_stream.argtypes = [C.c_int, C.c_int, C.c_int, i32p, i32p, C.c_int, C.c_int,
                                   C.c_int, C.c_int, C.c_int, C.c_int, i8p, u8p, C.c_longlong,
                                   C.POINTER(StreamStats)]
        L.or_cd_stream.restype = C.c_longlong
        L.or_complete_ab.argtypes = [C.c_int, C.c_int, C.c_int, i8p, i8p, C.c_longlong, C.c_int,
                                     C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, i8p, i8p,
                                     C.POINTER(C.c_longlong)]
        L.or_complete_ab.restype = C.c_int
        L.or_complete_ab_a2.argtypes = [C.c_int, C.c_int, C.c_int, i8p, i8p, C.c_longlong, C.c_int,
                                        C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_int, i8p,
                                        i8p, C.POINTER(C.c_longlong)]
        L.or_complete_ab_a2.restype = C.c_int
        L.or_outer_tables.argtypes = [u8p, u8p]
        L.or_gen_hall_pairs.argtypes = [C.c_int, C.c_longlong, C.c_uint64,
                                        np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS"),
                                        C.c_int]
        _lib = L
    return _lib


def hall_tables(n):
    w = n + 1
    ct = np.zeros(201 * w, np.float64)
    st = np.zeros(201 * w, np.float64)
    lib().or_hall_tables(n, ct, st)
    return ct.reshape(201, w), st.reshape(201, w)


def hall_pair(n, X, Y, tables=None, detail=False):
    X = np.ascontiguousarray(X, np.int8)
    Y = np.ascontiguousarray(Y, np.int8)
    ct, st = tables if tables is not None else hall_tables(n)
    ct = np.ascontiguousarray(ct).ravel()
    st = np.ascontiguousarray(st).ravel()
    if detail:
        mx, mm = C.c_double(), C.c_double()
        p = lib().or_hall_pair(n, X, Y, len(X), ct, st, C.byref(mx), C.byref(mm))
        return p, mx.value, mm.value
    return lib().or_hall_pair(n, X, Y, len(X), ct, st, None, None)


def hall_batch(n, XY, nthreads=1):
    """XY: int8 [npairs, 2, L] or [npairs, 2L]; returns uint8 pass mask."""
    XY = np.ascontiguousarray(XY, np.int8)
    npairs = XY.shape[0]
    L = XY.reshape(npairs, -1).shape[1] // 2
    out = np.zeros(npairs, np.uint8)
    lib().or_hall_batch(n, L, XY.reshape(-1), npairs, out, nthreads)
    return out


def npaf_at(A, B, C_, D, s):
    A, B, C_, D = (np.ascontiguousarray(v, np.int8) for v in (A, B, C_, D))
    return lib().or_npaf_at(A, B, len(A), C_, D, len(C_), s)


def flat_score(C_, D):
    C_, D = (np.ascontiguousarray(v, np.int8) for v in (C_, D))
    return lib().or_flat_score(C_, D, len(C_))


def autocorr_key(X, Y, n, negate):
    X, Y = (np.ascontiguousarray(v, np.int8) for v in (X, Y))
    return lib().or_autocorr_key(X, Y, len(X), n, int(negate))


def cd_stream(n, tx, ty, m=6, pinX=False, pinY=False, rev=False, endpos=False, cd_prune=0,
              keep_all=False, cap=None, ab_side=False):
    """Returns (rows [k, 2, L] int8 in DFS order, pass flags, stats dict); L = n, or n+1 for
    the A,B side (ab_side)."""
    tx = np.ascontiguousarray(tx, np.int32)
    ty = np.ascontiguousarray(ty, np.int32)
    st = StreamStats()
    L = n + 1 if ab_side else n
    # the walk writes at most `room` rows and returns the full count; a stream longer than
    # the first buffer is walked a second time into one of its size
    room = min(cap, 1 << 18) if cap is not None else 1 << 16
    for _ in range(2):
        out = np.zeros(max(1, room) * 2 * L, np.int8)
        flags = np.zeros(max(1, room), np.uint8)
        total = lib().or_cd_stream(n, L, m, tx, ty, int(pinX), int(pinY), int(rev), int(endpos),
                                   int(cd_prune), int(keep_all), out, flags, room, C.byref(st))
        want = min(total, cap) if cap is not None else total
        if want <= room:
            break
        room = want
        st = StreamStats()
    return (out[: want * 2 * L].reshape(want, 2, L), flags[:want],
            dict(nodes=st.nodes, leaves=st.leaves, ok=st.ok))


def complete_ab(n, sigA, sigB, C_, D, budget, rows=None, m=6, outer_k=3, early=True, canon=True,
                a2=0):
    C_, D = (np.ascontiguousarray(v, np.int8) for v in (C_, D))
    A = np.zeros(n + 1, np.int8)
    B = np.zeros(n + 1, np.int8)
    nodes = C.c_longlong()
    if rows is not None and len(rows):
        rows = np.ascontiguousarray(rows, np.int8).reshape(-1, 16)
        ptr, nr = rows.ctypes.data_as(C.c_void_p), rows.shape[0]
    else:
        ptr, nr = None, 0
    v = lib().or_complete_ab_a2(n, sigA, sigB, C_, D, budget, outer_k, int(early), int(canon), m,
                                ptr, nr, int(a2), A, B, C.byref(nodes))
    return v, nodes.value, A, B


def outer_tables():
    o2 = np.zeros(16 * 5 * 9, np.uint8)
    o3 = np.zeros(128 * 5 * 9 * 13, np.uint8)
    lib().or_outer_tables(o2, o3)
    return o2, o3


def gen_hall_pairs(n, npairs, seed=0xB545C2, nthreads=1):
    """Hall microbench words [npairs, 2] uint64 (the oracle's copy of the generator)."""
    w = np.zeros(2 * max(1, npairs), np.uint64)
    lib().or_gen_hall_pairs(n, npairs, seed, w, nthreads)
    return w[: 2 * npairs].reshape(npairs, 2)
