"""The reference's own CPU code, timed on this host's cores: bench.py's reference arm and its
CPU-baseline legs. TEST INFRASTRUCTURE ONLY: nothing in the product imports this file.

oracle/_ref/libref.so is the reference's src/solver/wz_match.cpp compiled unmodified with its
production flags (`make -C oracle ref`), plus ref_harness.cpp, which only calls into it. The
reference keeps its state in globals and runs one single-threaded arm per core, one process
each (cluster_firsthit_probe.sh; WZ_FH_SHARD/NSHARD, wz_match.cpp:1573-1586). Here each arm is
its own copy of the library loaded into this process (so it has its own globals) and driven
by its own host thread; ctypes releases the GIL for the duration of each call, so the arms
run in parallel like the reference's processes.
"""
import ctypes as C
import os
import shutil
import tempfile
import threading
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBREF = os.path.join(HERE, "_ref", "libref.so")


def available():
    return os.path.exists(LIBREF)


def _bind(lib):
    ip = C.POINTER(C.c_int)
    lib.refh_setup.argtypes = [C.c_int] * 6
    lib.refh_hall_batch.restype = C.c_longlong
    lib.refh_hall_batch.argtypes = [C.c_void_p, C.c_longlong, C.c_longlong, C.c_int, C.c_int,
                                    C.c_int, C.c_void_p]
    lib.refh_stream_for.restype = C.c_longlong
    lib.refh_stream_for.argtypes = [C.c_int, ip, ip, C.c_int, C.c_int, C.c_int, C.c_double,
                                    C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                    C.POINTER(C.c_longlong)]
    lib.refh_complete.restype = C.c_int
    lib.refh_complete.argtypes = [ip, ip, C.c_longlong, C.c_int, C.c_void_p, C.c_int, ip, ip,
                                  C.POINTER(C.c_longlong)]
    return lib


def _ints(a):
    a = np.ascontiguousarray(a, dtype=np.int32)
    return a, a.ctypes.data_as(C.POINTER(C.c_int))


class Arms:
    """`narms` independent instances of the reference, each set up for (n, sig) as
    wz_match.cpp's main does before its first-hit loop."""

    def __init__(self, narms, n, sig, outer_k=3):
        if not available():
            raise FileNotFoundError(f"{LIBREF} is not built (make -C oracle ref REF=...)")
        self.n, self.sig, self.narms = n, tuple(sig), narms
        self._tmp = tempfile.mkdtemp(prefix="bsfh-refarms-")
        self.libs = []
        for i in range(narms):
            path = os.path.join(self._tmp, f"libref_{i}.so")
            shutil.copyfile(LIBREF, path)
            lib = _bind(C.CDLL(path, mode=os.RTLD_LOCAL if hasattr(os, "RTLD_LOCAL") else 0))
            lib.refh_setup(n, *self.sig, outer_k)
            self.libs.append(lib)

    def close(self):
        self.libs = []
        shutil.rmtree(self._tmp, ignore_errors=True)

    def _parallel(self, fn, items):
        out = [None] * len(items)

        def run(i):
            out[i] = fn(i, items[i])
        th = [threading.Thread(target=run, args=(i,)) for i in range(len(items))]
        for t in th:
            t.start()
        for t in th:
            t.join()
        return out

    # ---- the Hall filter (wz_match.cpp:143-168) ----
    def hall_fast(self, words, L=None, out=None):
        """hall_ok_pair_fast on every pair of `words` ([npairs, 2] uint64), the pairs split
        into one contiguous share per arm. Returns (passed, seconds)."""
        L = L or self.n
        words = np.ascontiguousarray(words, dtype=np.uint64)
        npairs = len(words)
        bounds = np.linspace(0, npairs, self.narms + 1).astype(np.int64)
        optr = out.ctypes.data if out is not None else None
        t0 = time.perf_counter()
        got = self._parallel(lambda i, lohi: self.libs[i].refh_hall_batch(
            words.ctypes.data, int(lohi[0]), int(lohi[1]), L, 1, 1, optr),
            [(bounds[i], bounds[i + 1]) for i in range(self.narms)])
        return int(sum(got)), time.perf_counter() - t0

    def hall_conj(self, words, nthreads, L=None, out=None):
        """The WZ_FH_HALL_FAST=0 conjunction hall_ok_single(X) && hall_ok_single(Y) &&
        hall_ok(X, Y) over nthreads OpenMP threads of one instance. Returns (passed, s)."""
        L = L or self.n
        words = np.ascontiguousarray(words, dtype=np.uint64)
        t0 = time.perf_counter()
        got = self.libs[0].refh_hall_batch(words.ctypes.data, 0, len(words), L, 0, nthreads,
                                           out.ctypes.data if out is not None else None)
        return int(got), time.perf_counter() - t0

    # ---- the C,D stream (count_pairs22, wz_match.cpp:678-784) ----
    def stream_for(self, cells, seconds, m=6):
        """Each arm streams one cell ((tx, ty) of the C,D side) for `seconds`, as an arm in
        the middle of its range. Returns dict(nodes, leaves, ok, survivors, seconds)."""
        assert len(cells) <= self.narms

        def one(i, cell):
            tx, px = _ints(cell[0])
            ty, py = _ints(cell[1])
            nodes, leaves, ok = C.c_longlong(0), C.c_longlong(0), C.c_longlong(0)
            s = self.libs[i].refh_stream_for(self.n, px, py, m, 0, 0, seconds, C.byref(nodes),
                                             C.byref(leaves), C.byref(ok))
            return nodes.value, leaves.value, ok.value, s
        t0 = time.perf_counter()
        res = self._parallel(one, list(cells))
        dt = time.perf_counter() - t0
        return {"nodes": sum(r[0] for r in res), "leaves": sum(r[1] for r in res),
                "ok": sum(r[2] for r in res), "survivors": sum(r[3] for r in res), "seconds": dt}

    def stream_cells_for(self, cells, seconds, m=6):
        """The arms take cells ((tx, ty, pinX, pinY) of the C,D side) in order from a shared
        queue and stream each whole until `seconds` have passed (the cell in flight is cut at
        the deadline), as the reference's single-core arms work through a range. Returns
        dict(nodes, leaves, ok, survivors, cells_done, seconds)."""
        lock = threading.Lock()
        nxt = [0]
        t_end = time.perf_counter() + seconds

        def one(i, _):
            got = [0, 0, 0, 0, 0]
            while True:
                left = t_end - time.perf_counter()
                if left <= 0:
                    break
                with lock:
                    k = nxt[0]
                    nxt[0] += 1
                if k >= len(cells):
                    break
                tx, ty, pin_x, pin_y = cells[k]
                ax, px = _ints(tx)  # the arrays stay alive while their pointers are used
                ay, py = _ints(ty)
                nodes, leaves, ok = C.c_longlong(0), C.c_longlong(0), C.c_longlong(0)
                t0 = time.perf_counter()
                s = self.libs[i].refh_stream_for(self.n, px, py, m, int(pin_x), int(pin_y), left,
                                                 C.byref(nodes), C.byref(leaves), C.byref(ok))
                got[0] += nodes.value
                got[1] += leaves.value
                got[2] += ok.value
                got[3] += s
                got[4] += time.perf_counter() - t0 < left  # finished before the deadline
            return got
        t0 = time.perf_counter()
        res = self._parallel(one, [None] * self.narms)
        dt = time.perf_counter() - t0
        return {"nodes": sum(r[0] for r in res), "leaves": sum(r[1] for r in res),
                "ok": sum(r[2] for r in res), "survivors": sum(r[3] for r in res),
                "cells_done": sum(r[4] for r in res), "seconds": dt}

    # ---- the A,B completer (fh_complete_ab, wz_match.cpp:1298-1341) ----
    def complete_for(self, cands, budget, seconds, rows=None, m=6):
        """Completes candidates (int8 [K, 2, n]: C, D) in order from a shared queue on every
        arm until all are done or `seconds` have passed (a candidate in flight is finished).
        Returns dict(nodes, done, verdicts, seconds)."""
        n1 = self.n + 1
        lock = threading.Lock()
        nxt = [0]
        t_end = time.perf_counter() + seconds
        rows_arr = None if rows is None or len(rows) == 0 else np.ascontiguousarray(rows, dtype=np.int8)
        rptr = rows_arr.ctypes.data if rows_arr is not None else None
        nrows = 0 if rows_arr is None else len(rows_arr)

        def work(i, _):
            lib = self.libs[i]
            A, pa = _ints(np.zeros(n1))
            B, pb = _ints(np.zeros(n1))
            nodes, done, verdicts = 0, 0, []
            nd = C.c_longlong(0)
            while time.perf_counter() < t_end:
                with lock:
                    k = nxt[0]
                    nxt[0] += 1
                if k >= len(cands):
                    break
                Cc, pc = _ints(cands[k, 0])
                Dd, pd = _ints(cands[k, 1])
                v = lib.refh_complete(pc, pd, budget, m, rptr, nrows, pa, pb, C.byref(nd))
                nodes += nd.value
                done += 1
                verdicts.append((k, v, nd.value))
            return nodes, done, verdicts
        t0 = time.perf_counter()
        res = self._parallel(work, [None] * self.narms)
        dt = time.perf_counter() - t0
        return {"nodes": sum(r[0] for r in res), "done": sum(r[1] for r in res),
                "verdicts": sorted(v for r in res for v in r[2]), "seconds": dt}
