"""Host-side mirror of the reference's per-cell keep and A,B completion interfaces.

flat_topk(): flat_score + drain()'s stable sort and front-only cut
(src/solver/wz_match.cpp:2569-2583, 2656-2714) through bs_flat_topk.
complete_ab(): fh_complete_ab(C, D) (wz_match.cpp:1298-1341) for a batch through
bs_complete_ab_batch; same verdict codes, charged node counts and completions.
"""
import ctypes as C

import numpy as np

from ._lib import BS_STOPPED, AbCand, AbOpts, check, lib
from .hall import pack


def flat_topk(ctx, words, buf_cap, keep):
    """words: uint64 [k, 2] survivors in stream order. Returns (order, scores): stream
    indices per batch of buf_cap in (score, stream position) order, first `keep` per batch."""
    words = np.ascontiguousarray(words, np.uint64)
    nsurv = words.shape[0]
    nk = C.c_longlong()
    lib().bs_flat_topk(ctx.h, None, nsurv, buf_cap, keep, None, None, C.byref(nk))
    order = np.zeros(max(1, nk.value), np.int64)
    scores = np.zeros(max(1, nk.value), np.int32)
    check(lib().bs_flat_topk(ctx.h, words.ctypes.data, nsurv, buf_cap, keep, order.ctypes.data,
                             scores.ctypes.data, C.byref(nk)), "bs_flat_topk")
    return order[:nk.value], scores[:nk.value]


AB_CAND = np.dtype([("c", np.uint64), ("d", np.uint64), ("row_off", np.int64),
                    ("nrows", np.int32), ("reserved", np.int32)])
assert AB_CAND.itemsize == C.sizeof(AbCand)


def complete_ab(ctx, cands, budget, rows_per_cand=None, m=6, outer_k=3, early=True, canon=True,
                first_hit=False, max_seconds=0.0, rows=None, a2=0, blocks_per_sm=0):
    """cands: int8 [k, 2, n] (C, D) or uint64 words [k, 2]. Allowed A,B rows (int8 [r, 16]):
    `rows` shared by every candidate (one cell's list), or rows_per_cand, a list of arrays
    (empty = unconstrained); neither: unconstrained. a2 = 2: WZ_FH_A2=2, the A2 row prune.
    Returns (verdict int32 [k], nodes int64 [k], A int8 [k, n+1], B int8 [k, n+1]); when the
    context's stop flag stops the batch, the candidates it did not finish have verdict -1."""
    cands = np.asarray(cands)
    words = cands if cands.dtype == np.uint64 else pack(cands)
    words = np.ascontiguousarray(words.reshape(-1, 2), np.uint64)
    k = words.shape[0]
    arr = np.zeros(max(1, k), AB_CAND)
    arr["c"][:k], arr["d"][:k] = words[:, 0], words[:, 1]
    if rows is not None and len(rows):
        all_rows = np.ascontiguousarray(rows, np.int8).reshape(-1, 16)
        arr["nrows"][:k] = all_rows.shape[0]
        off = all_rows.shape[0]
    else:
        # one copy of each row set: candidates given the same array share its rows (and the
        # library builds its bitset masks once)
        parts, off, seen = [], 0, {}
        for i in range(k):
            r = None if rows_per_cand is None else rows_per_cand[i]
            if r is not None and len(r):
                key = id(r)
                if key not in seen:
                    rr = np.ascontiguousarray(r, np.int8).reshape(-1, 16)
                    seen[key] = (off, rr.shape[0], r)  # r kept alive so its id stays unique
                    parts.append(rr)
                    off += rr.shape[0]
                arr["row_off"][i], arr["nrows"][i] = seen[key][0], seen[key][1]
        all_rows = np.concatenate(parts) if parts else np.zeros((1, 16), np.int8)
    all_rows = np.ascontiguousarray(all_rows)
    opt = AbOpts(budget=budget, outer_k=outer_k, early=int(early), canon=int(canon), m=m,
                 first_hit=int(first_hit), a2=int(a2), max_seconds=max_seconds,
                 blocks_per_sm=int(blocks_per_sm), reserved=0)
    n1 = ctx.n + 1
    verdict = np.zeros(max(1, k), np.int32)
    nodes = np.zeros(max(1, k), np.int64)
    A = np.zeros((max(1, k), n1), np.int8)
    B = np.zeros((max(1, k), n1), np.int8)
    rc = lib().bs_complete_ab_batch(ctx.h, C.cast(arr.ctypes.data, C.POINTER(AbCand)), k,
                                    all_rows.ctypes.data, off, C.byref(opt), verdict.ctypes.data,
                                    nodes.ctypes.data, A.ctypes.data, B.ctypes.data)
    if rc != BS_STOPPED:  # stopped by the context's stop flag: candidates not run read -1
        check(rc, "bs_complete_ab_batch")
    return verdict[:k], nodes[:k], A[:k], B[:k]
