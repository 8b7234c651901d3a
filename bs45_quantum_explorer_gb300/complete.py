"""Host-side mirror of the reference's per-cell keep and A,B completion interfaces.

flat_topk(): flat_score + drain()'s stable sort and front-only cut
(src/solver/wz_match.cpp:2569-2583, 2656-2714) through bs_flat_topk.
complete_ab(): fh_complete_ab(C, D) (wz_match.cpp:1298-1341) for a batch through
bs_complete_ab_batch; same verdict codes, charged node counts and completions.
"""
import ctypes as C

import numpy as np

from ._lib import AbCand, AbOpts, check, lib
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


def complete_ab(ctx, cands, budget, rows_per_cand=None, m=6, outer_k=3, early=True, canon=True,
                first_hit=False, max_seconds=0.0):
    """cands: int8 [k, 2, n] (C, D) or uint64 words [k, 2]. rows_per_cand: None or a list of
    int8 [r, 16] arrays (the cell's allowed rows; empty = unconstrained).
    Returns (verdict int32 [k], nodes int64 [k], A int8 [k, n+1], B int8 [k, n+1])."""
    cands = np.asarray(cands)
    words = cands if cands.dtype == np.uint64 else pack(cands)
    words = np.ascontiguousarray(words.reshape(-1, 2), np.uint64)
    k = words.shape[0]
    arr = (AbCand * max(1, k))()
    all_rows = []
    off = 0
    for i in range(k):
        arr[i].c, arr[i].d = int(words[i, 0]), int(words[i, 1])
        r = None if rows_per_cand is None else rows_per_cand[i]
        if r is not None and len(r):
            r = np.ascontiguousarray(r, np.int8).reshape(-1, 16)
            arr[i].row_off, arr[i].nrows = off, r.shape[0]
            all_rows.append(r)
            off += r.shape[0]
        else:
            arr[i].row_off, arr[i].nrows = 0, 0
    rows = np.ascontiguousarray(np.concatenate(all_rows) if all_rows else np.zeros((1, 16), np.int8))
    opt = AbOpts(budget=budget, outer_k=outer_k, early=int(early), canon=int(canon), m=m,
                 first_hit=int(first_hit), reserved=0, max_seconds=max_seconds)
    n1 = ctx.n + 1
    verdict = np.zeros(max(1, k), np.int32)
    nodes = np.zeros(max(1, k), np.int64)
    A = np.zeros((max(1, k), n1), np.int8)
    B = np.zeros((max(1, k), n1), np.int8)
    check(lib().bs_complete_ab_batch(ctx.h, arr, k, rows.ctypes.data, off, C.byref(opt),
                                     verdict.ctypes.data, nodes.ctypes.data, A.ctypes.data,
                                     B.ctypes.data), "bs_complete_ab_batch")
    return verdict[:k], nodes[:k], A[:k], B[:k]
