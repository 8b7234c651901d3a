"""Host-side mirror of the reference's C,D stream interface.

The reference streams one cell with count_pairs22(n, px, py, false, pinC, pinD, leaves, ok,
&sink, m, stop) (src/solver/wz_match.cpp:678-784), calling sink(C, D) per survivor in DFS
order. cd_stream() returns the same survivors, in the same order, for a batch of cells,
computed on the GPU through bs_cd_stream (include/bsfh.h).
"""
import ctypes as C

import numpy as np

from ._lib import BS_OK, BsError, Cell, CellStats, StreamOpts, check, lib
from .hall import MODES, unpack


def make_cells(cells, m, pins=None):
    arr = (Cell * len(cells))()
    for i, (tx, ty) in enumerate(cells):
        for c in range(m):
            arr[i].tx[c] = int(tx[c])
            arr[i].ty[c] = int(ty[c])
        pX, pY = pins[i] if pins is not None else (0, 0)
        arr[i].pinX, arr[i].pinY = int(pX), int(pY)
    return arr


def cd_stream(ctx, cells, m=6, pins=None, rev=False, endpos=False, hall_mode="tc_fp16",
              target_prefixes=0, leaf_chunk=0, survivor_cap=0, cap=None, as_words=False):
    """cells: list of (tx, ty). Returns (survivors, cell index per survivor, per-cell stats).

    survivors: int8 [k, 2, n] (or uint64 words [k, 2] with as_words) in stream order.
    stats: list of dicts {nodes, leaves, ok} per cell (the reference's CDSTAT dfs_nodes and
    CELLSIZE leaves / hall_ok)."""
    ncells = len(cells)
    arr = make_cells(cells, m, pins)
    opt = StreamOpts(m=m, rev=int(rev), endpos=int(endpos), cd_prune=0,
                     hall_mode=MODES[hall_mode], reserved=0, target_prefixes=target_prefixes,
                     leaf_chunk=leaf_chunk, survivor_cap=survivor_cap)
    stats = (CellStats * ncells)()
    nout = C.c_longlong(0)
    cap = cap if cap is not None else (1 << 20)
    for _ in range(2):
        words = np.zeros((max(1, cap), 2), np.uint64)
        cidx = np.zeros(max(1, cap), np.uint32)
        rc = lib().bs_cd_stream(ctx.h, arr, ncells, C.byref(opt), words.ctypes.data,
                                cidx.ctypes.data, cap, C.byref(nout), stats)
        if rc == -6 and nout.value > cap:  # BS_ERR_CAP: retry with the size it reported
            cap = nout.value
            opt.survivor_cap = max(opt.survivor_cap, cap)
            continue
        check(rc, "bs_cd_stream")
        break
    k = nout.value
    st = [dict(nodes=s.nodes, leaves=s.leaves, ok=s.ok) for s in stats]
    words = words[:k]
    out = words if as_words else unpack(words, ctx.n)
    return out, cidx[:k], st


__all__ = ["cd_stream", "make_cells", "BsError", "BS_OK"]
