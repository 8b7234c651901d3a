"""Host-side mirror of the reference's C,D stream interface.

The reference streams one cell with count_pairs22(n, px, py, false, pinC, pinD, leaves, ok,
&sink, m, stop) (src/solver/wz_match.cpp:678-784), calling sink(C, D) per survivor in DFS
order. cd_stream() returns the same survivors, in the same order, for a batch of cells,
computed on the GPU through bs_cd_stream (include/bsfh.h).
"""
import ctypes as C

import numpy as np

from ._lib import BS_OK, BS_STOPPED, BS_WALLED, BsError, Cell, CellStats, StreamOpts, check, lib
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
              target_prefixes=0, leaf_chunk=0, survivor_cap=0, cap=None, as_words=False,
              ab_side=False, limit=0, round_us=0, cd_prune=0, wall_sec=0.0, fine_nodes=0.0,
              wave_nodes=0.0, dfs_blocks=0):
    """cells: list of (tx, ty). Returns (survivors, cell index per survivor, per-cell stats).

    survivors: int8 [k, 2, L] (or uint64 words [k, 2] with as_words) in stream order, L = n
    (C,D) or n+1 with ab_side (the reference's abSide stream of A,B pairs).
    stats: list of dicts {nodes, leaves, ok} per cell (the reference's CDSTAT dfs_nodes and
    CELLSIZE leaves / hall_ok; with limit > 0, of the part explored).
    limit > 0 returns only the first `limit` survivors and stops the search there.
    cd_prune: WZ_FH_CD_PRUNE (bit 1 root quad rule, bit 2 block reachability; C,D side, m = 6,
    even n only): the same survivors, fewer DFS nodes.
    wall_sec > 0: WZ_FH_WALL_SEC, abandon the stream after that long without a new survivor.
    fine_nodes, wave_nodes, dfs_blocks: work sizes (0 = defaults; see tune.py).
    A stream stopped early (the context's stop flag, or the wall) returns the survivors of the
    part it completed, and every stats dict then carries stopped = 1 (flag) or 2 (wall)."""
    ncells = len(cells)
    arr = make_cells(cells, m, pins)
    opt = StreamOpts(m=m, rev=int(rev), endpos=int(endpos), cd_prune=int(cd_prune),
                     hall_mode=MODES[hall_mode], ab_side=int(ab_side),
                     target_prefixes=target_prefixes, leaf_chunk=leaf_chunk,
                     survivor_cap=survivor_cap, limit=limit, round_us=round_us,
                     wall_sec=float(wall_sec), fine_nodes=float(fine_nodes),
                     wave_nodes=float(wave_nodes), dfs_blocks=int(dfs_blocks))
    stats = (CellStats * ncells)()
    nout = C.c_longlong(0)
    cap = cap if cap is not None else (min(1 << 20, limit) if limit > 0 else 1 << 20)
    for _ in range(4):
        words = np.zeros((max(1, cap), 2), np.uint64)
        cidx = np.zeros(max(1, cap), np.uint32)
        rc = lib().bs_cd_stream(ctx.h, arr, ncells, C.byref(opt), words.ctypes.data,
                                cidx.ctypes.data, cap, C.byref(nout), stats)
        if rc == -6:  # BS_ERR_CAP: retry with the sizes it reported
            cap = max(cap, nout.value)
            opt.survivor_cap = max(opt.survivor_cap, nout.value)
            continue
        if rc not in (BS_STOPPED, BS_WALLED):
            check(rc, "bs_cd_stream")
        break
    k = nout.value
    st = [dict(nodes=s.nodes, leaves=s.leaves, ok=s.ok) for s in stats]
    if rc > 0:  # stopped early: the counts cover the part explored
        for x in st:
            x["stopped"] = rc
    words = words[:k]
    out = words if as_words else unpack(words, ctx.n + (1 if ab_side else 0))
    return out, cidx[:k], st


def npaf_verify(ctx, quads):
    """quads: uint64 words [k, 4] (A, B, C, D). Returns max_s |NPAF(s)| per quad (0 = valid)."""
    quads = np.ascontiguousarray(quads, np.uint64).reshape(-1, 4)
    out = np.zeros(max(1, len(quads)), np.int32)
    check(lib().bs_npaf_verify_batch(ctx.h, quads.ctypes.data, len(quads), out.ctypes.data),
          "bs_npaf_verify_batch")
    return out[:len(quads)]


def join_quads(ctx, cd_words, ab_words, cap=1 << 16):
    """Every (A,B) x (C,D) pairing with AB[s] = -CD[s] for all s, verified exactly on the GPU.
    Returns (quads uint64 [k, 4], key_hits)."""
    cd_words = np.ascontiguousarray(cd_words, np.uint64).reshape(-1, 2)
    ab_words = np.ascontiguousarray(ab_words, np.uint64).reshape(-1, 2)
    nout, hits = C.c_longlong(0), C.c_longlong(0)
    while True:
        out = np.zeros((max(1, cap), 4), np.uint64)
        rc = lib().bs_join_quads(ctx.h, cd_words.ctypes.data, len(cd_words), ab_words.ctypes.data,
                                 len(ab_words), out.ctypes.data, cap, C.byref(nout), C.byref(hits))
        if rc == -6 and nout.value > cap:
            cap = nout.value
            continue
        check(rc, "bs_join_quads")
        return out[:nout.value], hits.value


__all__ = ["cd_stream", "make_cells", "npaf_verify", "join_quads", "BsError", "BS_OK"]
