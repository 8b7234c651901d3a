"""One first-hit lane over a window of raw cells, as a library call.

The reference runs this loop as a process (`WZ_FIRSTHIT=1 wz_match n a b c d`,
src/solver/wz_match.cpp:2101-2891); bin/bs_firsthit is the drop-in for that process. run_lane()
is the same search for callers that hold a GPU context and want a result object instead of a
stdout protocol: a scheduler serving many jobs, or a benchmark. For each raw cell pi of the
window that the arm owns (pi = shard + k*nshard, WZ_FH_PROF_SKIP <= k < WZ_FH_PROF_END) it
  - skips orbit duplicates (orbit canon) and cells whose allowed A,B row list is empty,
  - streams the cell on the GPU in the reference's DFS order (bs_cd_stream),
  - buffers survivors in batches of buf_cap, orders each batch by flat score (bs_flat_topk),
    completes the first drain_top of the first drain_batches batches (front-only cut;
    drain_top = 0 completes every survivor) with budgeted A,B search (bs_complete_ab_batch),
  - stops at the first hit.
Counts follow the reference's summary line (candidates_streamed, clean_no_AB, budget_aborted,
total_AB_nodes, cells_done, ...), so a run equals the lane's under the same settings.
Not carried over: checkpoints, SIGTERM handling and the stdout protocol (bs_firsthit has them),
WZ_FH_SCORE_MAX / WZ_FH_MAX_CAND and the unbuffered order (cell_order = 0).
"""
import time
from dataclasses import dataclass, field

import numpy as np

from .cells import ab_rows, cell_list
from .complete import complete_ab, flat_topk
from .hall import unpack
from .stream import cd_stream


@dataclass
class LaneResult:
    found: bool = False
    hit_idx: int = -1              # candidates_streamed when the hit's batch was drained
    profile_rank: int = -1         # raw cell index of the hit
    quad: tuple = None             # (A, B, C, D) int8 arrays on a hit
    nodes_this_cand: int = 0
    candidates_streamed: int = 0
    pre_filter_rejected: int = 0
    clean_no_ab: int = 0
    budget_aborted: int = 0
    total_ab_nodes: int = 0
    backtracks_entered: int = 0
    cells_done: int = 0
    cells_orbit_dup: int = 0
    cells_prof_dead: int = 0
    cells_prof_uncap: int = 0
    cells_empty: int = 0
    cells_capped: int = 0
    dfs_nodes: int = 0
    completions: int = 0
    stream_s: float = 0.0
    stream_device_ms: float = 0.0  # the stream's timed kernels (DFS waves and Hall filters)
    complete_s: float = 0.0
    complete_device_ms: float = 0.0
    timings: dict = field(default_factory=dict)


_LIST_CACHE = {}


def lane_list(n, sig, m6=None, thm211b=None, thm212=None, endpos=False, orbit_canon=True,
              orbit_q=1, qprune=True, prof_order=3):
    """The lane's cell list (bs_cell_list), cached per settings."""
    key = (n, tuple(sig), m6, thm211b, thm212, endpos, orbit_canon, orbit_q, qprune, prof_order)
    if key not in _LIST_CACHE:
        _LIST_CACHE[key] = cell_list(n, sig, m6=m6, thm211b=thm211b, thm212=thm212, endpos=endpos,
                                     orbit_canon=orbit_canon, orbit_q=orbit_q if orbit_canon else 0,
                                     qprune=qprune, prof_order=prof_order)
    return _LIST_CACHE[key]


def run_lane(ctx, n, sig, skip=0, end=0, shard=0, nshard=1, budget=200000, buf_cap=500000,
             drain_top=0, drain_batches=1, endpos=False, orbit_canon=True, orbit_q=1, qprune=True,
             prof_order=3, m6=None, thm211b=None, thm212=None, abp_cap=20000, outer_k=3,
             early=True, canon=True, rev=False, hall_mode="tc_fp16", chunk=65536,
             max_seconds=0.0, listing=None, batch_cells=None, cd_prune=0, a2=0, tuning=None,
             flush_cands=4096):
    """Runs the lane over raw cells [skip, end) of its shard (end = 0: to the list's end).
    The list options are the lane's WZ_FH_* list settings (cells.cell_list); the cells must
    be mod-6 cells (the lane's buffered order). max_seconds > 0 takes no new cell once
    exceeded; the cells already taken are completed (their queued candidates included, which
    can still give the hit), and the counts cover those cells.
    listing: a cell_list() result to reuse. batch_cells: cells streamed per device call
    (default 32 up to n = 30, where cells are small, else 1); a batch is streamed whole and
    each cell cut to its front-only prefix on the host, which is the same prefix.
    cd_prune: WZ_FH_CD_PRUNE for the streams (fewer DFS nodes, the same candidates).
    a2: WZ_FH_A2 (2 = the A2 row prune in the completer).
    tuning: work sizes from tune.py (stream fine_nodes / wave_nodes / dfs_blocks, completer
    blocks_per_sm and chunk); none of them changes a result.
    flush_cands: kept candidates queued (over whole cells) before one completer call."""
    tuning = dict(tuning or {})
    stream_kw = {k: tuning[k] for k in ("fine_nodes", "wave_nodes", "dfs_blocks") if k in tuning}
    ab_kw = {k: tuning[k] for k in ("blocks_per_sm",) if k in tuning}
    chunk = int(tuning.get("chunk", chunk))
    cells, kept, _, m = listing if listing is not None else lane_list(
        n, sig, m6, thm211b, thm212, endpos, orbit_canon, orbit_q, qprune, prof_order)
    if m != 6:
        raise ValueError("run_lane runs the buffered (mod-6 cell) order only")
    ncells = len(kept)
    stop = min(ncells, shard + end * nshard) if end > 0 else ncells
    owned = list(range(shard + skip * nshard, stop, nshard))
    res = LaneResult()
    t_start = time.perf_counter()
    live = [pi for pi in owned if kept[pi]]
    # allowed A,B rows of every owned kept cell (the reference's abpMap), one host call
    t_rows = time.perf_counter()
    rows, row_off, nrows = ab_rows(n, sig, m, [cells[pi] for pi in live]) if live else (None, [], [])
    res.timings["rows_s"] = time.perf_counter() - t_rows
    slot = {pi: j for j, pi in enumerate(live)}
    if batch_cells is None:
        batch_cells = 32 if n <= 30 else 1
    cut = drain_batches * buf_cap if drain_top > 0 else 0
    streamed = {}  # raw cell -> (survivors in stream order, stats), filled a batch at a time

    def stream_from(j0):
        """Streams the live cells live[j0:] with allowed rows, batch_cells at a time."""
        group = [pi for pi in live[j0:] if int(nrows[slot[pi]]) > 0][:batch_cells]
        args = [(list(cells[q].tx[:m]), list(cells[q].ty[:m])) for q in group]
        pins = [(cells[q].pinX, cells[q].pinY) for q in group]
        t0 = time.perf_counter()
        ctx.timing(True)
        surv, cidx, st = cd_stream(ctx, args, m=m, pins=pins, rev=rev, endpos=endpos,
                                   hall_mode=hall_mode, as_words=True, cd_prune=cd_prune,
                                   limit=cut if len(group) == 1 else 0, **stream_kw)
        ms, _, _ = ctx.timing_read()
        ctx.timing(False)
        res.stream_s += time.perf_counter() - t0
        res.stream_device_ms += ms
        if len(group) == 1:
            streamed[group[0]] = (surv, st[0])
            return
        bounds = np.searchsorted(cidx, np.arange(len(group) + 1))
        for k, q in enumerate(group):
            w = surv[int(bounds[k]):int(bounds[k + 1])]
            streamed[q] = (w[:cut] if cut else w, st[k])

    # The cells' effects go to a queue in cell order and are applied when the queued
    # completions have run: the kept candidates of several cells (each with its own allowed
    # rows) go to the completer in one call once at least FLUSH of them wait, so that small
    # per-cell keeps (DRAIN_TOP 64) fill the device. The call runs in first-hit mode over the
    # candidates in cell order, and the queue is replayed in that order up to the first hit,
    # so every count, the hit and its quad are those of completing cell by cell; cells after
    # a hit are streamed but never counted.
    FLUSH = max(1, int(flush_cands))
    queue = []    # ("count", {field: increment}) | ("batch", item) | ("cell", {...})
    pend = []     # the batch items waiting for the completer, in order
    npend = 0

    def flush():
        """Completes the queued candidates and replays the queue; True on a hit."""
        nonlocal npend
        if pend:
            words = np.concatenate([it["words"] for it in pend])
            rpc = []
            for it in pend:
                rpc.extend([it["rows"] if it["rows"] is not None else np.zeros((0, 16), np.int8)] *
                           len(it["words"]))
            out = []
            for c0 in range(0, len(words), chunk):
                t1 = time.perf_counter()
                ctx.timing(True)
                part = rpc[c0:c0 + chunk]
                # one shared row set (a lane's one large cell): no per-candidate list
                one = len({id(x) for x in part}) == 1
                out.append(complete_ab(ctx, words[c0:c0 + chunk], budget,
                                       rows=part[0] if one and len(part[0]) else None,
                                       rows_per_cand=None if one else part,
                                       m=m, outer_k=outer_k, early=early, canon=canon,
                                       first_hit=True, a2=a2, **ab_kw))
                ms, _, _ = ctx.timing_read()
                ctx.timing(False)
                res.complete_s += time.perf_counter() - t1
                res.complete_device_ms += ms
                if (out[-1][0] == 0).any():
                    break  # a hit: later chunks are never reached in cell order
            v = np.concatenate([o[0] for o in out])
            nd = np.concatenate([o[1] for o in out])
            A = np.concatenate([o[2] for o in out])
            B = np.concatenate([o[3] for o in out])
            base = 0
            for it in pend:
                it["v"], it["nd"], it["A"], it["B"] = (v[base:base + len(it["words"])],
                                                       nd[base:base + len(it["words"])],
                                                       A[base:base + len(it["words"])],
                                                       B[base:base + len(it["words"])])
                base += len(it["words"])
        found = False
        for kind, x in queue:
            if kind == "count":
                for f, inc in x.items():
                    setattr(res, f, getattr(res, f) + inc)
            elif kind == "cell":
                res.cells_capped += x["capped"]
                res.candidates_streamed = x["cand"]
                res.cells_done += 1
                res.cells_empty += x["empty"]
            else:
                # the batch's verdicts up to and including its first hit, tallied at once
                v, nd = x["v"], x["nd"]
                hits = np.flatnonzero(v == 0)
                stop = int(hits[0]) + 1 if len(hits) else len(x["words"])
                if len(v) < stop:
                    raise RuntimeError(f"candidate {len(v)} of a batch was not completed (-1)")
                seg, segn = v[:stop], nd[:stop]
                bad = np.flatnonzero((seg < 0) | (seg == 4))
                if len(bad):
                    t = int(bad[0])
                    if seg[t] == 4:
                        raise RuntimeError("completer found a quad whose NPAF recheck failed")
                    raise RuntimeError(f"candidate {t} of a batch was not completed ({int(seg[t])})")
                res.completions += stop
                res.total_ab_nodes += int(segn.sum())
                res.backtracks_entered += int(((seg >= 2) | (seg == 0)).sum())  # the hit too
                res.pre_filter_rejected += int((seg == 1).sum())
                res.clean_no_ab += int((seg == 2).sum())
                res.budget_aborted += int((seg == 3).sum())
                if len(hits):
                    t = int(hits[0])
                    cw = unpack(x["words"][t:t + 1], n)[0]
                    res.found, res.hit_idx, res.profile_rank = True, x["cand"], x["pi"]
                    res.quad = (x["A"][t].copy(), x["B"][t].copy(), cw[0].copy(), cw[1].copy())
                    res.nodes_this_cand = int(segn[t])
                    res.candidates_streamed = x["cand"]
                    found = True
                    break
        queue.clear()
        pend.clear()
        npend = 0
        return found

    cand = 0
    found = False
    for pi in owned:
        if max_seconds > 0 and time.perf_counter() - t_start > max_seconds:
            break
        if not kept[pi]:
            queue.append(("count", {"cells_orbit_dup": 1}))
            continue
        j = slot[pi]
        nr = int(nrows[j])
        if nr == 0:
            queue.append(("count", {"cells_prof_dead": 1, "cells_done": 1}))
            continue
        cell_rows = rows[row_off[j]:row_off[j] + nr] if nr <= abp_cap else None
        if cell_rows is None:
            queue.append(("count", {"cells_prof_uncap": 1}))
        if pi not in streamed:
            stream_from(j)
        surv, st0 = streamed.pop(pi)
        queue.append(("count", {"dfs_nodes": st0["nodes"]}))
        nout = len(surv)
        cs_start = cand
        nb = (nout + buf_cap - 1) // buf_cap
        if drain_top > 0:
            nb = min(nb, drain_batches)
        for b in range(nb):
            lo, hi = b * buf_cap, min(nout, (b + 1) * buf_cap)
            cand = cs_start + hi          # survivors counted when this batch is drained
            keep = min(hi - lo, drain_top) if drain_top > 0 else hi - lo
            t_k = time.perf_counter()
            order, _ = flat_topk(ctx, surv[lo:hi], hi - lo, keep)
            res.timings["topk_s"] = res.timings.get("topk_s", 0.0) + time.perf_counter() - t_k
            item = {"words": surv[lo + order], "rows": cell_rows, "cand": cand, "pi": pi}
            queue.append(("batch", item))
            pend.append(item)
            npend += len(order)
        # the lane counts a cell as capped once it has drained its last allowed batch
        cand = cs_start + (min(nout, drain_batches * buf_cap) if drain_top > 0 else nout)
        queue.append(("cell", {"capped": int(drain_top > 0 and nout > 0 and -(-nout // buf_cap) >= drain_batches),
                               "cand": cand, "empty": int(nout == 0)}))
        if npend >= FLUSH:
            found = flush()
            if found:
                break
    if not found:
        flush()
    res.timings["wall_s"] = time.perf_counter() - t_start
    return res
