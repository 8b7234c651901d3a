"""Work sizes chosen by measurement on the device at hand.

The reference has no counterpart (its work unit is one cell on one core). On the GPU the
stream's subtree granularity, its wave size and the DFS kernel's register budget, and the
completer's resident blocks per SM and batch size, change throughput but never a result: the
survivors, their order, the node counts and the verdicts are the same for every choice. So
these sizes are picked by timing short probes of the workload itself:

  tune_stream(ctx, cell)       fine_nodes x dfs_blocks on the first `probe` survivors of one
                               cell (a front-only prefix, the lane's own unit of work), then
                               wave_nodes for the best pair
  tune_completer(ctx, cands)   blocks_per_sm x chunk on a sample of drained candidates, each
                               charged at most 2^14 nodes

Each returns (choice, table of every probe's rate). tune_lane() runs both on a lane's first
kept cell and returns one dict for run_lane(tuning=...). Results are cached per (device,
n, signature, workload key) for the life of the process.
"""
import time

import numpy as np

from .complete import complete_ab
from .stream import cd_stream

FINE = (5e3, 2e4, 8e4)
BLOCKS = (4, 5, 6)
WAVES = (2e9, 8e9, 3.2e10)
AB_BLOCKS = (1, 2, 3)
CHUNKS = (8192, 65536)

_CACHE = {}


def _rate(fn, reps=2):
    """Best of `reps` timed calls of fn() -> work units; returns units per second."""
    best = 0.0
    for _ in range(reps):
        t0 = time.perf_counter()
        units = fn()
        dt = time.perf_counter() - t0
        best = max(best, units / dt if dt > 0 else 0.0)
    return best


def tune_stream(ctx, cell, m=6, probe=20000, pins=None):
    """cell = (tx, ty). Returns ({fine_nodes, wave_nodes, dfs_blocks}, probes)."""
    key = ("stream", ctx.n, ctx.sig, tuple(map(tuple, cell)), probe)
    if key in _CACHE:
        return _CACHE[key]
    pins = [pins] if pins is not None else None
    cd_stream(ctx, [cell], m=m, pins=pins, as_words=True, limit=min(probe, 100))  # warm-up
    probes = []

    def run(**kw):
        def fn():
            _, _, st = cd_stream(ctx, [cell], m=m, pins=pins, as_words=True, limit=probe, **kw)
            return st[0]["nodes"]
        return fn
    for fine in FINE:
        for blocks in BLOCKS:
            probes.append(dict(fine_nodes=fine, dfs_blocks=blocks,
                               nodes_per_s=_rate(run(fine_nodes=fine, dfs_blocks=blocks))))
    best = max(probes, key=lambda p: p["nodes_per_s"])
    choice = dict(fine_nodes=best["fine_nodes"], dfs_blocks=best["dfs_blocks"])
    wave_probes = []
    for wave in WAVES:
        wave_probes.append(dict(wave_nodes=wave, nodes_per_s=_rate(run(wave_nodes=wave, **choice))))
    choice["wave_nodes"] = max(wave_probes, key=lambda p: p["nodes_per_s"])["wave_nodes"]
    out = (choice, probes + wave_probes)
    _CACHE[key] = out
    return out


def tune_completer(ctx, cands, budget, rows=None, m=6, sample=16384, probe_budget=1 << 14):
    """cands: the drained candidates (int8 [k, 2, n] or words). Returns
    ({blocks_per_sm, chunk}, probes), timing each setting on the same first `sample`.

    The probes charge at most `probe_budget` nodes per candidate: at the lane's own budget a
    few candidates that run to it take seconds on one warp, and a probe that waits for them
    measures that tail, not the rate of a full device. A setting within 3 % of the best is
    taken as equal, and of equals the one with more resident warps wins."""
    cands = np.asarray(cands)[:sample]
    pb = min(budget, probe_budget) if budget > 0 else probe_budget
    key = ("complete", ctx.n, ctx.sig, pb, len(cands), hash(cands.tobytes()),
           None if rows is None else hash(np.asarray(rows).tobytes()))
    if key in _CACHE:
        return _CACHE[key]
    complete_ab(ctx, cands[:256], pb, rows=rows, m=m)  # warm-up
    probes = []
    for blocks in AB_BLOCKS:
        for chunk in CHUNKS:
            def fn(blocks=blocks, chunk=chunk):
                nodes = 0
                for c0 in range(0, len(cands), chunk):
                    _, nd, _, _ = complete_ab(ctx, cands[c0:c0 + chunk], pb, rows=rows, m=m,
                                              blocks_per_sm=blocks)
                    nodes += int(nd.sum())
                return nodes
            probes.append(dict(blocks_per_sm=blocks, chunk=chunk, nodes_per_s=_rate(fn, reps=2)))
    top = max(p["nodes_per_s"] for p in probes)
    near = [p for p in probes if p["nodes_per_s"] >= 0.97 * top]
    best = max(near, key=lambda p: (p["blocks_per_sm"], p["chunk"], p["nodes_per_s"]))
    out = (dict(blocks_per_sm=best["blocks_per_sm"], chunk=best["chunk"]), probes)
    _CACHE[key] = out
    return out


def tune_lane(ctx, n, sig, listing, skip, end, budget, buf_cap=500000, drain_top=50000,
              probe=20000, sample=16384):
    """Work sizes for a lane over raw cells [skip, end): both probes on its first kept cell
    that has allowed rows. Returns (tuning dict for run_lane, report)."""
    from .cells import ab_rows
    from .complete import flat_topk
    cells, kept, _, m = listing
    for pi in range(skip, end):
        if not kept[pi]:
            continue
        c = cells[pi]
        rows, off, nr = ab_rows(n, sig, m, [c])
        if nr[0] == 0:
            continue
        cell = (list(c.tx[:m]), list(c.ty[:m]))
        pins = (c.pinX, c.pinY)
        t0 = time.perf_counter()
        s_choice, s_probes = tune_stream(ctx, cell, m=m, probe=probe, pins=pins)
        surv, _, _ = cd_stream(ctx, [cell], m=m, pins=[pins], as_words=True,
                               limit=min(buf_cap, 4 * sample), **s_choice)
        order, _ = flat_topk(ctx, surv, len(surv), min(drain_top, len(surv)) if drain_top else len(surv))
        r = rows[off[0]:off[0] + nr[0]] if nr[0] <= 20000 else None
        c_choice, c_probes = tune_completer(ctx, surv[order], budget, rows=r, m=m, sample=sample)
        tuning = dict(s_choice, **c_choice)
        return tuning, dict(cell=int(pi), seconds=round(time.perf_counter() - t0, 2),
                            stream_probes=s_probes, completer_probes=c_probes, choice=tuning)
    return {}, dict(cell=None)
