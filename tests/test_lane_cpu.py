"""The library lane's control flow (lane.run_lane) on the host: its device calls are replaced
by the oracle (stream, flat score, completion), and its summary counts and first hit are
checked against the reference's own runs (tests/golden/lane_golden.json) at n <= 9. This
pins the buffer / drain / front-only-cut / first-hit bookkeeping without a GPU; the GPU
tests check the same runs through the real kernels."""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(HERE, "golden"))


class _Ctx:
    def __init__(self, n, sig):
        self.n, self.sig = n, tuple(sig)

    def timing(self, on):
        pass

    def timing_read(self):
        return 0.0, 0, 0


def _fakes(oracle):
    from bs45_quantum_explorer_gb300.hall import pack, unpack

    def stream(ctx, cells, m=6, pins=None, rev=False, endpos=False, hall_mode=None, as_words=False,
               limit=0, **kw):
        words, cidx, stats = [], [], []
        for i, (tx, ty) in enumerate(cells):
            r, _, st = oracle.cd_stream(ctx.n, tx, ty, m=m, pinX=pins[i][0], pinY=pins[i][1],
                                        rev=rev, endpos=endpos, cd_prune=kw.get("cd_prune", 0))
            words.append(pack(r) if len(r) else np.zeros((0, 2), np.uint64))
            cidx += [i] * len(r)
            stats.append(st)
        w = np.concatenate(words)
        cidx = np.array(cidx, np.uint32)
        return (w[:limit], cidx[:limit], stats) if limit else (w, cidx, stats)

    def topk(ctx, words, buf_cap, keep):
        X = unpack(words, ctx.n).astype(np.int64)
        n = ctx.n
        sc = np.array([sum(abs(int((C[:n - s] * C[s:]).sum() + (D[:n - s] * D[s:]).sum()))
                           for s in range(1, n + 1)) for C, D in X])
        order = np.argsort(sc, kind="stable")[:keep]
        return order, sc[order]

    def complete(ctx, words, budget, rows=None, m=6, outer_k=3, early=True, canon=True,
                 first_hit=False, rows_per_cand=None, **kw):
        X = unpack(np.asarray(words).reshape(-1, 2), ctx.n)
        out = [[], [], [], []]
        hit = False
        for i, (C, D) in enumerate(X):
            r = rows if rows_per_cand is None else rows_per_cand[i]
            if r is not None and not len(r):
                r = None
            if hit:
                v, nd, a, b = -1, 0, np.zeros(ctx.n + 1, np.int8), np.zeros(ctx.n + 1, np.int8)
            else:
                v, nd, a, b = oracle.complete_ab(ctx.n, ctx.sig[0], ctx.sig[1], C, D, budget, rows=r,
                                                 m=m, outer_k=outer_k, early=early, canon=canon)
                hit = first_hit and v == 0
            for lst, x in zip(out, (v, nd, a, b)):
                lst.append(x)
        return tuple(np.array(x) for x in out)

    return stream, topk, complete


def test_run_lane_control_flow_matches_reference_runs(built_lib, oracle, monkeypatch):
    import bs45_quantum_explorer_gb300.lane as lane
    from test_lane_gpu import check_run_lane, lane_kwargs, summary_of
    stream, topk, complete = _fakes(oracle)
    monkeypatch.setattr(lane, "cd_stream", stream)
    monkeypatch.setattr(lane, "flat_topk", topk)
    monkeypatch.setattr(lane, "complete_ab", complete)
    cases = [c for c in json.load(open(os.path.join(HERE, "golden", "lane_golden.json")))
             if not c.get("resume") and c["settings"].get("WZ_FH_M6") == 1 and c["n"] <= 9
             and not any(k in c["settings"] for k in ("WZ_FH_CELLSIZE", "WZ_FH_SCORE_MAX"))]
    assert len(cases) >= 40
    for c in cases:
        for batch in (1, 5):  # one cell per stream call, and batches cut per cell
            res = lane.run_lane(_Ctx(c["n"], c["sig"]), c["n"], tuple(c["sig"]), batch_cells=batch,
                                **lane_kwargs(c["settings"]))
            check_run_lane(res, summary_of(c["semantic"]), (c["n"], c["sig"], c["settings"], batch))


def test_run_lane_cd_prune_changes_only_the_node_count(built_lib, oracle, monkeypatch):
    """CD_PRUNE removes DFS nodes only: every lane summary is the one without it, and the
    lane's DFS node count does not grow (even n, mod-6 cells)."""
    import bs45_quantum_explorer_gb300.lane as lane
    from test_lane_gpu import check_run_lane, lane_kwargs, summary_of
    stream, topk, complete = _fakes(oracle)
    monkeypatch.setattr(lane, "cd_stream", stream)
    monkeypatch.setattr(lane, "flat_topk", topk)
    monkeypatch.setattr(lane, "complete_ab", complete)
    cases = [c for c in json.load(open(os.path.join(HERE, "golden", "lane_golden.json")))
             if not c.get("resume") and c["settings"].get("WZ_FH_M6") == 1 and c["n"] in (8, 10)
             and not any(k in c["settings"] for k in ("WZ_FH_CELLSIZE", "WZ_FH_SCORE_MAX"))]
    assert len(cases) >= 10
    fewer = 0
    for c in cases:
        kw = lane_kwargs(c["settings"])
        r0 = lane.run_lane(_Ctx(c["n"], c["sig"]), c["n"], tuple(c["sig"]), **kw)
        r3 = lane.run_lane(_Ctx(c["n"], c["sig"]), c["n"], tuple(c["sig"]), cd_prune=3, **kw)
        check_run_lane(r3, summary_of(c["semantic"]), (c["n"], c["sig"], c["settings"]))
        assert r3.dfs_nodes <= r0.dfs_nodes
        fewer += r3.dfs_nodes < r0.dfs_nodes
    assert fewer > 0
