"""The reference's archived n = 29 first-hit canary (tools/test_firsthit_telemetry.py:176-181:
`WZ_FIRSTHIT=1 WZ_FH_M6=1 wz_match 29 0 6 9 1`, orbit canon off, order 0, budget 200,000),
against the reference's own run of it today (tests/golden/canary_n29_golden.json, from
make_canary_golden.py: the summary, the quad, per raw cell the completions, verdicts and
charged nodes, and the hit cell's drain sequence).

The oracle rebuilds the run's stream and its hit: the lane's cell list (bs_cell_list) and
allowed rows, each live cell's stream up to the hit cell (their survivor counts sum to
FIRSTHIT idx), and the hit cell's survivors ordered by flat score (stable) and completed up to
the first hit: the same drain ranks, verdicts and node counts, the hit's nodes_this_cand and
the same quad. Both recorded runs, every completion of the cells before the hit and the hit
cell under the older completer (nodes_this_cand = 81,320) included, are replayed through the
lane binary's host logic in test_lane_host_cpu.py, and through the GPU in
test_z_canary_gpu.py."""
import concurrent.futures as cf
import json
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUDGET = 200000  # the lane's default WZ_FH_AB_BUDGET
NCPU = min(8, os.cpu_count() or 1)


def _golden():
    return json.load(open(os.path.join(HERE, "golden", "canary_n29_golden.json")))


def _setup(g):
    from bs45_quantum_explorer_gb300.cells import ab_rows
    from bs45_quantum_explorer_gb300.lane import lane_list
    n, sig = g["n"], tuple(g["sig"])
    cells, kept, _, m = lane_list(n, sig, m6=True, orbit_canon=False, orbit_q=0, qprune=False,
                                  prof_order=0)
    hit = re.match(r"FIRSTHIT: idx=(\d+) profile_rank=(\d+) nodes_this_cand=(\d+)",
                   next(s for s in g["runs"]["archived"]["semantic"] if s.startswith("FIRSTHIT")))
    idx, hit_pi, hit_nodes = (int(x) for x in hit.groups())
    upto = [cells[pi] for pi in range(hit_pi + 1)]
    rows, off, nr = ab_rows(n, sig, m, upto)
    return n, sig, m, cells, kept, rows, off, nr, idx, hit_pi, hit_nodes


def _stream(oracle, n, m, c):
    surv, _, _ = oracle.cd_stream(n, list(c.tx[:m]), list(c.ty[:m]), m=m, pinX=bool(c.pinX),
                                  pinY=bool(c.pinY))
    return surv


def _complete(oracle, n, sig, m, pairs, r, **kw):
    """(verdict, nodes, A, B) of each C,D pair, on the host cores (the oracle's C calls run
    outside the interpreter lock)."""
    def one(x):
        return oracle.complete_ab(n, sig[0], sig[1], x[0], x[1], BUDGET, rows=r, m=m, **kw)
    with cf.ThreadPoolExecutor(max_workers=NCPU) as ex:
        return list(ex.map(one, pairs))


def _drain(oracle, n, sig, m, surv, r, **kw):
    """The hit cell's drain: survivors by flat score (stable), completed in order up to the
    first hit (in blocks, each block's candidates completed in parallel)."""
    score = np.array([oracle.flat_score(x[0], x[1]) for x in surv])
    order = np.argsort(score, kind="stable")
    got = []
    for b0 in range(0, len(order), 1024):
        block = order[b0:b0 + 1024]
        for t, (v, nodes, A, B) in zip(block, _complete(oracle, n, sig, m, surv[block], r, **kw)):
            got.append([len(got), int(v), int(nodes)])
            if v == 0:
                return got, (A, B, surv[t][0], surv[t][1])
    return got, None


def test_canary_n29_stream_counts_and_hit_cell(built_lib, oracle):
    g = _golden()
    run = g["runs"]["archived"]
    n, sig, m, cells, kept, rows, off, nr, idx, hit_pi, hit_nodes = _setup(g)
    assert run["rc"] == 0 and f"RESULT: FOUND at idx={idx}" in run["semantic"]
    assert all(kept[:hit_pi + 1])  # orbit canon off: no orbit duplicates
    live = [pi for pi in range(hit_pi + 1) if nr[pi] > 0]
    summary = next(s for s in run["semantic"] if s.startswith("backtracks_entered="))
    dead = int(re.search(r"cells_prof_dead=(\d+)", summary).group(1))
    assert hit_pi + 1 - len(live) == dead  # cells without allowed rows are never streamed

    streamed = {pi: _stream(oracle, n, m, cells[pi]) for pi in live}
    assert sum(len(s) for s in streamed.values()) == idx  # candidates_streamed at the hit
    # the cells whose candidates were completed: every live cell with survivors
    assert [c["pi"] for c in run["cells"]] == [pi for pi in live if len(streamed[pi])]

    r = rows[off[hit_pi]:off[hit_pi] + nr[hit_pi]]
    got, quad = _drain(oracle, n, sig, m, streamed[hit_pi], r)
    want = [[ci, v, nodes] for ci, pi, v, nodes in run["hit_cell"]]
    assert got == want
    assert got[-1][1] == 0 and got[-1][2] == hit_nodes
    lines = {s.split(" =")[0]: s for s in run["semantic"] if s[:3] in ("A =", "B =", "C =", "D =")}
    for name, seq in zip("ABCD", quad):
        assert lines[name] == "%s = {%s};" % (name, ",".join(str(int(x)) for x in seq))
    A, B, C_, D = quad
    for s in range(1, n + 1):
        assert oracle.npaf_at(A, B, C_, D, s) == 0
