"""The per-cell flattest-256 keep of config C3 (n = 30, sig (1,7,6,6), whole cells) against
the reference's own drain on real cells (tests/golden/keep_n30_golden.json: its
WZ_FH_CAND_LOG lines, one per completed candidate in drain order with the drain rank, the
verdict and the charged nodes). Here the oracle streams each whole cell, scores every
survivor with the reference's flat score, keeps the 256 flattest by a stable sort and
completes them with the cell's allowed rows at the golden's budget: the same sequence. The
device keep (flat_topk) is checked against the same stable sort in test_complete_gpu.py, and
the lane binary's CAND lines against this golden in test_keep_gpu.py."""
import concurrent.futures as cf
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def test_keep_matches_reference_drain(built_lib, oracle):
    from bs45_quantum_explorer_gb300.cells import ab_rows
    from bs45_quantum_explorer_gb300.lane import lane_list
    g = json.load(open(os.path.join(HERE, "golden", "keep_n30_golden.json")))
    n, sig = g["n"], tuple(g["sig"])
    cells, kept, _, m = lane_list(n, sig, m6=True, thm211b=True, thm212=True, qprune=False)

    def one(case):
        st = case["settings"]
        pi = case["pi"]
        assert kept[pi]
        c = cells[pi]
        rows, off, nr = ab_rows(n, sig, m, [c])
        r = rows[off[0]:off[0] + nr[0]]
        surv, _, _ = oracle.cd_stream(n, list(c.tx[:m]), list(c.ty[:m]), m=m, pinX=bool(c.pinX),
                                      pinY=bool(c.pinY), cap=st["WZ_FH_BUF_CAP"])
        assert 256 <= len(surv) <= st["WZ_FH_BUF_CAP"]
        # flat scores of every survivor at once (sum over s of |N_C(s) + N_D(s)|), checked
        # against the oracle's flat_score on the first 512
        X = surv.astype(np.int64)
        score = np.zeros(len(surv), np.int64)
        for s in range(1, n):
            score += np.abs((X[:, 0, :-s] * X[:, 0, s:]).sum(1) + (X[:, 1, :-s] * X[:, 1, s:]).sum(1))
        assert all(score[i] == oracle.flat_score(surv[i][0], surv[i][1]) for i in range(512))
        order = np.argsort(score, kind="stable")[:st["WZ_FH_DRAIN_TOP"]]
        got = []
        for ci, t in enumerate(order):
            v, nodes, _, _ = oracle.complete_ab(n, sig[0], sig[1], surv[t][0], surv[t][1],
                                                st["WZ_FH_AB_BUDGET"], rows=r, m=m)
            got.append([ci, pi, int(v), int(nodes)])
        return got, case["cand"]

    with cf.ThreadPoolExecutor(max_workers=len(g["cases"])) as ex:
        for got, want in ex.map(one, g["cases"]):
            assert got == want
