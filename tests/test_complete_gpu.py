"""A,B completion (fh_complete_ab, src/solver/wz_match.cpp:1298-1341) and the per-cell
flattest-k keep (flat_score + drain(), :2569-2583, :2656-2714) on the GPU.

Bit-exact against the reference's own outputs (tests/golden/) and the oracle: verdict,
charged node count and the completion A,B of every candidate; the kept order of every batch.
"""
import json
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
G = os.path.join(HERE, "golden")


def unpack(w, L):
    w = np.asarray(w, np.uint64)
    bits = (w[..., None] >> np.arange(L, dtype=np.uint64)) & np.uint64(1)
    return np.where(bits == 1, 1, -1).astype(np.int8)


@pytest.mark.parametrize("blocks", [0, 3])
def test_completions_golden(gpu, blocks):
    """blocks: resident completer blocks per SM (0 = the default 2; 3 = the build whose
    register budget is cut for three), which must not change a result."""
    from bs45_quantum_explorer_gb300.complete import complete_ab
    from bs45_quantum_explorer_gb300.hall import Context
    g = np.load(os.path.join(G, "complete_golden.npz"))
    cases, cd, rows = g["cases"].astype(np.int64), g["cd"], g["rows"]
    groups = {}
    for i, row in enumerate(cases):
        n, a, b, budget, use_rows = (int(x) for x in row[:5])
        groups.setdefault((n, a, b, budget, use_rows), []).append(i)
    for (n, a, b, budget, use_rows), idx in groups.items():
        sig = (a, b) + _cd_sig(n, a, b)
        ctx = Context(n, sig)
        cands = np.stack([cd[int(cases[i, 9])] for i in idx])
        rr = [rows[int(cases[i, 5]):int(cases[i, 5]) + int(cases[i, 6])] if use_rows else None for i in idx]
        v, nodes, A, B = complete_ab(ctx, cands, budget, rows_per_cand=rr, blocks_per_sm=blocks)
        for t, i in enumerate(idx):
            assert (v[t], nodes[t]) == (cases[i, 7], cases[i, 8]), (n, a, b, budget, use_rows, t)
            if v[t] == 0:
                assert (A[t] == unpack(np.uint64(cases[i, 10]), n + 1)).all()
                assert (B[t] == unpack(np.uint64(cases[i, 11]), n + 1)).all()
        ctx.close()


def test_a2_completions_golden(gpu):
    """The A2 row prune on the device (bs_ab_opts.a2 = 2) against the reference's fh_complete_ab
    under WZ_FH_A2=2 (tests/golden/a2_complete_golden.npz): verdicts, charged nodes and the
    first completion."""
    from bs45_quantum_explorer_gb300.complete import complete_ab
    from bs45_quantum_explorer_gb300.hall import Context
    g = np.load(os.path.join(G, "a2_complete_golden.npz"))
    cases, cd, rows = g["cases"].astype(np.int64), g["cd"], g["rows"]
    groups = {}
    for i, row in enumerate(cases):
        n, a, b, budget = (int(x) for x in row[:4])
        groups.setdefault((n, a, b, budget), []).append(i)
    for (n, a, b, budget), idx in groups.items():
        ctx = Context(n, (a, b) + _cd_sig(n, a, b))
        cands = np.stack([cd[int(cases[i, 8])] for i in idx])
        rr = [rows[int(cases[i, 4]):int(cases[i, 4]) + int(cases[i, 5])] for i in idx]
        for a2, vcol, ncol in ((2, 6, 7), (0, 9, 10)):
            v, nodes, A, B = complete_ab(ctx, cands, budget, rows_per_cand=rr, a2=a2)
            for t, i in enumerate(idx):
                assert (v[t], nodes[t]) == (cases[i, vcol], cases[i, ncol]), (n, a, b, budget, a2, t)
                if a2 == 2 and v[t] == 0:
                    assert (A[t] == unpack(np.uint64(cases[i, 11]), n + 1)).all()
                    assert (B[t] == unpack(np.uint64(cases[i, 12]), n + 1)).all()
        ctx.close()


def _cd_sig(n, a, b):
    """Any (c, d) completing the signature norm; the completer only reads |a|, |b|."""
    rest = 4 * n + 2 - a * a - b * b
    for c in range(n % 2, n + 1, 2):
        d2 = rest - c * c
        if d2 < 0:
            break
        d = int(round(d2 ** 0.5))
        if d * d == d2 and (d - n) % 2 == 0:
            return (c, d)
    raise ValueError((n, a, b))


def test_controls_golden(gpu):
    """The six known C,D (ours and Wang-Zhu n=41..43) exactly and every banked quad at
    budgets 2e5 and 2^22, in batches."""
    from bs45_quantum_explorer_gb300.complete import complete_ab
    from bs45_quantum_explorer_gb300.hall import Context
    ctl = json.load(open(os.path.join(G, "controls_golden.json")))
    quads = {q["file"]: q for q in json.load(open(os.path.join(G, "known_quads.json")))}
    by = {}
    for c in ctl:
        by.setdefault((c["n"], tuple(c["sig"]), c["budget"]), []).append(c)
    for (n, sig, budget), cs in by.items():
        ctx = Context(n, sig)
        cands = np.stack([np.stack([np.array(quads[c["file"]]["C"], np.int8),
                                    np.array(quads[c["file"]]["D"], np.int8)]) for c in cs])
        v, nodes, A, B = complete_ab(ctx, cands, budget, max_seconds=600)
        for t, c in enumerate(cs):
            assert (v[t], nodes[t]) == (c["verdict"], c["nodes"]), (c["file"], budget)
            if v[t] == 0:
                assert A[t].tolist() == c["A"] and B[t].tolist() == c["B"]
        ctx.close()


def test_completion_vs_oracle_first_hit(gpu, oracle):
    """Random stream candidates with rows, small budgets (many aborts) and first-hit mode."""
    import sys
    sys.path.insert(0, G)
    from make_golden import abp_rows, classes, enum_cs
    from bs45_quantum_explorer_gb300.complete import complete_ab
    from bs45_quantum_explorer_gb300.hall import Context
    rng = np.random.default_rng(5)
    for n in (13, 16, 19, 24):
        cl = classes(n)
        sig = cl[len(cl) // 2]
        ctx = Context(n, sig)
        cells = [(x, y) for x in enum_cs(n, sig[2], 6) for y in enum_cs(n, sig[3], 6)]
        rng.shuffle(cells)
        cands, rows = [], []
        # the oracle walks each cell whole; the 60 walks run on all host threads
        with ThreadPoolExecutor(os.cpu_count() or 4) as ex:
            streams = list(ex.map(lambda c: oracle.cd_stream(n, c[0], c[1], m=6, cap=20)[0],
                                  cells[:60]))
        for (tx, ty), rs in zip(cells[:60], streams):
            if len(rs):
                r = abp_rows(n, sig[0], sig[1], tx, ty)
                for cand in rs[:8]:
                    cands.append(cand)
                    rows.append(r if len(r) else None)
        if not cands:
            continue
        cands = np.stack(cands)
        for budget in (0, 25, 300):
            v, nodes, A, B = complete_ab(ctx, cands, budget, rows_per_cand=rows)
            for t in range(len(cands)):
                ov, on, oa, ob = oracle.complete_ab(n, sig[0], sig[1], cands[t, 0], cands[t, 1], budget,
                                                    rows=rows[t])
                assert (v[t], nodes[t]) == (ov, on), (n, budget, t)
                if ov == 0:
                    assert (A[t] == oa).all() and (B[t] == ob).all()
            # first-hit mode: everything up to the first hit is identical
            fv, fnodes, _, _ = complete_ab(ctx, cands, budget, rows_per_cand=rows, first_hit=True)
            hits = np.nonzero(v == 0)[0]
            upto = hits[0] + 1 if len(hits) else len(cands)
            assert (fv[:upto] == v[:upto]).all() and (fnodes[:upto] == nodes[:upto]).all()
            assert ((fv[upto:] == -1) | (fv[upto:] == v[upto:])).all()
        ctx.close()


def test_flat_topk_matches_stable_sort(gpu, oracle):
    from bs45_quantum_explorer_gb300.complete import flat_topk
    from bs45_quantum_explorer_gb300.hall import Context, pack
    n = 30
    ctx = Context(n, (1, 7, 6, 6))
    words = oracle.gen_hall_pairs(n, 20000, nthreads=4)
    X = unpack(words, n)
    scores = np.array([oracle.flat_score(x[0], x[1]) for x in X])
    for buf_cap, keep in ((20000, 0), (5000, 256), (777, 50), (20000, 20000), (64, 1)):
        order, sc = flat_topk(ctx, words, buf_cap, keep)
        exp_o, exp_s = [], []
        for lo in range(0, len(words), buf_cap):
            idx = np.arange(lo, min(len(words), lo + buf_cap))
            srt = idx[np.argsort(scores[idx], kind="stable")]
            if keep > 0:
                srt = srt[:keep]
            exp_o += srt.tolist()
            exp_s += scores[srt].tolist()
        assert order.tolist() == exp_o, (buf_cap, keep)
        assert sc.tolist() == exp_s
