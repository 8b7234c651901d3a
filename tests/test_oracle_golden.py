"""The oracle pinned against the reference's own outputs (tests/golden/, generated by
tests/golden/make_golden.py from the reference compiled from its sources).

CPU only: these run in the default suite and need no GPU.
"""
import json
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
G = os.path.join(HERE, "golden")


def unpack(w, L):
    w = np.asarray(w, np.uint64)
    bits = (w[..., None] >> np.arange(L, dtype=np.uint64)) & np.uint64(1)
    return np.where(bits == 1, 1, -1).astype(np.int8)


def test_known_quads_npaf_and_hall(oracle):
    quads = json.load(open(os.path.join(G, "known_quads.json")))
    assert len(quads) >= 40
    for q in quads:
        n = q["n"]
        A, B, C_, D = (np.array(q[k], np.int8) for k in "ABCD")
        assert max(abs(oracle.npaf_at(A, B, C_, D, s)) for s in range(1, n + 2)) == 0, q["file"]
        assert oracle.hall_pair(n, C_, D) == q["hall_cd"], q["file"]
        assert sum(int(x.sum()) ** 2 for x in (A, B, C_, D)) == 4 * n + 2


def test_hall_decisions_match_reference(oracle):
    g = np.load(os.path.join(G, "hall_golden.npz"))
    n = int(g["n"])
    got = oracle.hall_batch(n, unpack(g["words"], n), nthreads=4)
    assert (got == g["decisions"]).all()
    got = oracle.hall_batch(n, unpack(g["near_words"], n), nthreads=4)
    assert (got == g["near_decisions"]).all()


@pytest.mark.parametrize("fixture,least", [("streams_golden.npz", 100), ("cd_prune_golden.npz", 150)])
def test_streams_match_reference(oracle, fixture, least):
    """count_pairs22 survivors and counts; cd_prune_golden.npz holds WZ_FH_CD_PRUNE 1, 2, 3."""
    g = np.load(os.path.join(G, fixture))
    cases, words = g["cases"], g["words"]
    assert len(cases) >= least
    for row in cases:
        n, a, b, c, d, m, rev, endpos, pinX, pinY, cdp, nodes, leaves, ok, off, cnt = (int(x) for x in row[:16])
        tx = [int(x) for x in row[16:16 + m]]
        ty = [int(x) for x in row[22:22 + m]]
        rows, _, st = oracle.cd_stream(n, tx, ty, m=m, pinX=pinX, pinY=pinY, rev=rev, endpos=endpos,
                                       cd_prune=cdp)
        assert len(rows) == cnt
        assert (rows == unpack(words[off:off + cnt], n)).all()
        assert (st["nodes"], st["leaves"], st["ok"]) == (nodes, leaves, ok)


def test_ab_side_streams_match_reference(oracle):
    g = np.load(os.path.join(G, "ab_streams_golden.npz"))
    cases, words = g["cases"], g["words"]
    assert len(cases) >= 50
    for row in cases:
        n, a, b, c, d, m, rev, pinX, pinY, nodes, leaves, ok, off, cnt = (int(x) for x in row[:14])
        tx = [int(x) for x in row[14:14 + m]]
        ty = [int(x) for x in row[20:20 + m]]
        rows, _, st = oracle.cd_stream(n, tx, ty, m=m, pinX=pinX, pinY=pinY, rev=rev, ab_side=True)
        assert len(rows) == cnt
        assert (rows == unpack(words[off:off + cnt], n + 1)).all()
        assert (st["nodes"], st["leaves"], st["ok"]) == (nodes, leaves, ok)


def _complete_cases():
    g = np.load(os.path.join(G, "complete_golden.npz"))
    return g["cases"].astype(np.int64), g["cd"], g["rows"]


def test_completions_match_reference(oracle):
    cases, cd, rows = _complete_cases()
    assert len(cases) >= 900
    for row in cases:
        n, a, b, budget, use_rows, roff, nrows, v, nodes, ci = (int(x) for x in row[:10])
        if budget == 0 and n > 17:
            continue  # exact completions at the larger n run in the GPU suite
        C_, D = unpack(cd[ci], n)
        rr = rows[roff:roff + nrows] if use_rows else None
        got_v, got_nodes, A, B = oracle.complete_ab(n, a, b, C_, D, budget, rows=rr)
        assert (got_v, got_nodes) == (v, nodes), (n, a, b, budget, use_rows)
        if v == 0:
            aw, bw = np.uint64(row[10]), np.uint64(row[11])
            assert (A == unpack(aw, n + 1)).all() and (B == unpack(bw, n + 1)).all()


def _a2_cases():
    g = np.load(os.path.join(G, "a2_complete_golden.npz"))
    return g["cases"].astype(np.int64), g["cd"], g["rows"]


def test_a2_completions_match_reference(oracle):
    """The A2 row prune (WZ_FH_A2=2): the reference's verdicts, charged node counts and
    completions with the prune on; and with it off, its node counts (never fewer)."""
    cases, cd, rows = _a2_cases()
    assert len(cases) >= 1000
    assert (cases[:, 7] < cases[:, 10]).sum() > 100  # the prune cuts real nodes
    for row in cases:
        n, a, b, budget, roff, nrows, v2, n2, ci, v0, n0 = (int(x) for x in row[:11])
        if budget == 0 and n > 17:
            continue  # exact completions at the larger n run in the GPU suite
        C_, D = unpack(cd[ci], n)
        rr = rows[roff:roff + nrows]
        got = oracle.complete_ab(n, a, b, C_, D, budget, rows=rr, a2=2)
        assert got[:2] == (v2, n2), (n, a, b, budget)
        if v2 == 0:
            assert (got[2] == unpack(np.uint64(row[11]), n + 1)).all()
            assert (got[3] == unpack(np.uint64(row[12]), n + 1)).all()
        assert oracle.complete_ab(n, a, b, C_, D, budget, rows=rr)[:2] == (v0, n0)
        assert n2 <= n0 or budget > 0


def test_controls_match_reference(oracle):
    ctl = json.load(open(os.path.join(G, "controls_golden.json")))
    quads = {q["file"]: q for q in json.load(open(os.path.join(G, "known_quads.json")))}
    checked = 0
    for c in ctl:
        if c["budget"] != 200000:
            continue  # the 2^22 and exact controls run in the GPU suite
        q = quads[c["file"]]
        C_, D = np.array(q["C"], np.int8), np.array(q["D"], np.int8)
        v, nodes, A, B = oracle.complete_ab(c["n"], c["sig"][0], c["sig"][1], C_, D, c["budget"])
        assert (v, nodes) == (c["verdict"], c["nodes"]), c["file"]
        if v == 0:
            assert A.tolist() == c["A"] and B.tolist() == c["B"]
        checked += 1
    assert checked >= 40


def test_bs7_6_full_set_is_closed_and_complete():
    """The brute-force BS(7,6) set: 4,736 ordered quads over 56 signed signatures, every one
    with NPAF 0 and every one in the Thm 2.2 encoding."""
    q = np.load(os.path.join(G, "bs7_6_all.npz"))["quads"]
    assert q.shape == (4736, 4)
    A, B = unpack(q[:, 0], 7), unpack(q[:, 1], 7)
    C_, D = unpack(q[:, 2], 6), unpack(q[:, 3], 6)
    for s in range(1, 7):
        tot = (A[:, :7 - s] * A[:, s:]).sum(1) + (B[:, :7 - s] * B[:, s:]).sum(1)
        if s < 6:
            tot += (C_[:, :6 - s] * C_[:, s:]).sum(1) + (D[:, :6 - s] * D[:, s:]).sum(1)
        assert (tot == 0).all()
    sigs = {(int(a), int(b), int(c), int(d)) for a, b, c, d in
            zip(A.sum(1), B.sum(1), C_.sum(1), D.sum(1))}
    assert len(sigs) == 56
    # Thm 2.2 encoding: A,B root quad product -1, the others +1 (verify_npaf.py:60-73)
    assert (A[:, 0] * B[:, 0] * A[:, 6] * B[:, 6] == -1).all()
    for d in range(1, 3):
        assert (A[:, d] * B[:, d] * A[:, 6 - d] * B[:, 6 - d] == 1).all()
        assert (C_[:, d] * D[:, d] * C_[:, 5 - d] * D[:, 5 - d] == 1).all()
