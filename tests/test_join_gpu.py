"""A,B-side stream (count_pairs22 with abSide, src/solver/wz_match.cpp:766-768), exact NPAF
verification (npaf_at, :184-192) and the autocorrelation join (WZ_JOIN22, :2894-3104) on the
GPU. The join test rebuilds the complete BS(7,6) set (4,736 ordered quads over 56 signed
signatures) from the mirror-quad streams and compares it with the brute force."""
import itertools
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _cells(L, total, m):
    cnt = [len(range(c, L, m)) for c in range(m)]
    out = []
    for v in itertools.product(*[range(-k, k + 1, 2) for k in cnt[:-1]]):
        last = total - sum(v)
        if abs(last) <= cnt[-1] and (last + cnt[-1]) % 2 == 0:
            out.append(list(v) + [last])
    return out


def _classes(n):
    out = []
    for a in range((n + 1) % 2, n + 2, 2):
        for b in range(a, n + 2, 2):
            for c in range(n % 2, n + 1, 2):
                rest = 4 * n + 2 - a * a - b * b - c * c
                if rest < c * c:
                    break
                d = int(round(rest ** 0.5))
                if d * d == rest and d >= c and (d - n) % 2 == 0:
                    out.append((a, b, c, d))
    return out


@pytest.mark.parametrize("n", [6, 9, 12, 15, 20])
def test_ab_stream_matches_oracle(gpu, oracle, n):
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.stream import cd_stream
    rng = np.random.default_rng(n)
    for sig in _classes(n)[:2]:
        ctx = Context(n, sig)
        for m in (3, 6):
            cells = [(x, y) for x in _cells(n + 1, sig[0], m) for y in _cells(n + 1, sig[1], m)]
            cells = [cells[i] for i in rng.permutation(len(cells))[:20]]
            for rev, pin in ((0, 0), (1, 1)):
                pins = [(int(pin and sig[0] == 0), int(pin and sig[1] == 0))] * len(cells)
                got, gidx, gst = cd_stream(ctx, cells, m=m, pins=pins, rev=rev, ab_side=True)
                rows, ridx, rst = [], [], []
                for i, (tx, ty) in enumerate(cells):
                    r, _, st = oracle.cd_stream(n, tx, ty, m=m, pinX=pins[i][0], pinY=pins[i][1],
                                                rev=rev, ab_side=True)
                    rows.append(r)
                    ridx += [i] * len(r)
                    rst.append(st)
                ref = np.concatenate(rows)
                assert got.shape == ref.shape and (got == ref).all(), (n, sig, m, rev)
                assert gidx.tolist() == ridx and gst == rst


def test_npaf_verify(gpu, oracle):
    from bs45_quantum_explorer_gb300.hall import Context, pack
    from bs45_quantum_explorer_gb300.stream import npaf_verify
    quads = json.load(open(os.path.join(HERE, "golden", "known_quads.json")))
    for q in quads[:12]:
        n = q["n"]
        ctx = Context(n, [abs(x) for x in q["sig"]])
        A, B, C_, D = (np.array(q[k], np.int8) for k in "ABCD")
        rng = np.random.default_rng(n)
        rows = [[pack(A), pack(B), pack(C_), pack(D)]]
        exp = [0]
        for _ in range(50):  # flip one element: NPAF is no longer zero
            A2 = A.copy()
            A2[rng.integers(0, n + 1)] *= -1
            rows.append([pack(A2), pack(B), pack(C_), pack(D)])
            exp.append(max(abs(oracle.npaf_at(A2, B, C_, D, s)) for s in range(1, n + 2)))
        got = npaf_verify(ctx, np.array(rows, np.uint64))
        assert got.tolist() == exp


def test_join_rebuilds_bs7_6_full_set(gpu):
    """C1: every BS(7,6) quad, found by joining the A,B and C,D mirror-quad streams of all
    56 signed signatures (no pins, no canonicalisation), equals the brute-force set."""
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.stream import cd_stream, join_quads
    n = 6
    truth = np.load(os.path.join(HERE, "golden", "bs7_6_all.npz"))["quads"]
    found = []
    sigs = set()
    for a, b, c, d in itertools.product(range(-7, 8), range(-7, 8), range(-6, 7), range(-6, 7)):
        if a * a + b * b + c * c + d * d != 4 * n + 2:
            continue
        if (a - 7) % 2 or (b - 7) % 2 or c % 2 or d % 2:
            continue
        sigs.add((a, b, c, d))
        ctx = Context(n, (a, b, c, d))
        m = 6
        ab_cells = [(x, y) for x in _cells(n + 1, a, m) for y in _cells(n + 1, b, m)]
        cd_cells = [(x, y) for x in _cells(n, c, m) for y in _cells(n, d, m)]
        ab, _, _ = cd_stream(ctx, ab_cells, m=m, ab_side=True, as_words=True)
        cd, _, _ = cd_stream(ctx, cd_cells, m=m, as_words=True)
        if len(ab) and len(cd):
            q, _ = join_quads(ctx, cd, ab)
            found.append(q)
        ctx.close()
    assert len(sigs) == 56
    got = np.concatenate(found)
    got_set = {tuple(int(x) for x in r) for r in got}
    truth_set = {tuple(int(x) for x in r) for r in truth}
    assert len(got) == len(got_set)  # no duplicates
    assert got_set == truth_set, (len(got_set), len(truth_set))
