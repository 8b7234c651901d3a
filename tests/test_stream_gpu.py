"""C,D stream (count_pairs22, src/solver/wz_match.cpp:678-784) on the GPU against the oracle
and against the reference's own outputs (tests/golden/streams_golden.npz).

Bit-exact: the surviving (C,D) sequence in stream order, and per cell the DFS node count,
the class-exact leaf count and the Hall-pass count.
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


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


def _cells(n, total, m):
    import itertools
    cnt = [len(range(c, n, m)) for c in range(m)]
    out = []
    for v in itertools.product(*[range(-k, k + 1, 2) for k in cnt[:-1]]):
        last = total - sum(v)
        if abs(last) <= cnt[-1] and (last + cnt[-1]) % 2 == 0:
            out.append(list(v) + [last])
    return out


def _oracle_batch(oracle, n, cells, m, pins, rev, endpos):
    rows, cidx, stats = [], [], []
    # one oracle walk per cell, on all host threads, joined in cell order
    with ThreadPoolExecutor(os.cpu_count() or 4) as ex:
        outs = list(ex.map(lambda i: oracle.cd_stream(n, cells[i][0], cells[i][1], m=m,
                                                      pinX=pins[i][0], pinY=pins[i][1],
                                                      rev=rev, endpos=endpos),
                           range(len(cells))))
    for i, (r, _, st) in enumerate(outs):
        rows.append(r)
        cidx += [i] * len(r)
        stats.append(st)
    rows = np.concatenate(rows) if rows else np.zeros((0, 2, n), np.int8)
    return rows, np.array(cidx, np.uint32), stats


def _compare(ctx, oracle, n, cells, m, pins, rev, endpos, **kw):
    from bs45_quantum_explorer_gb300.stream import cd_stream
    got, gidx, gst = cd_stream(ctx, cells, m=m, pins=pins, rev=rev, endpos=endpos, **kw)
    ref, ridx, rst = _oracle_batch(oracle, n, cells, m, pins, rev, endpos)
    assert got.shape == ref.shape, (got.shape, ref.shape)
    assert (got == ref).all()
    assert (gidx == ridx).all()
    assert gst == rst, [(i, a, b) for i, (a, b) in enumerate(zip(gst, rst)) if a != b][:3]
    return len(ref)


@pytest.mark.parametrize("n", [6, 7, 9, 10, 12, 13, 15, 16, 18, 19, 21, 22])
def test_stream_matches_oracle(gpu, oracle, n):
    from bs45_quantum_explorer_gb300.hall import Context
    rng = np.random.default_rng(100 + n)
    total = 0
    for sig in _classes(n)[:3]:
        ctx = Context(n, sig)
        for m in (3, 6):
            cells = [(x, y) for x in _cells(n, sig[2], m) for y in _cells(n, sig[3], m)]
            idx = rng.permutation(len(cells))[:24]
            cells = [cells[i] for i in idx]
            for rev, endpos, pin in ((0, 0, 0), (1, 0, 1), (0, 1, 1), (1, 1, 0)):
                pins = [(int(pin and sig[2] == 0), int(pin and sig[3] == 0))] * len(cells)
                total += _compare(ctx, oracle, n, cells, m, pins, rev, endpos)
        ctx.close()
    assert total >= 0


def test_stream_resume_and_split_invariance(gpu, oracle):
    """A tiny leaf buffer forces many suspend/resume rounds; the split depth varies."""
    from bs45_quantum_explorer_gb300.hall import Context
    n, sig = 18, (1, 5, 6, 6)
    if sig not in _classes(n):
        sig = _classes(n)[0]
    ctx = Context(n, sig)
    cells = [(x, y) for x in _cells(n, sig[2], 6) for y in _cells(n, sig[3], 6)][:200]
    pins = [(0, 0)] * len(cells)
    for kw in (dict(leaf_chunk=64), dict(leaf_chunk=1000, target_prefixes=16),
               dict(target_prefixes=1 << 20), dict(hall_mode="fp64"), dict(hall_mode="tc_bf16x2"),
               # 1 us launches: every walk suspends after 256 steps, so the rounds, the
               # resumption and the host's splitting of walks all run many times
               dict(round_us=1), dict(round_us=1, leaf_chunk=64, target_prefixes=16)):
        _compare(ctx, oracle, n, cells, 6, pins, 0, 0, **kw)


@pytest.mark.parametrize("n", [26, 30])
def test_stream_larger_n(gpu, oracle, n):
    from bs45_quantum_explorer_gb300.hall import Context
    sig = (1, 7, 6, 6) if n == 30 else _classes(n)[0]
    ctx = Context(n, sig)
    rng = np.random.default_rng(n)
    cells = [(x, y) for x in _cells(n, sig[2], 6) for y in _cells(n, sig[3], 6)]
    # cells whose class sums are small have the largest streams
    cells.sort(key=lambda c: sum(abs(v) for v in c[0]) + sum(abs(v) for v in c[1]))
    pick = [cells[i] for i in rng.integers(0, min(len(cells), 400), 3)]
    from bs45_quantum_explorer_gb300.stream import cd_stream
    ref, ridx, rst = _oracle_batch(oracle, n, pick, 6, [(0, 0)] * 3, 0, 0)
    # default launches, then short ones that force suspension and splitting inside these
    # large subtrees
    for kw in (dict(), dict(round_us=300)):
        got, gidx, gst = cd_stream(ctx, pick, m=6, pins=[(0, 0)] * 3, **kw)
        assert got.shape == ref.shape and (got == ref).all() and (gidx == ridx).all(), kw
        assert gst == rst, kw


@pytest.mark.parametrize("n,sig", [(16, (3, 5, 4, 4)), (20, (1, 7, 4, 4)), (22, (1, 3, 4, 8))])
def test_stream_cd_prune_matches_oracle(gpu, oracle, n, sig):
    """WZ_FH_CD_PRUNE 1, 2, 3: the same survivors as without it and the pruned node counts of
    the oracle (the reference's rec() calls), also with 1 us launches, so that suspended
    walks are split on the host under the prune; m = 3 cells are not pruned."""
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.stream import cd_stream
    ctx = Context(n, sig)
    rng = np.random.default_rng(n + 100)
    cells = [(x, y) for x in _cells(n, sig[2], 6) for y in _cells(n, sig[3], 6)]
    # cells whose class sums are small have the largest streams
    cells.sort(key=lambda c: sum(abs(v) for v in c[0]) + sum(abs(v) for v in c[1]))
    cells = [cells[i] for i in rng.permutation(min(len(cells), 200))[:16]]
    pins = [(0, 0)] * len(cells)
    base, _, _ = cd_stream(ctx, cells, m=6, pins=pins)
    for mode in (1, 2, 3):
        for kw in (dict(), dict(round_us=1), dict(rev=True, endpos=True)):
            okw = {k: v for k, v in kw.items() if k in ("rev", "endpos")}
            with ThreadPoolExecutor(os.cpu_count() or 4) as ex:
                want = list(ex.map(lambda c: oracle.cd_stream(n, c[0], c[1], m=6, cd_prune=mode,
                                                              **okw), cells))
            ref = np.concatenate([w[0] for w in want])
            got, _, gst = cd_stream(ctx, cells, m=6, pins=pins, cd_prune=mode, **kw)
            assert got.shape == ref.shape and (got == ref).all(), (mode, kw)
            assert gst == [w[2] for w in want], (mode, kw)
            if not okw:
                assert got.shape == base.shape and (got == base).all(), (mode, kw)
    # m = 3 cells are never pruned
    c3 = [(x, y) for x in _cells(n, sig[2], 3) for y in _cells(n, sig[3], 3)][:8]
    _, _, s0 = cd_stream(ctx, c3, m=3, pins=[(0, 0)] * len(c3))
    _, _, s3 = cd_stream(ctx, c3, m=3, pins=[(0, 0)] * len(c3), cd_prune=3)
    assert s0 == s3
    ctx.close()


@pytest.mark.parametrize("fixture", ["streams_golden.npz", "cd_prune_golden.npz"])
def test_stream_golden_reference(gpu, fixture):
    """Survivors and counts exactly as the reference's count_pairs22 produced them
    (cd_prune_golden.npz: under WZ_FH_CD_PRUNE 1, 2, 3)."""
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.stream import cd_stream
    g = np.load(os.path.join(HERE, "golden", fixture))
    cases, words = g["cases"], g["words"]
    ctxs = {}
    for row in cases:
        n, a, b, c, d, m, rev, endpos, pinX, pinY, cdp, nodes, leaves, ok, off, cnt = (int(x) for x in row[:16])
        tx = [int(x) for x in row[16:16 + m]]
        ty = [int(x) for x in row[22:22 + m]]
        key = (n, a, b, c, d)
        if key not in ctxs:
            ctxs[key] = Context(n, (a, b, c, d))
        got, _, st = cd_stream(ctxs[key], [(tx, ty)], m=m, pins=[(pinX, pinY)], rev=rev,
                               endpos=endpos, as_words=True, cd_prune=cdp)
        assert got.shape[0] == cnt
        assert (got == words[off:off + cnt]).all()
        assert st[0]["leaves"] == leaves and st[0]["ok"] == ok
        assert st[0]["nodes"] == nodes, (n, m, cdp, tx, ty)


def test_stream_limit_returns_the_stream_prefix(gpu, oracle):
    """limit = L returns exactly the first L survivors of the batch, in order (the lane's
    front-only cut), for limits inside one cell, across cells and past the end."""
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.stream import cd_stream
    n = 22
    sig = _classes(n)[0]
    ctx = Context(n, sig)
    rng = np.random.default_rng(7)
    cells = [(x, y) for x in _cells(n, sig[2], 6) for y in _cells(n, sig[3], 6)]
    cells = [cells[i] for i in rng.permutation(len(cells))[:40]]
    pins = [(0, 0)] * len(cells)
    ref, ridx, _ = _oracle_batch(oracle, n, cells, 6, pins, 0, 0)
    total = len(ref)
    assert total > 200
    for L, rus in ((1, 0), (5, 0), (100, 0), (total // 2, 0), (total // 2, 1), (total - 1, 0),
                   (total, 0), (total + 3, 0)):
        got, gidx, _ = cd_stream(ctx, cells, m=6, pins=pins, limit=L, round_us=rus)
        k = min(L, total)
        assert got.shape[0] == k, (L, got.shape)
        assert (got == ref[:k]).all() and (gidx == ridx[:k]).all(), L
    ctx.close()


def test_stream_limit_on_a_large_cell(gpu):
    """n = 30, the 176,414-survivor cell: the limited stream is the full stream's prefix."""
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.stream import cd_stream
    ctx = Context(30, (1, 7, 6, 6))
    cell = ([-1, 1, 1, 1, 1, 3], [-1, 1, 1, 1, 5, -1])
    full, _, st = cd_stream(ctx, [cell], m=6, as_words=True)
    assert len(full) == 176414 and st[0]["nodes"] == 599381729
    for L in (1000, 50000, 176414):
        got, _, _ = cd_stream(ctx, [cell], m=6, as_words=True, limit=L)
        assert np.array_equal(got, full[:L]), L
    ctx.close()
