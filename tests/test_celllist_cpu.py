"""The lane's cell list on the host, against the reference's own list stage
(tests/golden/list_golden.json: WZ_FH_LIST_ONLY runs of the reference binary under
WZ_FH_PROF_ORDER=3, whose digest covers every raw cell key in order and every kept flag).

Checked two ways: the drop-in binary bin/bs_firsthit prints the same bracketed lines and exit
code, and the host-only C ABI bs_cell_list returns the same cell count, kept count and digest.
bs_ab_rows is checked against a direct restatement of the abpMap rule at small n.
"""
import itertools
import json
import os
import re
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


def _cases(large=None):
    cs = json.load(open(os.path.join(HERE, "golden", "list_golden.json")))
    return [c for c in cs if large is None or c["large"] == large]


def _order_line(lines):
    for l in lines:
        m = re.match(r"\[order\] ord3 cells=(\d+) kept=(\d+) .*digest=([0-9a-f]+:[0-9a-f]+)", l)
        if m:
            return int(m.group(1)), int(m.group(2)), m.group(3)
    raise AssertionError("no [order] line")


def test_lane_binary_list_stage_matches_reference(built_lib):
    from make_list_golden import run
    from bs45_quantum_explorer_gb300.build import build_host
    exe = build_host()
    for c in _cases():
        if c["large"] and c["n"] != 42:
            continue
        rc, lines = run(exe, c["n"], c["sig"], c["settings"])
        assert (rc, lines) == (c["rc"], c["lines"]), (c["n"], c["sig"], c["settings"])


def _opts(c):
    st = c["settings"]
    big = c["n"] >= 36
    return dict(m6=bool(st.get("WZ_FH_M6", big)), thm211b=bool(st.get("WZ_THM211B", big)),
                thm212=bool(st.get("WZ_THM212", big)), endpos=bool(st.get("WZ_FH_ENDPOS", 0)),
                orbit_canon=True, orbit_q=int(st.get("WZ_FH_ORBIT_Q", 0)),
                qprune=bool(st.get("WZ_FH_ORBIT_QPRUNE", 0)), prof_order=3,
                nshard=int(st.get("WZ_FH_NSHARD", 1)))


def test_cell_list_capi_matches_reference(built_lib):
    from bs45_quantum_explorer_gb300.cells import cell_list
    for c in _cases():
        if c["large"] and c["n"] != 36:   # (n=42 is covered through the binary above)
            continue
        cells, kept, digest, m = cell_list(c["n"], tuple(c["sig"]), **_opts(c))
        ncell, nkept, want = _order_line(c["lines"])
        assert (len(kept), int(kept.sum()), digest) == (ncell, nkept, want), (c["n"], c["sig"], c["settings"])
        assert m == (6 if _opts(c)["m6"] else 3)


def test_cell_list_longer_than_its_first_buffer(built_lib, monkeypatch):
    """A list longer than the first buffer is built again at its reported size: the same
    cells, kept flags and digest as a single build."""
    import ctypes as C

    import bs45_quantum_explorer_gb300.cells as cl
    args = (17, _sigs(17)[0])
    kw = dict(m6=True, orbit_canon=True, orbit_q=1, prof_order=3)
    cells, kept, digest, m = cl.cell_list(*args, **kw)
    assert len(kept) > 8 and digest
    monkeypatch.setattr(cl, "LIST_GUESS", 8)
    cells2, kept2, digest2, m2 = cl.cell_list(*args, **kw)
    assert (digest2, m2) == (digest, m) and np.array_equal(kept2, kept)
    assert len(cells2) == len(cells)
    assert C.string_at(C.addressof(cells2), C.sizeof(cells2)) == \
        C.string_at(C.addressof(cells), C.sizeof(cells))


def test_cell_list_kept_after_a_short_buffer_serves_only_its_own_request(built_lib, monkeypatch):
    """The list a short-buffer call built is handed to the same request made again with room
    for it, never to another request; a request made in between gets its own list."""
    import bs45_quantum_explorer_gb300.cells as cl
    kw = dict(m6=True, orbit_canon=True, orbit_q=1, prof_order=3)
    a, b = (17, _sigs(17)[0]), (17, _sigs(17)[1])
    want_a, want_b = cl.cell_list(*a, **kw), cl.cell_list(*b, **kw)
    assert want_a[2] != want_b[2]
    monkeypatch.setattr(cl, "LIST_GUESS", 8)
    lib = cl.lib()
    o = cl.ListOpts(m6=1, thm211b=0, thm212=0, endpos=0, orbit_canon=1, orbit_q=1, qprune=0,
                    prof_order=3, nshard=1)
    ncells = cl.C.c_longlong(0)
    # a short call for a, then a whole call for b: b is built, not served a's list
    assert lib.bs_cell_list(17, *a[1], cl.C.byref(o), None, None, 1, cl.C.byref(ncells),
                            None) == cl.BS_ERR_CAP
    got_b = cl.cell_list(*b, **kw)
    assert got_b[2] == want_b[2] and np.array_equal(got_b[1], want_b[1])
    # a again, short twice, then whole: the same list as a single build
    for _ in range(2):
        assert lib.bs_cell_list(17, *a[1], cl.C.byref(o), None, None, 1, cl.C.byref(ncells),
                                None) == cl.BS_ERR_CAP
    got_a = cl.cell_list(*a, **kw)
    assert got_a[2] == want_a[2] and np.array_equal(got_a[1], want_a[1])


def _sigs(n):
    from make_golden import classes
    return [tuple(s) for s in classes(n)]


def test_cell_list_without_canon_keeps_every_cell_and_sets_pins(built_lib):
    from bs45_quantum_explorer_gb300.cells import cell_list
    cells, kept, digest, m = cell_list(12, (1, 7, 0, 0), m6=True)
    assert digest == "" and kept.all() and len(kept) > 0
    assert all(cells[i].pinX == 1 and cells[i].pinY == 1 for i in range(len(kept)))
    cells2, kept2, _, _ = cell_list(12, (1, 7, 0, 0), m6=True, orbit_canon=True)
    assert len(kept2) == len(kept) and 0 < kept2.sum() < len(kept2)
    assert all(cells2[i].pinX == 0 and cells2[i].pinY == 0 for i in range(len(kept2)))


def test_cell_list_refuses_bad_arguments(built_lib):
    from bs45_quantum_explorer_gb300._lib import BsError
    from bs45_quantum_explorer_gb300.cells import cell_list
    with pytest.raises(BsError):
        cell_list(12, (1, 7, 0, 2))                     # signature norm != 4n+2
    with pytest.raises(BsError):
        cell_list(12, (1, 7, 0, 0), prof_order=3)        # ORDER=3 without canon


# ---- allowed A,B rows, restated from the rule (wz_match.cpp:2318-2378) ----

def _enum_cs(L, target, m):
    cnt = [len(range(c, L, m)) for c in range(m)]
    out = []
    for v in itertools.product(*[range(-k, k + 1, 2) for k in cnt[:-1]]):
        last = target - sum(v)
        if abs(last) <= cnt[-1] and (last + cnt[-1]) % 2 == 0:
            out.append(list(v) + [last])
    return out


def _acf(v, s):
    return sum(v[i] * v[i + s] for i in range(len(v) - s))


def _ab_side_212(x, y, m, n):
    c1 = n % m
    want = 2 if c1 else 0
    if (x[0] + y[0] + x[c1] + y[c1]) % 4 != want:
        return False
    for j in range(2, m + 1):
        if j == c1 + 1:
            continue
        c = (n + 1 - j) % m
        if (x[j - 1] + y[j - 1] + x[c] + y[c]) % 4:
            return False
    return True


def _rows_brute(n, sig, m, px, py):
    tgt, hm = 4 * n + 2, m // 2
    need = tgt - sum(v * v for v in px) - sum(v * v for v in py)
    needT = [-(_acf(px, s) + _acf(py, s) + _acf(px, m - s) + _acf(py, m - s)) for s in range(1, hm + 1)]
    def side(sg):
        return [v for s in ((1, -1) if sg else (1,)) for v in _enum_cs(n + 1, s * sg, m)]
    rows = []
    for k in side(sig[0]):
        for r in side(sig[1]):
            if sum(v * v for v in k) + sum(v * v for v in r) != need:
                continue
            T = [_acf(k, s) + _acf(k, m - s) + _acf(r, s) + _acf(r, m - s) for s in range(1, hm + 1)]
            if T == needT and _ab_side_212(k, r, m, n):
                rows.append(tuple(k) + (0,) * (8 - m) + tuple(r) + (0,) * (8 - m))
    return rows


@pytest.mark.parametrize("n,sig,m6", [(12, (1, 7, 0, 0), True), (13, (0, 2, 1, 7), True),
                                      (12, (1, 3, 2, 6), False)])
def test_ab_rows_match_the_rule(built_lib, n, sig, m6):
    from bs45_quantum_explorer_gb300.cells import ab_rows, cell_list, cell_tuple
    cells, kept, _, m = cell_list(n, sig, m6=m6, thm211b=True, thm212=True)
    pick = list(range(0, len(kept), max(1, len(kept) // 40)))[:40]
    sub = [cells[i] for i in pick]
    rows, row_off, nrows = ab_rows(n, sig, m, sub)
    assert rows.shape[1] == 16
    for j, i in enumerate(pick):
        px, py = cell_tuple(cells[i], m)
        got = [tuple(int(x) for x in r) for r in rows[row_off[j]:row_off[j] + nrows[j]]]
        want = _rows_brute(n, sig, m, list(px), list(py))
        assert got == want, (n, sig, px, py)


def _rows_grouped(n, sig, m, cells):
    """The same rule at production n: a pair (k, r) is kept when its norms sum to the cell's
    need, its residues to the cell's needT, and Thm 2.12 holds, in k-then-r order. The r tuples
    are grouped by (norm, residues), so each k looks up only the r that can complete it."""
    tgt, hm = 4 * n + 2, m // 2

    def side(sg):
        return [v for s in ((1, -1) if sg else (1,)) for v in _enum_cs(n + 1, s * sg, m)]

    def info(v):
        return sum(x * x for x in v), tuple(_acf(v, s) + _acf(v, m - s) for s in range(1, hm + 1))
    K = [(v,) + info(v) for v in side(sig[0])]
    R = side(sig[1])
    by = {}
    for r in R:
        by.setdefault(info(r), []).append(r)
    out = []
    for px, py in cells:
        need = tgt - sum(v * v for v in px) - sum(v * v for v in py)
        needT = [-(_acf(px, s) + _acf(py, s) + _acf(px, m - s) + _acf(py, m - s)) for s in range(1, hm + 1)]
        rows = []
        for k, kn, kT in K:
            for r in by.get((need - kn, tuple(t - a for t, a in zip(needT, kT))), ()):
                if _ab_side_212(k, r, m, n):
                    rows.append(tuple(k) + (0,) * (8 - m) + tuple(r) + (0,) * (8 - m))
        out.append(rows)
    return out


@pytest.mark.parametrize("n,sig", [(30, (1, 7, 6, 6)), (36, (5, 11, 0, 0))])
def test_ab_rows_match_the_rule_at_production_n(built_lib, n, sig):
    from bs45_quantum_explorer_gb300.cells import ab_rows, cell_tuple
    from bs45_quantum_explorer_gb300.lane import lane_list
    cells, kept, _, m = lane_list(n, sig, m6=True, thm211b=True, thm212=True)
    idx = [i for i in range(len(kept)) if kept[i]]
    pick = idx[:: max(1, len(idx) // 6)][:6]
    sub = [cells[i] for i in pick]
    rows, row_off, nrows = ab_rows(n, sig, m, sub)
    want = _rows_grouped(n, sig, m, [tuple(map(list, cell_tuple(c, m))) for c in sub])
    assert sum(len(w) for w in want) > 0
    for j in range(len(sub)):
        got = [tuple(int(x) for x in r) for r in rows[row_off[j]:row_off[j] + nrows[j]]]
        assert got == want[j], (n, sig, j)


def test_lane_binary_qprune_audit_files_match_reference(built_lib):
    """WZ_FH_QPRUNE_DUMP: the lane binary writes the same audit files as the reference (the
    raw index of every cell the Q-closure prune removes, and one certificate per dead orbit;
    tests/golden/qprune_dump_golden.json, from make_qprune_dump_golden.py), byte for byte."""
    from make_qprune_dump_golden import record
    from bs45_quantum_explorer_gb300.build import build_host
    exe = build_host()
    cases = json.load(open(os.path.join(HERE, "golden", "qprune_dump_golden.json")))
    assert len(cases) >= 8 and all(c["files"]["dump"][1] > 0 for c in cases)
    for c in cases:
        rc, files = record(exe, c["n"], tuple(c["sig"]))
        assert (rc, files) == (c["rc"], c["files"]), (c["n"], c["sig"])
