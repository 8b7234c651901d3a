"""The lane list's prunes remove only cells that hold no candidate (the reference's gate
tools/test_endpos_q.py (4) and (6), there checked with its CELLSIZE counts).

Over every signature class at small odd n, with mod-6 cells:
  * the ENDPOS cell filter (wz_match.cpp:1598-1622): every cell it removes from the plain list
    streams no survivor under ENDPOS (without 2.11b and 2.12, which leave it nothing to
    remove at these n);
  * the Q-closure prune (wz_match.cpp:1745-1802) at odd n under ENDPOS with Q: every cell kept
    by orbit canon with Q but not kept once the prune runs streams no survivor.
The lists are the library's (bs_cell_list); the streams are the oracle's restatement of the
reference's DFS with ENDPOS (count_pairs22, wz_match.cpp:678-784)."""
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


def _cells(lst):
    cells, kept, _, m = lst
    return {(tuple(cells[i].tx[:m]), tuple(cells[i].ty[:m])): (cells[i], int(kept[i]))
            for i in range(len(kept))}


def _survivors(oracle, n, cell):
    """The cell's survivor count under ENDPOS (only the count is kept)."""
    _, _, st = oracle.cd_stream(n, list(cell.tx[:6]), list(cell.ty[:6]), m=6, pinX=bool(cell.pinX),
                                pinY=bool(cell.pinY), endpos=True, cap=1)
    return st["ok"]


@pytest.mark.parametrize("n", [7, 9, 13])
def test_endpos_cell_filter_removes_only_empty_cells(built_lib, oracle, n):
    from make_golden import classes
    from bs45_quantum_explorer_gb300.cells import cell_list
    removed = 0
    for sig in classes(n):
        kw = dict(m6=True, thm211b=False, thm212=False)
        plain = _cells(cell_list(n, sig, **kw))
        kept = _cells(cell_list(n, sig, endpos=True, **kw))
        assert set(kept) <= set(plain)
        for key in set(plain) - set(kept):
            assert _survivors(oracle, n, plain[key][0]) == 0, (n, sig, key)
            removed += 1
    assert removed > 0


@pytest.mark.parametrize("n", [9, 11, 13])
def test_q_closure_prune_removes_only_empty_cells(built_lib, oracle, n):
    from make_golden import classes
    from bs45_quantum_explorer_gb300.cells import cell_list
    pruned = 0
    for sig in classes(n):
        kw = dict(m6=True, thm211b=True, thm212=True, endpos=True, orbit_canon=True, orbit_q=1)
        canon = _cells(cell_list(n, sig, **kw))
        after = _cells(cell_list(n, sig, qprune=True, **kw))
        assert set(canon) == set(after)  # the prune only clears kept flags
        for key, (cell, k) in canon.items():
            if k and not after[key][1]:
                assert _survivors(oracle, n, cell) == 0, (n, sig, key)
                pruned += 1
    assert pruned > 0  # 2, 14 and 200 kept cells pruned at n = 9, 11, 13
