"""Every known solution survives the lane's cell list (the reference's soundness gate
tools/test_endpos_q.py (3), which LOCATEs banked odd-n solutions in the production ORDER=3
list under ENDPOS + Q + Q-prune and requires retained=YES).

For each of the 43 banked and published quads (tests/golden/known_quads.json, from the
reference's results/champions and results/reference), the cell of its C,D (class sums mod 6)
is looked up in the list bs_cell_list builds for its class with the production settings:
mod-6 cells, Thm 2.11b and 2.12, orbit canon with the quad switch Q where it is proven safe,
the Q-closure prune and ORDER=3, with WZ_FH_ENDPOS at odd n as the reference's n = 45 lanes
run. Retained means that some cell of the solution's orbit (under the 32- or 64-element group
the reference's canonicalisation uses, wz_match.cpp:1714-1730) is in the list and kept.
At odd n the solution's endpoint quad is positive, as ENDPOS requires."""
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def _class_sums(x, m):
    return tuple(int(sum(x[i] for i in range(c, len(x), m))) for c in range(m))


def _rev(p, n, m):
    """Class sums of the reversed sequence: position i goes to n-1-i, so class c goes to class
    (n-1-c) mod m."""
    return tuple(p[(n - 1 - c) % m] for c in range(m))


def _quad_switch(px, py, n, m):
    """The quad switch on class sums: with U = (C+D)/2 and V = (C-D)/2 it maps (C, D) to
    (U + rev V, U - rev V); on class sums the halves are always whole numbers."""
    rx, ry = _rev(px, n, m), _rev(py, n, m)
    two_x = [px[c] + py[c] + rx[c] - ry[c] for c in range(m)]
    two_y = [px[c] + py[c] - rx[c] + ry[c] for c in range(m)]
    assert all(v % 2 == 0 for v in two_x + two_y)
    return tuple(v // 2 for v in two_x), tuple(v // 2 for v in two_y)


def _orbit(px0, py0, n, m, nvar):
    """The orbit of a cell under the lane's symmetry group: negating either side, reversing
    either side, swapping the sides, and (nvar = 64) the quad switch. Built as the closure
    under those generators; it equals the set of 32 or 64 variants the reference's
    canonicalisation ranges over (wz_match.cpp:1714-1730)."""
    start = (tuple(px0), tuple(py0))
    seen, todo = {start}, [start]
    while todo:
        x, y = todo.pop()
        images = [(tuple(-v for v in x), y), (x, tuple(-v for v in y)),
                  (_rev(x, n, m), y), (x, _rev(y, n, m)), (y, x)]
        if nvar == 64:
            images.append(_quad_switch(x, y, n, m))
        for im in images:
            if im not in seen:
                seen.add(im)
                todo.append(im)
    return seen


def test_known_solutions_are_retained_by_the_lane_list(built_lib):
    from bs45_quantum_explorer_gb300.cells import cell_list
    quads = json.load(open(os.path.join(HERE, "golden", "known_quads.json")))
    assert len(quads) == 43
    lists = {}
    retained = 0
    for q in quads:
        n, C, D = q["n"], q["C"], q["D"]
        a, b = sorted(abs(sum(x)) for x in (q["A"], q["B"]))
        c, d = sorted(abs(sum(x)) for x in (C, D))
        assert a * a + b * b + c * c + d * d == 4 * n + 2
        endpos = n % 2 == 1
        if endpos:  # ENDPOS keeps only C,D whose endpoint quad is positive
            assert C[0] * D[0] * C[-1] * D[-1] == 1, q["file"]
        key = (n, a, b, c, d)
        if key not in lists:
            cells, kept, digest, m = cell_list(n, (a, b, c, d), m6=True, thm211b=True, thm212=True,
                                               endpos=endpos, orbit_canon=True, orbit_q=1,
                                               qprune=True, prof_order=3)
            assert m == 6 and digest
            lists[key] = {(tuple(cells[i].tx[:6]), tuple(cells[i].ty[:6])): int(kept[i])
                          for i in range(len(kept))}
        listed = lists[key]
        q_on = endpos or (c + d) % 4 == 0  # where the reference's WZ_FH_ORBIT_Q=1 is active
        orbit = _orbit(_class_sums(C, 6), _class_sums(D, 6), n, 6, 64 if q_on else 32)
        members = [cell for cell in orbit if cell in listed]
        assert members, (q["file"], "no cell of the solution's orbit is listed")
        assert any(listed[cell] for cell in members), (q["file"], "the solution's orbit is not kept")
        retained += 1
    assert retained == 43
