"""Every true solution at small n is kept by the lane's cell list (the reference's gate
tools/test_orbit_q_retention.py, which brute-forces every BS(n+1, n) at n = 6, 8, 10 and asks
its LOCATE instrument whether some image of each solution lies in a kept cell).

Here the solutions come from the same brute force, restated (every C,D pair's summed
aperiodic autocorrelation against the negated vectors of every A,B pair), one per
(signed A,B sums, 64-orbit of C,D). For each, with mod-3 and mod-6 cells, 2.11b and 2.12, orbit
canon, and the 32-group, the 64-group (Q, where the reference enables it: c + d = 0 mod 4)
and Q with the closure prune, the list bs_cell_list builds for the solution's own signed
signature must hold the solution's cell, and some cell of its orbit must be kept."""
import itertools

import numpy as np
import pytest


def _all_seqs(L):
    idx = np.arange(1 << L, dtype=np.int64)[:, None]
    return (1 - 2 * ((idx >> np.arange(L)) & 1)).astype(np.int8)


def _acf(X, n):
    L = X.shape[1]
    return np.stack([(X[:, :L - s].astype(np.int32) * X[:, s:]).sum(1) if s < L
                     else np.zeros(len(X), np.int32) for s in range(1, n + 1)], 1).astype(np.int32)


def _solutions(n):
    """[(C, D, {(sum A, sum B), ...})]: every C,D pair (C <= D in enumeration order) with an
    A,B pair whose autocorrelation cancels it at every shift 1..n."""
    S, T = _all_seqs(n), _all_seqs(n + 1)
    aS, aT = _acf(S, n), _acf(T, n)
    ia = np.triu_indices(len(T))
    ab = aT[ia[0]] + aT[ia[1]]
    sums = np.stack([T[ia[0]].sum(1), T[ia[1]].sum(1)], 1).astype(int)
    want = {}
    for k in range(len(ab)):
        want.setdefault(ab[k].tobytes(), set()).add((int(sums[k, 0]), int(sums[k, 1])))
    iu = np.triu_indices(len(S))
    neg = -(aS[iu[0]] + aS[iu[1]])
    out = []
    for k in range(len(neg)):
        hit = want.get(neg[k].tobytes())
        if hit:
            out.append((S[iu[0][k]].astype(int), S[iu[1][k]].astype(int), hit))
    return out


def _canon64(C, D):
    """The smallest form of (C, D) under negations, reversals, the swap and (where it maps
    +-1 sequences to +-1 sequences) the quad switch: one representative per orbit."""
    L = len(C)
    C, D = tuple(int(x) for x in C), tuple(int(x) for x in D)
    forms = {(C, D)}
    qc = tuple((C[i] + D[i] + C[L - 1 - i] - D[L - 1 - i]) // 2 for i in range(L))
    qd = tuple((C[i] + D[i] - C[L - 1 - i] + D[L - 1 - i]) // 2 for i in range(L))
    if all(x in (1, -1) for x in qc + qd):
        forms.add((qc, qd))
    best = None
    for c, d in forms:
        for nc, nd, rc, rd, sw in itertools.product(range(2), repeat=5):
            x = tuple(-v for v in c) if nc else c
            y = tuple(-v for v in d) if nd else d
            x = x[::-1] if rc else x
            y = y[::-1] if rd else y
            k = (y, x) if sw else (x, y)
            best = k if best is None or k < best else best
    return best


@pytest.mark.parametrize("n", [6, 8, 10])
def test_every_solution_orbit_is_kept(built_lib, n):
    from test_retention_cpu import _class_sums, _orbit
    from bs45_quantum_explorer_gb300.cells import cell_list
    reps = {}
    for C, D, abs_ in _solutions(n):
        for a, b in abs_:
            reps.setdefault((a, b, _canon64(C, D)), (C, D, a, b))
    assert reps
    lists = {}
    checked = 0
    for C, D, a, b in reps.values():
        c, d = int(C.sum()), int(D.sum())
        for m6, q in itertools.product((0, 1), (0, 1, 2)):
            key = (a, b, c, d, m6, q)
            if key not in lists:
                cells, kept, _, m = cell_list(n, (a, b, c, d), m6=bool(m6), thm211b=True,
                                              thm212=True, orbit_canon=True, orbit_q=min(q, 1),
                                              qprune=q == 2)
                lists[key] = (m, {(tuple(cells[i].tx[:m]), tuple(cells[i].ty[:m])): int(kept[i])
                                  for i in range(len(kept))})
            m, listed = lists[key]
            own = (_class_sums(C, m), _class_sums(D, m))
            assert own in listed, (n, a, b, c, d, m6, "a true solution's cell is not listed")
            nvar = 64 if q and (c + d) % 4 == 0 else 32
            orbit = _orbit(own[0], own[1], n, m, nvar)
            assert any(listed.get(cell, 0) for cell in orbit), (n, a, b, c, d, m6, q, own)
            checked += 1
    assert checked == 6 * len(reps)
