"""Every true solution at small n is kept by the lane's cell list (the reference's gate
tools/test_orbit_q_retention.py, which brute-forces every BS(n+1, n) at n = 6, 8, 10 and asks
its LOCATE instrument whether some image of each solution lies in a kept cell).

Here every solution comes from a brute force of our own: every unordered C,D pair whose
summed aperiodic autocorrelation (packed exactly into one integer) is the negation of some
unordered A,B pair's. For each, with mod-3 and mod-6 cells, 2.11b and 2.12, orbit
canon, and the 32-group, the 64-group (Q, where the reference enables it: c + d = 0 mod 4)
and Q with the closure prune, the list bs_cell_list builds for the solution's own signed
signature must hold the solution's cell, and some cell of its orbit must be kept."""
import itertools

import numpy as np
import pytest


def _seqs(L):
    """Every +-1 sequence of length L, one per row."""
    return np.array(list(itertools.product((1, -1), repeat=L)), dtype=np.int8)


def _keys(X, Y, n, negate=False):
    """For every pair (X[i], Y[i]), its summed aperiodic autocorrelation at shifts 1..n (values
    within +-2(n+1)) packed exactly into one int64, negated first when asked."""
    base, off = 4 * n + 9, 2 * n + 4
    key = np.zeros(len(X), np.int64)
    for s in range(n, 0, -1):
        v = np.zeros(len(X), np.int64)
        for Z in (X, Y):
            if s < Z.shape[1]:
                v += np.einsum("ij,ij->i", Z[:, :-s].astype(np.int64), Z[:, s:].astype(np.int64))
        key = key * base + ((-v if negate else v) + off)
    return key


def _solutions(n):
    """[(C, D, sum A, sum B)] over every base sequence quad of BS(n+1, n): each unordered C,D
    pair whose summed autocorrelation is cancelled by some unordered A,B pair, with the signed
    sums of every such A,B."""
    S, T = _seqs(n), _seqs(n + 1)
    i, j = np.triu_indices(len(T))
    ab = _keys(T[i], T[j], n)
    p, q = np.triu_indices(len(S))
    cd = _keys(S[p], S[q], n, negate=True)
    hit = np.isin(cd, ab)
    wanted = np.isin(ab, cd[hit])
    sums = {}
    for k, a, b in zip(ab[wanted], T[i[wanted]].sum(1), T[j[wanted]].sum(1)):
        sums.setdefault(int(k), set()).add((int(a), int(b)))
    out = []
    for k in np.flatnonzero(hit):
        C, D = S[p[k]].astype(int), S[q[k]].astype(int)
        for a, b in sorted(sums[int(cd[k])]):
            out.append((C, D, a, b))
    return out


@pytest.mark.parametrize("n", [6, 8, 10])
def test_every_solution_orbit_is_kept(built_lib, n):
    from test_retention_cpu import _class_sums, _orbit
    from bs45_quantum_explorer_gb300.cells import cell_list
    sols = _solutions(n)
    assert sols
    lists, orbits = {}, {}
    checked = 0
    for C, D, a, b in sols:
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
            if (own, m, nvar) not in orbits:
                orbits[own, m, nvar] = _orbit(own[0], own[1], n, m, nvar)
            orbit = orbits[own, m, nvar]
            assert any(listed.get(cell, 0) for cell in orbit), (n, a, b, c, d, m6, q, own)
            checked += 1
    assert checked == 6 * len(sols)
