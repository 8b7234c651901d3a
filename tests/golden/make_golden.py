#!/usr/bin/env python3
"""Generates the golden fixtures in this folder from the reference itself.

Run on a machine that holds the reference sources (DanielGord0n/BS45_Quantum_Explorer at
REF, given on the command line) after `make -C oracle ref REF=...`, which compiles the reference's own
src/solver/wz_match.cpp, unmodified, with its production flags into oracle/_ref/ (the binary,
and a harness library that exposes hall_ok_pair_fast, count_pairs22, fh_complete_ab, npaf_at
and autocorr_key). Every expected value below is computed by that reference code, except the
BS(7,6) full set, which is a numpy brute force over all 2^26 (A,B) x ... pairs as the
reference's own test_orbit_q_retention.py does it (join of pair autocorrelations).

    python tests/golden/make_golden.py REF             # everything below but the two that follow
    python tests/golden/make_golden.py REF ab          # ab_streams_golden.npz
    python tests/golden/make_golden.py REF cdprune     # cd_prune_golden.npz

Outputs (small, committed): known_quads.json, hall_golden.npz, streams_golden.npz,
complete_golden.npz, controls_golden.json, bs7_6_all.npz, ab_streams_golden.npz,
cd_prune_golden.npz.
"""
import ctypes as C
import functools
import itertools
import json
import os
import random
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = None  # the reference repository's root, from the command line (main)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def load_ref():
    R = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref.so"))
    R.refh_setup.argtypes = [C.c_int] * 6
    R.refh_hall_fast.argtypes = [ip, ip, C.c_int]
    R.refh_hall_conj.argtypes = [ip, ip, C.c_int]
    R.refh_npaf.argtypes = [ip, ip, C.c_int, ip, ip, C.c_int, C.c_int]
    R.refh_autocorr_key.argtypes = [ip, ip, C.c_int, C.c_int]
    R.refh_autocorr_key.restype = C.c_ulonglong
    R.refh_stream.argtypes = [C.c_int, ip, ip] + [C.c_int] * 7 + [ip, C.c_longlong] + \
        [C.POINTER(C.c_longlong)] * 3
    R.refh_stream.restype = C.c_longlong
    R.refh_complete.argtypes = [ip, ip, C.c_longlong, C.c_int, C.c_void_p, C.c_int, ip, ip,
                                C.POINTER(C.c_longlong)]
    return R


def classes(n):
    out = []
    for a, b, c, d in itertools.product(range(n + 2), range(n + 2), range(n + 1), range(n + 1)):
        if a > b or c > d:
            continue
        if (a - (n + 1)) % 2 or (b - (n + 1)) % 2 or (c - n) % 2 or (d - n) % 2:
            continue
        if a * a + b * b + c * c + d * d == 4 * n + 2:
            out.append((a, b, c, d))
    return out


def enum_cs(L, target, m):
    cnt = [len(range(c, L, m)) for c in range(m)]
    out = []

    def rec(c, acc, cur):
        if c == m - 1:
            last = target - acc
            if last < -cnt[c] or last > cnt[c] or (last + cnt[c]) & 1:
                return
            out.append(cur + [last])
            return
        for v in range(-cnt[c], cnt[c] + 1, 2):
            rec(c + 1, acc + v, cur + [v])
    rec(0, 0, [])
    return out


def norm(v):
    return sum(x * x for x in v)


def acv(v, s):
    m = len(v)
    return 0 if s >= m else sum(v[i] * v[i + s] for i in range(m - s))


def thm212(x, y, m, n, ab):
    m4 = lambda v: ((v % 4) + 4) % 4  # noqa: E731
    if ab:
        c1 = n % m
        want = 2 if n % m else 0
        if m4(x[0] + y[0] + x[c1] + y[c1]) != want:
            return False
        for j in range(2, m + 1):
            if j == c1 + 1:
                continue
            c = ((n + 1 - j) % m + m) % m
            if m4(x[j - 1] + y[j - 1] + x[c] + y[c]) != 0:
                return False
    else:
        for j in range(1, m + 1):
            c = ((n - j) % m + m) % m
            if m4(x[j - 1] + y[j - 1] + x[c] + y[c]) != 0:
                return False
    return True


def abp_rows(n, a, b, px, py, m=6):
    """The cell's allowed A,B rows as the reference's abpMap builds them
    (wz_match.cpp:2318-2371): both signed targets, norm, 2.11b tuple, then eq 2.12."""
    need = 4 * n + 2 - norm(px) - norm(py)
    half = m // 2
    T = [-(acv(px, s) + acv(py, s) + acv(px, m - s) + acv(py, m - s)) for s in range(1, half + 1)]
    # the pairs (kv, rv) with kn + rn == need and kc + rc == T, in the reference's nested
    # order: rv looked up by (rn, rc) among b's tuples, which keep their enumeration order
    by_key = _tuples_by_key(n, b, m)
    rows = []
    for kv, kn, kc in _tuples(n, a, m):
        want = (need - kn, tuple(T[s] - kc[s] for s in range(half)))
        for rv in by_key.get(want, ()):
            if not thm212(kv, rv, m, n, True):
                continue
            rows.append(list(kv) + [0] * (8 - m) + list(rv) + [0] * (8 - m))
    return np.array(rows, np.int8).reshape(-1, 16)


@functools.lru_cache(maxsize=None)
def _tuples(n, sig, m):
    """(v, norm, the half-period combined autocorrelations) of every class tuple of length
    n+1 and class sum +sig or -sig, in enumeration order (wz_match.cpp:2318-2340)."""
    half = m // 2
    out = []
    for sgn in ([1, -1] if sig else [1]):
        for v in enum_cs(n + 1, sgn * sig, m):
            if norm(v) > 4 * n + 2:
                continue
            out.append((tuple(v), norm(v), [acv(v, s) + acv(v, m - s) for s in range(1, half + 1)]))
    return out


@functools.lru_cache(maxsize=None)
def _tuples_by_key(n, sig, m):
    by = {}
    for v, vn, vc in _tuples(n, sig, m):
        by.setdefault((vn, tuple(vc)), []).append(v)
    return by


def pack(seqs):
    seqs = np.asarray(seqs)
    L = seqs.shape[-1]
    return ((seqs == 1).astype(np.uint64) * (np.uint64(1) << np.arange(L, dtype=np.uint64))).sum(-1, dtype=np.uint64)


def parse_quad(path):
    vals = []
    for line in open(path):
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        vals.append([int(x) for x in line.split()])
    n = vals[0][0]
    sig = vals[1]
    A, B, Cc, D = vals[2], vals[3], vals[4], vals[5]
    assert len(A) == n + 1 and len(Cc) == n, path
    return {"file": os.path.relpath(path, REF), "n": n, "sig": sig, "A": A, "B": B, "C": Cc, "D": D}


def ab_streams(R):
    """A,B-side streams (count_pairs22 with abSide = true, length n+1)."""
    rng = random.Random(0xB546)
    cases, surv = [], []
    for n in (6, 8, 9, 11, 12, 14, 15, 17):
        for sig in rng.sample(classes(n), min(2, len(classes(n)))):
            a, b, c, d = sig
            R.refh_setup(n, a, b, c, d, 3)
            L = n + 1
            for m in (3, 6):
                cells = [(x, y) for x in enum_cs(L, a, m) for y in enum_cs(L, b, m)]
                rng.shuffle(cells)
                for (tx, ty) in cells[:3]:
                    rev, pin = rng.choice([(0, 0), (1, 1), (1, 0)])
                    pinX, pinY = int(pin and a == 0), int(pin and b == 0)
                    cap = 1 << 20
                    out = np.zeros(cap * 2 * L, np.int32)
                    nd, lv, ok = C.c_longlong(), C.c_longlong(), C.c_longlong()
                    w = R.refh_stream(L, np.array(tx, np.int32), np.array(ty, np.int32), m, pinX, pinY, rev,
                                      0, 0, 1, out, cap, C.byref(nd), C.byref(lv), C.byref(ok))
                    off = sum(len(s) for s in surv)
                    cases.append([n, a, b, c, d, m, rev, pinX, pinY, nd.value, lv.value, ok.value, off, w] +
                                 list(tx) + [0] * (6 - m) + list(ty) + [0] * (6 - m))
                    surv.append(pack(out[:w * 2 * L].reshape(w, 2, L)).reshape(-1, 2))
    np.savez_compressed(os.path.join(HERE, "ab_streams_golden.npz"), cases=np.array(cases, np.int64),
                        words=np.concatenate(surv) if surv else np.zeros((0, 2), np.uint64))
    print("A,B streams", len(cases), sum(len(s) for s in surv))


def cd_prune_streams(R):
    """C,D streams under WZ_FH_CD_PRUNE 1, 2 and 3 (count_pairs22 with G_CD_PRUNE set): even n,
    m = 6 cells, where the prunes apply, and m = 3 cells, where they do not. Same row layout as
    streams_golden.npz."""
    rng = random.Random(0xCDB)
    cases, surv = [], []
    for n in (8, 10, 12, 14, 16, 18, 20):
        cl = classes(n)
        for sig in rng.sample(cl, min(2, len(cl))):
            a, b, c, d = sig
            R.refh_setup(n, a, b, c, d, 3)
            for m in (6, 3):
                cells = [(x, y) for x in enum_cs(n, c, m) for y in enum_cs(n, d, m)]
                # small class sums first: the cells with the largest streams
                cells.sort(key=lambda t: sum(map(abs, t[0])) + sum(map(abs, t[1])))
                pick = cells[:40]
                rng.shuffle(pick)
                for (tx, ty) in pick[:2]:
                    rev, endpos, pin = rng.choice([(0, 0, 0), (1, 0, 1), (0, 1, 0), (1, 1, 1)])
                    pinX, pinY = int(pin and c == 0), int(pin and d == 0)
                    for cdp in (1, 2, 3):
                        cap = 1 << 20
                        out = np.zeros(cap * 2 * n, np.int32)
                        nd, lv, ok = C.c_longlong(), C.c_longlong(), C.c_longlong()
                        w = R.refh_stream(n, np.array(tx, np.int32), np.array(ty, np.int32), m, pinX,
                                          pinY, rev, endpos, cdp, 1, out, cap, C.byref(nd), C.byref(lv),
                                          C.byref(ok))
                        off = sum(len(t) for t in surv)
                        cases.append([n, a, b, c, d, m, rev, endpos, pinX, pinY, cdp, nd.value, lv.value,
                                      ok.value, off, w] + list(tx) + [0] * (6 - m) + list(ty) + [0] * (6 - m))
                        surv.append(pack(out[:w * 2 * n].reshape(w, 2, n)).reshape(-1, 2))
    np.savez_compressed(os.path.join(HERE, "cd_prune_golden.npz"), cases=np.array(cases, np.int64),
                        words=np.concatenate(surv) if surv else np.zeros((0, 2), np.uint64))
    print("CD_PRUNE streams", len(cases), sum(len(t) for t in surv))


def main():
    global REF
    if len(sys.argv) < 2:
        sys.exit("usage: make_golden.py REF [ab|cdprune]   (REF: root of the reference repository)")
    REF = sys.argv[1]
    R = load_ref()
    if len(sys.argv) > 2 and sys.argv[2] == "ab":
        ab_streams(R)
        return
    if len(sys.argv) > 2 and sys.argv[2] == "cdprune":
        cd_prune_streams(R)
        return
    rng = random.Random(0xB545)

    # ---- known-answer quads: banked champions and the published WZ controls ----
    quads = []
    for sub in ("results/champions", "results/reference"):
        d = os.path.join(REF, sub)
        for f in sorted(os.listdir(d)):
            if f.endswith(".txt"):
                try:
                    quads.append(parse_quad(os.path.join(d, f)))
                except Exception:
                    pass
    for q in quads:
        n = q["n"]
        A, B, Cc, D = (np.array(q[k], np.int32) for k in "ABCD")
        R.refh_setup(n, *[abs(x) for x in q["sig"]], 3)
        q["npaf_max"] = max(abs(R.refh_npaf(A, B, n + 1, Cc, D, n, s)) for s in range(1, n + 2))
        q["hall_cd"] = R.refh_hall_fast(Cc, D, n)
    json.dump(quads, open(os.path.join(HERE, "known_quads.json"), "w"))
    print("known quads", len(quads), "all NPAF 0:", all(q["npaf_max"] == 0 for q in quads))

    # ---- completer controls: the six known C,D (and the other banked ones) ----
    six = ["results/champions/champion_firsthit_bs42_41.txt", "results/champions/champion_firsthit_bs43_42.txt",
           "results/champions/champion_firsthit_bs44_43.txt", "results/reference/wz_table1_bs42_41.txt",
           "results/reference/wz_table1_bs43_42.txt", "results/reference/wz_table1_bs44_43.txt"]
    controls = []
    for q in quads:
        n = q["n"]
        sig = [abs(x) for x in q["sig"]]
        Cc, D = np.array(q["C"], np.int32), np.array(q["D"], np.int32)
        for budget in (0, 200000, 1 << 22):
            if budget == 0 and q["file"] not in six:
                continue
            R.refh_setup(n, *sig, 3)
            A = np.zeros(n + 1, np.int32)
            B = np.zeros(n + 1, np.int32)
            nodes = C.c_longlong()
            v = R.refh_complete(Cc, D, budget, 6, None, 0, A, B, C.byref(nodes))
            controls.append({"file": q["file"], "n": n, "sig": sig, "budget": budget, "verdict": v,
                             "nodes": nodes.value, "A": A.tolist() if v == 0 else None,
                             "B": B.tolist() if v == 0 else None})
    json.dump(controls, open(os.path.join(HERE, "controls_golden.json"), "w"))
    print("controls", len(controls))

    # ---- Hall decisions (the reference's hall_ok_pair_fast, production build) ----
    import pyoracle
    n = 42
    words = pyoracle.gen_hall_pairs(n, 1 << 14, nthreads=8)
    R.refh_setup(42, 7, 11, 0, 0, 3)
    from bs45_quantum_explorer_gb300.workloads import unpack_pairs
    X = unpack_pairs(words, n).astype(np.int32)
    dec = np.array([R.refh_hall_fast(np.ascontiguousarray(X[i, 0]), np.ascontiguousarray(X[i, 1]), n)
                    for i in range(len(X))], np.uint8)
    # near-threshold pairs: max pair PSD within 1 of the limit
    big = pyoracle.gen_hall_pairs(n, 1 << 19, seed=0xB545C7, nthreads=8)
    ct, st = pyoracle.hall_tables(n)
    Xb = unpack_pairs(big, n).astype(np.float64)
    f = ((Xb @ ct[1:, :n].T) ** 2 + (Xb @ st[1:, :n].T) ** 2).sum(axis=1).max(axis=1)
    near = big[np.abs(f - (4 * n + 2.5)) < 1.0][:2000]
    Xn = unpack_pairs(near, n).astype(np.int32)
    dec_near = np.array([R.refh_hall_fast(np.ascontiguousarray(Xn[i, 0]), np.ascontiguousarray(Xn[i, 1]), n)
                         for i in range(len(Xn))], np.uint8)
    np.savez_compressed(os.path.join(HERE, "hall_golden.npz"), n=n, words=words, decisions=dec,
                        near_words=near, near_decisions=dec_near)
    print("hall", dec.mean(), len(near), dec_near.mean())

    # ---- C,D streams (count_pairs22 with the real sink) ----
    cases = []
    surv = []
    for n in (6, 7, 9, 10, 12, 13, 15, 16, 18, 19):
        cl = classes(n)
        for sig in rng.sample(cl, min(2, len(cl))):
            a, b, c, d = sig
            R.refh_setup(n, a, b, c, d, 3)
            for m in (3, 6):
                cells = [(x, y) for x in enum_cs(n, c, m) for y in enum_cs(n, d, m)]
                rng.shuffle(cells)
                for (tx, ty) in cells[:3]:
                    rev, endpos, pin, cdp = rng.choice([(0, 0, 0, 0), (1, 0, 1, 0), (0, 1, 0, 3), (1, 1, 1, 3)])
                    pinX, pinY = int(pin and c == 0), int(pin and d == 0)
                    cap = 1 << 20
                    out = np.zeros(cap * 2 * n, np.int32)
                    nd, lv, ok = C.c_longlong(), C.c_longlong(), C.c_longlong()
                    w = R.refh_stream(n, np.array(tx, np.int32), np.array(ty, np.int32), m, pinX, pinY,
                                      rev, endpos, cdp, 1, out, cap, C.byref(nd), C.byref(lv), C.byref(ok))
                    rows = out[:w * 2 * n].reshape(w, 2, n)
                    cases.append([n, a, b, c, d, m, rev, endpos, pinX, pinY, cdp, nd.value, lv.value,
                                  ok.value, len(surv) and sum(len(s) for s in surv), w] + list(tx) + [0] * (6 - m) +
                                 list(ty) + [0] * (6 - m))
                    surv.append(pack(rows).reshape(-1, 2))
    offs = np.cumsum([0] + [len(s) for s in surv])
    for i, cse in enumerate(cases):
        cse[14] = int(offs[i])
    np.savez_compressed(os.path.join(HERE, "streams_golden.npz"), cases=np.array(cases, np.int64),
                        words=np.concatenate(surv) if surv else np.zeros((0, 2), np.uint64))
    print("streams", len(cases), offs[-1])

    # ---- completions with and without the cell's allowed rows ----
    comp = []
    comp_rows = []
    comp_cd = []
    for n in (8, 10, 11, 13, 14, 16, 17, 19, 20, 22):
        cl = classes(n)
        for sig in rng.sample(cl, min(3, len(cl))):
            a, b, c, d = sig
            R.refh_setup(n, a, b, c, d, 3)
            cells = [(x, y) for x in enum_cs(n, c, 6) for y in enum_cs(n, d, 6)]
            rng.shuffle(cells)
            done = 0
            for tx, ty in cells:
                rows_s, _, _ = pyoracle.cd_stream(n, tx, ty, m=6, cap=200)
                if not len(rows_s):
                    continue
                rows = abp_rows(n, a, b, tx, ty)
                for cand in rows_s[:4]:
                    for budget in (0, 40, 700):
                        for use_rows in (0, 1):
                            if use_rows and not len(rows):
                                continue
                            A = np.zeros(n + 1, np.int32)
                            B = np.zeros(n + 1, np.int32)
                            nodes = C.c_longlong()
                            rr = np.ascontiguousarray(rows) if use_rows else None
                            v = R.refh_complete(cand[0].astype(np.int32), cand[1].astype(np.int32), budget, 6,
                                                rr.ctypes.data_as(C.c_void_p) if use_rows else None,
                                                len(rows) if use_rows else 0, A, B, C.byref(nodes))
                            roff = sum(len(r) for r in comp_rows)
                            comp.append([n, a, b, budget, use_rows, roff if use_rows else 0,
                                         len(rows) if use_rows else 0, v, nodes.value, len(comp_cd)] +
                                        [int(x) for x in pack(A.astype(np.int8)).reshape(1)] +
                                        [int(x) for x in pack(B.astype(np.int8)).reshape(1)])
                            if use_rows:
                                comp_rows.append(rows)
                    comp_cd.append(pack(cand).reshape(2))
                done += 1
                if done >= 2:
                    break
    np.savez_compressed(os.path.join(HERE, "complete_golden.npz"),
                        cases=np.array(comp, np.uint64), cd=np.array(comp_cd, np.uint64),
                        rows=np.concatenate(comp_rows) if comp_rows else np.zeros((0, 16), np.int8))
    print("completions", len(comp))

    # ---- BS(7,6): every ordered quad by brute force (join of pair autocorrelations) ----
    n = 6
    def pair_auto(L):
        seqs = np.array(list(itertools.product((-1, 1), repeat=L)), np.int64)
        ac = np.stack([(seqs[:, :L - s] * seqs[:, s:]).sum(1) for s in range(1, n + 1)] if L > n else
                      [(seqs[:, :L - s] * seqs[:, s:]).sum(1) if s < L else np.zeros(len(seqs), np.int64)
                       for s in range(1, n + 1)], 1)
        return seqs, ac
    sab, aab = pair_auto(n + 1)
    scd, acd = pair_auto(n)
    from collections import defaultdict
    cd_by = defaultdict(list)
    for i in range(len(scd)):
        for j in range(len(scd)):
            cd_by[tuple(-(acd[i] + acd[j]))].append((i, j))
    found = []
    for i in range(len(sab)):
        for j in range(len(sab)):
            key = tuple(aab[i] + aab[j])
            for (k, l) in cd_by.get(key, ()):
                found.append((i, j, k, l))
    quads76 = np.array([[pack(sab[i].astype(np.int8)), pack(sab[j].astype(np.int8)),
                         pack(scd[k].astype(np.int8)), pack(scd[l].astype(np.int8))] for i, j, k, l in found],
                       np.uint64)
    np.savez_compressed(os.path.join(HERE, "bs7_6_all.npz"), quads=quads76)
    print("BS(7,6) quads", len(quads76))
    ab_streams(R)


if __name__ == "__main__":
    main()
