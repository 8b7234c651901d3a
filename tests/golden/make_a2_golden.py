#!/usr/bin/env python3
"""Golden fixtures for the A2 row-reachability prune (WZ_FH_A2=2, src/solver/wz_match.cpp:
977-1047 and 1069-1072), from the reference itself (oracle/_ref, `make -C oracle ref`):

  a2_complete_golden.npz   fh_complete_ab with the cell's allowed rows under A2 = 2 (and the
                           same candidates with A2 off, whose node counts must not be lower):
                           verdict, charged nodes and the first completion, at n = 8..22
  a2_lane_golden.json      full first-hit lane runs of the reference binary with WZ_FH_A2=2
                           over every signature class at n = 6..13 (the lane's semantic
                           lines, as make_lane_golden.py records them)

Modelled on the reference's own identity gate tools/test_a2_rows.py (3): the prune keeps the
verdict of every uncapped candidate and never adds nodes.

    python tests/golden/make_a2_golden.py
"""
import ctypes as C
import json
import os
import random
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import ROOT, abp_rows, classes, enum_cs, load_ref, pack  # noqa: E402
from make_lane_golden import cellsize_lines, run, semantic  # noqa: E402

sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle  # noqa: E402

LANE_SETTINGS = [
    dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=0, WZ_FH_A2=2),
    dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=30, WZ_FH_A2=2, WZ_FH_STREAM_REV=1),
    dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=5, WZ_FH_BUF_CAP=7, WZ_FH_DRAIN_TOP=3, WZ_FH_DRAIN_BATCHES=2,
         WZ_FH_A2=2),
    dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=0, WZ_FH_ORBIT_CANON=1, WZ_FH_ORBIT_Q=1, WZ_FH_PROF_ORDER=3,
         WZ_FH_ORD3_NODIGEST_OK=1, WZ_FH_A2=2),
]


def completions(R):
    R.refh_set_a2.argtypes = [C.c_int, C.c_int]
    rng = random.Random(0xB545A2)
    comp, comp_rows, comp_cd = [], [], []
    for n in (8, 10, 11, 13, 14, 16, 17, 19, 20, 22):
        cl = classes(n)
        for sig in rng.sample(cl, min(3, len(cl))):
            a, b, c, d = sig
            R.refh_setup(n, a, b, c, d, 3)
            cells = [(x, y) for x in enum_cs(n, c, 6) for y in enum_cs(n, d, 6)]
            rng.shuffle(cells)
            done = 0
            for tx, ty in cells:
                rows = abp_rows(n, a, b, tx, ty)
                if not len(rows):
                    continue
                surv, _, _ = pyoracle.cd_stream(n, tx, ty, m=6, cap=200)
                if not len(surv):
                    continue
                roff = sum(len(r) for r in comp_rows)
                comp_rows.append(rows)
                rr = np.ascontiguousarray(rows)
                for cand in surv[:6]:
                    for budget in (0, 40, 700, 20000):
                        out = []
                        for mode in (2, 0):
                            R.refh_set_a2(mode, 6)
                            A = np.zeros(n + 1, np.int32)
                            B = np.zeros(n + 1, np.int32)
                            nodes = C.c_longlong()
                            v = R.refh_complete(cand[0].astype(np.int32), cand[1].astype(np.int32),
                                                budget, 6, rr.ctypes.data_as(C.c_void_p), len(rows),
                                                A, B, C.byref(nodes))
                            out.append((v, nodes.value, A, B))
                        (v2, n2, A2, B2), (v0, n0, _, _) = out
                        comp.append([n, a, b, budget, roff, len(rows), v2, n2, len(comp_cd), v0, n0,
                                     int(pack(A2.astype(np.int8))), int(pack(B2.astype(np.int8)))])
                    comp_cd.append(pack(cand).reshape(2))
                done += 1
                if done >= 2:
                    break
    R.refh_set_a2(0, 6)
    np.savez_compressed(os.path.join(HERE, "a2_complete_golden.npz"),
                        cases=np.array(comp, np.int64).astype(np.uint64),
                        cd=np.array(comp_cd, np.uint64), rows=np.concatenate(comp_rows))
    pruned = sum(1 for x in comp if x[7] < x[10])
    print("A2 completions", len(comp), "with fewer nodes than A2 off:", pruned)


def lanes():
    cases = []
    with tempfile.TemporaryDirectory(prefix="bsfh-a2-") as tmp:
        for n in range(6, 14):
            for sig in classes(n):
                for st in LANE_SETTINGS:
                    rc, out, dh, dl = run(n, sig, st, tmp)
                    cases.append(dict(n=n, sig=list(sig), settings=st, rc=rc, semantic=semantic(out),
                                      cells=cellsize_lines(out), dump_sha256=dh, dump_len=dl))
    json.dump(cases, open(os.path.join(HERE, "a2_lane_golden.json"), "w"))
    print("A2 lane cases", len(cases), "found", sum(1 for c in cases if c["rc"] == 0))


if __name__ == "__main__":
    R = load_ref()
    completions(R)
    lanes()
