#!/usr/bin/env python3
"""More lane settings from full first-hit runs of the reference binary at small n: the
WZ_FH_* knobs lane_golden.json leaves at their defaults -- the candidate cap (MAX_CAND), the
unbuffered stream order (CELL_ORDER=0), allowed rows off or capped (AB_PROF, AB_PROF_CAP), the
completer's canon off (NO_CANON), a shard of a skip/end range (SHARD, NSHARD, PROF_SKIP,
PROF_END), the production list settings (canon + Q + Q-prune, ORDER=3), buffered mod-3 cells,
HALL_FAST=0 and a score gate on the unbuffered order -- and an interrupted run resumed with
WZ_FH_RESUME=0 (a fresh start beside the old checkpoint). Same record as lane_golden.json.

Runs oracle/_ref/wz_match (the reference's wz_match.cpp compiled unmodified by
`make -C oracle ref`); about a minute.

    python tests/golden/make_lane_knobs_golden.py  ->  tests/golden/lane_knobs_golden.json
"""
import json
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_golden import classes  # noqa: E402
from make_lane_golden import cellsize_lines, run, semantic  # noqa: E402

SETTINGS = [
    dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=30, WZ_FH_MAX_CAND=40),
    dict(WZ_FH_M6=1, WZ_FH_CELL_ORDER=0, WZ_FH_AB_BUDGET=30),
    dict(WZ_FH_M6=1, WZ_FH_AB_PROF=0, WZ_FH_AB_BUDGET=30),
    dict(WZ_FH_M6=1, WZ_FH_AB_PROF_CAP=5, WZ_FH_AB_BUDGET=30),
    dict(WZ_FH_M6=1, WZ_FH_NO_CANON=1, WZ_FH_AB_BUDGET=30),
    dict(WZ_FH_M6=1, WZ_FH_NSHARD=3, WZ_FH_SHARD=1, WZ_FH_PROF_SKIP=2, WZ_FH_PROF_END=40,
         WZ_FH_AB_BUDGET=30),
    dict(WZ_FH_M6=1, WZ_FH_ORBIT_CANON=1, WZ_FH_ORBIT_Q=1, WZ_FH_ORBIT_QPRUNE=1,
         WZ_FH_PROF_ORDER=3, WZ_FH_ORD3_NODIGEST_OK=1, WZ_FH_AB_BUDGET=30),
    dict(WZ_FH_M6=0, WZ_FH_CELL_ORDER=1, WZ_FH_AB_BUDGET=30),
    dict(WZ_FH_M6=1, WZ_FH_HALL_FAST=0, WZ_FH_AB_BUDGET=0),
    dict(WZ_FH_M6=1, WZ_FH_SCORE_MAX=40, WZ_FH_CELL_ORDER=0, WZ_FH_AB_BUDGET=30),
]


def main():
    cases = []
    with tempfile.TemporaryDirectory(prefix="bsfh-knobs-") as tmp:
        for n in range(8, 14):
            for sig in classes(n):
                for st in SETTINGS:
                    rc, out, dh, dl = run(n, sig, st, tmp)
                    cases.append(dict(n=n, sig=list(sig), settings=st, rc=rc, semantic=semantic(out),
                                      cells=cellsize_lines(out), dump_sha256=dh, dump_len=dl))
        for n in (11, 13):
            for sig in classes(n)[:2]:
                st = dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=50, WZ_FH_TEST_STOP_AFTER=3)
                ck = tempfile.mkdtemp(dir=tmp)
                rc1, out1, _, _ = run(n, sig, st, tmp, ck)
                files = sorted(os.listdir(ck))
                ckpt1 = open(os.path.join(ck, files[0])).read() if files else ""
                st2 = dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=50, WZ_FH_RESUME=0)
                rc2, out2, dh, dl = run(n, sig, st2, tmp, ck)
                ckpt2 = open(os.path.join(ck, files[0])).read() if files else ""
                cases.append(dict(n=n, sig=list(sig), settings=st, settings2=st2, resume=True, rc=rc1,
                                  semantic=semantic(out1), ckpt=ckpt1, rc2=rc2, semantic2=semantic(out2),
                                  ckpt2=ckpt2, dump_sha256=dh, dump_len=dl, cells=[]))
    json.dump(cases, open(os.path.join(HERE, "lane_knobs_golden.json"), "w"))
    print("cases", len(cases), "found", sum(1 for c in cases if c["rc"] == 0),
          "exit codes", sorted({c["rc"] for c in cases}))


if __name__ == "__main__":
    main()
