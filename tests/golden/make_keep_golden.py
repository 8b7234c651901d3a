#!/usr/bin/env python3
"""The per-cell flattest-256 keep of config C3 as the reference drains it: whole cells of the
n = 30, sig (1,7,6,6) ORDER=3 list (Thm 2.11b + 2.12, orbit canon with the quad switch),
each cell's stream buffered whole (BUF_CAP 500,000 holds every survivor), its 256 flattest
completed (DRAIN_TOP 256, budget 2^16), with the reference's WZ_FH_CAND_LOG on: one line per
completed candidate, in drain order, with its drain rank, verdict and charged nodes
(wz_match.cpp:2584-2598, 2656-2705). The node counts differ from candidate to candidate, so
the sequence pins the drained order as well as the completions.

Runs oracle/_ref/wz_match (the reference's wz_match.cpp compiled unmodified by
`make -C oracle ref`), one process per cell, in parallel; about 30 s.

    python tests/golden/make_keep_golden.py  ->  tests/golden/keep_n30_golden.json
"""
import concurrent.futures as cf
import json
import os
import re
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "wz_match")

N, SIG = 30, (1, 7, 6, 6)
BASE = dict(WZ_FIRSTHIT=1, WZ_FH_M6=1, WZ_THM211B=1, WZ_THM212=1, WZ_FH_ORBIT_CANON=1,
            WZ_FH_ORBIT_Q=1, WZ_FH_PROF_ORDER=3, WZ_FH_ORD3_NODIGEST_OK=1, WZ_FH_BUF_CAP=500000,
            WZ_FH_DRAIN_TOP=256, WZ_FH_AB_BUDGET=1 << 16, WZ_FH_CAND_LOG=1, WZ_FH_PROG_SEC=99999)
CELLS = (3005, 3045, 3085, 3093)  # kept cells of cells_n30_golden.json, 1.5e5-1.8e5 survivors


def cand_lines(out):
    """(drain rank, raw cell, verdict, charged nodes) of every CAND line, in order."""
    return [[int(x) for x in m.groups()]
            for m in re.finditer(r"^CAND idx=\d+ ci=(\d+) pi=(\d+) r=(-?\d+) nodes=(\d+)", out, re.M)]


def one(pi):
    import sys
    sys.path.insert(0, HERE)
    from make_lane_golden import semantic
    settings = dict(BASE, WZ_FH_PROF_SKIP=pi, WZ_FH_PROF_END=pi + 1)
    env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
    env.update({k: str(v) for k, v in settings.items()})
    p = subprocess.run([REF_BIN, str(N), *map(str, SIG)], env=env, capture_output=True, text=True)
    return dict(pi=pi, settings=settings, rc=p.returncode, cand=cand_lines(p.stdout),
                semantic=semantic(p.stdout))


def main():
    with cf.ThreadPoolExecutor(max_workers=len(CELLS)) as ex:
        cases = list(ex.map(one, CELLS))
    for c in cases:
        print(c["pi"], "rc", c["rc"], "completions", len(c["cand"]), "distinct node counts",
              len({x[3] for x in c["cand"]}))
    json.dump(dict(n=N, sig=SIG, cases=cases), open(os.path.join(HERE, "keep_n30_golden.json"), "w"))


if __name__ == "__main__":
    main()
