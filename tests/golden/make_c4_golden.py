#!/usr/bin/env python3
"""First-hit goldens at the production lane settings: n = 36, sig (5,11,0,0), budget 2^22,
BUF_CAP 500,000, DRAIN_TOP 50,000 (the lane defaults of cluster_firsthit_probe.sh), orbit
canon + quad switch + Q-closure prune, ORDER=3 with the list digest.

The window is the head of the first-hit workload's seeded range of 4,096 raw cells
([158570, 162666), 85 kept cells): the raw cells before and including each of its first
eight kept cells, one window per kept cell, so that the reference's eight runs go in
parallel on the host's cores. Each window runs oracle/_ref/wz_match (the reference's
src/solver/wz_match.cpp compiled unmodified by `make -C oracle ref`) as one lane arm and
records what the drop-in must reproduce: exit code, semantic stdout lines (summary counts
including total_AB_nodes, FIRSTHIT on a hit), CDSTAT/CELLSIZE lines and the WZ_FH_DUMP bytes
(sha256). One window takes the reference about half an hour on one core.

    python tests/golden/make_c4_golden.py   ->  tests/golden/c4_golden.json
"""
import concurrent.futures as cf
import json
import os
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_lane_golden import cellsize_lines, run, semantic  # noqa: E402

N, SIG = 36, (5, 11, 0, 0)
DIGEST = "36d184528757c9e9:715445ba72775867"   # canon + Q + Q-prune, ORDER=3
LANE = dict(WZ_FH_ORBIT_CANON=1, WZ_FH_ORBIT_Q=1, WZ_FH_ORBIT_QPRUNE=1, WZ_FH_PROF_ORDER=3,
            WZ_FH_EXPECT_DIGEST=DIGEST, WZ_FH_AB_BUDGET=1 << 22, WZ_FH_BUF_CAP=500000,
            WZ_FH_DRAIN_TOP=50000)
START = 158570
# the first eight kept raw cells of [158570, 162666) in the ORDER=3 list above
KEPT = [158597, 158629, 158693, 158757, 158789, 158821, 158885, 158949]


def windows():
    lo = START
    for pi in KEPT:
        yield dict(LANE, WZ_FH_PROF_SKIP=lo, WZ_FH_PROF_END=pi + 1)
        lo = pi + 1


def one(st):
    with tempfile.TemporaryDirectory(prefix="bsfh-c4-") as tmp:
        t0 = time.time()
        rc, out, dh, dl = run(N, SIG, st, tmp, timeout=None)
        return dict(n=N, sig=list(SIG), settings=st, rc=rc, semantic=semantic(out),
                    cells=cellsize_lines(out), dump_sha256=dh, dump_len=dl,
                    ref_seconds=round(time.time() - t0, 1))


def main():
    sts = list(windows())
    with cf.ThreadPoolExecutor(max_workers=len(sts)) as ex:
        cases = list(ex.map(one, sts))
    for c in cases:
        print(c["settings"]["WZ_FH_PROF_SKIP"], c["rc"], c["ref_seconds"], "s", flush=True)
    with open(os.path.join(HERE, "c4_golden.json"), "w") as f:
        json.dump(cases, f, indent=0)


if __name__ == "__main__":
    main()
