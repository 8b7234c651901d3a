#!/usr/bin/env python3
"""Lane golden fixtures at the first-hit workload's size: n = 36, sig (5,11,0,0).

Runs oracle/_ref/wz_match (the reference's src/solver/wz_match.cpp, compiled unmodified by
`make -C oracle ref`) as one production-style lane -- orbit canon with the quad switch and its
Q-closure prune, the orbit-deterministic order checked against the list digest, budget 2^22 --
over windows of raw cells, with the per-cell buffer and drain cut small enough for the CPU
reference to finish in minutes (about seven in all). Records what the drop-in must reproduce: exit code, semantic
stdout lines, CELLSIZE/CDSTAT counts and the WZ_FH_DUMP stream bytes (sha256).

    python tests/golden/make_lane36_golden.py   ->  tests/golden/lane36_golden.json
"""
import json
import os
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_lane_golden import REF_BIN, cellsize_lines, run, semantic  # noqa: E402

N, SIG = 36, (5, 11, 0, 0)
DIGEST = "36d184528757c9e9:715445ba72775867"   # canon + Q + Q-prune, ORDER=3
LANE = dict(WZ_FH_ORBIT_CANON=1, WZ_FH_ORBIT_Q=1, WZ_FH_ORBIT_QPRUNE=1, WZ_FH_PROF_ORDER=3,
            WZ_FH_EXPECT_DIGEST=DIGEST, WZ_FH_AB_BUDGET=1 << 22)
SETTINGS = [
    dict(LANE, WZ_FH_PROF_SKIP=3000, WZ_FH_PROF_END=3400, WZ_FH_BUF_CAP=2000, WZ_FH_DRAIN_TOP=64),
    dict(LANE, WZ_FH_PROF_SKIP=3400, WZ_FH_PROF_END=3800, WZ_FH_BUF_CAP=1000, WZ_FH_DRAIN_TOP=16,
         WZ_FH_DRAIN_BATCHES=2, WZ_FH_STREAM_REV=1),
    dict(LANE, WZ_FH_PROF_SKIP=3800, WZ_FH_PROF_END=4300, WZ_FH_BUF_CAP=300, WZ_FH_DRAIN_TOP=32,
         WZ_FH_OUTER_K=2),
]
# (CELLSIZE measurement runs are left out here: a whole n = 36 cell takes the CPU reference
# longer than ten minutes.)


def main():
    cases = []
    with tempfile.TemporaryDirectory() as tmp:
        for st in SETTINGS:
            t0 = time.time()
            rc, out, dh, dl = run(N, SIG, st, tmp)
            cases.append(dict(n=N, sig=list(SIG), settings=st, rc=rc, semantic=semantic(out),
                              cells=cellsize_lines(out), dump_sha256=dh, dump_len=dl,
                              ref_seconds=round(time.time() - t0, 1)))
            print(st, rc, cases[-1]["ref_seconds"], "s", flush=True)
    with open(os.path.join(HERE, "lane36_golden.json"), "w") as f:
        json.dump(cases, f, indent=0)


if __name__ == "__main__":
    main()
