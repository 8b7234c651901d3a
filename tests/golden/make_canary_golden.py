#!/usr/bin/env python3
"""The reference's archived n = 29 first-hit canary, as the reference runs it today.

The reference keeps one larger end-to-end check beside its n <= 13 identity gates: the
command `WZ_FIRSTHIT=1 WZ_FH_M6=1 OMP_NUM_THREADS=1 wz_match 29 0 6 9 1` (orbit canon off,
order 0, budget 200,000, every other setting at its default) must re-find the same quad
(tools/test_firsthit_telemetry.py:176-181, archived fingerprint idx=26694 profile_rank=588
nodes_this_cand=81320, recorded before the outer-lag tables and the early check became the
completer's defaults; HANDOFF.md:910-913).

This script runs oracle/_ref/wz_match (the reference's wz_match.cpp compiled unmodified by
`make -C oracle ref`) twice, in parallel, with WZ_FH_CAND_LOG=1 (one line per completed
candidate, wz_match.cpp:2584-2598):
  * the whole archived command: its semantic lines (FIRSTHIT, the summary counts, the quad),
    and per raw cell the completions, their verdict histogram and charged nodes, plus the
    hit cell's CAND lines in drain order;
  * the hit cell alone (WZ_FH_PROF_SKIP=588, PROF_END=589) with WZ_FH_OUTER_K=0 and
    WZ_FH_EARLY_CHECK=0, the completer as it was when the fingerprint was archived: its CAND
    lines and FIRSTHIT line (nodes_this_cand = 81,320 pins that older node count too).
About two minutes on one core each.

    python tests/golden/make_canary_golden.py  ->  tests/golden/canary_n29_golden.json
"""
import concurrent.futures as cf
import json
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "wz_match")
sys.path.insert(0, HERE)
from make_lane_golden import semantic  # noqa: E402

N, SIG = 29, (0, 6, 9, 1)
BASE = dict(WZ_FIRSTHIT=1, WZ_FH_M6=1, OMP_NUM_THREADS=1, WZ_FH_CAND_LOG=1, WZ_FH_PROG_SEC=99999)
RUNS = {
    "archived": dict(BASE),
    "hit_cell_outer0": dict(BASE, WZ_FH_PROF_SKIP=588, WZ_FH_PROF_END=589, WZ_FH_OUTER_K=0,
                            WZ_FH_EARLY_CHECK=0),
}


def cand_lines(out):
    """(drain rank, raw cell, verdict, charged nodes) of every CAND line, in order."""
    return [[int(x) for x in m.groups()]
            for m in re.finditer(r"^CAND idx=\d+ ci=(\d+) pi=(\d+) r=(-?\d+) nodes=(\d+)", out, re.M)]


def record(binary, name, cwd, timeout=None):
    """One of RUNS through `binary` (the reference's wz_match, or a drop-in with its argv,
    environment and stdout): the fields the golden holds."""
    settings = RUNS[name]
    env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
    env.update({k: str(v) for k, v in settings.items()})
    p = subprocess.run([binary, str(N), *map(str, SIG)], env=env, capture_output=True, text=True,
                       cwd=cwd, timeout=timeout)
    cand = cand_lines(p.stdout)
    hit = re.search(r"^FIRSTHIT: idx=(\d+) profile_rank=(\d+) nodes_this_cand=(\d+)", p.stdout, re.M)
    hit_pi = int(hit.group(2)) if hit else -1
    cells = {}
    for _, pi, r, nodes in cand:
        c = cells.setdefault(pi, dict(pi=pi, completions=0, nodes=0, verdicts=[0] * 5))
        c["completions"] += 1
        c["nodes"] += nodes
        c["verdicts"][r] += 1
    return dict(settings=settings, rc=p.returncode, semantic=semantic(p.stdout),
                cells=[cells[k] for k in sorted(cells)], hit_cell=[x for x in cand if x[1] == hit_pi])


def main():
    cwd = os.path.join(ROOT, "oracle", "_ref")
    with cf.ThreadPoolExecutor(max_workers=len(RUNS)) as ex:
        runs = dict(zip(RUNS, ex.map(lambda name: record(REF_BIN, name, cwd), RUNS)))
    for name, r in runs.items():
        print(name, "rc", r["rc"], "cells completed", len(r["cells"]), "hit-cell completions",
              len(r["hit_cell"]), [s for s in r["semantic"] if s.startswith("FIRSTHIT")])
    json.dump(dict(n=N, sig=SIG, runs=runs),
              open(os.path.join(HERE, "canary_n29_golden.json"), "w"))


if __name__ == "__main__":
    main()
