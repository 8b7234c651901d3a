#!/usr/bin/env python3
"""Cell-list golden fixtures: the reference lane's list stage under WZ_FH_PROF_ORDER=3.

Runs oracle/_ref/wz_match (the reference's own src/solver/wz_match.cpp, compiled unmodified
by `make -C oracle ref`) with WZ_FIRSTHIT=1 WZ_FH_LIST_ONLY=1 and the orbit-deterministic
order, which prints the list digest "<list>:<kept>" (an FNV-1a over every raw cell key in
order, and over every kept flag) and exits. Settings cover mod-3 and mod-6 cells, with and
without 2.11b/2.12, the quad switch Q (proven and forced), its Q-closure prune and ENDPOS.

    python tests/golden/make_list_golden.py   ->  tests/golden/list_golden.json
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "wz_match")
sys.path.insert(0, HERE)
from make_golden import classes  # noqa: E402

ORD3 = dict(WZ_FIRSTHIT=1, WZ_FH_LIST_ONLY=1, WZ_FH_PROF_ORDER=3, WZ_FH_ORBIT_CANON=1)
SETTINGS = [
    dict(WZ_FH_M6=1, WZ_THM211B=1, WZ_THM212=1),
    dict(WZ_FH_M6=1),
    dict(WZ_FH_M6=0, WZ_THM211B=1, WZ_THM212=1),
    dict(WZ_FH_M6=1, WZ_THM211B=1, WZ_THM212=1, WZ_FH_ORBIT_Q=2, WZ_FH_ORBIT_QPRUNE=1),
    dict(WZ_FH_M6=1, WZ_THM211B=1, WZ_THM212=1, WZ_FH_ORBIT_Q=1, WZ_FH_ENDPOS=1,
         WZ_FH_ORBIT_QPRUNE=1, WZ_FH_NSHARD=3),
]
SMALL_N = [12, 13, 17, 20, 23]
# full-size lists of the first-hit workloads (n >= 36 forces 2.11b/2.12 and mod-6 cells)
LARGE = [(36, (5, 11, 0, 0)), (42, (7, 11, 0, 0))]
LARGE_SETTINGS = [dict(WZ_FH_M6=1, WZ_FH_ORBIT_Q=1, WZ_FH_ORBIT_QPRUNE=1)]


def list_lines(out):
    return [l for l in out.splitlines() if l.startswith(("[", "RESULT"))]


def run(bin_path, n, sig, settings, timeout=1200):
    env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
    env.update({k: str(v) for k, v in {**ORD3, **settings}.items()})
    p = subprocess.run([bin_path, str(n), *map(str, sig)], env=env, capture_output=True, text=True,
                       timeout=timeout)
    return p.returncode, list_lines(p.stdout)


def main():
    cases = []
    for n in SMALL_N:
        for sig in classes(n)[:2]:
            for st in SETTINGS:
                rc, lines = run(REF_BIN, n, sig, st)
                cases.append(dict(n=n, sig=list(sig), settings=st, rc=rc, lines=lines, large=False))
    for n, sig in LARGE:
        for st in LARGE_SETTINGS:
            rc, lines = run(REF_BIN, n, sig, st)
            cases.append(dict(n=n, sig=list(sig), settings=st, rc=rc, lines=lines, large=True))
    with open(os.path.join(HERE, "list_golden.json"), "w") as f:
        json.dump(cases, f, indent=0)
    print(len(cases), "cases")


if __name__ == "__main__":
    main()
