#!/usr/bin/env python3
"""Whole-cell stream counts of the reference at full size (config C3: n = 30, signature
(1,7,6,6), Thm 2.11b + 2.12, orbit canon with the quad switch, ORDER=3).

Runs oracle/_ref/wz_match (the reference's own source, built by `make -C oracle ref`) in
WZ_FH_CELLSIZE mode over the raw cells [3000, 3100) and records, per kept cell, the cell's
class sums, candidate count, leaf count, Hall-pass count and DFS node count, plus the
WZ_FH_DUMP stream bytes' sha256 per cell. About 7 minutes on one core.

    python tests/golden/make_cell_golden.py  ->  tests/golden/cells_n30_golden.json
"""
import hashlib
import json
import os
import re
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "wz_match")

N, SIG = 30, (1, 7, 6, 6)
ENV = dict(WZ_FIRSTHIT=1, WZ_FH_M6=1, WZ_THM211B=1, WZ_THM212=1, WZ_FH_ORBIT_CANON=1, WZ_FH_ORBIT_Q=1,
           WZ_FH_PROF_ORDER=3, WZ_FH_CELLSIZE=10 ** 9, WZ_FH_PROF_SKIP=3000, WZ_FH_PROF_END=3100,
           WZ_FH_PROG_SEC=99999)


def main():
    env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
    env.update({k: str(v) for k, v in ENV.items()})
    with tempfile.TemporaryDirectory() as tmp:
        dump = os.path.join(tmp, "dump.txt")
        env["WZ_FH_DUMP"] = dump
        p = subprocess.run([REF_BIN, str(N), *map(str, SIG)], env=env, capture_output=True, text=True)
        lines = open(dump).read().splitlines()
    cells, pos = [], 0
    out = p.stdout.splitlines()
    for i, line in enumerate(out):
        m = re.match(r"CELLSIZE pi=(\d+) cand=(\d+) capped=(\d+) partial=(\d+) .* leaves=(\d+) hall_ok=(\d+)", line)
        if not m:
            continue
        pi, cand, capped, partial, leaves, ok = (int(x) for x in m.groups())
        nodes = int(re.match(r"CDSTAT pi=\d+ dfs_nodes=(\d+)", out[i + 1]).group(1))
        body = "\n".join(lines[pos:pos + cand]) + "\n"
        pos += cand
        cells.append(dict(pi=pi, cand=cand, capped=capped, partial=partial, leaves=leaves, hall_ok=ok,
                          dfs_nodes=nodes, dump_sha256=hashlib.sha256(body.encode()).hexdigest()))
    digest = re.search(r"digest=(\S+)", p.stdout).group(1)
    json.dump(dict(n=N, sig=SIG, env=ENV, digest=digest, cells=cells),
              open(os.path.join(HERE, "cells_n30_golden.json"), "w"), indent=1)
    print("cells", len(cells), "digest", digest)


if __name__ == "__main__":
    main()
