#!/usr/bin/env python3
"""Lane-level golden fixtures: full first-hit runs of the reference binary at small n.

Runs oracle/_ref/wz_match (the reference's own src/solver/wz_match.cpp, compiled unmodified
by `make -C oracle ref`) with WZ_FIRSTHIT=1 over every signature class at n = 6..13 and a set
of lane settings modelled on the reference's own identity gates (tools/test_cd_prune.py,
test_hall_fast.py, test_resume_boundary.py, test_firsthit_cellsize.py), and records what a
drop-in must reproduce: exit code, the semantic stdout lines (RESULT / candidates_streamed /
backtracks_entered / FIRSTHIT without elapsed / A,B,C,D), CELLSIZE and CDSTAT counts, the
WZ_FH_DUMP stream bytes (sha256) and the checkpoint file.

    python tests/golden/make_lane_golden.py   ->  tests/golden/lane_golden.json
"""
import hashlib
import itertools
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "wz_match")
sys.path.insert(0, HERE)
from make_golden import classes  # noqa: E402

BASE = dict(WZ_FIRSTHIT=1, WZ_THM211B=1, WZ_THM212=1, WZ_FH_PROG_SEC=9999)

SETTINGS = [
    dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=0),
    dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=30, WZ_FH_STREAM_REV=1),
    dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=0, WZ_FH_PROF_ORDER=1, WZ_FH_ORBIT_CANON=1),
    dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=0, WZ_FH_PROF_ORDER=2, WZ_FH_STREAM_REV=1, WZ_FH_ORBIT_CANON=1),
    dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=5, WZ_FH_BUF_CAP=7, WZ_FH_DRAIN_TOP=3, WZ_FH_DRAIN_BATCHES=2),
    dict(WZ_FH_M6=1, WZ_FH_CELLSIZE=10 ** 9),
    dict(WZ_FH_M6=1, WZ_FH_CELLSIZE=10 ** 9, WZ_FH_STREAM_REV=1, WZ_FH_ENDPOS=1),
    dict(WZ_FH_M6=1, WZ_FH_CELLSIZE=10 ** 9, WZ_FH_CD_PRUNE=3),
    dict(WZ_FH_M6=1, WZ_FH_CELLSIZE=10 ** 9, WZ_FH_CD_PRUNE=1, WZ_FH_STREAM_REV=1),
    dict(WZ_FH_M6=1, WZ_FH_CELLSIZE=10 ** 9, WZ_FH_CD_PRUNE=2, WZ_FH_ENDPOS=1),
    dict(WZ_FH_M6=0, WZ_FH_AB_BUDGET=0),
    dict(WZ_FH_M6=0, WZ_FH_AB_BUDGET=20, WZ_FH_OUTER_K=0, WZ_FH_EARLY_CHECK=0),
    dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=0, WZ_FH_ORBIT_CANON=1, WZ_FH_ORBIT_Q=1, WZ_FH_PROF_ORDER=3,
         WZ_FH_ORD3_NODIGEST_OK=1, WZ_FH_SCORE_MAX=30),
]


def semantic(out):
    keep = []
    for line in out.splitlines():
        if line.startswith(("RESULT:", "candidates_streamed=", "backtracks_entered=", "FIRSTHIT:",
                            "A =", "B =", "C =", "D =", "[order]", "[orbitcanon]", "[firsthit] profiles=")):
            keep.append(re.sub(r" elapsed=.*", "", line))
    return keep


def cellsize_lines(out):
    rows = []
    for line in out.splitlines():
        m = re.match(r"CELLSIZE pi=(\d+) cand=(\d+) capped=(\d+) partial=(\d+) .* leaves=(\d+) hall_ok=(\d+)", line)
        if m:
            rows.append(["CELLSIZE"] + [int(x) for x in m.groups()])
        m = re.match(r"CDSTAT pi=(\d+) dfs_nodes=(\d+)", line)
        if m:
            rows.append(["CDSTAT"] + [int(x) for x in m.groups()])
    return rows


def run(n, sig, settings, tmp, ckdir=None, timeout=600):
    env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
    env.update({k: str(v) for k, v in {**BASE, **settings}.items()})
    dump = os.path.join(tmp, "dump.txt")
    env["WZ_FH_DUMP"] = dump
    if ckdir:
        env["WZ_FH_CKPT_DIR"] = ckdir
    p = subprocess.run([REF_BIN, str(n), *map(str, sig)], env=env, capture_output=True, text=True, timeout=timeout)
    data = open(dump, "rb").read() if os.path.exists(dump) else b""
    return p.returncode, p.stdout, hashlib.sha256(data).hexdigest(), len(data)


def main():
    cases = []
    with tempfile.TemporaryDirectory(prefix="bsfh-lane-") as tmp:
        for n in range(6, 14):
            for sig in classes(n):
                for k, st in enumerate(SETTINGS):
                    rc, out, dh, dl = run(n, sig, st, tmp)
                    cases.append(dict(n=n, sig=list(sig), settings=st, rc=rc, semantic=semantic(out),
                                      cells=cellsize_lines(out), dump_sha256=dh, dump_len=dl))
        # checkpoint interrupt + resume (the reference's test_resume_boundary shape)
        for n in (9, 11, 12, 13):
            for sig in classes(n)[:3]:
                for st in (dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=50, WZ_FH_TEST_STOP_AFTER=3),
                           dict(WZ_FH_M6=1, WZ_FH_AB_BUDGET=50, WZ_FH_BUF_CAP=5, WZ_FH_DRAIN_TOP=2,
                                WZ_FH_TEST_STOP_AFTER=2)):
                    ck = tempfile.mkdtemp(dir=tmp)
                    rc1, out1, _, _ = run(n, sig, st, tmp, ck)
                    files = sorted(os.listdir(ck))
                    ckpt1 = open(os.path.join(ck, files[0])).read() if files else ""
                    st2 = {k: v for k, v in st.items() if k != "WZ_FH_TEST_STOP_AFTER"}
                    rc2, out2, dh, dl = run(n, sig, st2, tmp, ck)
                    ckpt2 = open(os.path.join(ck, files[0])).read() if files else ""
                    cases.append(dict(n=n, sig=list(sig), settings=st, resume=True, rc=rc1, semantic=semantic(out1),
                                      ckpt=ckpt1, rc2=rc2, semantic2=semantic(out2), ckpt2=ckpt2,
                                      dump_sha256=dh, dump_len=dl, cells=[]))
    json.dump(cases, open(os.path.join(HERE, "lane_golden.json"), "w"))
    print("lane cases", len(cases), "found", sum(1 for c in cases if c["rc"] == 0))


if __name__ == "__main__":
    main()
