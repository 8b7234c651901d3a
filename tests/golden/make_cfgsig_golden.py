#!/usr/bin/env python3
"""The checkpoint namespace (CFGSIG) the reference derives from a lane's settings, for every
field it holds.

An arm's checkpoint file starts with `CFGSIG=<string>`, built from n, the signature and the
lane settings (wz_match.cpp:2241-2287: the fixed fields, then suffixes appended only when a
setting is not at its default). An arm resumes only from a checkpoint whose CFGSIG equals its
own (wz_match.cpp:2288-2314), so GPU and CPU arms share checkpoints only if they derive the
same string. Each case below gives the reference binary (oracle/_ref/wz_match, compiled
unmodified by `make -C oracle ref`) a forged checkpoint whose CFGSIG matches nothing; the
reference prints `[firsthit ckpt] STALE/MISMATCHED checkpoint IGNORED (<forged> != <its
CFGSIG>)` before it searches. Recorded per case: that line, the `[firsthit] profiles=` line
and the `[abprof]` line without its build time. The search is stopped after one completion
(WZ_FH_TEST_STOP_AFTER=1).

    python tests/golden/make_cfgsig_golden.py  ->  tests/golden/cfgsig_golden.json
"""
import concurrent.futures as cf
import json
import os
import re
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "wz_match")
FORGED = "n0.forged"

BASE = dict(WZ_FIRSTHIT=1, WZ_FH_PROG_SEC=99999, WZ_FH_TEST_STOP_AFTER=1, WZ_FH_AB_BUDGET=50)
# (n, sig, settings): every fixed CFGSIG field away from its default once, and every suffix
CASES = [
    (12, (1, 3, 2, 6), {}),
    (12, (1, 3, 2, 6), dict(WZ_FH_M6=1)),
    (12, (1, 3, 2, 6), dict(WZ_FH_M6=1, WZ_FH_CELL_ORDER=0, WZ_FH_AB_PROF=0)),
    (12, (1, 3, 2, 6), dict(WZ_FH_NSHARD=3, WZ_FH_SHARD=1)),
    (12, (1, 3, 2, 6), dict(WZ_FH_M6=1, WZ_FH_SCORE_MAX=60, WZ_FH_BUF_CAP=7, WZ_FH_PROF_SKIP=2)),
    (12, (1, 3, 2, 6), dict(WZ_THM211B=1, WZ_THM212=1, WZ_FH_M6=1)),
    (12, (1, 3, 2, 6), dict(WZ_FH_M6=1, WZ_FH_DRAIN_TOP=3, WZ_FH_DRAIN_BATCHES=2)),
    (12, (1, 3, 2, 6), dict(WZ_FH_M6=1, WZ_FH_STREAM_REV=1, WZ_FH_WALL_SEC=100)),
    (12, (1, 3, 2, 6), dict(WZ_FH_M6=1, WZ_FH_PROF_ORDER=1, WZ_FH_ORBIT_CANON=1)),
    (12, (1, 3, 2, 6), dict(WZ_FH_M6=1, WZ_FH_PROF_ORDER=2, WZ_FH_ORBIT_CANON=1)),
    (12, (1, 7, 0, 0), dict(WZ_FH_M6=1, WZ_FH_ORBIT_CANON=1)),               # pins dropped
    (12, (1, 7, 0, 0), dict(WZ_FH_M6=1)),                                    # pins kept
    (13, (0, 2, 1, 7), dict(WZ_FH_M6=1, WZ_FH_ENDPOS=1)),
    (13, (0, 2, 1, 7), dict(WZ_FH_M6=1, WZ_FH_ORBIT_CANON=1, WZ_FH_ORBIT_Q=1)),
    (13, (0, 2, 1, 7), dict(WZ_FH_M6=1, WZ_FH_ORBIT_CANON=1, WZ_FH_ORBIT_Q=1,
                            WZ_FH_ORBIT_QPRUNE=1)),
    (13, (0, 2, 1, 7), dict(WZ_FH_M6=1, WZ_FH_ORBIT_CANON=1, WZ_FH_ORBIT_Q=1, WZ_FH_PROF_ORDER=3,
                            WZ_FH_ORD3_NODIGEST_OK=1)),
    (13, (0, 2, 1, 7), dict(WZ_FH_M6=1, WZ_FH_ORBIT_CANON=1, WZ_FH_ORBIT_Q=1, WZ_FH_ORBIT_QPRUNE=1,
                            WZ_FH_PROF_ORDER=3, WZ_FH_ORD3_NODIGEST_OK=1, WZ_THM211B=1,
                            WZ_THM212=1, WZ_FH_NSHARD=2, WZ_FH_SHARD=1, WZ_FH_DRAIN_TOP=5,
                            WZ_FH_STREAM_REV=1, WZ_FH_WALL_SEC=7, WZ_FH_ENDPOS=1)),
    (10, (1, 5, 0, 4), dict(WZ_FH_M6=1, WZ_FH_ORBIT_CANON=1, WZ_FH_PROF_ORDER=3,
                            WZ_FH_ORD3_NODIGEST_OK=1, WZ_FH_AB_BUDGET=0)),
]


def lines_of(out):
    """The CFGSIG-bearing and list-stage lines (build time dropped)."""
    keep = []
    for line in out.splitlines():
        if line.startswith(("[firsthit ckpt]", "[firsthit] profiles=", "[abprof]")):
            keep.append(re.sub(r" build=\S+", "", line))
    return keep


def record(binary, n, sig, settings, timeout=120):
    """Runs `binary` (the reference's wz_match or a drop-in) on one case with the forged
    checkpoint; returns its exit code and lines_of() its stdout."""
    st = {**BASE, **settings}
    with tempfile.TemporaryDirectory() as ck:
        shard = int(st.get("WZ_FH_SHARD", 0))
        with open(os.path.join(ck, f"arm_{shard}.ckpt"), "w") as f:
            f.write(f"CFGSIG={FORGED}\nresume_pi=0\nresume_batch=0\nresume_k=0\ntested_cum=0\n")
        env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
        env.update({k: str(v) for k, v in st.items()})
        env["WZ_FH_CKPT_DIR"] = ck
        p = subprocess.run([binary, str(n), *map(str, sig)], env=env, capture_output=True,
                           text=True, timeout=timeout, cwd=ck)
    return p.returncode, lines_of(p.stdout)


def main():
    def one(case):
        n, sig, settings = case
        rc, lines = record(REF_BIN, n, sig, settings)
        return dict(n=n, sig=sig, settings=settings, rc=rc, lines=lines)

    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        cases = list(ex.map(one, CASES))
    for c in cases:
        sig = [l for l in c["lines"] if l.startswith("[firsthit ckpt]")]
        print(c["n"], c["sig"], c["rc"], sig[0].split(" != ")[1].split(")")[0] if sig else "NO CKPT LINE")
    json.dump(cases, open(os.path.join(HERE, "cfgsig_golden.json"), "w"), indent=0)


if __name__ == "__main__":
    main()
