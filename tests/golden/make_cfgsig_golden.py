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
and the `[abprof]` line without its build time. Each run is ended once those lines are out (small
cases also carry WZ_FH_TEST_STOP_AFTER=1). Besides settings chosen to move every field, the cases
include edge values (empty, zero and negative settings, presence-only flags), n = 36 defaults
and one arm of the reference's first n = 44 and n = 45 production lanes, with the environment
its lane driver gives it.

    python tests/golden/make_cfgsig_golden.py REF  ->  tests/golden/cfgsig_golden.json
(REF: the reference repository's root, for its production submission files)
"""
import concurrent.futures as cf
import json
import os
import re
import subprocess
import sys
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
    # edge values: Q forced at odd n, empty or zero or negative values, presence-only flags
    (13, (0, 2, 1, 7), dict(WZ_FH_M6=1, WZ_FH_ORBIT_CANON=1, WZ_FH_ORBIT_Q=2)),
    (12, (1, 3, 2, 6), dict(WZ_FH_M6=1, WZ_FH_SCORE_MAX="", WZ_THM211B="0", WZ_THM212="0")),
    (12, (1, 3, 2, 6), dict(WZ_FH_M6=1, WZ_FH_STREAM_REV="0", WZ_FH_DRAIN_BATCHES="0",
                            WZ_FH_WALL_SEC="-5", WZ_FH_NSHARD="0")),
    # n >= 36: mod-6 cells, 2.11b and 2.12 forced
    (36, (5, 11, 0, 0), {}),
]

# The production lanes' arms (the reference's Pass H submissions, docs/plans/passh_submit_fir.txt
# and passh45_submit_fir.txt, through cluster_firsthit_probe.sh): the first line of each, as
# arm 1 of its lane with an empty per-arm WZ_FH_SCORE_MAX (the lane driver's ungated tier).
SUBMITS = (("docs/plans/passh_submit_fir.txt", 44), ("docs/plans/passh45_submit_fir.txt", 45))
DRIVER_EXPORTS = ("WZ_FH_AB_BUDGET", "WZ_FH_PROF_ORDER", "WZ_FH_SCORE_MAX", "WZ_FH_STREAM_TOTAL",
                  "WZ_FH_PROF_SKIP", "WZ_FH_AB_PROF", "WZ_FH_RESUME", "WZ_FH_BUF_CAP",
                  "WZ_FH_ORBIT_CANON", "WZ_FH_DRAIN_TOP", "WZ_FH_DRAIN_BATCHES", "WZ_FH_STREAM_REV",
                  "WZ_FH_WALL_SEC", "WZ_FH_PROF_END", "WZ_FH_EARLY_CHECK", "WZ_FH_TELEMETRY",
                  "WZ_FH_ORBIT_Q", "WZ_FH_ORBIT_QPRUNE", "WZ_FH_EXPECT_DIGEST", "WZ_FH_ENDPOS")


def production_cases(ref_root):
    out = []
    for path, n in SUBMITS:
        line = open(os.path.join(ref_root, path)).readline()
        env = dict(kv.split("=", 1) for kv in re.search(r"--export=ALL,(\S+)", line).group(1).split(","))
        assert int(env["WZ_N"]) == n
        sig = tuple(int(env["WZ_" + k]) for k in "ABCD")
        st = {k: env[k] for k in DRIVER_EXPORTS if k in env}
        st.update(WZ_FH_SHARD=1, WZ_FH_NSHARD=env["FH_NARMS"], WZ_FH_SCORE_MAX="",
                  OMP_NUM_THREADS=1, PRODUCTION=path)
        out.append((n, sig, st))
    return out


def lines_of(out):
    """The CFGSIG-bearing and list-stage lines (build time dropped)."""
    keep = []
    for line in out.splitlines():
        if line.startswith(("[firsthit ckpt]", "[firsthit] profiles=", "[abprof]")):
            keep.append(re.sub(r" build=\S+", "", line))
    return keep


def record(binary, n, sig, settings, timeout=600):
    """Runs `binary` (the reference's wz_match or a drop-in) on one case with the forged
    checkpoint, up to the last line compared (the [abprof] line when the allowed rows are on,
    else the checkpoint line; the search that follows is not waited for: the process is then
    ended); returns its exit code (None when ended) and lines_of() its stdout."""
    st = {k: v for k, v in {**BASE, **settings}.items() if k != "PRODUCTION"}
    m6 = int(st["WZ_FH_M6"] or 0) != 0 if "WZ_FH_M6" in st else n >= 36
    ab_prof = int(st["WZ_FH_AB_PROF"] or 0) != 0 if "WZ_FH_AB_PROF" in st else m6
    last = "[abprof]" if ab_prof else "[firsthit ckpt]"
    with tempfile.TemporaryDirectory() as ck:
        shard = int(st.get("WZ_FH_SHARD", 0) or 0)
        with open(os.path.join(ck, f"arm_{shard}.ckpt"), "w") as f:
            f.write(f"CFGSIG={FORGED}\nresume_pi=0\nresume_batch=0\nresume_k=0\ntested_cum=0\n")
        env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
        env.update({k: str(v) for k, v in st.items()})
        env["WZ_FH_CKPT_DIR"] = ck
        p = subprocess.Popen([binary, str(n), *map(str, sig)], env=env, stdout=subprocess.PIPE,
                             stderr=subprocess.DEVNULL, text=True, cwd=ck)
        out = []
        try:
            for line in p.stdout:
                out.append(line)
                if line.startswith(last):
                    break
        finally:
            if p.poll() is None:
                p.kill()
            p.stdout.close()
            rc = p.wait(timeout=timeout)
    return (rc if rc >= 0 else None), lines_of("".join(out))


def main():
    def one(case):
        n, sig, settings = case
        rc, lines = record(REF_BIN, n, sig, settings)
        return dict(n=n, sig=sig, settings=settings, lines=lines)

    ref_root = sys.argv[1] if len(sys.argv) > 1 else None
    if not ref_root:
        sys.exit("usage: make_cfgsig_golden.py REF   (REF: root of the reference repository)")
    with cf.ThreadPoolExecutor(max_workers=8) as ex:
        cases = list(ex.map(one, CASES + production_cases(ref_root)))
    for c in cases:
        sig = [l for l in c["lines"] if l.startswith("[firsthit ckpt]")]
        print(c["n"], c["sig"], sig[0].split(" != ")[1].split(")")[0] if sig else "NO CKPT LINE")
    json.dump(cases, open(os.path.join(HERE, "cfgsig_golden.json"), "w"), indent=0)


if __name__ == "__main__":
    main()
