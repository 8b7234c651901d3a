#!/usr/bin/env python3
"""How the reference's first-hit lane answers bad or unusual arguments, before it searches:
the exit code (1 usage, 2 refusal; wz_match.cpp:1344-1362, 1584, 1595, 1851, 1870, 1878),
the refusal line it prints, and, for settings it accepts, the lines of its list stage.

Runs oracle/_ref/wz_match (the reference's wz_match.cpp compiled unmodified by
`make -C oracle ref`) on each case; a case it accepts is searched to the end (n = 12, a few
milliseconds).

    python tests/golden/make_refusal_golden.py  ->  tests/golden/refusal_golden.json
"""
import json
import os
import re
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "wz_match")

FH = dict(WZ_FIRSTHIT=1)
O3 = dict(WZ_FIRSTHIT=1, WZ_FH_M6=1, WZ_FH_PROF_ORDER=3, WZ_FH_ORBIT_CANON=1)
SIG = ["12", "1", "3", "2", "6"]
# (name, argv after the program, environment)
CASES = [
    ("too few arguments", ["12", "1", "3"], FH),
    ("signature norm is not 4n+2", ["12", "1", "3", "2", "5"], FH),
    ("n below 4", ["3", "1", "1", "1", "1"], FH),
    ("shard beyond the shard count", SIG, dict(FH, WZ_FH_SHARD=3, WZ_FH_NSHARD=2)),
    ("negative shard", SIG, dict(FH, WZ_FH_SHARD=-1, WZ_FH_NSHARD=2)),
    ("order 3 without orbit canon", SIG, dict(FH, WZ_FH_M6=1, WZ_FH_PROF_ORDER=3)),
    ("order 3 search without a digest", SIG, O3),
    ("order 3 with a wrong digest", SIG, dict(O3, WZ_FH_EXPECT_DIGEST="00:00")),
    ("order 3 list only", SIG, dict(O3, WZ_FH_LIST_ONLY=1)),
    ("telemetry mode not 0, 1 or 64", SIG, dict(FH, WZ_FH_TELEMETRY=5)),
    ("outer-lag K = 1 (runs without the tables)", SIG, dict(FH, WZ_FH_OUTER_K=1)),
    ("outer-lag K = -1 (runs without the tables)", SIG, dict(FH, WZ_FH_OUTER_K=-1)),
    ("shard count 0 (taken as 1)", SIG, dict(FH, WZ_FH_NSHARD=0)),
]


def lines_of(out):
    """The refusal and list-stage lines of a run's stdout."""
    return [l for l in out.splitlines()
            if l.startswith(("RESULT:", "[firsthit] BAD SHARD", "[firsthit] profiles=", "[order]"))]


def record(binary, argv, settings, timeout=120):
    env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
    env.update({k: str(v) for k, v in settings.items()})
    with tempfile.TemporaryDirectory() as tmp:
        p = subprocess.run([binary, *argv], env=env, capture_output=True, text=True,
                           timeout=timeout, cwd=tmp)
    return p.returncode, lines_of(p.stdout)


def main():
    cases = []
    for name, argv, settings in CASES:
        rc, lines = record(REF_BIN, argv, settings)
        cases.append(dict(name=name, argv=argv, settings=settings, rc=rc, lines=lines))
        print(f"{name}: rc {rc} {[l for l in lines if not l.startswith('[order]')][:2]}")
    json.dump(cases, open(os.path.join(HERE, "refusal_golden.json"), "w"), indent=0)


if __name__ == "__main__":
    main()
