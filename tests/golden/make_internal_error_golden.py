#!/usr/bin/env python3
"""The first-hit lane's internal-error exit as the reference takes it: with the test hook
WZ_FH_TEST_INTERNAL_ERROR set, its completer reports its first completion as failing the
independent NPAF check (wz_match.cpp:1328-1335), and the lane prints FH_INTERNAL_ERROR and
"RESULT: INTERNAL ERROR at candidate ..." and exits 5 without advancing its checkpoint
(wz_match.cpp:2591-2595). Recorded per case: exit code, those lines and the protocol lines
before them, and the checkpoint file left in WZ_FH_CKPT_DIR, from oracle/_ref/wz_match (the
reference's wz_match.cpp compiled unmodified by `make -C oracle ref`).

    python tests/golden/make_internal_error_golden.py  ->  tests/golden/internal_error_golden.json
"""
import json
import os
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "wz_match")

BASE = dict(WZ_FIRSTHIT=1, WZ_FH_TEST_INTERNAL_ERROR=1, WZ_FH_PROG_SEC=9999)
CASES = [(6, (1, 5, 0, 0), dict(WZ_FH_M6=1)), (8, (3, 5, 0, 0), dict(WZ_FH_M6=1)),
         (10, (1, 5, 0, 4), dict(WZ_FH_M6=1)), (12, (3, 5, 0, 4), dict(WZ_FH_M6=1)),
         (10, (1, 5, 0, 4), dict(WZ_FH_M6=0)),
         (12, (3, 5, 0, 4), dict(WZ_FH_M6=1, WZ_FH_BUF_CAP=7, WZ_FH_DRAIN_TOP=3))]


def lines_of(out):
    return [l for l in out.splitlines()
            if l.startswith(("FH_INTERNAL_ERROR", "RESULT:", "[firsthit] profiles=", "FIRSTHIT:"))]


def record(binary, n, sig, settings):
    """Runs `binary` (the reference's wz_match or a drop-in) with the hook and a checkpoint
    directory; returns (exit code, lines_of(stdout), {checkpoint file: text})."""
    with tempfile.TemporaryDirectory() as ck:
        env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
        env.update({k: str(v) for k, v in {**BASE, **settings}.items()})
        env["WZ_FH_CKPT_DIR"] = ck
        p = subprocess.run([binary, str(n), *map(str, sig)], env=env, capture_output=True,
                           text=True, cwd=ck, timeout=600)
        files = {f: open(os.path.join(ck, f)).read() for f in sorted(os.listdir(ck))}
    return p.returncode, lines_of(p.stdout), files


def main():
    cases = []
    for n, sig, settings in CASES:
        rc, lines, files = record(REF_BIN, n, sig, settings)
        cases.append(dict(n=n, sig=sig, settings=settings, rc=rc, lines=lines, files=files))
        print(n, sig, settings, rc, lines[-1][:60] if lines else None, list(files))
    json.dump(cases, open(os.path.join(HERE, "internal_error_golden.json"), "w"), indent=0)


if __name__ == "__main__":
    main()
