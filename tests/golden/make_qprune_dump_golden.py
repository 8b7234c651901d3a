#!/usr/bin/env python3
"""The Q-closure prune's audit files as the reference writes them: with WZ_FH_QPRUNE_DUMP=path
its list stage writes the raw list index of every cell the prune removes to `path` and one
certificate per dead orbit to `path.certs` (wz_match.cpp:1785-1797). Recorded per case: the
sha256 and line count of both files, from list-only runs (ORDER=3, orbit canon + Q +
Q-prune, mod-6 cells, 2.11b and 2.12; ENDPOS at odd n) of oracle/_ref/wz_match, the reference's
wz_match.cpp compiled unmodified by `make -C oracle ref`.

    python tests/golden/make_qprune_dump_golden.py  ->  tests/golden/qprune_dump_golden.json
"""
import concurrent.futures as cf
import hashlib
import json
import os
import subprocess
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_BIN = os.path.join(ROOT, "oracle", "_ref", "wz_match")

CASES = [(13, (0, 2, 1, 7)), (15, (0, 6, 1, 5)), (17, (2, 4, 5, 5)), (20, (1, 9, 0, 0)),
         (22, (1, 7, 2, 6)), (25, (2, 8, 3, 5)), (30, (1, 7, 6, 6)), (36, (5, 11, 0, 0))]


def settings(n):
    return dict(WZ_FIRSTHIT=1, WZ_FH_M6=1, WZ_THM211B=1, WZ_THM212=1, WZ_FH_ORBIT_CANON=1,
                WZ_FH_ORBIT_Q=1, WZ_FH_ORBIT_QPRUNE=1, WZ_FH_PROF_ORDER=3, WZ_FH_LIST_ONLY=1,
                WZ_FH_ENDPOS=n % 2)


def record(binary, n, sig):
    """Runs `binary` (the reference's wz_match or a drop-in) list-only with the dump on;
    returns {file: [sha256, lines]} for the dump and its certificates, and the exit code."""
    with tempfile.TemporaryDirectory() as tmp:
        dump = os.path.join(tmp, "qprune.txt")
        env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
        env.update({k: str(v) for k, v in settings(n).items()})
        env["WZ_FH_QPRUNE_DUMP"] = dump
        p = subprocess.run([binary, str(n), *map(str, sig)], env=env, capture_output=True,
                           text=True, cwd=tmp, timeout=600)
        files = {}
        for name, path in (("dump", dump), ("certs", dump + ".certs")):
            data = open(path, "rb").read() if os.path.exists(path) else b""
            files[name] = [hashlib.sha256(data).hexdigest(), data.count(b"\n")]
    return p.returncode, files


def main():
    def one(case):
        n, sig = case
        assert sum(x * x for x in sig) == 4 * n + 2, case
        rc, files = record(REF_BIN, n, sig)
        return dict(n=n, sig=sig, rc=rc, files=files)

    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        cases = list(ex.map(one, CASES))
    for c in cases:
        print(c["n"], c["sig"], c["rc"], {k: v[1] for k, v in c["files"].items()})
    json.dump(cases, open(os.path.join(HERE, "qprune_dump_golden.json"), "w"), indent=0)


if __name__ == "__main__":
    main()
