#!/usr/bin/env python3
"""Golden for lane manifests: the reference solver's list-only mode (WZ_FH_LIST_ONLY=1 with the
planner's settings of tools/passh_manifest.py: ORDER=3, orbit canon + quad switch + Q-closure
prune, WZ_FH_NSHARD = NARMS) run by oracle/_ref/wz_match, its `[order]` line parsed into the
raw list length, kept count, window count, digest and kept cells per arm.

    python tests/golden/make_manifest_golden.py   ->  tests/golden/manifest_golden.json
"""
import json
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
from make_lane_golden import REF_BIN  # noqa: E402

CASES = [(30, (1, 7, 6, 6), 177), (36, (5, 11, 0, 0), 177), (36, (5, 11, 0, 0), 191),
         (42, (7, 11, 0, 0), 177)]


def main():
    out = []
    for n, sig, narms in CASES:
        env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
        env.update(WZ_FIRSTHIT="1", WZ_FH_ORBIT_CANON="1", WZ_FH_ORBIT_Q="1", WZ_FH_ORBIT_QPRUNE="1",
                   WZ_FH_PROF_ORDER="3", WZ_FH_LIST_ONLY="1", WZ_FH_NSHARD=str(narms))
        p = subprocess.run([REF_BIN, str(n), *map(str, sig)], env=env, capture_output=True, text=True,
                           timeout=3600)
        m = re.search(r"^\[order\] ord3 cells=(\d+) kept=(\d+) windows=(\d+) digest=(\S+) arms=(\d+) "
                      r"kept_per_arm_min=(\d+) max=(\d+)", p.stdout, re.M)
        assert p.returncode == 0 and m, p.stdout[-500:]
        out.append(dict(n=n, sig=list(sig), narms=narms, cells=int(m[1]), kept=int(m[2]),
                        windows=int(m[3]), digest=m[4], kept_per_arm_min=int(m[6]),
                        kept_per_arm_max=int(m[7])))
        print(out[-1], flush=True)
    json.dump(out, open(os.path.join(HERE, "manifest_golden.json"), "w"), indent=0)


if __name__ == "__main__":
    main()
