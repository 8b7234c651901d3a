#!/usr/bin/env python3
"""The reference's production lane manifests as fixtures: Pass H at n = 44 and n = 45
(docs/plans/passh_manifest.json and passh45_manifest.json in the reference repository), which
its planner tools/passh_manifest.py built from list-only runs of the reference solver (ORDER=3,
orbit canon + Q + Q-prune, 177 arms; the n = 45 lanes also with WZ_FH_ENDPOS=1, as their
submission lines carry it). Kept per class: signature, letter, raw cells, kept cells, windows,
lane size S, the list:kept digest and the lanes.

    python tests/golden/make_production_golden.py REF  ->  tests/golden/production_manifest_golden.json
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PASSES = (("docs/plans/passh_manifest.json", 44, False), ("docs/plans/passh45_manifest.json", 45, True))
FIELDS = ("sig", "letter", "cells", "kept", "windows", "S", "digest", "lanes")


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_production_golden.py REF   (REF: root of the reference repository)")
    out = []
    for path, n, endpos in PASSES:
        m = json.load(open(os.path.join(sys.argv[1], path)))
        assert m.get("n", n) == n
        out.append(dict(source=path, n=n, endpos=endpos, narms=m["narms"],
                        classes=[{k: c[k] for k in FIELDS} for c in m["classes"]]))
    json.dump(out, open(os.path.join(HERE, "production_manifest_golden.json"), "w"), indent=0)
    print(sum(len(p["classes"]) for p in out), "classes")


if __name__ == "__main__":
    main()
