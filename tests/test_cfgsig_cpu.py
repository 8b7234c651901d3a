"""The drop-in lane binary's checkpoint namespace against the reference's
(tests/golden/cfgsig_golden.json, from make_cfgsig_golden.py). For every CFGSIG field and
suffix the reference derives from a lane's settings (wz_match.cpp:2241-2287), both binaries
are given the same forged checkpoint and must print the same `[firsthit ckpt] STALE/MISMATCHED
checkpoint IGNORED (<forged> != <CFGSIG>)` line, so a checkpoint written by either one resumes
on the other exactly when the reference would resume it. The `[firsthit] profiles=` and
`[abprof]` lines (list size, settings, allowed-row counts) are compared too. All of this runs
before the binary opens its GPU context; the search that follows needs the GPU and is checked
by the -m gpu lane tests (checkpoint bytes included). The cases include one arm of the
reference's first n = 44 and n = 45 production lanes with the environment its lane driver
gives it (the manifest's digest is expected, and matches)."""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


def test_lane_binary_cfgsig_matches_reference(built_lib):
    from make_cfgsig_golden import FORGED, record
    from bs45_quantum_explorer_gb300.build import build_host
    exe = build_host()
    cases = json.load(open(os.path.join(HERE, "golden", "cfgsig_golden.json")))
    assert len(cases) >= 20 and sum("PRODUCTION" in c["settings"] for c in cases) == 2
    suffixes = set()
    for c in cases:
        want = c["lines"]
        stale = [l for l in want if l.startswith("[firsthit ckpt]")]
        assert len(stale) == 1 and f"({FORGED} != " in stale[0]
        cfgsig = stale[0].split(" != ")[1].split(")")[0]
        suffixes.update("dg" if x.startswith("dg") else re.match(r"[a-z]+", x).group(0)
                        for x in cfgsig.split(".")[18:])
        _, got = record(exe, c["n"], tuple(c["sig"]), c["settings"])
        assert got == want, (c["n"], c["sig"], c["settings"])
    # every optional suffix of the reference's CFGSIG is among the cases
    assert suffixes == {"db", "sr", "np", "ws", "ep", "oq", "qp", "bud", "dg"}
