"""The drop-in lane binary's answers to bad or unusual arguments against the reference's
(tests/golden/refusal_golden.json, from make_refusal_golden.py): the same exit code (1 usage,
2 refusal) and refusal line for a short argv, a wrong signature norm, n below 4, a bad shard,
ORDER=3 without orbit canon or without / with a wrong digest, a bad telemetry mode; list-only
exits 0; and settings the reference accepts (outer-lag K below 2 runs without the tables, a
shard count of 0 is taken as 1) are accepted with the same list-stage lines. Everything
compared happens before the binary opens its GPU context; on a host without a GPU an accepted
case then ends with exit 5 (no CPU fallback), which the test allows."""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


def test_lane_binary_refusals_match_reference(built_lib):
    from make_refusal_golden import record
    from bs45_quantum_explorer_gb300.build import build_host
    exe = build_host()
    cases = json.load(open(os.path.join(HERE, "golden", "refusal_golden.json")))
    assert {c["rc"] for c in cases} >= {0, 1, 2}
    for c in cases:
        rc, lines = record(exe, c["argv"], c["settings"])
        searched = any(l.startswith("[firsthit] profiles=") for l in c["lines"])
        if searched and rc == 5:  # no GPU here: the list stage matches, the search cannot run
            assert [l for l in lines if not l.startswith("RESULT:")] == \
                [l for l in c["lines"] if not l.startswith("RESULT:")], c["name"]
            continue
        assert (rc, lines) == (c["rc"], c["lines"]), c["name"]
