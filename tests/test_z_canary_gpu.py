"""The drop-in lane binary (bin/bs_firsthit) on the reference's archived n = 29 first-hit
canary (`WZ_FIRSTHIT=1 WZ_FH_M6=1 wz_match 29 0 6 9 1`, tools/test_firsthit_telemetry.py:176-181)
against the reference's own run of it (tests/golden/canary_n29_golden.json): exit code,
semantic lines (FIRSTHIT idx=26694 profile_rank=588, the summary counts, the quad), per raw cell
the completions, verdicts and charged nodes, and the hit cell's drain sequence with
WZ_FH_CAND_LOG on; and the hit cell alone with the outer-lag tables and the early check off,
where nodes_this_cand is the archived 81,320. (The file name has it collected after the other
lane tests and before the allocation-free filter's test, which is collected last.)"""
import json
import os
import sys
import tempfile

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


def test_lane_binary_replays_the_n29_canary(gpu):
    from make_canary_golden import RUNS, record
    from bs45_quantum_explorer_gb300.build import build_all
    _, exe = build_all()
    g = json.load(open(os.path.join(HERE, "golden", "canary_n29_golden.json")))
    assert set(g["runs"]) == set(RUNS)
    with tempfile.TemporaryDirectory() as tmp:
        for name, want in g["runs"].items():
            got = record(exe, name, tmp, timeout=600)
            assert got["settings"] == want["settings"]
            assert got["rc"] == want["rc"], name
            assert got["semantic"] == want["semantic"], name
            assert got["cells"] == want["cells"], name
            assert got["hit_cell"] == want["hit_cell"], name
