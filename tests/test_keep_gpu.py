"""The lane binary's per-cell flattest-256 keep on whole n = 30 cells (config C3) against the
reference's own drain (tests/golden/keep_n30_golden.json): with WZ_FH_CAND_LOG on, every
completed candidate's drain rank, cell, verdict and charged nodes, in drain order, and the
summary lines must equal the reference's."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


def test_lane_binary_keep_matches_reference_drain(gpu):
    from make_keep_golden import cand_lines
    from make_lane_golden import semantic
    from bs45_quantum_explorer_gb300.build import build_all
    _, exe = build_all()
    g = json.load(open(os.path.join(HERE, "golden", "keep_n30_golden.json")))
    for c in g["cases"]:
        env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
        env.update({k: str(v) for k, v in c["settings"].items()})
        p = subprocess.run([exe, str(g["n"]), *map(str, g["sig"])], env=env, capture_output=True,
                           text=True, timeout=600)
        assert p.returncode == c["rc"], (c["pi"], p.stdout[-2000:])
        assert cand_lines(p.stdout) == c["cand"], c["pi"]
        assert semantic(p.stdout) == c["semantic"], c["pi"]
