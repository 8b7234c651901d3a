"""The first-hit workload at its production size: n = 36, sig (5,11,0,0), orbit canon + quad
switch + Q-closure prune, ORDER=3 with the list digest, budget 2^22, BUF_CAP 500,000,
DRAIN_TOP 50,000. The reference binary ran the head of the seeded 4,096-cell window (its first
eight kept cells, one window each; tests/golden/c4_golden.json, make_c4_golden.py), about half
an hour of CPU per cell. The drop-in binary and the library lane must reproduce every summary
count (total_AB_nodes, budget_aborted, cells_done, ...), the CDSTAT/CELLSIZE lines, the
streamed candidates (WZ_FH_DUMP bytes) and any FIRSTHIT line."""
import json
import os
import sys
import tempfile

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(HERE, "golden"))


def _cases():
    return json.load(open(os.path.join(HERE, "golden", "c4_golden.json")))


def test_c4_lane_binary_matches_reference(gpu):
    from make_lane_golden import cellsize_lines, semantic
    from test_lane_gpu import _bin, _run
    exe = _bin()
    cases = _cases()
    assert len(cases) == 8
    with tempfile.TemporaryDirectory() as tmp:
        for c in cases:
            rc, out, dh, dl = _run(exe, c["n"], c["sig"], c["settings"], tmp)
            ctx = c["settings"]["WZ_FH_PROF_SKIP"]
            assert rc == c["rc"], (ctx, out[-3000:])
            assert semantic(out) == c["semantic"], ctx
            assert cellsize_lines(out) == c["cells"], ctx
            assert (dh, dl) == (c["dump_sha256"], c["dump_len"]), ctx


def test_c4_library_lane_matches_reference(gpu):
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.lane import run_lane
    from test_lane_gpu import check_run_lane, lane_kwargs, summary_of
    ctx = Context(36, (5, 11, 0, 0))
    for c in _cases():
        res = run_lane(ctx, 36, (5, 11, 0, 0), **lane_kwargs(c["settings"]))
        check_run_lane(res, summary_of(c["semantic"]), c["settings"]["WZ_FH_PROF_SKIP"])
    ctx.close()
