"""The lane at the first-hit workload's size (n = 36, sig (5,11,0,0), orbit canon + quad switch
+ Q-closure prune, ORDER=3 with the list digest, budget 2^22) against the reference binary's
runs over windows of raw cells (tests/golden/lane36_golden.json, make_lane36_golden.py):
the drop-in binary's exit code, semantic lines, CELLSIZE/CDSTAT counts and stream bytes, and
the library lane's (lane.run_lane) summary counts."""
import json
import os
import sys

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(HERE, "golden"))


def _cases():
    return json.load(open(os.path.join(HERE, "golden", "lane36_golden.json")))


def test_lane_binary_n36_windows_match_reference(gpu):
    import tempfile
    from make_lane_golden import cellsize_lines, semantic
    from test_lane_gpu import _bin, _run
    exe = _bin()
    with tempfile.TemporaryDirectory() as tmp:
        for c in _cases():
            rc, out, dh, dl = _run(exe, c["n"], c["sig"], c["settings"], tmp)
            ctx = c["settings"]
            assert rc == c["rc"], (ctx, out[-3000:])
            assert semantic(out) == c["semantic"], ctx
            assert cellsize_lines(out) == c["cells"], ctx
            assert (dh, dl) == (c["dump_sha256"], c["dump_len"]), ctx


def test_run_lane_n36_windows_match_reference(gpu):
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.lane import run_lane
    from test_lane_gpu import check_run_lane, lane_kwargs, summary_of
    ctx = Context(36, (5, 11, 0, 0))
    ran = 0
    for c in _cases():
        if "WZ_FH_CELLSIZE" in c["settings"]:
            continue
        res = run_lane(ctx, 36, (5, 11, 0, 0), **lane_kwargs(c["settings"]))
        check_run_lane(res, summary_of(c["semantic"]), c["settings"])
        ran += 1
    assert ran >= 2
    ctx.close()
