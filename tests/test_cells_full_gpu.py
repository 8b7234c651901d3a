"""Full-size stream parity (config C3: n = 30, signature (1,7,6,6)): whole cells of the
ORDER=3 list streamed on the GPU must reproduce the reference's own CELLSIZE / CDSTAT counts
and its WZ_FH_DUMP stream bytes (tests/golden/cells_n30_golden.json, from the reference
binary). Cells here hold 1e5-3e5 survivors, 1e7-3e7 leaves and 6e8-1.6e9 DFS nodes."""
import hashlib
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _golden():
    path = os.path.join(HERE, "golden", "cells_n30_golden.json")
    if not os.path.exists(path):
        pytest.fail("cells_n30_golden.json missing")
    return json.load(open(path))


def _cell_list(g, lo, hi):
    """(px, py) of raw cells [lo, hi) from the lane binary's own list (checked by digest)."""
    from bs45_quantum_explorer_gb300.build import build_all
    _, exe = build_all()
    env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
    env.update({k: str(v) for k, v in g["env"].items() if k not in ("WZ_FH_CELLSIZE",)})
    env["WZ_FH_LIST_CELLS"] = f"{lo},{hi}"
    env["WZ_FH_ORD3_NODIGEST_OK"] = "1"
    out = subprocess.run([exe, str(g["n"]), *map(str, g["sig"])], env=env, capture_output=True,
                         text=True, timeout=900).stdout
    assert f"digest={g['digest']}" in out
    cells = {}
    for line in out.splitlines():
        if line.startswith("CELL pi="):
            f = dict(kv.split("=") for kv in line.split()[1:])
            cells[int(f["pi"])] = ([int(x) for x in f["px"].split(",")], [int(x) for x in f["py"].split(",")])
    return cells


def test_n30_cells_match_reference(gpu):
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.stream import cd_stream
    g = _golden()
    cells = _cell_list(g, 3000, 3100)
    ctx = Context(g["n"], g["sig"])
    gold = [c for c in g["cells"] if not c["capped"] and not c["partial"]]
    assert len(gold) >= 10
    batch = [cells[c["pi"]] for c in gold]
    surv, cidx, stats = cd_stream(ctx, batch, m=6, cap=1 << 23)
    for i, c in enumerate(gold):
        rows = surv[cidx == i]
        assert (len(rows), stats[i]["leaves"], stats[i]["ok"], stats[i]["nodes"]) == \
            (c["cand"], c["leaves"], c["hall_ok"], c["dfs_nodes"]), c["pi"]
        body = "".join(" ".join(str(int(v)) for v in r[0]) + " | " +
                       " ".join(str(int(v)) for v in r[1]) + " \n" for r in rows)
        assert hashlib.sha256(body.encode()).hexdigest() == c["dump_sha256"], c["pi"]
