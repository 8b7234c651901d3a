"""bench.py's reference arm runs on the host alone: one JSON line with the contract's keys, the
same metric, unit and workload as the GPU arm, and a positive rate."""
import json
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_reference_arm_prints_one_contract_line(built_lib):
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "3", "--warmup", "3", "--pairs", "65536"], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "impl",
              "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 3
    assert d["metric"].startswith("spectral-filtered C,D cands/s at n=42")
    assert d["unit"] == "pairs/s" and d["config"]["workload"] == "hall_filter_n42_2^24_pairs"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
    # the reference's own code where oracle/_ref was built here, else the oracle restatement
    import refarm
    assert d["cpu_baseline"]["kind"] == ("reference" if refarm.available() else "port")
    assert d["config"]["pairs_per_step"] == 65536


def test_reference_arm_under_torchrun_prints_on_rank0_only(built_lib):
    """Launched like the multi-GPU bench (two ranks over 127.0.0.1): rank 0 alone does the
    work and prints the line; the other rank exits 0 without output."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    p = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                        "--nproc-per-node", "2", "--master-addr", "127.0.0.1", "--master-port",
                        str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--gpus", "2", "--steps", "3", "--warmup", "3", "--pairs", "65536"],
                       capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0


def test_reference_arms_stream_a_range_of_cells(built_lib, oracle):
    """The C3 baseline's arms (refarm.Arms.stream_cells_for): cells taken in order from a
    shared queue and streamed whole through the reference's count_pairs22; with a generous
    bound every cell finishes and the summed node and leaf counts equal the oracle's."""
    import refarm
    if not refarm.available():
        pytest.skip("oracle/_ref/libref.so was not built here (the reference sources are absent)")
    from bs45_quantum_explorer_gb300.cells import cell_list
    n, sig = 20, (1, 9, 0, 0)  # 1 + 81 = 4n + 2
    cells, kept, _, m = cell_list(n, sig, m6=True, thm211b=True, thm212=True)
    live = [cells[i] for i in range(len(kept)) if kept[i]][:12]
    todo = [(list(c.tx[:m]), list(c.ty[:m]), c.pinX, c.pinY) for c in live]
    arms = refarm.Arms(3, n, sig)
    try:
        r = arms.stream_cells_for(todo, 120.0, m=m)
    finally:
        arms.close()
    assert r["cells_done"] == len(todo)
    want_nodes = want_leaves = 0
    for tx, ty, px, py in todo:
        _, _, st = oracle.cd_stream(n, tx, ty, m=m, pinX=bool(px), pinY=bool(py))
        want_nodes += st["nodes"]
        want_leaves += st["leaves"]
    assert (r["nodes"], r["leaves"]) == (want_nodes, want_leaves)
