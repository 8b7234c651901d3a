"""Stopping device work from the host: the context's stop flag (SIGTERM in the lane) and the
stream's wall limit (WZ_FH_WALL_SEC). The reference polls g_fh_sigterm and its wall clock
inside the DFS (src/solver/wz_match.cpp:640-653, 712-718) because an arm that ignored SIGTERM
inside a long cell hung its lane driver past walltime; here the flag is mapped host memory
that the stream's host loop reads between launches (each at most 25 ms) and the completer's
warps read every 1,024 steps. A stopped call returns the part it completed, which must be
exactly what the unstopped call returns for that part."""
import os
import signal
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

CELL42 = ([-1, -1, 1, 1, 1, -1], [-1, -3, 1, 1, 3, -1])  # n = 42, sig (7,11,0,0): > 10^13 nodes


def _stop_after(ctx, seconds):
    t = threading.Timer(seconds, ctx.request_stop)
    t.start()
    return t


def test_stream_stops_within_a_round(gpu):
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.stream import cd_stream
    ctx = Context(42, (7, 11, 0, 0))
    cd_stream(ctx, [CELL42], m=6, as_words=True, limit=100)  # warm-up
    timer = _stop_after(ctx, 0.5)
    t0 = time.perf_counter()
    # bounded even if the flag were ignored: 2,000,000 survivors take about a minute
    part, _, st = cd_stream(ctx, [CELL42], m=6, as_words=True, limit=2000000)
    dt = time.perf_counter() - t0
    timer.join()
    ctx.clear_stop()
    assert st[0].get("stopped", 0) == 1
    assert dt < 0.5 + 0.5, dt  # the flag is seen after the launch in flight (<= 25 ms)
    # the survivors returned are the stream's first ones, in order
    assert 0 < len(part) < 2000000
    ref, _, st2 = cd_stream(ctx, [CELL42], m=6, as_words=True, limit=len(part))
    assert st2[0].get("stopped", 0) == 0
    assert np.array_equal(part, ref)
    ctx.close()


def test_stream_wall_limit(gpu):
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.stream import cd_stream
    ctx = Context(42, (7, 11, 0, 0))
    # a wall far below one launch: the stream is abandoned at its first check
    part, _, st = cd_stream(ctx, [CELL42], m=6, as_words=True, limit=200000, wall_sec=1e-4)
    assert st[0].get("stopped", 0) == 2
    if len(part):
        ref, _, _ = cd_stream(ctx, [CELL42], m=6, as_words=True, limit=len(part))
        assert np.array_equal(part, ref)
    # a wall that survivors keep resetting: the stream completes as without one
    full, _, st = cd_stream(ctx, [CELL42], m=6, as_words=True, limit=20000, wall_sec=30.0)
    ref, _, _ = cd_stream(ctx, [CELL42], m=6, as_words=True, limit=20000)
    assert st[0].get("stopped", 0) == 0 and np.array_equal(full, ref)
    ctx.close()


def test_completer_stops_and_keeps_finished_verdicts(gpu):
    from bs45_quantum_explorer_gb300.cells import ab_rows
    from bs45_quantum_explorer_gb300.complete import complete_ab
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.lane import lane_list
    from bs45_quantum_explorer_gb300.stream import cd_stream
    n, sig = 36, (5, 11, 0, 0)
    cells, kept, _, m = lane_list(n, sig)
    pi = 158597  # the first kept cell of the first-hit workload's window
    assert kept[pi]
    c = cells[pi]
    rows, off, nr = ab_rows(n, sig, m, [c])
    ctx = Context(n, sig)
    cand, _, _ = cd_stream(ctx, [(list(c.tx[:m]), list(c.ty[:m]))], m=m, limit=16384)
    r = rows[off[0]:off[0] + nr[0]]
    want, wnodes, _, _ = complete_ab(ctx, cand, 1 << 22, rows=r, m=m)
    t0 = time.perf_counter()
    full_s = None
    timer = _stop_after(ctx, 0.05)
    got, gnodes, _, _ = complete_ab(ctx, cand, 1 << 22, rows=r, m=m)
    dt = time.perf_counter() - t0
    timer.join()
    ctx.clear_stop()
    t1 = time.perf_counter()
    complete_ab(ctx, cand, 1 << 22, rows=r, m=m)
    full_s = time.perf_counter() - t1
    done = got >= 0
    assert (~done).any(), "the flag came after the batch finished: make the batch longer"
    assert dt < full_s, (dt, full_s)
    assert np.array_equal(got[done], want[done]) and np.array_equal(gnodes[done], wnodes[done])
    ctx.close()


def test_lane_binary_exits_on_sigterm_mid_cell(gpu):
    """The lane at the first-hit workload's production settings, SIGTERM while it streams or
    completes its first cell: it exits 3 with the INTERRUPTED result line within a second or
    two and leaves a checkpoint at the cell it was in."""
    from test_lane_gpu import _bin
    from make_lane_golden import BASE
    exe = _bin()
    settings = dict(BASE, WZ_FH_ORBIT_CANON=1, WZ_FH_ORBIT_Q=1, WZ_FH_ORBIT_QPRUNE=1,
                    WZ_FH_PROF_ORDER=3, WZ_FH_AB_BUDGET=1 << 22, WZ_FH_BUF_CAP=500000,
                    WZ_FH_DRAIN_TOP=50000, WZ_FH_PROF_SKIP=158570, WZ_FH_PROF_END=162666,
                    WZ_FH_ORD3_NODIGEST_OK=1)
    env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
    env.update({k: str(v) for k, v in settings.items()})
    with tempfile.TemporaryDirectory() as ck:
        env["WZ_FH_CKPT_DIR"] = ck
        p = subprocess.Popen([exe, "36", "5", "11", "0", "0"], env=env, stdout=subprocess.PIPE,
                             stderr=subprocess.PIPE, text=True)
        time.sleep(8.0)  # list build and context, then the first cell's work
        assert p.poll() is None, p.communicate()[0][-2000:]
        t0 = time.perf_counter()
        p.send_signal(signal.SIGTERM)
        try:
            out, _ = p.communicate(timeout=30)
        except subprocess.TimeoutExpired:
            p.kill()
            raise
        dt = time.perf_counter() - t0
        assert p.returncode == 3, out[-2000:]
        assert "RESULT: INTERRUPTED (SIGTERM)" in out
        assert dt < 3.0, dt
        ckpts = os.listdir(ck)
        assert ckpts and "resume_pi=" in open(os.path.join(ck, ckpts[0])).read()
