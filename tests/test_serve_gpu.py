"""Serving on the GPU (serve.Server): a seeded Poisson mix of first-hit jobs runs on three
slots at once, each job's result (counts, first hit, quad) is identical to its run alone on
one context, the jobs really overlapped on the device, and every emitted quad passes the exact
integer NPAF check."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.gpu


def _classes(n):
    from test_stream_gpu import _classes as cl
    return cl(n)


def _trace():
    from bs45_quantum_explorer_gb300.serve import poisson_trace, serving_list
    return poisson_trace(nj=10, rate=40.0, seed=0xB545, n_range=(18, 24), max_cells=24, tail_n42=0,
                         classes=lambda n: _classes(n)[:2],
                         ncells_of=lambda n, s: len(serving_list(n, s)[1]),
                         budget=1 << 12, buf_cap=400, drain_top=8)


def test_jobs_in_a_mix_equal_their_runs_alone(gpu, oracle):
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.serve import Server, result_key, run_job
    jobs = _trace()
    alone = {}
    ctx = None
    for j in jobs:
        if ctx is None:
            ctx = Context(j.n, j.sig)
        else:
            ctx.retarget(j.n, j.sig)
        alone[j.jid] = result_key(run_job(ctx, j))
    ctx.close()
    mix = _trace()
    srv = Server(slots=3)
    out, st = srv.run_trace(mix)
    assert all(j.error is None for j in out), [j.error for j in out if j.error]
    for j in out:
        assert result_key(j.result) == alone[j.jid], j.jid
    # the work overlapped: some pair of jobs ran at the same time
    iv = sorted((j.admitted, j.finished) for j in out)
    assert any(b[0] < a[1] for a, b in zip(iv, iv[1:]))
    assert st.p99_s >= st.p50_s > 0
    for j in out:
        if j.result.found:
            A, B, C, D = (np.asarray(x, np.int8) for x in j.result.quad)
            for s in range(1, j.n + 1):
                assert oracle.npaf_at(A, B, C, D, s) == 0
