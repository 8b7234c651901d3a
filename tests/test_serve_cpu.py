"""Serving logic on the host (serve.Server with a stand-in runner, no GPU): admission by HBM
footprint never oversubscribes the budget, a job that arrives while others run is admitted
once room frees up, every job finishes, a job that can never fit is refused, latencies are
measured from arrival, and the seeded Poisson trace is reproducible."""
import threading
import time

import pytest


def _server(budget_slots_extra, slots, runner):
    from bs45_quantum_explorer_gb300.serve import SLOT_BASE_BYTES, Server
    return Server(slots=slots, hbm_budget=slots * SLOT_BASE_BYTES + budget_slots_extra,
                  runner=runner)


def test_admission_respects_the_hbm_budget_and_finishes_every_job():
    from bs45_quantum_explorer_gb300.lane import LaneResult
    from bs45_quantum_explorer_gb300.serve import Job
    lock = threading.Lock()
    live, peak = [0], [0]
    jobs = [Job(jid=i, n=20, sig=(1, 5, 2, 6), skip=0, end=1, buf_cap=[1000, 200000, 50000][i % 3],
                drain_batches=1, arrival=0.01 * i) for i in range(30)]
    extra = max(j.footprint() for j in jobs) * 2  # room for about two large jobs at once

    def runner(slot, job):
        with lock:
            live[0] += job.footprint()
            peak[0] = max(peak[0], live[0])
        time.sleep(0.02)
        with lock:
            live[0] -= job.footprint()
        return LaneResult(cells_done=1, total_ab_nodes=job.jid)

    srv = _server(extra, 4, runner)
    out, st = srv.run_trace(jobs)
    assert all(j.result is not None and j.error is None for j in out)
    assert peak[0] <= extra
    assert srv.peak_in_use <= srv.hbm_budget
    assert st.jobs == 30 and st.cells == 30
    assert all(j.latency >= 0 and j.finished >= j.admitted >= j.arrival - 1e-3 for j in out)
    assert st.p99_s >= st.p50_s > 0


def test_jobs_overlap_when_slots_and_memory_allow():
    from bs45_quantum_explorer_gb300.lane import LaneResult
    from bs45_quantum_explorer_gb300.serve import Job
    lock = threading.Lock()
    live, peak = [0], [0]

    def runner(slot, job):
        with lock:
            live[0] += 1
            peak[0] = max(peak[0], live[0])
        time.sleep(0.05)
        with lock:
            live[0] -= 1
        return LaneResult()

    jobs = [Job(jid=i, n=20, sig=(1, 5, 2, 6), skip=0, end=1, buf_cap=1000, arrival=0.0) for i in range(8)]
    srv = _server(10 ** 9, 3, runner)
    srv.run_trace(jobs)
    assert peak[0] == 3  # three slots busy at once


def test_a_job_that_can_never_fit_is_refused():
    from bs45_quantum_explorer_gb300.lane import LaneResult
    from bs45_quantum_explorer_gb300.serve import Job
    big = Job(jid=0, n=20, sig=(1, 5, 2, 6), skip=0, end=1, buf_cap=1 << 22)
    small = Job(jid=1, n=20, sig=(1, 5, 2, 6), skip=0, end=1, buf_cap=10, arrival=0.01)
    srv = _server(small.footprint() + 1, 1, lambda k, j: LaneResult())
    out, _ = srv.run_trace([big, small])
    assert big.error and big.result is None
    assert small.error is None and small.result is not None


def test_poisson_trace_is_seeded():
    from bs45_quantum_explorer_gb300.serve import poisson_trace
    classes = lambda n: [(1, 3, 2, 6), (3, 3, 4, 4)]
    kw = dict(nj=20, rate=5.0, seed=11, n_range=(20, 26), max_cells=64, tail_n42=3, classes=classes,
              ncells_of=lambda n, s: 1000 + n)
    a, b = poisson_trace(**kw), poisson_trace(**kw)
    assert [(j.n, j.sig, j.skip, j.end, j.arrival) for j in a] == [(j.n, j.sig, j.skip, j.end, j.arrival) for j in b]
    assert all(j.n == 42 for j in a[-3:]) and all(20 <= j.n <= 26 for j in a[:-3])
    assert all(0 <= j.skip < j.end <= 1000 + j.n and j.end - j.skip <= 64 for j in a)
    assert all(x.arrival < y.arrival for x, y in zip(a, a[1:]))


def test_admission_waits_for_measured_device_memory():
    """The footprint is an estimate: a job is also held until the driver reports its footprint
    free on the device. A fake probe reports room for the first job only until it finishes
    (as when a buffer grew), so the second job, which fits the budget, waits for it; the peak
    measured use is recorded."""
    from bs45_quantum_explorer_gb300.lane import LaneResult
    from bs45_quantum_explorer_gb300.serve import SLOT_BASE_BYTES, Job, Server
    first_done = threading.Event()
    order = []
    jobs = [Job(jid=0, n=20, sig=(1, 5, 2, 6), skip=0, end=1, buf_cap=1000, arrival=0.0),
            Job(jid=1, n=20, sig=(1, 5, 2, 6), skip=0, end=1, buf_cap=1 << 20, arrival=0.01)]
    assert jobs[0].footprint() < jobs[1].footprint()
    total = 1 << 36
    busy = total - (jobs[0].footprint() + (1 << 20))  # leaves room for job 0 only

    def probe():
        used = 1 << 20 if first_done.is_set() else busy
        return total - used, total

    def runner(slot, job):
        order.append(("start", job.jid))
        time.sleep(0.05)
        order.append(("end", job.jid))
        if job.jid == 0:
            first_done.set()
        return LaneResult()

    srv = Server(slots=2, hbm_budget=2 * SLOT_BASE_BYTES + (1 << 34), runner=runner, mem_probe=probe)
    out, _ = srv.run_trace(jobs)
    assert all(j.result is not None and j.error is None for j in out)
    assert order.index(("end", 0)) < order.index(("start", 1))
    assert srv.waits_on_device_memory > 0
    assert srv.peak_device_used == busy
