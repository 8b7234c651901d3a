"""Serving first-hit jobs on one GPU: continuous batching of (n, signature, cell range) lanes.

The reference serves this load as SLURM lanes, one process per (n, signature, cell range) on
one CPU core each (cluster/deploy/cluster_firsthit_probe.sh). Here a job is one lane over a
contiguous raw cell range (lane.run_lane) and one server runs many of them on one GPU:

  - a fixed set of slots, each a host thread with its own GPU context: its own CUDA stream and
    device buffers (frontier and suspended DFS walks, leaf and survivor buffers, completer
    stacks). A slot keeps its context across jobs and retargets it (bs_ctx_retarget), so the
    buffers stay resident and a job allocates only when it needs a buffer larger than any
    job before it on that slot (the buffer then grows once);
  - admission by HBM footprint: a job starts when a slot is free, its estimated device
    footprint fits the budget beside the jobs already running, and that many bytes are free
    on the device as the driver reports them (the estimate alone cannot see a buffer that
    grows); a job that arrives while others run is admitted as soon as that holds (first
    fitting job in arrival order);
  - jobs on different slots overlap on the device (different streams).
A job's result does not depend on what runs beside it: the stream, the keep and the
completions are deterministic per job, so its counts and its quad equal its run alone.
"""
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from .hall import Context
from .lane import LaneResult, lane_list, run_lane

# device bytes a slot holds whatever it runs: leaf buffer (2^24 leaves x 25 B), survivor
# buffer (2^22 x 24 B), suspended walks, Hall scratch, completer outer tables and counters
SLOT_BASE_BYTES = (1 << 24) * 25 + (1 << 22) * 24 + 2 * 233472 * 32 + (64 << 20)


@dataclass
class Job:
    jid: int
    n: int
    sig: tuple
    skip: int                      # raw cells [skip, end) of the ORDER=3 list
    end: int
    budget: int = 1 << 22          # A,B nodes per candidate
    buf_cap: int = 500000
    drain_top: int = 50000
    drain_batches: int = 1
    arrival: float = 0.0           # seconds after the trace starts
    # filled by the server
    slot: int = -1
    admitted: float = None
    finished: float = None
    result: LaneResult = None
    error: str = None

    def footprint(self):
        """Device bytes the job adds to its slot: survivors of the front-only cut (words,
        keys, order and scores) and the completer's per-candidate state for one chunk."""
        surv = min(self.buf_cap * self.drain_batches, 1 << 22)
        return surv * 40 + 65536 * 64

    @property
    def latency(self):
        return None if self.finished is None else self.finished - self.arrival


@dataclass
class ServeStats:
    jobs: int = 0
    makespan_s: float = 0.0
    cells: int = 0
    dfs_nodes: int = 0
    ab_nodes: int = 0
    p50_s: float = 0.0
    p99_s: float = 0.0
    latencies: list = field(default_factory=list)

    def as_dict(self):
        d = dict(self.__dict__)
        d.pop("latencies")
        d["cells_per_s"] = self.cells / self.makespan_s if self.makespan_s else 0.0
        d["dfs_nodes_per_s"] = self.dfs_nodes / self.makespan_s if self.makespan_s else 0.0
        d["ab_nodes_per_s"] = self.ab_nodes / self.makespan_s if self.makespan_s else 0.0
        return d


class Server:
    def __init__(self, slots=4, hbm_budget=None, device=0, lane_opts=None, runner=None,
                 mem_probe=None):
        """runner(slot_index, job) -> LaneResult replaces the GPU lane (host-side tests of
        the admission and queueing logic); hbm_budget defaults to 80% of the free memory.

        mem_probe() -> (free, total) device bytes as the driver reports them (by default
        cudaMemGetInfo through torch; none with a runner unless given). Admission then also
        needs the job's footprint free on the device: the footprint is an estimate, and a
        slot's buffers grow when a job needs more than the slot has held, so the measured free
        memory is checked as well. The largest measured use is reported (peak_device_used)."""
        if mem_probe is None and runner is None:
            import torch
            mem_probe = lambda: torch.cuda.mem_get_info(device)  # noqa: E731
        self._mem_probe = mem_probe
        if hbm_budget is None:
            free, _ = mem_probe()
            hbm_budget = int(0.8 * free)
        self.hbm_budget = hbm_budget
        self._runner = runner
        self.peak_in_use = 0
        self.peak_device_used = 0
        self.waits_on_device_memory = 0  # admissions held back by the measured check
        if slots * SLOT_BASE_BYTES > self.hbm_budget:
            raise ValueError(f"{slots} slots need {slots * SLOT_BASE_BYTES} B, budget {self.hbm_budget} B")
        self.device = device
        self.lane_opts = dict(lane_opts or {})
        self.nslots = slots
        self._cv = threading.Condition()
        self._pending = []          # arrived, not admitted, in arrival order
        self._in_use = slots * SLOT_BASE_BYTES
        self._closing = False
        self._threads = []
        self._t0 = None
        self._list_locks = {}
        self.done = []

    # ---- lifecycle ----
    def start(self):
        self._t0 = time.perf_counter()
        for k in range(self.nslots):
            t = threading.Thread(target=self._slot_main, args=(k,), daemon=True)
            t.start()
            self._threads.append(t)

    def now(self):
        return time.perf_counter() - self._t0

    def submit(self, job):
        with self._cv:
            if self.nslots * SLOT_BASE_BYTES + job.footprint() > self.hbm_budget:
                # it would never fit: refuse it now rather than hold the queue
                job.error = "footprint exceeds the HBM budget"
                job.admitted = job.finished = self.now()
                self.done.append(job)
                return
            self._pending.append(job)
            self._cv.notify_all()

    def close(self):
        with self._cv:
            self._closing = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()

    # ---- admission: first pending job, in arrival order, whose footprint fits ----
    def _measured_free(self):
        """Free device bytes now (None without a probe); records the peak measured use."""
        if self._mem_probe is None:
            return None
        free, total = self._mem_probe()
        self.peak_device_used = max(self.peak_device_used, total - free)
        return free

    def _take(self):
        with self._cv:
            while True:
                free = self._measured_free() if self._pending else None
                for i, job in enumerate(self._pending):
                    if self._in_use + job.footprint() <= self.hbm_budget:
                        if free is not None and free < job.footprint():
                            self.waits_on_device_memory += 1
                            continue
                        self._pending.pop(i)
                        self._in_use += job.footprint()
                        self.peak_in_use = max(self.peak_in_use, self._in_use)
                        job.admitted = self.now()
                        return job
                if self._closing and not self._pending:
                    return None
                self._cv.wait(timeout=0.05)

    def _release(self, job):
        with self._cv:
            self._measured_free()
            self._in_use -= job.footprint()
            self.done.append(job)
            self._cv.notify_all()

    def _listing(self, job):
        key = (job.n, job.sig)
        with self._cv:
            lock = self._list_locks.setdefault(key, threading.Lock())
        with lock:  # one build per list; other slots wait for it
            return serving_list(job.n, job.sig, **self.lane_opts)

    def _slot_main(self, k):
        ctx = None
        while True:
            job = self._take()
            if job is None:
                break
            job.slot = k
            try:
                if self._runner is not None:
                    job.result = self._runner(k, job)
                elif ctx is None:
                    ctx = Context(job.n, job.sig, device=self.device)
                if self._runner is None:
                    if ctx.n != job.n or ctx.sig != tuple(job.sig):
                        ctx.retarget(job.n, job.sig)
                    job.result = run_job(ctx, job, self._listing(job), **self.lane_opts)
            except Exception as e:  # a failed job is reported, the slot keeps serving
                job.error = f"{type(e).__name__}: {e}"
            job.finished = self.now()
            self._release(job)
        if ctx is not None:
            ctx.close()

    # ---- a whole trace ----
    def run_trace(self, jobs):
        """Submits each job at its arrival time (seconds after start), waits for all, and
        returns (jobs in submission order, ServeStats)."""
        self.start()
        for job in sorted(jobs, key=lambda j: j.arrival):
            delay = job.arrival - self.now()
            if delay > 0:
                time.sleep(delay)
            self.submit(job)
        self.close()
        return jobs, summarize(jobs, self.now())


LIST_KEYS = ("endpos", "orbit_q", "qprune")


def serving_list(n, sig, **lane_opts):
    """The cell list a served job's raw range indexes: mod-6 cells with 2.11b and 2.12, orbit
    canon with the quad switch and its Q-closure prune, ORDER=3 (the production lane's list)."""
    o = {k: lane_opts[k] for k in LIST_KEYS if k in lane_opts}
    return lane_list(n, sig, m6=True, thm211b=True, thm212=True, endpos=o.get("endpos", False),
                     orbit_canon=True, orbit_q=o.get("orbit_q", 1), qprune=o.get("qprune", True),
                     prof_order=3)


def run_job(ctx, job, listing=None, **lane_opts):
    """One job alone on a context: the lane over its range."""
    if listing is None:
        listing = serving_list(job.n, job.sig, **lane_opts)
    opts = {k: v for k, v in lane_opts.items() if k not in LIST_KEYS}
    return run_lane(ctx, job.n, job.sig, skip=job.skip, end=job.end, budget=job.budget,
                    buf_cap=job.buf_cap, drain_top=job.drain_top,
                    drain_batches=job.drain_batches, listing=listing,
                    endpos=lane_opts.get("endpos", False), **opts)


def summarize(jobs, makespan):
    st = ServeStats(jobs=len(jobs), makespan_s=makespan)
    for j in jobs:
        if j.result is None:
            continue
        r = j.result
        st.cells += r.cells_done
        st.dfs_nodes += r.dfs_nodes
        st.ab_nodes += r.total_ab_nodes
        st.latencies.append(j.latency)
    if st.latencies:
        st.p50_s = float(np.percentile(st.latencies, 50))
        st.p99_s = float(np.percentile(st.latencies, 99))
    return st


def result_key(r):
    """What must not change between a job's run alone and in a mix."""
    quad = None if r.quad is None else tuple(tuple(int(v) for v in x) for x in r.quad)
    return (r.found, r.hit_idx, r.profile_rank, quad, r.nodes_this_cand, r.candidates_streamed,
            r.pre_filter_rejected, r.clean_no_ab, r.budget_aborted, r.total_ab_nodes,
            r.backtracks_entered, r.cells_done, r.cells_orbit_dup, r.cells_prof_dead,
            r.cells_prof_uncap, r.cells_empty, r.cells_capped, r.dfs_nodes)


def poisson_trace(nj, rate, seed, n_range=(20, 42), max_cells=4096, tail_n42=0, classes=None,
                  ncells_of=None, **job_kw):
    """A seeded Poisson stream of jobs: n uniform in n_range, a signature drawn from
    classes(n), a contiguous raw range of 1..max_cells cells at a seeded start, plus
    `tail_n42` n = 42 ranges at the end. ncells_of(n, sig) gives the list length."""
    rng = np.random.default_rng(seed)
    jobs, t = [], 0.0
    for k in range(nj + tail_n42):
        t += float(rng.exponential(1.0 / rate))
        n = 42 if k >= nj else int(rng.integers(n_range[0], n_range[1] + 1))
        cls = classes(n)
        sig = tuple(cls[int(rng.integers(0, len(cls)))])
        total = ncells_of(n, sig)
        width = int(rng.integers(1, max_cells + 1))
        width = min(width, total)
        skip = int(rng.integers(0, total - width + 1))
        jobs.append(Job(jid=k, n=n, sig=sig, skip=skip, end=skip + width, arrival=t, **job_kw))
    return jobs
