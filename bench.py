#!/usr/bin/env python3
"""Benchmark: the Thm 2.4 spectral (Hall) filter at n = 42 on 2^24 C,D pairs.

The metric is spectral-filtered C,D candidates per second with zero false rejects (the
reference's hall_ok_pair_fast decision on every pair, src/solver/wz_match.cpp:143-168). One
step filters one batch of 2^24 seeded synthetic pairs (half i.i.d. +-1, half mirror-quad
pairs with sum C = sum D = 0) resident in HBM (268 MB of packed words, larger than L2).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Rank 0 prints one JSON line. --impl reference times the reference's own filter on all host
cores over the same 2^24-pair batch: its default predicate hall_ok_pair_fast from
src/solver/wz_match.cpp compiled unmodified into oracle/_ref/libref.so (one arm per core, as
the reference's lanes run), or, where that library was not built, the oracle restatement.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N = 42
SIG = (7, 11, 0, 0)
SEED = 0xB545C2
FLOPS_PER_PAIR = 800 * N * 2  # 4 DFT terms x n MACs x 200 angles, counted once
METRIC = "spectral-filtered C,D cands/s at n=42 (0 false rejects)"
UNIT = "pairs/s"


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return p, "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


def load_traffic():
    """DRAM bytes per Hall filter step (screen + full test) from the committed ncu figure."""
    path = os.path.join(ROOT, "profiles", "hall_filter_n42_traffic.txt")
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].strip().split()[0])
    except Exception:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms in the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    pyoracle.build()
    return pyoracle


def _ref_arms(narms, n=N, sig=SIG):
    """The reference's own code as `narms` single-threaded arms (oracle/refarm.py), or None
    when oracle/_ref/libref.so was not built on this machine."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import refarm
    return refarm.Arms(narms, n, sig) if refarm.available() else None


def cpu_hall_rate(nthreads, words, target_s=10.0):
    """The reference's Hall filter on all host cores over the whole 2^24-pair batch, repeated
    until about target_s of work is timed. Returns (pairs/s, pairs filtered, cores, seconds,
    kind, sample, pass mask of one pass)."""
    arms = _ref_arms(nthreads)
    if arms is not None:
        mask = np.zeros(len(words), np.uint8)
        arms.hall_fast(words[: 1 << 16])  # the arms' angle orders adapt, as in a running lane
        done, dt, reps = 0, 0.0, 0
        while dt < target_s:
            _, t = arms.hall_fast(words, out=mask if reps == 0 else None)
            done += len(words)
            dt += t
            reps += 1
        arms.close()
        return (done / dt, done, nthreads, dt, "reference",
                f"the whole {len(words)}-pair batch x{reps} through hall_ok_pair_fast "
                f"(src/solver/wz_match.cpp compiled unmodified, {nthreads} single-threaded arms, "
                f"{dt:.1f} s)", mask)
    pyoracle = _oracle()
    from bs45_quantum_explorer_gb300.workloads import unpack_pairs
    X = unpack_pairs(words, N)
    done, dt, mask = 0, 0.0, None
    while dt < target_s:
        t0 = time.perf_counter()
        got = pyoracle.hall_batch(N, X, nthreads=nthreads)
        dt += time.perf_counter() - t0
        mask = got if mask is None else mask
        done += len(words)
    return (done / dt, done, nthreads, dt, "port",
            f"the whole {len(words)}-pair batch through the oracle restatement ({dt:.1f} s, all threads)",
            mask)


def cpu_search_rate(ncpu, cell, seconds=10.0):
    """The reference's C,D stream (count_pairs22 with hall_ok_pair_fast at the leaves,
    src/solver/wz_match.cpp:678-784) on all host cores: every arm streams the same n = 42 cell
    from its start for `seconds`, the same stretch of the DFS that the GPU search covers, so
    the sum over arms is the reference's nodes/s on this workload."""
    arms = _ref_arms(ncpu)
    if arms is None:
        return {"unavailable": "oracle/_ref/libref.so was not built on this machine"}
    r = arms.stream_for([cell] * ncpu, seconds)
    arms.close()
    return {"value": r["nodes"] / r["seconds"], "unit": "DFS nodes/s", "cores": ncpu,
            "kind": "reference", "leaves_per_s": r["leaves"] / r["seconds"],
            "sample": f"{ncpu} single-threaded arms of count_pairs22 (src/solver/wz_match.cpp "
                      f"compiled unmodified), each streaming the cell from its start for "
                      f"{seconds:.0f} s ({r['nodes']} nodes, {r['leaves']} leaves, "
                      f"{r['survivors']} survivors in all)"}


def run_reference(args, rank, world):
    if rank != 0:
        return
    import numpy as np
    ncpu = os.cpu_count() or 1
    pyoracle = _oracle()
    w = pyoracle.gen_hall_pairs(N, args.pairs, seed=SEED, nthreads=ncpu)  # the same batch as ours
    arms = _ref_arms(ncpu)
    conj = None
    if arms is not None:
        kind = "reference"
        what = (f"hall_ok_pair_fast, the reference's default predicate (src/solver/wz_match.cpp "
                f"compiled unmodified), {ncpu} single-threaded arms, each on 1/{ncpu} of the batch")

        def step():
            arms.hall_fast(w)
        # the WZ_FH_HALL_FAST=0 conjunction under OpenMP, once, for the record
        nconj = min(len(w), 1 << 20)
        _, tc = arms.hall_conj(w[:nconj], ncpu)
        conj = {"value": nconj / tc, "unit": UNIT, "threads": ncpu,
                "sample": f"the first {nconj} pairs of the batch",
                "predicate": "hall_ok_single(X) && hall_ok_single(Y) && hall_ok(X,Y) (WZ_FH_HALL_FAST=0)"}
    else:
        kind = "port"
        what = "the oracle restatement of the reference's FP64 test (oracle/_ref not built here), all threads"
        from bs45_quantum_explorer_gb300.workloads import unpack_pairs
        X = unpack_pairs(w, N)

        def step():
            pyoracle.hall_batch(N, X, nthreads=ncpu)
    for _ in range(args.warmup):
        step()
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step()
        times.append(time.perf_counter() - t0)
    if arms is not None:
        arms.close()
    total = sum(times)
    npairs = len(w)
    value = npairs * args.steps / total
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": "hall_filter_n42_2^24_pairs", "n": N, "sig": list(SIG),
                   "pairs_per_step": npairs, "sample": f"the whole {npairs}-pair batch every step"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": ncpu, "kind": kind, "sample": what},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "p50_ms": 1e3 * statistics.median(times),
        "p99_ms": 1e3 * sorted(times)[min(len(times) - 1, int(0.99 * len(times)))],
    }
    if conj:
        line["hall_fast_0_conjunction"] = conj
    print(json.dumps(line), flush=True)


# Built-in cells of the ORDER=3 lists (orbit canon + quad switch): (n, sig, px, py, raw index)
STREAM_CELLS = {
    "n30": (30, (1, 7, 6, 6), [-1, 1, 1, 1, 1, 3], [-1, 1, 1, 1, 5, -1], 3005),
    "n42": (42, (7, 11, 0, 0), [-1, -1, 1, 1, 1, -1], [-1, -3, 1, 1, 3, -1], 3056),
}


def run_stream_only(args):
    """Stream one cell (the DFS, the Hall filter of its leaves and the ordering) and print
    the per-cell counts and rates."""
    import torch
    from bs45_quantum_explorer_gb300 import build_library
    build_library()
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.stream import cd_stream
    n, sig, px, py, pi = STREAM_CELLS[args.stream_only]
    limit = args.limit if args.limit is not None else (0 if n <= 30 else 500000)
    ctx = Context(n, sig)
    cd_stream(ctx, [(px, py)], m=6, as_words=True, limit=min(limit, 1000) if limit else 0)  # warm-up
    torch.cuda.synchronize()
    ctx.timing(True)
    t0 = time.perf_counter()
    surv, _, st = cd_stream(ctx, [(px, py)], m=6, as_words=True, limit=limit)
    dt = time.perf_counter() - t0
    kms, kl, _ = ctx.timing_read()
    what = "whole cell" if not limit else f"first {limit} survivors (front-only cut)"
    print(json.dumps({"workload": f"C,D stream, n={n} sig={sig} raw cell {pi} px={px} py={py}, {what}",
                      "dfs_nodes": st[0]["nodes"], "leaves": st[0]["leaves"], "survivors": len(surv),
                      "seconds": dt, "nodes_per_s": st[0]["nodes"] / dt, "device_kernel_ms": kms,
                      "timed_launches": kl}), flush=True)
    ctx.close()


# ---- first-hit pipeline at n = 36: a seeded window of 4096 raw cells ----
FH_N, FH_SIG = 36, (5, 11, 0, 0)


def _classes(n):
    out = []
    for a in range((n + 1) % 2, n + 2, 2):
        for b in range(a, n + 2, 2):
            for c in range(n % 2, n + 1, 2):
                rest = 4 * n + 2 - a * a - b * b - c * c
                if rest < c * c:
                    break
                d = int(round(rest ** 0.5))
                if d * d == rest and d >= c and (d - n) % 2 == 0:
                    out.append((a, b, c, d))
    return out


def run_first_hit(seconds, cpu_seconds=10.0, with_cpu=True, drain_top=50000, tune=True):
    """One production lane (orbit canon + quad switch + Q-prune, ORDER=3; budget 2^22,
    BUF_CAP 500,000, DRAIN_TOP 50,000) over raw cells [s, s+4096) of n = 36, sig (5,11,0,0),
    s drawn from the seed; stopped between cells after `seconds`. Reports the completer's
    A,B nodes/s (the reference's node definition) on the device and through the API, the
    stream's DFS nodes/s, and the oracle completer on the same candidates on one host core."""
    import numpy as np
    import torch
    from bs45_quantum_explorer_gb300.complete import flat_topk
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.serve import serving_list
    from bs45_quantum_explorer_gb300.lane import run_lane
    from bs45_quantum_explorer_gb300.stream import cd_stream
    t0 = time.perf_counter()
    listing = serving_list(FH_N, FH_SIG)
    list_s = time.perf_counter() - t0
    cells, kept, digest, m = listing
    rng = np.random.default_rng(SEED)
    s = int(rng.integers(0, len(kept) - 4096))
    ctx = Context(FH_N, FH_SIG)
    kw = dict(budget=1 << 22, buf_cap=500000, drain_top=drain_top, listing=listing)
    tune_report = None
    if tune:  # work sizes picked by timing probes of this window's first kept cell
        from bs45_quantum_explorer_gb300.tune import tune_lane
        kw["tuning"], tune_report = tune_lane(ctx, FH_N, FH_SIG, listing, s, s + 4096, 1 << 22,
                                              buf_cap=500000, drain_top=drain_top, probe=20000,
                                              sample=2048)
    run_lane(ctx, FH_N, FH_SIG, skip=s, end=s + 1, **kw)  # warm-up: buffers, first cell
    torch.cuda.synchronize()
    res = run_lane(ctx, FH_N, FH_SIG, skip=s, end=s + 4096, max_seconds=seconds, **kw)
    out = {"workload": f"first-hit lane, n={FH_N} sig={FH_SIG}, raw cells [{s}, {s + 4096}) of the "
                       f"ORDER=3 list (digest {digest}, {int(kept[s:s + 4096].sum())} kept cells), "
                       f"budget 2^22, BUF_CAP 500000, DRAIN_TOP {drain_top}",
           "bounded_seconds": seconds, "list_build_s": round(list_s, 2),
           "cells_done": res.cells_done, "cells_orbit_dup": res.cells_orbit_dup,
           "cells_prof_dead": res.cells_prof_dead, "completions": res.completions,
           "ab_nodes": res.total_ab_nodes, "budget_aborted": res.budget_aborted,
           "completer_device_s": res.complete_device_ms * 1e-3, "completer_api_s": res.complete_s,
           "ab_nodes_per_s_device": res.total_ab_nodes / (res.complete_device_ms * 1e-3)
           if res.complete_device_ms > 0 else None,
           "ab_nodes_per_s_api": res.total_ab_nodes / res.complete_s if res.complete_s > 0 else None,
           "dfs_nodes": res.dfs_nodes, "stream_s": res.stream_s,
           "stream_device_s": res.stream_device_ms * 1e-3,
           "gpu_busy_frac": ((res.complete_device_ms + res.stream_device_ms) * 1e-3 /
                             res.timings["wall_s"]) if res.timings.get("wall_s") else None,
           "dfs_nodes_per_s": res.dfs_nodes / res.stream_s if res.stream_s > 0 else None,
           "wall_s": res.timings.get("wall_s"), "found": res.found}
    if tune_report is not None:
        out["autotune"] = {"choice": tune_report.get("choice"), "seconds": tune_report.get("seconds"),
                           "probe_cell": tune_report.get("cell"),
                           "stream_probes": tune_report.get("stream_probes"),
                           "completer_probes": tune_report.get("completer_probes")}
    if res.found:
        out["hit"] = {"idx": res.hit_idx, "profile_rank": res.profile_rank,
                      "quad": [list(map(int, x)) for x in res.quad]}
    if with_cpu:
        # the reference's completer on the first drained candidates of the window's first
        # kept cell, on all host cores (the oracle's on one core where it was not built)
        from bs45_quantum_explorer_gb300.cells import ab_rows
        from bs45_quantum_explorer_gb300.hall import unpack
        pi = next(i for i in range(s, s + 4096) if kept[i])
        c = cells[pi]
        rows, off, nr = ab_rows(FH_N, FH_SIG, m, [c])
        surv, _, _ = cd_stream(ctx, [(list(c.tx[:m]), list(c.ty[:m]))], m=m, as_words=True, limit=500000)
        order, _ = flat_topk(ctx, surv, len(surv), drain_top)
        cand = unpack(surv[order], FH_N)
        r = rows[off[0]:off[0] + nr[0]] if 0 < nr[0] <= 20000 else None
        ncpu = os.cpu_count() or 1
        arms = _ref_arms(ncpu, FH_N, FH_SIG)
        if arms is not None:
            rr = arms.complete_for(cand, 1 << 22, cpu_seconds, rows=r, m=m)
            arms.close()
            out["cpu_baseline"] = {
                "value": rr["nodes"] / rr["seconds"], "unit": "A,B nodes/s", "cores": ncpu,
                "kind": "reference",
                "sample": f"fh_complete_ab (src/solver/wz_match.cpp compiled unmodified) on the "
                          f"first {rr['done']} drained candidates of raw cell {pi}, {ncpu} "
                          f"single-threaded arms ({rr['seconds']:.1f} s, budget 2^22, the cell's "
                          f"allowed rows)"}
        else:
            pyoracle = _oracle()
            nodes, done, t1 = 0, 0, time.perf_counter()
            while done < len(cand) and time.perf_counter() - t1 < cpu_seconds:
                _, nd, _, _ = pyoracle.complete_ab(FH_N, FH_SIG[0], FH_SIG[1], cand[done, 0],
                                                   cand[done, 1], 1 << 22, rows=r, m=m)
                nodes += nd
                done += 1
            dt = time.perf_counter() - t1
            out["cpu_baseline"] = {"value": nodes / dt, "unit": "A,B nodes/s", "cores": 1,
                                   "kind": "port",
                                   "sample": f"the oracle completer on the first {done} drained "
                                             f"candidates of raw cell {pi} ({dt:.1f} s, budget 2^22)"}
    ctx.close()
    return out


def guarded(fn, *a, **kw):
    """One extra leg of the default run: an exception in it is reported in its place, so the
    headline line (measured before the extras) is still printed."""
    try:
        return fn(*a, **kw)
    except Exception as e:  # noqa: BLE001 - any failure of an extra leg
        return {"error": f"{type(e).__name__}: {e}"}


def run_spike(budget=1 << 20, ncand=2048):
    """The reference's own GPU completer (src/solver/gpu/fh_gpu_spike.cu, compiled unmodified
    for sm_103a into oracle/_ref/fh_gpu_spike) beside ours on the same candidates: the first
    `ncand` drained candidates (flattest first) of the first-hit workload's first kept cell,
    at the same node budget. The spike has no allowed rows, no outer-lag tables and no early
    check, so ours runs with those off here too (rows=None, outer_k=0, early=False): the two
    searches then charge the same nodes, which the line checks (verdict histogram and total)."""
    import re
    import subprocess
    import tempfile
    import torch
    from bs45_quantum_explorer_gb300.complete import complete_ab, flat_topk
    from bs45_quantum_explorer_gb300.hall import Context, unpack
    from bs45_quantum_explorer_gb300.serve import serving_list
    from bs45_quantum_explorer_gb300.stream import cd_stream
    exe = os.path.join(ROOT, "oracle", "_ref", "fh_gpu_spike")
    if not os.path.exists(exe):
        return {"unavailable": "oracle/_ref/fh_gpu_spike was not built on this machine"}
    cells, kept, _, m = serving_list(FH_N, FH_SIG)
    rng = np.random.default_rng(SEED)
    s = int(rng.integers(0, len(kept) - 4096))
    pi = next(i for i in range(s, s + 4096) if kept[i])
    c = cells[pi]
    ctx = Context(FH_N, FH_SIG)
    surv, _, _ = cd_stream(ctx, [(list(c.tx[:m]), list(c.ty[:m]))], m=m, as_words=True,
                           pins=[(c.pinX, c.pinY)], limit=500000)
    order, _ = flat_topk(ctx, surv, len(surv), ncand)
    cand = unpack(surv[order[:ncand]], FH_N)
    complete_ab(ctx, cand[:64], budget, outer_k=0, early=False)  # warm-up
    torch.cuda.synchronize()
    ctx.timing(True)
    t0 = time.perf_counter()
    v, nodes, _, _ = complete_ab(ctx, cand, budget, outer_k=0, early=False)
    api_s = time.perf_counter() - t0
    dev_ms, _, _ = ctx.timing_read()
    ctx.close()
    ours_hist = [int((v == k).sum()) for k in range(4)]
    with tempfile.TemporaryDirectory() as tmp:
        dump = os.path.join(tmp, "cands.txt")
        with open(dump, "w") as f:
            for x in cand:
                f.write(" ".join(map(str, x[0])) + " | " + " ".join(map(str, x[1])) + "\n")
        p = subprocess.run([exe, str(FH_N), *map(str, FH_SIG), dump, str(budget), str(ncand), "4"],
                           capture_output=True, text=True, timeout=900)
    out = p.stdout
    ref = {}
    mm = re.search(r"GPU_SPIKE: cpu_cands_per_s=([\d.]+) gpu_cands_per_s=([\d.]+)", out)
    if mm:
        ref["cpu_1core_cands_per_s"], ref["thread_per_cand_cands_per_s"] = float(mm[1]), float(mm[2])
    mm = re.search(r"GPU_SPIKE_V2A_SORTED: cands_per_s=([\d.]+)", out)
    if mm:
        ref["thread_per_cand_sorted_cands_per_s"] = float(mm[1])
    mm = re.search(r"GPU_SPIKE_V2B_WARP: cands_per_s=([\d.]+).*hist (\d+)/(\d+)/(\d+)/(\d+) nodes=(\d+)", out)
    if mm:
        ref["warp_per_cand_cands_per_s"] = float(mm[1])
        ref["hist"] = [int(mm[k]) for k in range(2, 6)]
        ref["nodes"] = int(mm[6])
    total = int(nodes.sum())
    return {"workload": f"the first {ncand} drained candidates (flattest first) of raw cell {pi}, "
                        f"n={FH_N} sig={FH_SIG}, budget {budget}; no allowed rows, no outer-lag "
                        "tables, no early check (the spike's search)",
            "rc": p.returncode, "reference_spike": ref,
            "ours": {"cands_per_s_device": ncand / (dev_ms * 1e-3) if dev_ms > 0 else None,
                     "cands_per_s_api": ncand / api_s, "nodes": total,
                     "nodes_per_s_device": total / (dev_ms * 1e-3) if dev_ms > 0 else None,
                     "hist": ours_hist},
            "same_verdicts": ref.get("hist") == ours_hist,
            "node_rule": "the same charge per placed quad; after a budget abort the reference's "
                         "solver (and ours) charges one more node per ancestor with an eligible "
                         "quad left, which the spike does not, so totals differ by those when "
                         "candidates abort"}


def run_c3(max_cells=0, batch=32, topk=256, workers=3):
    """C3: the full C,D stream at n = 30, sig (1,7,6,6): every kept cell of the ORDER=3 list
    (2.11b + 2.12, orbit canon with the quad switch: 97,141 cells, 7,987 kept) streamed whole,
    with its flattest-256 keep. Batches of `batch` cells go to `workers` host threads, each with
    its own context (own CUDA stream and buffers), so one batch's host work (ordering its
    survivors, the keeps) overlaps the next batch's DFS on the device. Reports DFS nodes/s and
    the stream's algorithmic HBM rate: 32 B per DFS node (a 16 B frontier record written and
    read once) + 16 B per leaf handed to the filter + 24 B per survivor (packed C,D, DFS rank,
    score)."""
    import concurrent.futures as cf
    import torch
    from bs45_quantum_explorer_gb300.cells import cell_list
    from bs45_quantum_explorer_gb300.complete import flat_topk
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.stream import cd_stream
    n, sig = 30, (1, 7, 6, 6)
    cells, kept, digest, m = cell_list(n, sig, m6=True, thm211b=True, thm212=True, orbit_canon=True,
                                       orbit_q=1, qprune=False, prof_order=3)
    live = [i for i in range(len(kept)) if kept[i]]
    if max_cells:
        live = live[:max_cells]
    ctxs = [Context(n, sig) for _ in range(workers)]
    for ctx in ctxs:  # warm-up: buffers of every context
        cd_stream(ctx, [(list(cells[live[0]].tx[:m]), list(cells[live[0]].ty[:m]))], m=m, as_words=True)
    torch.cuda.synchronize()
    batches = [live[b:b + batch] for b in range(0, len(live), batch)]
    free = list(range(workers))
    import threading
    lock = threading.Lock()

    def one(group):
        with lock:
            k = free.pop()
        ctx = ctxs[k]
        try:
            batch_cells = [(list(cells[i].tx[:m]), list(cells[i].ty[:m])) for i in group]
            surv, cidx, st = cd_stream(ctx, batch_cells, m=m, as_words=True, cap=1 << 23,
                                       survivor_cap=1 << 23)
            kept_n = 0
            bounds = np.searchsorted(cidx, np.arange(len(group) + 1))
            for j in range(len(group)):  # each cell's flattest 256 (one batch: the whole cell)
                lo, hi = int(bounds[j]), int(bounds[j + 1])
                if hi > lo:
                    order, _ = flat_topk(ctx, surv[lo:hi], hi - lo, topk)
                    kept_n += len(order)
            return (sum(x["nodes"] for x in st), sum(x["leaves"] for x in st), len(surv), kept_n)
        finally:
            with lock:
                free.append(k)
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        parts = list(ex.map(one, batches))
    dt = time.perf_counter() - t0
    for ctx in ctxs:
        ctx.close()
    nodes = sum(p[0] for p in parts)
    leaves = sum(p[1] for p in parts)
    surv_total = sum(p[2] for p in parts)
    kept_total = sum(p[3] for p in parts)
    alg = 32 * nodes + 16 * leaves + 24 * surv_total
    cpu = c3_reference_rate([cells[i] for i in live], m)
    return {"workload": f"C,D stream n={n} sig={sig}: {len(live)} kept cells of the ORDER=3 list "
                        f"({len(kept)} cells, digest {digest}) streamed whole, flattest-{topk} per cell; "
                        f"batches of {batch} cells on {workers} host threads with their own contexts",
            "cells": len(live), "dfs_nodes": nodes, "leaves": leaves, "survivors": surv_total,
            "kept_topk": kept_total, "seconds": dt, "dfs_nodes_per_s": nodes / dt,
            "filtered_cands_per_s": leaves / dt, "cells_per_s": len(live) / dt,
            "algorithmic_bytes": alg, "algorithmic_gb_per_s": alg / dt / 1e9, "cpu_baseline": cpu}


def c3_reference_rate(cells, m, seconds=20.0, n=30, sig=(1, 7, 6, 6)):
    """The reference's C,D stream (count_pairs22 with hall_ok_pair_fast, wz_match.cpp:678-784)
    over the same kept cells in list order, one single-threaded arm per host core taking the
    next cell from a shared queue, bounded to `seconds` (the cells in flight are cut there):
    DFS nodes/s and whole cells/s, as the reference's arms work through a range."""
    ncpu = os.cpu_count() or 1
    arms = _ref_arms(ncpu, n=n, sig=sig)
    if arms is None:
        return {"unavailable": "oracle/_ref/libref.so was not built on this machine"}
    todo = [(list(c.tx[:m]), list(c.ty[:m]), c.pinX, c.pinY) for c in cells]
    r = arms.stream_cells_for(todo, seconds, m=m)
    arms.close()
    return {"value": r["nodes"] / r["seconds"], "unit": "DFS nodes/s", "cores": ncpu,
            "kind": "reference", "cells_per_s": r["cells_done"] / r["seconds"],
            "sample": f"{ncpu} single-threaded arms of count_pairs22 (src/solver/wz_match.cpp "
                      f"compiled unmodified) over the same kept cells in list order for "
                      f"{r['seconds']:.0f} s: {r['cells_done']} whole cells, {r['nodes']} nodes"}


def run_join(n=24):
    """The full-space exact join (the reference's JOIN22 semantics) for one signature of
    BS(n+1, n): every A,B pair of every mod-3 cell (length n+1) and every C,D pair of every
    cell (length n), streamed on the GPU, then joined on AB[s] = -CD[s] with every match
    verified by the exact NPAF. Reports the counts, the stream and join times and the join
    probe kernel's algorithmic rate (8 B per key inserted + 8 B per probed slot)."""
    import itertools
    import numpy as np
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.stream import cd_stream, join_quads

    def cells(L, total, m=6):
        cnt = [len(range(c, L, m)) for c in range(m)]
        out = []
        for v in itertools.product(*[range(-k, k + 1, 2) for k in cnt[:-1]]):
            last = total - sum(v)
            if abs(last) <= cnt[-1] and (last + cnt[-1]) % 2 == 0:
                out.append(list(v) + [last])
        return out

    sig = _classes(n)[0]
    ctx = Context(n, sig)
    # mod-3 cells: every (A,B) and every (C,D) of the signature falls in exactly one
    ab_cells = [(x, y) for x in cells(n + 1, sig[0], 3) for y in cells(n + 1, sig[1], 3)]
    cd_cells = [(x, y) for x in cells(n, sig[2], 3) for y in cells(n, sig[3], 3)]
    t0 = time.perf_counter()
    ab = np.concatenate([cd_stream(ctx, ab_cells[i:i + 512], m=3, ab_side=True, as_words=True,
                                   cap=1 << 22)[0] for i in range(0, len(ab_cells), 512)])
    cd = np.concatenate([cd_stream(ctx, cd_cells[i:i + 512], m=3, as_words=True, cap=1 << 22)[0]
                         for i in range(0, len(cd_cells), 512)])
    stream_s = time.perf_counter() - t0
    ctx.timing(True)
    t1 = time.perf_counter()
    quads, hits = join_quads(ctx, cd, ab)
    join_s = time.perf_counter() - t1
    probe_ms, _, _ = ctx.timing_read()
    ctx.close()
    slots = 1024
    while slots < 2 * len(cd):
        slots *= 2
    alg = 8 * len(cd) + 8 * len(ab)
    return {"workload": f"full-space join BS({n + 1},{n}) sig={sig}: {len(ab_cells)} A,B cells and "
                        f"{len(cd_cells)} C,D cells, all pairs passing the Thm 2.2-2.4 stream",
            "ab_pairs": int(len(ab)), "cd_pairs": int(len(cd)), "table_slots": slots,
            "key_matches": int(hits), "verified_quads": int(len(quads)),
            "stream_s": stream_s, "join_s": join_s, "probe_kernel_ms": probe_ms,
            "probe_algorithmic_gb_per_s": alg / (probe_ms * 1e-3) / 1e9 if probe_ms > 0 else None}


def run_serving(n_jobs=12, tail=2, rate=2.0, slots=4, max_cells=4096, ref_seconds=0.0,
                lane_opts=None):
    """C5: a seeded Poisson stream of first-hit jobs, n uniform in 20..42 with a signature from
    classes(n) and a contiguous ORDER=3 range of 1..max_cells raw cells, plus `tail` n = 42
    ranges; per-job budget 2^16, BUF_CAP 2000, DRAIN_TOP 64 (the per-cell work reduced from the
    production lane). Lists are built before the clock starts, in parallel (a service keeps
    them). Reports cells/s, nodes/s and p50/p99 job latency.

    With ref_seconds > 0 the same jobs also run as the reference's own lane processes, all at
    once on the host cores, stopped after ref_seconds; then our server runs exactly the raw
    cells each reference process completed (all jobs submitted at once), so the two are timed
    on the same work, and every job the reference finished is compared count for count."""
    import concurrent.futures as cf
    from bs45_quantum_explorer_gb300.serve import Job, Server, poisson_trace, serving_list
    plan = poisson_trace(nj=n_jobs, rate=rate, seed=SEED, n_range=(20, 42), max_cells=max_cells,
                         tail_n42=tail, classes=_classes, ncells_of=lambda n, sg: 1 << 30)
    t0 = time.perf_counter()
    keys = sorted({(j.n, j.sig) for j in plan})
    with cf.ThreadPoolExecutor(max_workers=min(16, len(keys))) as ex:
        lists = dict(zip(keys, ex.map(lambda k: serving_list(*k), keys)))
    list_s = time.perf_counter() - t0
    jobs = poisson_trace(nj=n_jobs, rate=rate, seed=SEED, n_range=(20, 42), max_cells=max_cells,
                         tail_n42=tail, classes=_classes, ncells_of=lambda n, sg: len(lists[(n, sg)][1]),
                         budget=1 << 16, buf_cap=2000, drain_top=64)
    srv = Server(slots=slots, lane_opts=lane_opts)
    out, st = srv.run_trace(jobs)
    d = st.as_dict()
    d.update({"workload": f"{len(jobs)} jobs ({tail} of them n=42), Poisson rate {rate}/s, seed {SEED:#x}, "
                          f"{slots} slots; ranges of 1..{max_cells} raw cells; budget 2^16, BUF_CAP 2000, "
                          "DRAIN_TOP 64", "lists_prebuilt_s": round(list_s, 2),
              "errors": sum(1 for j in out if j.error), "found": sum(1 for j in out if j.result and j.result.found),
              "peak_hbm_admitted_bytes": srv.peak_in_use,
              "peak_device_used_bytes": srv.peak_device_used,
              "admissions_held_by_measured_memory": srv.waits_on_device_memory})
    if ref_seconds > 0:
        ref, per_job = serving_reference(jobs, ref_seconds, out)
        d["cpu_baseline"] = ref
        if per_job:
            # the same work on our server: each job's cells the reference completed
            same = [Job(jid=j.jid, n=j.n, sig=j.sig, skip=j.skip, end=j.end if fin else rpi,
                        budget=j.budget, buf_cap=j.buf_cap, drain_top=j.drain_top,
                        drain_batches=j.drain_batches, arrival=0.0)
                    for j, (fin, rpi) in zip(jobs, per_job) if fin or (rpi is not None and rpi > j.skip)]
            # one slot per job, as the reference runs one process per job
            out2, st2 = Server(slots=min(len(same), 16), lane_opts=lane_opts).run_trace(same)
            d["same_work"] = {
                "jobs": len(same), "slots": min(len(same), 16),
                "reference_cells_done": ref["cells_done"], "our_cells_done": st2.cells,
                "reference_seconds": ref["seconds"], "reference_cores": ref["cores"],
                "our_seconds": round(st2.makespan_s, 2),
                "speedup": ref["seconds"] / st2.makespan_s if st2.makespan_s > 0 else None,
                "errors": sum(1 for j in out2 if j.error),
                "what": "the raw cells each reference lane process completed within its bound "
                        "(its whole range when it finished), on our server with every job "
                        "submitted at once, against the reference's wall time for them"}
    return d


def serving_reference(jobs, seconds, ours):
    """The same jobs through the reference's own lane binary (oracle/_ref/wz_match, the
    reference's wz_match.cpp compiled unmodified), one process per job as its SLURM lanes run
    them, all at once on the host cores, each stopped by SIGTERM after `seconds` (the
    reference then prints its summary with the raw cell it would resume from). Returns (the
    report: jobs that finished, their latency from their start, the cells done per second over
    the bound, and for every finished job whether its summary counts equal ours; per job
    (finished, resume_pi))."""
    import re
    import signal
    import subprocess
    exe = os.path.join(ROOT, "oracle", "_ref", "wz_match")
    if not os.path.exists(exe):
        return {"unavailable": "oracle/_ref/wz_match was not built on this machine"}, None
    base = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
    procs = []
    t0 = time.perf_counter()
    for j in jobs:
        env = dict(base, WZ_FIRSTHIT="1", WZ_FH_M6="1", WZ_THM211B="1", WZ_THM212="1",
                   WZ_FH_ORBIT_CANON="1", WZ_FH_ORBIT_Q="1", WZ_FH_ORBIT_QPRUNE="1",
                   WZ_FH_PROF_ORDER="3", WZ_FH_ORD3_NODIGEST_OK="1", WZ_FH_AB_BUDGET=str(j.budget),
                   WZ_FH_BUF_CAP=str(j.buf_cap), WZ_FH_DRAIN_TOP=str(j.drain_top),
                   WZ_FH_PROF_SKIP=str(j.skip), WZ_FH_PROF_END=str(j.end), WZ_FH_PROG_SEC="99999")
        procs.append(subprocess.Popen([exe, str(j.n), *map(str, j.sig)], env=env, text=True,
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL))
    finish = [None] * len(procs)
    while time.perf_counter() - t0 < seconds and any(f is None for f in finish):
        for i, p in enumerate(procs):
            if finish[i] is None and p.poll() is not None:
                finish[i] = time.perf_counter() - t0
        time.sleep(0.05)
    for i, p in enumerate(procs):
        if finish[i] is None:
            p.send_signal(signal.SIGTERM)
    wall = time.perf_counter() - t0
    cells, same, done = 0, 0, 0
    per_job = []
    for i, p in enumerate(procs):
        out, _ = p.communicate(timeout=600)
        m = re.search(r"cells_done=(\d+)", out)
        cells += int(m[1]) if m else 0
        rp = re.search(r"resume_pi=(-?\d+)", out)
        per_job.append((finish[i] is not None, int(rp[1]) if rp else None))
        if finish[i] is not None:
            done += 1
            r = ours[i].result
            keys = dict(re.findall(r"(candidates_streamed|total_AB_nodes|cells_done|budget_aborted)=(\d+)", out))
            if r is not None and keys and (int(keys.get("candidates_streamed", -1)) == r.candidates_streamed and
                                           int(keys.get("total_AB_nodes", -1)) == r.total_ab_nodes and
                                           int(keys.get("cells_done", -1)) == r.cells_done):
                same += 1
    lat = sorted(f for f in finish if f is not None)
    return {"value": cells / wall, "unit": "cells/s", "cores": os.cpu_count() or 1, "kind": "reference",
            "sample": f"the same {len(jobs)} jobs as reference lane processes (wz_match.cpp compiled "
                      f"unmodified), all started at once, stopped after {seconds:.0f} s",
            "jobs_finished": done, "cells_done": cells, "seconds": round(wall, 1),
            "finished_p50_s": float(np.percentile(lat, 50)) if lat else None,
            "finished_jobs_equal_to_ours": same}, per_job


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--pairs", type=int, default=1 << 24)
    ap.add_argument("--mode", default="tc_fp16", choices=["tc_fp16", "tc_bf16x2", "fp64"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--limit", type=int, default=None,
                    help="with --stream-only: stop after this many survivors (0: whole cell)")
    ap.add_argument("--stream-only", choices=["n30", "n42"], default=None,
                    help="stream one built-in cell only (a small case for profiling)")
    ap.add_argument("--first-hit", type=float, default=None, metavar="SECONDS",
                    help="run only the n=36 first-hit lane for about SECONDS and print its line")
    ap.add_argument("--serve", action="store_true", help="run only the serving mix and print its line")
    ap.add_argument("--join", type=int, default=None, metavar="N",
                    help="run only the full-space join for BS(N+1, N), one signature")
    ap.add_argument("--c3", type=int, default=None, metavar="CELLS",
                    help="run only the n=30 full stream over the first CELLS kept cells (0: all)")
    ap.add_argument("--no-tune", action="store_true",
                    help="first-hit lane with the default work sizes instead of the autotuner's")
    ap.add_argument("--spike", action="store_true",
                    help="run only the reference's GPU completer spike beside ours and print its line")
    ap.add_argument("--fh-drain", type=int, default=50000,
                    help="DRAIN_TOP of the first-hit lane (a smaller value makes a small profiling case)")
    ap.add_argument("--fh-seconds", type=float, default=30.0,
                    help="bound on the first-hit lane inside the default run")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank = env_int("RANK", 0)
    world = env_int("WORLD_SIZE", 1)
    local = env_int("LOCAL_RANK", 0)

    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.stream_only:
        run_stream_only(args)
        return
    if args.first_hit is not None or args.serve or args.c3 is not None or args.join is not None \
            or args.spike:
        from bs45_quantum_explorer_gb300 import build_library
        build_library()
        if args.first_hit is not None:
            print(json.dumps(run_first_hit(args.first_hit, with_cpu=not args.no_cpu_baseline,
                                           drain_top=args.fh_drain, tune=not args.no_tune)), flush=True)
        if args.serve:
            print(json.dumps(run_serving(ref_seconds=0.0 if args.no_cpu_baseline else 60.0)), flush=True)
        if args.c3 is not None:
            print(json.dumps(run_c3(args.c3)), flush=True)
        if args.join is not None:
            print(json.dumps(run_join(args.join)), flush=True)
        if args.spike:
            print(json.dumps(run_spike()), flush=True)
        return

    import numpy as np
    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from bs45_quantum_explorer_gb300 import build_library
    build_library()
    from bs45_quantum_explorer_gb300._lib import lib
    from bs45_quantum_explorer_gb300.hall import Context

    npairs = args.pairs
    ctx = Context(N, SIG, device=local)
    # a dedicated stream: the library launches on it and the events below are recorded on it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    assert stream.cuda_stream != 0
    ctx.set_stream(stream.cuda_stream)
    d_words = torch.empty(2 * npairs, dtype=torch.int64, device="cuda")
    d_pass = torch.empty(npairs, dtype=torch.uint8, device="cuda")
    ctx.gen_hall_pairs_dev(npairs, d_words.data_ptr(), seed=SEED + rank)
    torch.cuda.synchronize()

    def step():
        ctx.hall_filter_dev(d_words.data_ptr(), npairs, d_pass.data_ptr(), args.mode, stats=False)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    st = ctx.hall_filter_dev(d_words.data_ptr(), npairs, d_pass.data_ptr(), args.mode, stats=True)

    # ---- timed region: K steps, device events on the launching stream ----
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    clocks = ClockSampler(local)
    ctx.timing(True)
    _, _, launches0 = ctx.timing_read()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for k in range(args.steps):
        ev[k][0].record(stream)
        step()
        ev[k][1].record(stream)
    t_end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    elapsed_ms = t_start.elapsed_time(t_end)
    kern_ms, kern_launches, launches1 = ctx.timing_read()
    ctx.timing(False)
    if dist:
        t = torch.tensor([elapsed_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed_ms = float(t.item())
        dist.barrier()
    per_step = [a.elapsed_time(b) for a, b in ev]
    value = world * npairs * args.steps / (elapsed_ms * 1e-3)

    peaks, peak_src = load_peaks()
    avg_kernel_ms = kern_ms / max(1, kern_launches)
    if args.mode == "fp64":
        roof = None
    else:
        achieved = FLOPS_PER_PAIR * npairs / (avg_kernel_ms * 1e-3) / 1e12
        sustained = elapsed_ms > 2000
        peak = peaks.get("bf16_tflops_sustained" if sustained else "bf16_tflops", 1900.0)
        traffic = load_traffic()
        roof = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": traffic,
                "kernel": "hall_screen_kernel + hall_tc_kernel (one timed section per step)",
                "kernel_ms": avg_kernel_ms,
                "peak_source": f"{peak_src} {'bf16_tflops_sustained' if sustained else 'bf16_tflops'}",
                "algorithmic_flops_per_launch": FLOPS_PER_PAIR * npairs,
                "screen_tensor_flops_per_launch": 2 * 2 * npairs * 64 * 48 * (2 if args.mode == "tc_bf16x2" else 1)}

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f16" if args.mode == "tc_fp16" else
        ("bf16" if args.mode == "tc_bf16x2" else "f64"), "data": "synthetic",
        "config": {"workload": "hall_filter_n42_2^24_pairs", "n": N, "sig": list(SIG),
                   "pairs_per_step": npairs, "mode": args.mode,
                   "inputs": f"{16 * npairs / 1e6:.0f} MB packed words resident in HBM, larger than L2 (no flush)",
                   "parallelism": f"replica x{world}"},
        "p50_ms": statistics.median(per_step),
        "p99_ms": sorted(per_step)[min(len(per_step) - 1, int(0.99 * len(per_step)))],
        "rechecked_pairs_per_step": st["rechecked"], "fp64_rechecked_pairs_per_step": st["fp64_rechecked"],
        "passed_pairs_per_step": st["passed"],
        "certified_band": [st["pass_below"], st["reject_above"]],
        "gpu_launches": int(launches1 - launches0),
        "roofline": roof,
        "clocks": clk,
    }

    if rank == 0 and not args.no_extras:
        # ---- e2e: the C-ABI host entry point, pinned host buffers, copies inside ----
        h_words = d_words.cpu().pin_memory()
        h_pass = torch.empty(npairs, dtype=torch.uint8).pin_memory()
        from bs45_quantum_explorer_gb300._lib import HallStats
        import ctypes as C
        hs = HallStats()
        mode_id = {"fp64": 0, "tc_fp16": 1, "tc_bf16x2": 2}[args.mode]
        ctx2 = Context(N, SIG, device=local)
        e2e_times = []
        for k in range(args.warmup + min(args.steps, 10)):
            t0 = time.perf_counter()
            rc = lib().bs_hall_filter_packed(ctx2.h, C.c_void_p(h_words.data_ptr()), npairs,
                                             mode_id, C.c_void_p(h_pass.data_ptr()), C.byref(hs))
            dt = time.perf_counter() - t0
            assert rc == 0, rc
            if k >= args.warmup:
                e2e_times.append(dt)
        e2e_ok = bool(torch.equal(h_pass.cuda(), d_pass))
        ctx2.close()
        line["e2e"] = {"value": npairs * len(e2e_times) / sum(e2e_times), "unit": UNIT,
                       "h2d_bytes_per_step": 16 * npairs, "d2h_bytes_per_step": npairs,
                       "api": "bs_hall_filter_packed (host pinned words in, host mask out)",
                       "matches_device_path": e2e_ok}
        # ---- the FP64-only GPU form of the same filter, for the tensor-core speed-up ----
        if args.mode != "fp64":
            fp_steps = 3
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            d_pass64 = torch.empty_like(d_pass)
            ctx.hall_filter_dev(d_words.data_ptr(), npairs, d_pass64.data_ptr(), "fp64", stats=False)
            a.record(stream)
            for _ in range(fp_steps):
                ctx.hall_filter_dev(d_words.data_ptr(), npairs, d_pass64.data_ptr(), "fp64",
                                    stats=False)
            b.record(stream)
            torch.cuda.synchronize()
            fp_rate = npairs * fp_steps / (a.elapsed_time(b) * 1e-3)
            line["fp64_gpu_form"] = {"value": fp_rate, "unit": UNIT,
                                     "tc_speedup": value / world / fp_rate,
                                     "masks_identical": bool(torch.equal(d_pass64, d_pass))}
            # the other tensor-core form (split-BF16 hi + lo, or fp16) of the same filter
            other = "tc_bf16x2" if args.mode == "tc_fp16" else "tc_fp16"
            d_pass2 = torch.empty_like(d_pass)
            ctx.hall_filter_dev(d_words.data_ptr(), npairs, d_pass2.data_ptr(), other, stats=False)
            torch.cuda.synchronize()
            a.record(stream)
            for _ in range(10):
                ctx.hall_filter_dev(d_words.data_ptr(), npairs, d_pass2.data_ptr(), other, stats=False)
            b.record(stream)
            torch.cuda.synchronize()
            o_rate = npairs * 10 / (a.elapsed_time(b) * 1e-3)
            st2 = ctx.hall_filter_dev(d_words.data_ptr(), npairs, d_pass2.data_ptr(), other, stats=True)
            line[f"{other}_form"] = {"value": o_rate, "unit": UNIT, "speedup_vs_fp64_gpu_form": o_rate / fp_rate,
                                     "masks_identical": bool(torch.equal(d_pass2, d_pass)),
                                     "rechecked_pairs_per_step": st2["rechecked"],
                                     "certified_band": [st2["pass_below"], st2["reject_above"]]}
        # ---- the tensor-core PSD error against FP64 on 4,096 pairs (tables as the reference
        # builds them: cos/sin(i * (j pi / 100))); the false-reject count against the oracle is
        # taken in the CPU-baseline leg below ----
        from bs45_quantum_explorer_gb300.workloads import unpack_pairs
        lo = (1 << 23) - (1 << 15) if npairs >= (1 << 24) else 0
        w = d_words[2 * lo:2 * (lo + 4096)].cpu().numpy().view(np.uint64).reshape(-1, 2)
        acc = torch.zeros((2 * 4096, 208), dtype=torch.float32, device="cuda")
        ctx.hall_tc_dump_dev(d_words[2 * lo:].data_ptr(), 4096, acc.data_ptr(),
                             args.mode if args.mode != "fp64" else "tc_fp16")
        torch.cuda.synchronize()
        a = acc.cpu().numpy().astype(np.float64)
        f_tc = (a[:, :101] ** 2 + a[:, 104:205] ** 2).reshape(4096, 2, 101).sum(axis=1)
        jj = np.arange(201, dtype=np.float64)[:, None] * np.pi / 100.0
        ii = np.arange(N, dtype=np.float64)[None, :]
        ct, stb = np.cos(ii * jj), np.sin(ii * jj)
        X = unpack_pairs(w[:4096], N).astype(np.float64)
        js = list(range(1, 101)) + [200]
        re = X @ ct[js, :N].T
        im = X @ stb[js, :N].T
        f64 = (re * re + im * im).sum(axis=1)
        line["parity_sample"] = {"psd_pairs": 4096,
                                 "max_psd_err_vs_fp64": float(np.abs(f_tc - f64).max()),
                                 "psd_err_bound_at_limit": float(4 * st["quant_err"] * (4 * N + 2.5) ** 0.5
                                                                 + 4 * st["quant_err"] ** 2)}
        # ---- search nodes/s: the C,D stream of one n = 42 cell (DFS + Hall + order) ----
        from bs45_quantum_explorer_gb300.stream import cd_stream
        cell42 = ([-1, -1, 1, 1, 1, -1], [-1, -3, 1, 1, 3, -1])  # ORDER=3 raw cell 3056, sig (7,11,0,0)
        SEARCH_LIMIT = 50000  # the cell holds > 10^13 nodes: stream its first survivors
        cd_stream(ctx, [cell42], m=6, as_words=True, limit=100)  # warm-up (frontier, buffers)
        torch.cuda.synchronize()
        ctx.timing(True)
        t0 = time.perf_counter()
        surv, _, sst = cd_stream(ctx, [cell42], m=6, as_words=True, limit=SEARCH_LIMIT)
        dt = time.perf_counter() - t0
        dfs_ms, dfs_launches, _ = ctx.timing_read()
        ctx.timing(False)
        nodes = sst[0]["nodes"]
        # the tensor-core and FP64-only Hall forms on the same shorter search (the FP64 form
        # filters ~2e7 leaves/s, so the full 50,000-survivor search would take minutes)
        CMP_LIMIT = 500
        t1 = time.perf_counter()
        surv_c, _, sst_c = cd_stream(ctx, [cell42], m=6, as_words=True, limit=CMP_LIMIT)
        dt_c = time.perf_counter() - t1
        t1 = time.perf_counter()
        surv64, _, sst64 = cd_stream(ctx, [cell42], m=6, as_words=True, limit=CMP_LIMIT,
                                     hall_mode="fp64")
        dt64 = time.perf_counter() - t1
        t1 = time.perf_counter()
        survb, _, sstb = cd_stream(ctx, [cell42], m=6, as_words=True, limit=CMP_LIMIT,
                                   hall_mode="tc_bf16x2")
        dtb = time.perf_counter() - t1
        line["search"] = {
            "workload": "C,D stream of the n=42 cell px=(-1,-1,1,1,1,-1) py=(-1,-3,1,1,3,-1) "
                        "(ORDER=3 raw cell 3056 of sig (7,11,0,0)), its first 50,000 survivors "
                        "in stream order (the lane's front-only cut)",
            "dfs_nodes": nodes, "leaves": sst[0]["leaves"], "survivors": int(len(surv)),
            "seconds": dt, "nodes_per_s": nodes / dt, "leaves_per_s": sst[0]["leaves"] / dt,
            "device_kernel_ms": dfs_ms, "timed_launches": dfs_launches,
            "device_nodes_per_s": nodes / (dfs_ms * 1e-3) if dfs_ms > 0 else None,
            "filtered_cands_per_s": sst[0]["leaves"] / dt,
            "hall_forms_on_first_500": {
                "tc_fp16": {"seconds": dt_c, "nodes_per_s": sst_c[0]["nodes"] / dt_c,
                            "filtered_cands_per_s": sst_c[0]["leaves"] / dt_c},
                "fp64": {"seconds": dt64, "nodes_per_s": sst64[0]["nodes"] / dt64,
                         "filtered_cands_per_s": sst64[0]["leaves"] / dt64},
                "tc_bf16x2": {"seconds": dtb, "nodes_per_s": sstb[0]["nodes"] / dtb,
                              "filtered_cands_per_s": sstb[0]["leaves"] / dtb,
                              "speedup_vs_fp64": dt64 / dtb},
                "tc_speedup": dt64 / dt_c,
                "survivors_identical": bool(np.array_equal(surv64, surv_c)) and
                bool(np.array_equal(survb, surv_c)),
                "same_as_50000_prefix": bool(np.array_equal(surv_c, surv[:CMP_LIMIT]))},
        }
        if not args.no_cpu_baseline:
            line["search"]["cpu_baseline"] = guarded(cpu_search_rate, os.cpu_count() or 1, cell42)
        # the batch and its mask on the host for the CPU-baseline leg below, taken before the
        # extra legs so that a failing leg cannot cost the headline its baseline
        if not args.no_cpu_baseline:
            words = d_words.cpu().numpy().view(np.uint64).reshape(-1, 2)
            got = d_pass.cpu().numpy()
        # ---- the n = 36 first-hit lane (bounded) and the serving mix ----
        line["first_hit"] = guarded(run_first_hit, args.fh_seconds,
                                    with_cpu=not args.no_cpu_baseline)
        # ranges of 1..256 cells here so that the default run ends in minutes; `--serve`
        # runs the stated 1..4096
        line["serving"] = guarded(run_serving, max_cells=256,
                                  ref_seconds=0.0 if args.no_cpu_baseline else 45.0)
        line["completer_vs_reference_gpu_spike"] = guarded(run_spike)
        if not args.no_cpu_baseline:
            def cpu_leg():
                ncpu = os.cpu_count() or 1
                rate, samp, thr, dt, kind, what, rmask = cpu_hall_rate(ncpu, words)
                # parity of the device mask on every pair of the batch: against the oracle (the
                # checker) and against the reference's own decisions from the timed leg
                from bs45_quantum_explorer_gb300.workloads import unpack_pairs
                omask = _oracle().hall_batch(N, unpack_pairs(words, N), nthreads=ncpu)
                line["parity_sample"].update(
                    pairs=int(len(omask)), false_rejects=int(((omask == 1) & (got == 0)).sum()),
                    false_accepts=int(((omask == 0) & (got == 1)).sum()),
                    differs_from_reference_arm=int((rmask != got).sum()) if kind == "reference" else None)
                return {"value": rate, "unit": UNIT, "cores": thr, "kind": kind, "sample": what}
            line["cpu_baseline"] = guarded(cpu_leg)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
