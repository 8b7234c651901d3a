"""Lane manifests shared with the reference's campaigns, and GPU lanes that resume CPU arms.

The reference plans a campaign with tools/passh_manifest.py: per signature class it runs the
solver in list-only mode (ORDER=3, orbit canon + quad switch + Q-closure prune), reads the
raw list length, kept count, window count and digest from the `[order]` line, and splits the
windows [0, ceil(cells / NARMS)) into lanes of S windows. Raw cell i belongs to window
i // NARMS and arm i % NARMS; a lane runs NARMS single-core arms (WZ_FH_SHARD = arm,
WZ_FH_NSHARD = NARMS, WZ_FH_PROF_SKIP/END = its windows), and cluster_firsthit_probe.sh can
run a sub-range of arms [FH_SHARD_LO, FH_SHARD_HI) of a lane. Arm checkpoints live in one
directory per lane (arm_<shard>.ckpt).

Here the same manifest is built from the library's own list (bs_cell_list: the same counts
and digests, without running the solver), and a lane, or any sub-range of its arms, runs on
the GPU through the drop-in binary with the arm's exact environment and checkpoint file, so
a lane started on CPU cores resumes on the GPU arm by arm and the other way round (the
checkpoint files are byte-identical).

    python -m bs45_quantum_explorer_gb300.manifest plan --n 44 --narms 177 --out DIR
    python -m bs45_quantum_explorer_gb300.manifest run DIR/passh_manifest.json --class A \\
        --lane 0 [--rev] [--shard-lo LO --shard-hi HI] --ckpt-dir DIR
"""
import argparse
import json
import math
import os
import subprocess
import sys

from .cells import cell_list

# the lane settings every arm of a planned lane runs with (cluster_firsthit_probe.sh and the
# reference planner's ENV_COMMON)
LANE_ENV = dict(WZ_FIRSTHIT=1, WZ_FH_PROF_ORDER=3, WZ_FH_ORBIT_CANON=1, WZ_FH_ORBIT_Q=1,
                WZ_FH_ORBIT_QPRUNE=1, WZ_FH_DRAIN_TOP=50000, WZ_FH_AB_BUDGET=2000000,
                WZ_FH_DRAIN_BATCHES=1)


def plan_class(n, sig, S, narms, endpos=False):
    """One class of a manifest: the list's counts and digest, and its lanes of S windows,
    with the planner's ownership check (every raw index owned once)."""
    # the lane's own defaults for the modulus and the 2.11b / 2.12 filters (forced at n >= 36)
    cells, kept, digest, _ = cell_list(n, sig, endpos=endpos, orbit_canon=True, orbit_q=1,
                                       qprune=True, prof_order=3, nshard=narms)
    ncells, nkept = len(kept), int(kept.sum())
    windows = math.ceil(ncells / narms)
    lanes = [{"skip": k, "end": min(k + S, windows)} for k in range(0, windows, S)]
    owner = [0] * ncells
    for ln in lanes:
        for i in range(ln["skip"] * narms, min(ln["end"] * narms, ncells)):
            owner[i] += 1
    if any(o != 1 for o in owner):
        raise AssertionError(f"{sig}: ownership gap or duplicate")
    per_arm = [0] * narms
    for i in range(ncells):
        per_arm[i % narms] += int(kept[i])
    return {"sig": list(sig), "cells": ncells, "kept": nkept, "windows": windows, "S": S,
            "digest": digest, "lanes": lanes, "kept_per_arm_min": min(per_arm),
            "kept_per_arm_max": max(per_arm)}


def plan(n, classes, narms, endpos=False):
    """classes: [(sig, S, cluster, letter)] as the reference planner lists them."""
    if narms % 2 == 0:
        # under ORDER=3 every kept cell sits at an even raw index: an even arm count leaves
        # the odd arms idle (the reference planner's rule)
        raise ValueError("NARMS must be odd")
    out = {"narms": narms, "n": n, "classes": []}
    for sig, S, cluster, letter in classes:
        c = plan_class(n, sig, S, narms, endpos=endpos)
        c.update(cluster=cluster, letter=letter)
        out["classes"].append(c)
    return out


def arm_env(n, cls, lane, narms, arm, rev=0, ckpt_dir=None, extra=None):
    """The environment of one arm of a lane, as cluster_firsthit_probe.sh exports it."""
    env = {k: str(v) for k, v in LANE_ENV.items()}
    env.update(WZ_FH_STREAM_REV=str(int(rev)), WZ_FH_PROF_SKIP=str(lane["skip"]),
               WZ_FH_PROF_END=str(lane["end"]), WZ_FH_EXPECT_DIGEST=cls["digest"],
               WZ_FH_SHARD=str(arm), WZ_FH_NSHARD=str(narms))
    if ckpt_dir:
        env["WZ_FH_CKPT_DIR"] = ckpt_dir
    env.update({k: str(v) for k, v in (extra or {}).items()})
    return env


def run_arms(exe, manifest, letter, lane_index, rev=0, shard_lo=0, shard_hi=None,
             ckpt_dir=None, extra=None, timeout=None):
    """Runs arms [shard_lo, shard_hi) of one lane, one after the other, through the drop-in
    binary (one GPU). Returns [(arm, exit code, stdout)]."""
    narms, n = manifest["narms"], manifest["n"]
    cls = next(c for c in manifest["classes"] if c["letter"] == letter)
    lane = cls["lanes"][lane_index]
    shard_hi = narms if shard_hi is None else shard_hi
    base = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
    out = []
    for arm in range(shard_lo, shard_hi):
        env = dict(base, **arm_env(n, cls, lane, narms, arm, rev, ckpt_dir, extra))
        p = subprocess.run([exe, str(n), *map(str, cls["sig"])], env=env, capture_output=True,
                           text=True, timeout=timeout)
        out.append((arm, p.returncode, p.stdout))
        if p.returncode == 0:  # FOUND: the lane's driver stops the other arms
            break
    return out


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)
    p1 = sub.add_parser("plan")
    p1.add_argument("--n", type=int, required=True)
    p1.add_argument("--narms", type=int, default=177)
    p1.add_argument("--classes", required=True,
                    help='JSON list of [[a,b,c,d], S, "cluster", "letter"]')
    p1.add_argument("--endpos", action="store_true")
    p1.add_argument("--out", required=True)
    p2 = sub.add_parser("run")
    p2.add_argument("manifest")
    p2.add_argument("--class", dest="letter", required=True)
    p2.add_argument("--lane", type=int, required=True)
    p2.add_argument("--rev", action="store_true")
    p2.add_argument("--shard-lo", type=int, default=0)
    p2.add_argument("--shard-hi", type=int, default=None)
    p2.add_argument("--ckpt-dir", default=None)
    a = ap.parse_args(argv)
    if a.cmd == "plan":
        classes = [(tuple(c[0]), int(c[1]), c[2], c[3]) for c in json.loads(a.classes)]
        m = plan(a.n, classes, a.narms, endpos=a.endpos)
        os.makedirs(a.out, exist_ok=True)
        with open(os.path.join(a.out, "passh_manifest.json"), "w") as f:
            json.dump(m, f, indent=1)
        for c in m["classes"]:
            print(f"{tuple(c['sig'])} {c['letter']}: cells={c['cells']} kept={c['kept']} "
                  f"windows={c['windows']} S={c['S']} lanes={len(c['lanes'])}x2 digest={c['digest']}")
        return 0
    from .build import build_all
    _, exe = build_all()
    man = json.load(open(a.manifest))
    for arm, rc, out in run_arms(exe, man, a.letter, a.lane, int(a.rev), a.shard_lo, a.shard_hi,
                                 a.ckpt_dir):
        tail = [ln for ln in out.splitlines() if ln.startswith(("RESULT:", "FIRSTHIT:"))]
        print(f"arm {arm}: rc={rc} {' | '.join(tail)}", flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
