"""The lane binary's host logic against the reference's own lane runs, on the CPU.

bin/bs_firsthit is the reference's first-hit control flow (cell list, allowed rows, probe
order, buffers, drain, front-only cut, checkpoint file, stdout protocol, exit codes) around
device calls. Here the same firsthit_main.cpp is built with those device calls answered by
the oracle (tests/hostcheck/oracle_device.cpp: the oracle's stream, flat score and completer,
which test_oracle_golden.py pins to the reference) into tests/_build/bs_firsthit_hostcheck, a
test-only binary, and replayed against every n <= 13 reference run of
tests/golden/lane_golden.json and a2_lane_golden.json: exit code, semantic lines, CELLSIZE /
CDSTAT counts, WZ_FH_DUMP bytes, and the checkpoint files across an interrupted run and its
resume. The GPU tests (test_lane_gpu.py) replay the same runs through the product binary."""
import concurrent.futures as cf
import functools
import hashlib
import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(HERE, "golden"))
BUILD = os.path.join(HERE, "_build")


@functools.lru_cache(maxsize=1)
def _hostcheck_binary():
    pkg = os.path.join(ROOT, "bs45_quantum_explorer_gb300")
    exe = os.path.join(BUILD, "bs_firsthit_hostcheck")
    srcs = [os.path.join(pkg, "host", "firsthit_main.cpp"), os.path.join(pkg, "host", "celllist.cpp"),
            os.path.join(HERE, "hostcheck", "oracle_device.cpp")]
    os.makedirs(BUILD, exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", f"-I{os.path.join(ROOT, 'include')}",
           f"-I{os.path.join(pkg, 'host')}", "-o", exe, *srcs, f"-L{os.path.join(ROOT, 'oracle')}",
           "-loracle", f"-Wl,-rpath,{os.path.join(ROOT, 'oracle')}", "-lpthread"]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _run(exe, n, sig, settings, tmp, ckdir=None):
    from make_lane_golden import BASE
    env = {k: v for k, v in os.environ.items() if not k.startswith(("WZ_", "FH_"))}
    env.update({k: str(v) for k, v in {**BASE, **settings}.items()})
    dump = os.path.join(tmp, "dump.txt")
    if os.path.exists(dump):
        os.remove(dump)
    env["WZ_FH_DUMP"] = dump
    if ckdir:
        env["WZ_FH_CKPT_DIR"] = ckdir
    p = subprocess.run([exe, str(n), *map(str, sig)], env=env, capture_output=True, text=True,
                       timeout=600)
    data = open(dump, "rb").read() if os.path.exists(dump) else b""
    return p.returncode, p.stdout, hashlib.sha256(data).hexdigest(), len(data)


def _replay(exe, cases):
    """Every case in its own directory, the processes run on all host cores."""
    from make_lane_golden import cellsize_lines, semantic

    def one(c):
        with tempfile.TemporaryDirectory() as tmp:
            return c, _run(exe, c["n"], c["sig"], c["settings"], tmp)

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        for c, (rc, out, dh, dl) in ex.map(one, cases):
            ctx = (c["n"], c["sig"], c["settings"])
            assert rc == c["rc"], (ctx, out[-2000:])
            assert semantic(out) == c["semantic"], ctx
            assert (dh, dl) == (c["dump_sha256"], c["dump_len"]), ctx
            assert cellsize_lines(out) == c["cells"], ctx


def test_lane_host_logic_matches_reference_runs(oracle):
    exe = _hostcheck_binary()
    cases = json.load(open(os.path.join(HERE, "golden", "lane_golden.json")))
    runs = [c for c in cases if not c.get("resume")]
    assert len(runs) > 250
    _replay(exe, runs)


def test_lane_host_logic_a2_matches_reference_runs(oracle):
    exe = _hostcheck_binary()
    cases = json.load(open(os.path.join(HERE, "golden", "a2_lane_golden.json")))
    assert len(cases) >= 100
    _replay(exe, cases)


def test_lane_host_logic_checkpoint_resume_matches_reference(oracle):
    from make_lane_golden import semantic
    exe = _hostcheck_binary()
    cases = [c for c in json.load(open(os.path.join(HERE, "golden", "lane_golden.json")))
             if c.get("resume")]
    assert len(cases) >= 10
    def one(c):
        with tempfile.TemporaryDirectory() as tmp:
            ck = tempfile.mkdtemp(dir=tmp)
            rc1, out1, _, _ = _run(exe, c["n"], c["sig"], c["settings"], tmp, ck)
            files = sorted(os.listdir(ck))
            ckpt1 = open(os.path.join(ck, files[0])).read() if files else ""
            st2 = {k: v for k, v in c["settings"].items() if k != "WZ_FH_TEST_STOP_AFTER"}
            rc2, out2, dh, dl = _run(exe, c["n"], c["sig"], st2, tmp, ck)
            ckpt2 = open(os.path.join(ck, files[0])).read() if files else ""
            return c, (rc1, semantic(out1), ckpt1), (rc2, semantic(out2), ckpt2), (dh, dl)

    with cf.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        for c, first, second, dump in ex.map(one, cases):
            ctx = (c["n"], c["sig"], c["settings"])
            assert first == (c["rc"], c["semantic"], c["ckpt"]), ctx
            assert second == (c["rc2"], c["semantic2"], c["ckpt2"]), ctx
            assert dump == (c["dump_sha256"], c["dump_len"]), ctx


def test_lane_host_logic_internal_error_exit_matches_reference(oracle):
    """WZ_FH_TEST_INTERNAL_ERROR (tests/golden/internal_error_golden.json): the first completion
    is reported as failing the NPAF check, and the binary prints the reference's
    FH_INTERNAL_ERROR and RESULT lines, exits 5 and leaves the same checkpoint file."""
    from make_internal_error_golden import record
    exe = _hostcheck_binary()
    cases = json.load(open(os.path.join(HERE, "golden", "internal_error_golden.json")))
    assert len(cases) >= 6 and all(c["rc"] == 5 for c in cases)
    for c in cases:
        rc, lines, files = record(exe, c["n"], tuple(c["sig"]), c["settings"])
        assert (rc, lines, files) == (c["rc"], c["lines"], c["files"]), (c["n"], c["sig"], c["settings"])


def test_lane_host_logic_other_knobs_match_reference(oracle):
    """The knobs lane_golden.json leaves at their defaults (tests/golden/lane_knobs_golden.json:
    MAX_CAND, CELL_ORDER=0, AB_PROF off or capped, NO_CANON, a shard of a skip/end range, the
    production list settings, buffered mod-3 cells, HALL_FAST=0, a score gate) and a resume
    with WZ_FH_RESUME=0."""
    from make_lane_golden import semantic
    exe = _hostcheck_binary()
    cases = json.load(open(os.path.join(HERE, "golden", "lane_knobs_golden.json")))
    runs = [c for c in cases if not c.get("resume")]
    assert len(runs) >= 200
    _replay(exe, runs)
    with tempfile.TemporaryDirectory() as tmp:
        for c in [c for c in cases if c.get("resume")]:
            ck = tempfile.mkdtemp(dir=tmp)
            rc1, out1, _, _ = _run(exe, c["n"], c["sig"], c["settings"], tmp, ck)
            files = sorted(os.listdir(ck))
            ckpt1 = open(os.path.join(ck, files[0])).read() if files else ""
            rc2, out2, dh, dl = _run(exe, c["n"], c["sig"], c["settings2"], tmp, ck)
            ckpt2 = open(os.path.join(ck, files[0])).read() if files else ""
            ctx = (c["n"], c["sig"], c["settings"], c["settings2"])
            assert (rc1, semantic(out1), ckpt1) == (c["rc"], c["semantic"], c["ckpt"]), ctx
            assert (rc2, semantic(out2), ckpt2) == (c["rc2"], c["semantic2"], c["ckpt2"]), ctx
            assert (dh, dl) == (c["dump_sha256"], c["dump_len"]), ctx


def test_lane_host_logic_replays_the_n29_canary(oracle):
    """The reference's archived n = 29 canary (tests/golden/canary_n29_golden.json) through the
    binary's host logic: 588 raw cells, 584 of them without allowed rows, the hit cell's 4,349
    completions in drain order, the summary and the quad; and the hit cell alone with the
    completer the archived fingerprint was recorded with."""
    from make_canary_golden import RUNS, record
    exe = _hostcheck_binary()
    g = json.load(open(os.path.join(HERE, "golden", "canary_n29_golden.json")))
    assert set(g["runs"]) == set(RUNS)
    with tempfile.TemporaryDirectory() as tmp:
        for name, want in g["runs"].items():
            got = record(exe, name, tmp, timeout=900)
            assert got == want, name
