"""The drop-in lane binary (bin/bs_firsthit) against full runs of the reference binary
(tests/golden/lane_golden.json): same exit code, same semantic stdout lines, same CELLSIZE /
CDSTAT counts, same WZ_FH_DUMP stream bytes, and the same checkpoint files across an
interrupted run and its resume."""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))


def _bin():
    from bs45_quantum_explorer_gb300.build import build_all
    _, exe = build_all()
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
    p = subprocess.run([exe, str(n), *map(str, sig)], env=env, capture_output=True, text=True, timeout=600)
    data = open(dump, "rb").read() if os.path.exists(dump) else b""
    return p.returncode, p.stdout, hashlib.sha256(data).hexdigest(), len(data)


def _cases():
    return json.load(open(os.path.join(HERE, "golden", "lane_golden.json")))


def test_lane_matches_reference_runs(gpu):
    cases = [c for c in _cases() if not c.get("resume") and "WZ_FH_CD_PRUNE" not in c["settings"]]
    assert len(cases) > 200
    _replay(cases)


def test_lane_cd_prune_matches_reference_runs(gpu):
    """WZ_FH_CD_PRUNE 1, 2, 3 with CELLSIZE on: the same lane output and the pruned CDSTAT
    dfs_nodes of every cell."""
    cases = [c for c in _cases() if not c.get("resume") and "WZ_FH_CD_PRUNE" in c["settings"]]
    assert len(cases) >= 80
    _replay(cases)


def test_lane_a2_matches_reference_runs(gpu):
    """WZ_FH_A2=2 (the A2 row prune) in the drop-in binary and in the library lane against
    the reference binary's runs (tests/golden/a2_lane_golden.json)."""
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.lane import run_lane
    cases = json.load(open(os.path.join(HERE, "golden", "a2_lane_golden.json")))
    assert len(cases) >= 100
    _replay(cases)
    ctxs = {}
    for c in cases:
        key = (c["n"], tuple(c["sig"]))
        if key not in ctxs:
            ctxs[key] = Context(*key)
        res = run_lane(ctxs[key], c["n"], tuple(c["sig"]), **lane_kwargs(c["settings"]))
        check_run_lane(res, summary_of(c["semantic"]), (c["n"], c["sig"], c["settings"]))
    for x in ctxs.values():
        x.close()


def _replay(cases):
    from make_lane_golden import cellsize_lines, semantic
    exe = _bin()
    with tempfile.TemporaryDirectory() as tmp:
        for c in cases:
            rc, out, dh, dl = _run(exe, c["n"], c["sig"], c["settings"], tmp)
            ctx = (c["n"], c["sig"], c["settings"])
            assert rc == c["rc"], (ctx, out[-2000:])
            assert semantic(out) == c["semantic"], ctx
            assert (dh, dl) == (c["dump_sha256"], c["dump_len"]), ctx
            assert cellsize_lines(out) == c["cells"], ctx


def test_lane_checkpoint_resume_matches_reference(gpu):
    from make_lane_golden import semantic
    exe = _bin()
    cases = [c for c in _cases() if c.get("resume")]
    assert len(cases) >= 10
    with tempfile.TemporaryDirectory() as tmp:
        for c in cases:
            ck = tempfile.mkdtemp(dir=tmp)
            rc1, out1, _, _ = _run(exe, c["n"], c["sig"], c["settings"], tmp, ck)
            files = sorted(os.listdir(ck))
            ckpt1 = open(os.path.join(ck, files[0])).read() if files else ""
            st2 = {k: v for k, v in c["settings"].items() if k != "WZ_FH_TEST_STOP_AFTER"}
            rc2, out2, dh, dl = _run(exe, c["n"], c["sig"], st2, tmp, ck)
            ckpt2 = open(os.path.join(ck, files[0])).read() if files else ""
            ctx = (c["n"], c["sig"], c["settings"])
            assert (rc1, semantic(out1), ckpt1) == (c["rc"], c["semantic"], c["ckpt"]), ctx
            assert (rc2, semantic(out2), ckpt2) == (c["rc2"], c["semantic2"], c["ckpt2"]), ctx
            assert (dh, dl) == (c["dump_sha256"], c["dump_len"]), ctx


# ---- the library form of the lane (lane.run_lane) against the same reference runs ----

_SUMMARY_KEYS = {"candidates_streamed": "candidates_streamed", "backtracks_entered": "backtracks_entered",
                 "clean_no_AB": "clean_no_ab", "budget_aborted": "budget_aborted",
                 "total_AB_nodes": "total_ab_nodes", "cells_done": "cells_done",
                 "cells_prof_dead": "cells_prof_dead", "cells_prof_uncap": "cells_prof_uncap",
                 "cells_orbit_dup": "cells_orbit_dup", "cells_empty": "cells_empty",
                 "cells_capped": "cells_capped", "pre_filter_rejected": "pre_filter_rejected"}


def summary_of(semantic_lines):
    """The reference summary's counts, the FIRSTHIT fields and the quad, from semantic lines."""
    import re
    out = {}
    for line in semantic_lines:
        for k, v in re.findall(r"(\w+)=(-?\d+)", line):
            if k in _SUMMARY_KEYS:
                out[_SUMMARY_KEYS[k]] = int(v)
        m = re.match(r"FIRSTHIT: idx=(\d+) profile_rank=(\d+) nodes_this_cand=(\d+)", line)
        if m:
            out["hit"] = tuple(int(x) for x in m.groups())
        m = re.match(r"([ABCD]) = \{(.*)\};", line)
        if m:
            out[m.group(1)] = [int(x) for x in m.group(2).split(",")]
    return out


def lane_kwargs(st):
    """run_lane arguments for a lane's WZ_* settings (buffered mod-6 order only)."""
    return dict(budget=int(st.get("WZ_FH_AB_BUDGET", 200000)), buf_cap=int(st.get("WZ_FH_BUF_CAP", 500000)),
                drain_top=int(st.get("WZ_FH_DRAIN_TOP", 0)), drain_batches=int(st.get("WZ_FH_DRAIN_BATCHES", 1)),
                skip=int(st.get("WZ_FH_PROF_SKIP", 0)), end=int(st.get("WZ_FH_PROF_END", 0)),
                rev=bool(int(st.get("WZ_FH_STREAM_REV", 0))), endpos=bool(int(st.get("WZ_FH_ENDPOS", 0))),
                orbit_canon=bool(int(st.get("WZ_FH_ORBIT_CANON", 0))), orbit_q=int(st.get("WZ_FH_ORBIT_Q", 0)),
                qprune=bool(int(st.get("WZ_FH_ORBIT_QPRUNE", 0))), prof_order=int(st.get("WZ_FH_PROF_ORDER", 0)),
                outer_k=int(st.get("WZ_FH_OUTER_K", 3)), early=int(st.get("WZ_FH_EARLY_CHECK", 1)) != 0,
                canon="WZ_FH_NO_CANON" not in st, m6=True, thm211b=True, thm212=True,
                a2=int(st.get("WZ_FH_A2", 0)))


def check_run_lane(res, want, ctx):
    got = {v: getattr(res, v) for v in _SUMMARY_KEYS.values() if v in want}
    assert got == {k: want[k] for k in got}, ctx
    if "hit" in want:
        assert res.found and (res.hit_idx, res.profile_rank, res.nodes_this_cand) == want["hit"], ctx
        A, B, C, D = res.quad
        assert [list(map(int, x)) for x in (A, B, C, D)] == [want[k] for k in "ABCD"], ctx
    else:
        assert not res.found, ctx


def test_run_lane_matches_reference_runs(gpu):
    from bs45_quantum_explorer_gb300.hall import Context
    from bs45_quantum_explorer_gb300.lane import run_lane
    cases = [c for c in _cases() if not c.get("resume") and c["settings"].get("WZ_FH_M6") == 1
             and not any(k in c["settings"] for k in ("WZ_FH_CELLSIZE", "WZ_FH_SCORE_MAX"))]
    assert len(cases) >= 100
    ctxs = {}
    for c in cases:
        key = (c["n"], tuple(c["sig"]))
        if key not in ctxs:
            ctxs[key] = Context(c["n"], tuple(c["sig"]))
        res = run_lane(ctxs[key], c["n"], tuple(c["sig"]), **lane_kwargs(c["settings"]))
        check_run_lane(res, summary_of(c["semantic"]), (c["n"], c["sig"], c["settings"]))
    for x in ctxs.values():
        x.close()


def test_lane_resumes_across_cpu_and_gpu_arms(gpu):
    """An arm interrupted on CPU cores (the reference binary, oracle/_ref/wz_match) resumes on
    the GPU from its checkpoint file, and the other way round, with the same result and the
    same final checkpoint as the reference's own interrupted-and-resumed run."""
    from make_lane_golden import REF_BIN, semantic
    if not os.path.exists(REF_BIN):
        pytest.skip("the reference binary was not built on this machine (oracle/_ref)")
    exe = _bin()
    cases = [c for c in _cases() if c.get("resume")]
    assert len(cases) >= 10
    with tempfile.TemporaryDirectory() as tmp:
        for first, second in ((REF_BIN, exe), (exe, REF_BIN)):
            for c in cases:
                ck = tempfile.mkdtemp(dir=tmp)
                rc1, out1, _, _ = _run(first, c["n"], c["sig"], c["settings"], tmp, ck)
                st2 = {k: v for k, v in c["settings"].items() if k != "WZ_FH_TEST_STOP_AFTER"}
                rc2, out2, dh, dl = _run(second, c["n"], c["sig"], st2, tmp, ck)
                files = sorted(os.listdir(ck))
                ckpt2 = open(os.path.join(ck, files[0])).read() if files else ""
                ctx = (os.path.basename(first), c["n"], c["sig"], c["settings"])
                assert (rc1, semantic(out1)) == (c["rc"], c["semantic"]), ctx
                assert (rc2, semantic(out2), ckpt2) == (c["rc2"], c["semantic2"], c["ckpt2"]), ctx
