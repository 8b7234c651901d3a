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
    from make_lane_golden import cellsize_lines, semantic
    exe = _bin()
    cases = [c for c in _cases() if not c.get("resume")]
    assert len(cases) > 200
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
