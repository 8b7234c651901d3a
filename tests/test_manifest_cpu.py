"""Lane manifests (the reference's tools/passh_manifest.py planning, bs45_quantum_explorer_gb300.
manifest): the library's list gives the reference solver's list-only figures (raw cells, kept
cells, windows, digest, kept cells per arm; tests/golden/manifest_golden.json from
make_manifest_golden.py), lanes partition the windows with one owner per raw cell, and an arm's
environment is the one cluster_firsthit_probe.sh gives it. No GPU."""
import json
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _golden():
    return json.load(open(os.path.join(HERE, "golden", "manifest_golden.json")))


@pytest.mark.parametrize("case", range(4))
def test_plan_matches_reference_list_only(case):
    from bs45_quantum_explorer_gb300.manifest import plan_class
    g = _golden()
    if case >= len(g):
        pytest.skip("no such golden case")
    c = g[case]
    p = plan_class(c["n"], tuple(c["sig"]), 300, c["narms"])
    for k in ("cells", "kept", "windows", "digest", "kept_per_arm_min", "kept_per_arm_max"):
        assert p[k] == c[k], k
    # lanes of 300 windows, contiguous, covering [0, windows)
    assert p["lanes"][0]["skip"] == 0 and p["lanes"][-1]["end"] == c["windows"]
    assert all(a["end"] == b["skip"] for a, b in zip(p["lanes"], p["lanes"][1:]))


def test_plan_refuses_even_arm_counts_and_builds_arm_env():
    from bs45_quantum_explorer_gb300.manifest import arm_env, plan
    with pytest.raises(ValueError):
        plan(30, [((1, 7, 6, 6), 2, "x", "A")], 178)
    m = plan(30, [((1, 7, 6, 6), 2, "x", "A")], 177)
    cls = m["classes"][0]
    assert [ln["skip"] for ln in cls["lanes"]] == list(range(0, cls["windows"], 2))
    env = arm_env(30, cls, cls["lanes"][1], 177, 5, rev=1, ckpt_dir="/ck")
    assert env["WZ_FH_SHARD"] == "5" and env["WZ_FH_NSHARD"] == "177"
    assert env["WZ_FH_PROF_SKIP"] == "2" and env["WZ_FH_PROF_END"] == str(min(4, cls["windows"]))
    assert env["WZ_FH_STREAM_REV"] == "1" and env["WZ_FH_EXPECT_DIGEST"] == cls["digest"]
    assert env["WZ_FH_CKPT_DIR"] == "/ck" and env["WZ_FH_PROF_ORDER"] == "3"


def _production():
    g = json.load(open(os.path.join(HERE, "golden", "production_manifest_golden.json")))
    return [(p, c) for p in g for c in p["classes"]]


@pytest.mark.parametrize("i", range(22))
def test_plan_matches_reference_production_manifest(i):
    """The reference's own production manifests (Pass H, n = 44 and n = 45, from its planner's
    list-only solver runs; tests/golden/production_manifest_golden.json): the same raw and
    kept cell counts, windows, list:kept digest and lanes for each class."""
    from bs45_quantum_explorer_gb300.manifest import plan_class
    cases = _production()
    assert len(cases) == 22
    p, c = cases[i]
    got = plan_class(p["n"], tuple(c["sig"]), c["S"], p["narms"], endpos=p["endpos"])
    for k in ("cells", "kept", "windows", "digest", "lanes"):
        assert got[k] == c[k], (c["sig"], k)
