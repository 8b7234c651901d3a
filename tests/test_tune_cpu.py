"""The autotuner's choice rules on the host (tune.py), with the device calls replaced: the
completer probes run every (blocks_per_sm, chunk) setting on the same capped-budget sample,
take the fastest, and among settings within 3 % of it prefer the one with more resident
warps; the stream probes take the fastest (fine_nodes, dfs_blocks) pair, then the fastest
wave size. Results are cached per workload."""
import numpy as np
import pytest


def _fake_rates(monkeypatch, rate_of):
    """tune._rate -> rate_of(setting) for the probe closure's bound defaults (no timing)."""
    import bs45_quantum_explorer_gb300.tune as tune

    def fake_rate(fn, reps=2):
        fn()  # the probe still runs (against the stand-in device calls)
        return rate_of(fn.__defaults__)
    monkeypatch.setattr(tune, "_rate", fake_rate)
    return tune


class _Ctx:
    n, sig = 36, (5, 11, 0, 0)


@pytest.mark.parametrize("rates,want", [
    # blocks 3 within 3 % of the best: more resident warps win the tie
    ({1: 6.0e8, 2: 1.00e9, 3: 0.98e9}, 3),
    # blocks 3 clearly slower (its register cut spills): blocks 2
    ({1: 6.0e8, 2: 1.00e9, 3: 0.70e9}, 2),
    # one block per SM only wins when it is clearly fastest
    ({1: 1.2e9, 2: 1.00e9, 3: 0.90e9}, 1),
])
def test_completer_choice(monkeypatch, rates, want):
    calls = []

    def fake_complete(ctx, cands, budget, rows=None, m=6, blocks_per_sm=0, **kw):
        calls.append((len(cands), budget, blocks_per_sm))
        k = len(cands)
        return (np.full(k, 2, np.int32), np.full(k, 100, np.int64), None, None)

    tune = _fake_rates(monkeypatch, lambda d: rates[d[0]])
    monkeypatch.setattr(tune, "complete_ab", fake_complete)
    tune._CACHE.clear()
    cands = np.arange(2 * 20000, dtype=np.uint64).reshape(-1, 2)
    choice, probes = tune.tune_completer(_Ctx(), cands, budget=1 << 22, sample=16384)
    assert choice["blocks_per_sm"] == want
    assert {p["blocks_per_sm"] for p in probes} == set(tune.AB_BLOCKS)
    # every probe ran the same capped sample: at most 2^14 nodes per candidate, 16,384 of them
    probe_calls = [c for c in calls if c[2] != 0]
    assert probe_calls and all(b == 1 << 14 for _, b, _ in probe_calls)
    assert sum(n for n, _, blk in probe_calls if blk == want) % 16384 == 0
    # cached: a second call runs nothing
    n_before = len(calls)
    assert tune.tune_completer(_Ctx(), cands, budget=1 << 22, sample=16384)[0] == choice
    assert len(calls) == n_before


def test_stream_choice(monkeypatch):
    def fake_stream(ctx, cells, m=6, pins=None, as_words=True, limit=0, **kw):
        return np.zeros((0, 2), np.uint64), np.zeros(0, np.uint32), [{"nodes": 10, "leaves": 0, "ok": 0}]

    import bs45_quantum_explorer_gb300.tune as tune
    table = {(5e3, 4): 9e8, (5e3, 5): 8e8, (2e4, 4): 6e8, (2e4, 6): 9.5e8}
    waves = {2e9: 9e8, 8e9: 9.6e8, 3.2e10: 9.1e8}
    seen = []

    def fake_rate(fn, reps=2):
        fn()
        kw = seen[-1]
        if "wave_nodes" in kw:
            return waves[kw["wave_nodes"]]
        return table.get((kw["fine_nodes"], kw["dfs_blocks"]), 1e8)

    def recording_stream(ctx, cells, m=6, pins=None, as_words=True, limit=0, **kw):
        if limit and limit > 100:
            seen.append(kw)
        return fake_stream(ctx, cells, m=m, pins=pins, as_words=as_words, limit=limit, **kw)

    monkeypatch.setattr(tune, "_rate", fake_rate)
    monkeypatch.setattr(tune, "cd_stream", recording_stream)
    tune._CACHE.clear()
    choice, probes = tune.tune_stream(_Ctx(), ([1, 1, 1, 1, 1, 1], [1, 1, 1, 1, 1, 1]), probe=20000)
    assert (choice["fine_nodes"], choice["dfs_blocks"]) == (2e4, 6)
    assert choice["wave_nodes"] == 8e9
    assert len(probes) == len(tune.FINE) * len(tune.BLOCKS) + len(tune.WAVES)
