"""Hall (Thm 2.4) filter: the CUDA forms against the oracle, through the C ABI.

Decisions must be bit-identical to the oracle (itself pinned to the reference's
hall_ok_pair_fast, src/solver/wz_match.cpp:143-168) for the FP64 form and for both
tensor-core forms after their FP64 recheck of the margin band. For the tensor-core forms the
raw TMEM accumulators must equal the exact quantised DFT, and the PSD error against FP64 must
stay inside the certified bound 4 e sqrt(pf) + 4 e^2 (+ fp32 rounding, rho = 2^-20).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MODES = ("fp64", "tc_fp16", "tc_bf16x2")


def _ctx(n, sig):
    from bs45_quantum_explorer_gb300.hall import Context
    return Context(n, sig)


def _sig_for(n):
    """The first admissible signature class (a <= b, c <= d, parities of n+1 and n)."""
    tgt = 4 * n + 2
    for a in range((n + 1) % 2, n + 2, 2):
        for b in range(a, n + 2, 2):
            for c in range(n % 2, n + 1, 2):
                rest = tgt - a * a - b * b - c * c
                if rest < c * c:
                    break
                d = int(round(rest ** 0.5))
                if d * d == rest and d >= c and (d - n) % 2 == 0:
                    return (a, b, c, d)
    raise ValueError(n)


def _check_all_modes(ctx, words, ref):
    for mode in MODES:
        got, st = ctx.hall_filter_packed(words, mode)
        bad = np.nonzero(got != ref)[0]
        assert bad.size == 0, (mode, bad[:10], st)
        assert st["passed"] == int(ref.sum()), (mode, st)


def test_hall_microbench_parity(gpu, oracle):
    n = 42
    words = oracle.gen_hall_pairs(n, 1 << 17, nthreads=8)
    from bs45_quantum_explorer_gb300.workloads import unpack_pairs
    ref = oracle.hall_batch(n, unpack_pairs(words, n), nthreads=8)
    ctx = _ctx(n, (7, 11, 0, 0))
    _check_all_modes(ctx, words, ref)
    # the int8 host entry point (reference layout) agrees with the packed one
    got, _ = ctx.hall_filter(unpack_pairs(words[:4096], n), "tc_fp16")
    assert (got == ref[:4096]).all()


def test_device_generator_matches_oracle(gpu, oracle):
    import torch
    n = 42
    ctx = _ctx(n, (7, 11, 0, 0))
    d = torch.empty((1 << 16) * 2, dtype=torch.int64, device="cuda")
    ctx.gen_hall_pairs_dev(1 << 16, d.data_ptr())
    torch.cuda.synchronize()
    got = d.cpu().numpy().view(np.uint64).reshape(-1, 2)
    ref = oracle.gen_hall_pairs(n, 1 << 16, nthreads=8)
    assert (got == ref).all()


@pytest.mark.parametrize("n", [10, 13, 16, 21, 24])
def test_hall_stream_leaves_parity(gpu, oracle, n):
    """Every class-exact leaf of real C,D streams (what the DFS hands the filter)."""
    from bs45_quantum_explorer_gb300.hall import pack
    sig = _sig_for(n)
    rng = np.random.default_rng(n)
    rows_all, pass_all = [], []
    c, d = sig[2], sig[3]
    cells = [(x, y) for x in _all_cells(n, c) for y in _all_cells(n, d)]
    rng.shuffle(cells)
    total = 0
    for tx, ty in cells:
        rows, flags, _ = oracle.cd_stream(n, tx, ty, m=6, keep_all=True, cap=20000)
        if len(rows):
            rows_all.append(rows)
            pass_all.append(flags)
            total += len(rows)
        if total > 30000:
            break
    rows = np.concatenate(rows_all)
    ref = np.concatenate(pass_all)
    assert len(rows) > 20
    words = pack(rows)
    ctx = _ctx(n, sig)
    _check_all_modes(ctx, words, ref)


def _all_cells(n, total, m=6):
    """Every class-sum vector (m classes) of a +-1 sequence of length n summing to total."""
    import itertools
    cnt = [len(range(c, n, m)) for c in range(m)]
    out = []
    for v in itertools.product(*[range(-k, k + 1, 2) for k in cnt[:-1]]):
        last = total - sum(v)
        if abs(last) <= cnt[-1] and (last + cnt[-1]) % 2 == 0:
            out.append(list(v) + [last])
    return out


def _exact_psd(words, n, oracle):
    from bs45_quantum_explorer_gb300.workloads import unpack_pairs
    ct, st = oracle.hall_tables(n)
    X = unpack_pairs(words, n).astype(np.float64)  # [P, 2, n]
    re = X @ ct[1:, :n].T  # [P, 2, 200]
    im = X @ st[1:, :n].T
    f = re * re + im * im
    return f.sum(axis=1)  # pair PSD per angle j=1..200


def test_hall_near_threshold_parity(gpu, oracle):
    """Pairs whose max pair PSD lies within +-2 of the limit: the margin band is exercised."""
    n = 42
    words = oracle.gen_hall_pairs(n, 1 << 19, seed=0xB545C7, nthreads=8)
    mx = _exact_psd(words, n, oracle).max(axis=1)
    lim = 4 * n + 2.5
    sel = np.nonzero(np.abs(mx - lim) < 2.0)[0]
    assert sel.size > 50
    near = np.ascontiguousarray(words[sel])
    from bs45_quantum_explorer_gb300.workloads import unpack_pairs
    ref = oracle.hall_batch(n, unpack_pairs(near, n), nthreads=8)
    ctx = _ctx(n, (7, 11, 0, 0))
    _check_all_modes(ctx, near, ref)
    _, st = ctx.hall_filter_packed(near, "tc_fp16")
    assert st["rechecked"] > 0  # the tensor-core band is really used on these inputs
    # the exact fixed-point test decides nearly all of them; FP64 takes what is left
    assert 0 <= st["fp64_rechecked"] <= st["rechecked"]


def _quantised_tables(n, oracle, mode):
    ct, st = oracle.hall_tables(n)
    js = list(range(1, 101)) + [200]
    out = []
    for tab in (ct, st):
        t = tab[js, :n]  # [101, n]
        if mode == "tc_fp16":
            q = np.rint(t * 2048.0) / 2048.0
        else:
            hi = np.rint(t * 256.0) / 256.0
            q = hi + np.rint((t - hi) * 131072.0) / 131072.0
        out.append(q)
    return out


@pytest.mark.parametrize("mode", ["tc_fp16", "tc_bf16x2"])
@pytest.mark.parametrize("n", [42, 13, 63])
def test_tc_accumulators_exact_and_error_bound(gpu, oracle, mode, n):
    import torch
    npairs = 4096
    words = oracle.gen_hall_pairs(n, npairs, seed=0xB545C9, nthreads=4)
    ctx = _ctx(n, _sig_for(n))
    d_words = torch.from_numpy(words.view(np.int64).reshape(-1).copy()).cuda()
    acc = torch.zeros((2 * npairs, 208), dtype=torch.float32, device="cuda")
    ctx.hall_tc_dump_dev(d_words.data_ptr(), npairs, acc.data_ptr(), mode)
    torch.cuda.synchronize()
    acc = acc.cpu().numpy().astype(np.float64)
    from bs45_quantum_explorer_gb300.workloads import unpack_pairs
    X = unpack_pairs(words, n).reshape(2 * npairs, n).astype(np.float64)
    qc, qs = _quantised_tables(n, oracle, mode)
    re_q = X @ qc.T  # exact: multiples of 2^-17 below 64
    im_q = X @ qs.T
    assert np.array_equal(acc[:, :101], re_q), np.abs(acc[:, :101] - re_q).max()
    assert np.array_equal(acc[:, 104:205], im_q), np.abs(acc[:, 104:205] - im_q).max()
    assert not acc[:, 101:104].any() and not acc[:, 205:].any()
    # PSD error of the tensor-core values against FP64 at the same angles
    f_q = (re_q ** 2 + im_q ** 2).reshape(npairs, 2, 101).sum(axis=1)
    f64 = _exact_psd(words, n, oracle)[:, list(range(100)) + [199]]
    _, st = ctx.hall_filter_packed(words[:64], mode)
    e = st["quant_err"]
    bound = 4 * e * np.sqrt(f_q) + 4 * e * e + 1e-9
    err = np.abs(f_q - f64)
    assert (err <= bound).all(), (err.max(), e)


def test_hall_edge_cases(gpu, oracle):
    from bs45_quantum_explorer_gb300._lib import BsError
    n = 42
    ctx = _ctx(n, (7, 11, 0, 0))
    words = oracle.gen_hall_pairs(n, 200, nthreads=2)
    from bs45_quantum_explorer_gb300.workloads import unpack_pairs
    ref = oracle.hall_batch(n, unpack_pairs(words, n))
    for k in (0, 1, 63, 64, 65, 127, 200):
        for mode in MODES:
            got, st = ctx.hall_filter_packed(words[:k], mode)
            assert (got == ref[:k]).all(), (k, mode)
            assert st["pairs"] == k
    bad = unpack_pairs(words[:4], n).copy()
    bad[2, 1, 7] = 0  # not a +-1 value
    with pytest.raises(BsError):
        ctx.hall_filter(bad, "tc_fp16")
    # the context still works after the rejected call
    got, _ = ctx.hall_filter_packed(words, "tc_fp16")
    assert (got == ref).all()
