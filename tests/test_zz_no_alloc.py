"""The allocation-free Hall filter entry point (bs_hall_filter_noalloc).

It serves callers that may not allocate device memory (a device-memory budget owned by a
scheduler or host framework; latency-sensitive code that cannot afford cudaMalloc's device
synchronisation). Its scratch is a fixed static device array, so the test checks that two
calls in a row, through the C ABI, give exactly the decisions of the allocating entry point
bs_hall_filter_dev on the same inputs, that a third call with another sequence length
rebuilds its tables correctly, and that an oversized request is refused. This file is
collected last so a stop-at-first-failure run has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PAIRS = 1 << 20


def _reference_mask(n, sig, d_words, npairs):
    """Decisions of the existing (allocating) entry point on the same device input."""
    import torch
    from bs45_quantum_explorer_gb300.hall import Context
    ctx = Context(n, sig)
    d_pass = torch.zeros(max(1, npairs), dtype=torch.uint8, device="cuda")
    ctx.hall_filter_dev(d_words.data_ptr(), npairs, d_pass.data_ptr(), "tc_fp16", stats=True)
    torch.cuda.synchronize()
    out = d_pass[:npairs].cpu().numpy().copy()
    ctx.close()
    return out


def _noalloc(n, d_words, npairs, d_pass, stream=None):
    from bs45_quantum_explorer_gb300._lib import lib
    return lib().bs_hall_filter_noalloc(n, C.c_void_p(d_words.data_ptr()), npairs,
                                        C.c_void_p(d_pass.data_ptr()), C.c_void_p(stream))


def test_noalloc_matches_allocating_entry_point(gpu, oracle):
    import torch
    from bs45_quantum_explorer_gb300.workloads import unpack_pairs
    runs = [(42, (7, 11, 0, 0), 200003, 0xB545C2), (42, (7, 11, 0, 0), 65536, 0xB545C7),
            (30, (1, 7, 6, 6), 50000, 0xB545C3)]
    for n, sig, npairs, seed in runs:
        words = oracle.gen_hall_pairs(n, npairs, seed=seed, nthreads=8)
        d_words = torch.from_numpy(words.view(np.int64).reshape(-1).copy()).cuda()
        d_pass = torch.full((npairs,), 7, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        rc = _noalloc(n, d_words, npairs, d_pass)
        assert rc == 0, rc
        got = d_pass.cpu().numpy()
        want = _reference_mask(n, sig, d_words, npairs)
        assert np.array_equal(got, want), (n, npairs, int((got != want).sum()))
        # and both equal the oracle on a sample
        ref = oracle.hall_batch(n, unpack_pairs(words[:4096], n), nthreads=8)
        assert np.array_equal(got[:4096], ref)


def _near_threshold(n, oracle, npairs, seed, width):
    """Pairs whose exact max pair PSD lies within +-width of the limit 4n+2.5, so that the
    margin band and the FP64 recheck run."""
    from bs45_quantum_explorer_gb300.workloads import unpack_pairs
    words = oracle.gen_hall_pairs(n, npairs, seed=seed, nthreads=8)
    ct, st = oracle.hall_tables(n)
    X = unpack_pairs(words, n).astype(np.float64)
    re, im = X @ ct[1:, :n].T, X @ st[1:, :n].T
    mx = (re * re + im * im).sum(axis=1).max(axis=1)
    return np.ascontiguousarray(words[np.abs(mx - (4 * n + 2.5)) < width])


def test_noalloc_on_caller_stream_longest_length_and_full_size(gpu, oracle):
    """A caller-supplied stream, the longest accepted length (n = 63, where the FP64 recheck
    uses the most shared memory), a call at the maximum size, and an empty call."""
    import torch
    s = torch.cuda.Stream()
    cases = [(63, (12, 10, 3, 1), _near_threshold(63, oracle, 1 << 18, 0xB545D1, 16.0)),
             (42, (7, 11, 0, 0), oracle.gen_hall_pairs(42, MAX_PAIRS, seed=0xB545D2, nthreads=8))]
    for n, sig, words in cases:
        npairs = len(words)
        assert npairs > 20
        d_words = torch.from_numpy(words.view(np.int64).reshape(-1).copy()).cuda()
        d_pass = torch.full((npairs,), 7, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        for _ in range(2):
            with torch.cuda.stream(s):
                rc = _noalloc(n, d_words, npairs, d_pass, s.cuda_stream)
            assert rc == 0, rc
            s.synchronize()
            got = d_pass.cpu().numpy()
            want = _reference_mask(n, sig, d_words, npairs)
            assert np.array_equal(got, want), (n, npairs, int((got != want).sum()))
    d_pass = torch.zeros(1, dtype=torch.uint8, device="cuda")
    assert _noalloc(42, d_words, 0, d_pass, s.cuda_stream) == 0


def test_noalloc_refuses_oversized_request(gpu):
    import torch
    d_words = torch.zeros(2, dtype=torch.int64, device="cuda")
    d_pass = torch.zeros(1, dtype=torch.uint8, device="cuda")
    from bs45_quantum_explorer_gb300._lib import lib
    rc = lib().bs_hall_filter_noalloc(42, C.c_void_p(d_words.data_ptr()), MAX_PAIRS + 1,
                                      C.c_void_p(d_pass.data_ptr()), None)
    assert rc == -6  # BS_ERR_CAP, nothing launched
    rc = lib().bs_hall_filter_noalloc(3, C.c_void_p(d_words.data_ptr()), 1,
                                      C.c_void_p(d_pass.data_ptr()), None)
    assert rc == -1  # BS_ERR_ARG
