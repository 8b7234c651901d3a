"""Host-side mirror of the reference's Hall (Thm 2.4) filter interface.

The reference tests one pair at a time with `hall_ok_pair_fast(X, L, Y, L)`
(src/solver/wz_match.cpp:143-168); here the same decision is made for a batch on the GPU
through the C ABI (include/bsfh.h). Context is the reference's global state (n, signature,
G_HALL_COS/SIN tables) held per object instead of in globals.
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import HALL_FP64, HALL_TC_BF16X2, HALL_TC_FP16, HallStats, check, lib

MODES = {"fp64": HALL_FP64, "tc_fp16": HALL_TC_FP16, "tc_bf16x2": HALL_TC_BF16X2}


def pack(seqs):
    """+-1 int8 rows [..., L] -> uint64 words [...] (bit i set when element i is +1)."""
    seqs = np.asarray(seqs)
    if seqs.size and not np.all((seqs == 1) | (seqs == -1)):
        raise ValueError("sequences must be +-1")
    L = seqs.shape[-1]
    if L > 64:
        raise ValueError("sequences longer than 64 do not fit a word")
    bits = (seqs == 1).astype(np.uint64)
    weights = (np.uint64(1) << np.arange(L, dtype=np.uint64))
    return (bits * weights).sum(axis=-1, dtype=np.uint64)


def unpack(words, L):
    words = np.asarray(words, dtype=np.uint64)
    bits = (words[..., None] >> np.arange(L, dtype=np.uint64)) & np.uint64(1)
    return np.where(bits == 1, 1, -1).astype(np.int8)


class Context:
    """One BS(n+1,n) search context on one GPU (bs_ctx in the C ABI)."""

    def __init__(self, n, sig, device=0):
        a, b, c, d = sig
        self.n, self.sig = n, tuple(sig)
        h = C.c_void_p()
        check(lib().bs_ctx_create(n, a, b, c, d, device, C.byref(h)), "bs_ctx_create")
        self.h = h

    def close(self):
        if self.h:
            lib().bs_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def request_stop(self, value=1):
        """Raise (or, with value 0, clear) the context's stop flag: running and later stream
        and completion calls stop within one device round and return what they completed."""
        lib().bs_ctx_stop_flag(self.h)[0] = int(value)

    def clear_stop(self):
        self.request_stop(0)

    def set_stream(self, stream_handle):
        check(lib().bs_ctx_set_stream(self.h, C.c_void_p(stream_handle)), "bs_ctx_set_stream")

    def retarget(self, n, sig):
        """Point the context at another (n, signature), keeping its stream and buffers. If it
        fails, n becomes None until a retarget succeeds (the tables are half loaded)."""
        a, b, c, d = sig
        rc = lib().bs_ctx_retarget(self.h, n, a, b, c, d)
        if rc != 0:
            self.n = self.sig = None
        check(rc, "bs_ctx_retarget")
        self.n, self.sig = n, tuple(sig)

    # ---- Hall filter ----
    def hall_filter(self, XY, mode="tc_fp16"):
        """XY: int8 [npairs, 2, n] (C, D). Returns (pass uint8 [npairs], stats dict)."""
        XY = np.ascontiguousarray(XY, dtype=np.int8)
        npairs = XY.shape[0]
        out = np.zeros(max(1, npairs), np.uint8)
        st = HallStats()
        check(lib().bs_hall_filter_batch(self.h, XY.ctypes.data, npairs, MODES[mode],
                                         out.ctypes.data, C.byref(st)), "bs_hall_filter_batch")
        return out[:npairs], st.as_dict()

    def hall_filter_packed(self, words, mode="tc_fp16"):
        """words: uint64 [npairs, 2] host. Returns (pass, stats)."""
        words = np.ascontiguousarray(words, dtype=np.uint64)
        npairs = words.shape[0]
        out = np.zeros(max(1, npairs), np.uint8)
        st = HallStats()
        check(lib().bs_hall_filter_packed(self.h, words.ctypes.data, npairs, MODES[mode],
                                          out.ctypes.data, C.byref(st)), "bs_hall_filter_packed")
        return out[:npairs], st.as_dict()

    def hall_filter_dev(self, d_words_ptr, npairs, d_pass_ptr, mode="tc_fp16", stats=True):
        """Device pointers (e.g. torch tensor data_ptr()). Enqueued on the context stream."""
        st = HallStats()
        check(lib().bs_hall_filter_dev(self.h, C.c_void_p(d_words_ptr), npairs, MODES[mode],
                                       C.c_void_p(d_pass_ptr), C.byref(st) if stats else None),
              "bs_hall_filter_dev")
        return st.as_dict() if stats else None

    def gen_hall_pairs_dev(self, npairs, d_words_ptr, seed=0xB545C2):
        check(lib().bs_gen_hall_pairs_dev(self.h, npairs, seed, C.c_void_p(d_words_ptr)),
              "bs_gen_hall_pairs_dev")

    def timing(self, enable=True):
        check(lib().bs_ctx_timing(self.h, int(enable)), "bs_ctx_timing")

    def timing_read(self):
        ms, t, a = C.c_double(), C.c_longlong(), C.c_longlong()
        check(lib().bs_ctx_timing_read(self.h, C.byref(ms), C.byref(t), C.byref(a)),
              "bs_ctx_timing_read")
        return ms.value, t.value, a.value

    def device_status(self):
        return lib().bs_ctx_device_status(self.h)

    def hall_tc_dump_dev(self, d_words_ptr, npairs, d_acc_ptr, mode="tc_fp16"):
        check(lib().bs_hall_tc_dump_dev(self.h, C.c_void_p(d_words_ptr), npairs, MODES[mode],
                                        C.c_void_p(d_acc_ptr)), "bs_hall_tc_dump_dev")


def device_status(ctx):
    return lib().bs_ctx_device_status(ctx.h)


__all__ = ["Context", "pack", "unpack", "MODES", "device_status", "_lib"]
