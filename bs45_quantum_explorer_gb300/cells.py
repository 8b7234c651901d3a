"""The lane's cell list and per-cell allowed A,B rows, through the host-only C ABI
(bs_cell_list, bs_ab_rows in include/bsfh.h). No device is touched: a scheduler can plan a
lane (its cells, their rows and so its HBM footprint) before it opens a GPU context.

cell_list() reproduces the first-hit lane's list block (src/solver/wz_match.cpp:1388-1886):
raw cell i of the returned list is the lane's raw cell index i (WZ_FH_SHARD ownership,
WZ_FH_PROF_SKIP/END windows and checkpoints count in it).
"""
import ctypes as C

import numpy as np

from ._lib import BS_OK, BsError, Cell, ListOpts, check, lib

BS_ERR_CAP = -6


def lane_defaults(n):
    """The lane's defaults at this n (WZ_FH_M6, 2.11b and 2.12 forced at n >= 36)."""
    return dict(m6=n >= 36, thm211b=n >= 36, thm212=n >= 36)


LIST_GUESS = 1 << 20


def cell_list(n, sig, m6=None, thm211b=None, thm212=None, endpos=False, orbit_canon=False,
              orbit_q=0, qprune=False, prof_order=0, nshard=1):
    """Returns (cells, kept, digest, m): cells a ctypes array of bs_cell, kept a uint8 array,
    digest the ORDER=3 "<list>:<kept>" string ('' otherwise)."""
    d = lane_defaults(n)
    o = ListOpts(m6=int(d["m6"] if m6 is None else m6),
                 thm211b=int(d["thm211b"] if thm211b is None else thm211b or n >= 36),
                 thm212=int(d["thm212"] if thm212 is None else thm212 or n >= 36),
                 endpos=int(endpos), orbit_canon=int(orbit_canon), orbit_q=int(orbit_q),
                 qprune=int(qprune), prof_order=int(prof_order), nshard=int(nshard))
    a, b, c, dd = sig
    ncells = C.c_longlong(0)
    dig = C.create_string_buffer(40)
    # one build into a buffer of LIST_GUESS cells (24 MB); a longer list is built a second
    # time into a buffer of the size the first call reported
    cap = LIST_GUESS
    for _ in range(2):
        cells = (Cell * cap)()
        kept = np.zeros(cap, dtype=np.uint8)
        rc = lib().bs_cell_list(n, a, b, c, dd, C.byref(o), cells, kept.ctypes.data, cap,
                                C.byref(ncells), dig)
        if rc == 2:
            raise BsError(rc, "cell_list: the reference refuses this list")
        if rc != BS_ERR_CAP:
            break
        cap = max(1, ncells.value)
    check(rc, "cell_list")
    if ncells.value < cap:
        cells = (Cell * max(1, ncells.value)).from_buffer_copy(cells)
    return cells, kept[:ncells.value].copy(), dig.value.decode(), 6 if o.m6 else 3


def ab_rows(n, sig, m, cells):
    """(rows int8 [R,16], row_off int64 [N], nrows int32 [N]) for the given cells."""
    ncell = len(cells)
    arr = cells if isinstance(cells, C.Array) else (Cell * max(1, ncell))(*cells)
    row_off = np.zeros(max(1, ncell), dtype=np.int64)
    nrows = np.zeros(max(1, ncell), dtype=np.int32)
    total = C.c_longlong(0)
    a, b = sig[0], sig[1]
    # one call when the rows fit a first guess; the call reports the size when they do not
    cap = max(1 << 16, 4096 * max(1, ncell))
    rows = np.zeros((cap, 16), dtype=np.int8)
    rc = lib().bs_ab_rows(n, a, b, m, arr, ncell, rows.ctypes.data, cap, row_off.ctypes.data,
                          nrows.ctypes.data, C.byref(total))
    if rc == BS_ERR_CAP:
        rows = np.zeros((max(1, total.value), 16), dtype=np.int8)
        rc = lib().bs_ab_rows(n, a, b, m, arr, ncell, rows.ctypes.data, total.value,
                              row_off.ctypes.data, nrows.ctypes.data, C.byref(total))
    check(rc, "ab_rows")
    return rows[:total.value], row_off[:ncell], nrows[:ncell]


def cell_tuple(cell, m):
    return (tuple(cell.tx[:m]), tuple(cell.ty[:m]))
