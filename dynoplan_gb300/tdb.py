"""tdb-A*'s pair checks (include/dpg_tdb.h) from Python."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check

CONSTRAINT_VIOLATION = 3


class TdbArgs(C.Structure):
    _fields_ = [("reverse", C.c_int32), ("node_g", C.c_void_p), ("n_constraints", C.c_int32),
                ("c_time", C.c_void_p), ("c_state", C.c_void_p), ("goal", C.c_void_p), ("delta", C.c_double)]


def check_pairs(ctx, x, node, prim, reverse=False, node_g=None, c_time=None, c_state=None, goal=None, delta=0.5):
    """verdict, first_invalid, end_state of the pairs (node[i], prim[i]) of the
    states x, forward or reverse, with the constraints (c_time[k], c_state[k])"""
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, ctx.nx)
    node = np.ascontiguousarray(node, dtype=np.uint32)
    prim = np.ascontiguousarray(prim, dtype=np.uint32)
    nc = 0 if c_time is None else len(c_time)
    keep = []

    def ptr(a, dt):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return a.ctypes.data

    args = TdbArgs(1 if reverse else 0, ptr(node_g, np.float32), nc, ptr(c_time, np.float32),
                   ptr(c_state, np.float64), ptr(goal, np.float64), delta)
    n = len(node)
    verdict = np.empty(n, np.uint8)
    fi = np.empty(n, np.int32)
    end = np.empty((n, ctx.nx))
    check(_lib.load().dpg_tdb_check_pairs(ctx.h, C.byref(args), len(x), x.ctypes.data, n, node.ctypes.data,
                                          prim.ctypes.data, verdict.ctypes.data, fi.ctypes.data, end.ctypes.data),
          ctx.h)
    return verdict, fi, end
