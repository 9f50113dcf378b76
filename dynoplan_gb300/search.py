"""db-A* over the batched GPU expansion (include/dpg_search.h) from Python."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check

HEU_BLIND, HEU_EUCLIDEAN, HEU_MLP, HEU_ROADMAP = -1, 0, 1, 2
STATUS = {0: "SOLVED", 1: "MAX_EXPANDS", 2: "EMPTY_QUEUE", 3: "MAX_TIME"}


class SearchOpts(C.Structure):
    _fields_ = [("delta", C.c_double), ("alpha", C.c_double), ("delta_factor_goal", C.c_double),
                ("cost_delta_factor", C.c_double), ("limit_branching_factor", C.c_int32), ("batch", C.c_int32),
                ("max_expands", C.c_int64), ("time_limit_ms", C.c_double), ("heuristic", C.c_int32),
                ("precision", C.c_int32), ("shuffle", C.c_int32), ("max_neighbors", C.c_int32),
                ("seed", C.c_uint64), ("roadmap", C.c_void_p), ("connect_radius_h", C.c_double)]


class SearchResult(C.Structure):
    _fields_ = [("solved", C.c_int32), ("status", C.c_int32), ("cost", C.c_double), ("g", C.c_float),
                ("path_len", C.c_int32), ("expands", C.c_int64), ("nodes", C.c_int64),
                ("checked_pairs", C.c_int64), ("time_ms", C.c_double), ("expand_ms", C.c_double),
                ("novelty_ms", C.c_double), ("mlp_ms", C.c_double), ("prepare_ms", C.c_double),
                ("insert_ms", C.c_double), ("rounds", C.c_int64), ("table_ms", C.c_double),
                ("query_ms", C.c_double)]


def options(delta, alpha=0.5, batch=1, heuristic=HEU_EUCLIDEAN, limit_branching_factor=20,
            max_expands=100000, time_limit_ms=60000.0, precision=0, shuffle=0, seed=0, max_neighbors=64,
            delta_factor_goal=1.0, cost_delta_factor=1.0, roadmap=None, connect_radius_h=0.5) -> SearchOpts:
    """roadmap: a dynoplan_gb300.roadmap.Roadmap for HEU_ROADMAP"""
    return SearchOpts(delta, alpha, delta_factor_goal, cost_delta_factor, limit_branching_factor, batch,
                      max_expands, time_limit_ms, heuristic, precision, shuffle, max_neighbors, seed,
                      roadmap.h if roadmap is not None else None, connect_radius_h)


def search(ctx, start, goal, opts: SearchOpts, mlp=None, max_path=4096):
    """Runs dpg_search on a gpu.Context; returns (result dict, motions, states)."""
    lib = _lib.load()
    start = np.ascontiguousarray(start, dtype=np.float64)
    goal = np.ascontiguousarray(goal, dtype=np.float64)
    res = SearchResult()
    motions = np.zeros(max_path, np.int32)
    states = np.zeros((max_path + 1, ctx.nx))
    check(lib.dpg_search(ctx.h, C.byref(opts), start.ctypes.data, goal.ctypes.data,
                         mlp.h if mlp is not None else None, C.byref(res), motions.ctypes.data,
                         states.ctypes.data, max_path), ctx.h)
    d = {k: getattr(res, k) for k, _ in SearchResult._fields_}
    d["status_str"] = STATUS.get(res.status, "?")
    n = res.path_len if res.solved else 0
    return d, motions[:n].copy(), states[:n + 1].copy()
