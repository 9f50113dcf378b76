"""The roadmap heuristic (include/dpg_roadmap.h) from Python: sample
collision-free states, build the roadmap (GPU edge checks, Dijkstra from the
goal), evaluate h for batches of states."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from . import workloads as W
from ._lib import check


def _ptr(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def states_valid(ctx, x: np.ndarray) -> np.ndarray:
    """bounds and obstacle separation of each row of x, on the GPU"""
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, ctx.nx)
    out = np.empty(len(x), np.uint8)
    check(_lib.load().dpg_states_valid(ctx.h, len(x), _ptr(x), _ptr(out)), ctx.h)
    return out.astype(bool)


def sample_free(ctx, model, env, n: int, trials: int, seed: int = 0) -> np.ndarray:
    """Up to n collision-free states, velocities zero, from `trials` uniform
    draws in the bounds (generate_heuristic_map, heuristics.cpp:17-35)"""
    rng = W.Rng(seed)
    pd = 3 if model.kind == W.QUAD3D else 2
    x = np.zeros((trials, model.nx))
    x[:, :pd] = env.lo + (env.hi - env.lo) * rng.uniform((trials, pd))
    if model.kind == W.QUAD3D:
        x[:, 3:7] = rng.unit_quaternions(trials)
    else:
        x[:, 2] = rng.uniform(trials, -np.pi, np.pi)
        if model.kind == W.CAR1:
            x[:, 3] = x[:, 2] + rng.uniform(trials, -np.pi / 4, np.pi / 4)
    return x[states_valid(ctx, x)][:n]


class Roadmap:
    def __init__(self, ctx, samples: np.ndarray, connection_radius: float = 1.0, resolution: float = 0.5):
        """samples: start first, goal last (velocities zero)"""
        self.lib = _lib.load()
        s = np.ascontiguousarray(samples, dtype=np.float64)
        h = C.c_void_p()
        check(self.lib.dpg_roadmap_build(ctx.h, len(s), _ptr(s), connection_radius, resolution, C.byref(h)), ctx.h)
        self.h, self.S = h, len(s)

    def close(self):
        if getattr(self, "h", None):
            self.lib.dpg_roadmap_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def edges(self):
        n = C.c_int64()
        check(self.lib.dpg_roadmap_edges(self.h, C.byref(n), None, None, 0))
        ij = np.empty((n.value, 2), np.int32)
        w = np.empty(n.value)
        check(self.lib.dpg_roadmap_edges(self.h, C.byref(n), _ptr(ij), _ptr(w), n.value))
        return ij, w

    def distances(self):
        d = np.empty(self.S)
        p = np.empty(self.S, np.int32)
        check(self.lib.dpg_roadmap_distances(self.h, _ptr(d), _ptr(p)))
        return d, p

    def heuristic(self, x: np.ndarray, goal: np.ndarray, connect_radius: float = 0.5) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        g = np.ascontiguousarray(goal, dtype=np.float64)
        out = np.empty(len(x))
        check(self.lib.dpg_roadmap_heuristic(self.h, len(x), _ptr(x), _ptr(g), connect_radius, _ptr(out)))
        return out
