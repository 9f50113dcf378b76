"""Python handle over the C ABI (include/dpg.h): one context per robot,
primitive set and environment; ``expand`` runs the batched expansion.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import ExpandOpts, ExpandOut, LazyStats, RobotDesc, TuneReport, Tuning, check

VALID, COLLISION, OUT_OF_BOUNDS = 0, 1, 2


def robot_desc(model) -> RobotDesc:
    """dpg_robot_desc from a workloads.RobotModel (or the library default for
    an int kind)."""
    lib = _lib.load()
    d = RobotDesc()
    if isinstance(model, int):
        check(lib.dpg_robot_default(model, C.byref(d)))
        return d
    check(lib.dpg_robot_default(model.kind, C.byref(d)))
    d.dt = model.dt
    for i in range(4):
        d.w[i] = model.w[i]
    d.box[0], d.box[1] = model.box
    d.hitch, d.wheelbase, d.radius = model.hitch, model.wheelbase, model.radius
    d.mass, d.arm, d.t2t = model.mass, model.arm, model.t2t
    for i in range(3):
        d.inertia[i] = model.inertia[i]
    d.ang_gain, d.g = model.ang_gain, model.g
    return d


def _ptr(a: np.ndarray):
    return C.c_void_p(a.ctypes.data) if a is not None else None


class PinnedArray:
    """numpy view of a page-locked host buffer (dpg_host_alloc)."""

    def __init__(self, shape, dtype):
        lib = _lib.load()
        self.dtype = np.dtype(dtype)
        self.shape = tuple(np.atleast_1d(shape))
        nbytes = int(np.prod(self.shape)) * self.dtype.itemsize
        self._p = lib.dpg_host_alloc(max(nbytes, 1))
        if not self._p:
            raise MemoryError("dpg_host_alloc failed")
        buf = (C.c_char * max(nbytes, 1)).from_address(self._p)
        self.array = np.frombuffer(buf, dtype=self.dtype, count=int(np.prod(self.shape))).reshape(self.shape)

    def free(self):
        if self._p:
            self.array = None
            _lib.load().dpg_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class ExpandResult(dict):
    """numpy arrays per pair: node, prim, verdict, first_invalid, end_state,
    min_gap, flags; plus counters."""


class Context:
    """A dpg_ctx: robot + primitives + environment on one GPU."""

    def __init__(self, model, device: int = 0):
        self.lib = _lib.load()
        self.model = model
        self.desc = robot_desc(model)
        self.nx, self.nu = self.desc.nx, self.desc.nu
        h = C.c_void_p()
        check(self.lib.dpg_create(C.byref(h), device, C.byref(self.desc)))
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.dpg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def upload_primitives(self, prims):
        length = np.ascontiguousarray(prims.length, dtype=np.int32)
        states = np.ascontiguousarray(prims.states, dtype=np.float64)
        actions = np.ascontiguousarray(prims.actions, dtype=np.float64)
        if actions.size == 0:
            actions = np.zeros((1, self.nu))
        check(self.lib.dpg_upload_primitives(self.h, len(length), _ptr(length), _ptr(states),
                                             _ptr(actions)), self.h)
        self.P = len(length)

    def prepend_primitives(self, prims):
        """Insert motions in front of the uploaded set (new indices 0..P-1,
        the old ones shifted by P), as idbA* adds its optimised motions."""
        length = np.ascontiguousarray(prims.length, dtype=np.int32)
        states = np.ascontiguousarray(prims.states, dtype=np.float64)
        actions = np.ascontiguousarray(prims.actions, dtype=np.float64)
        if actions.size == 0:
            actions = np.zeros((1, self.nu))
        check(self.lib.dpg_prepend_primitives(self.h, len(length), _ptr(length), _ptr(states),
                                              _ptr(actions)), self.h)
        self.P = getattr(self, "P", 0) + len(length)

    def upload_env(self, env):
        lo = np.ascontiguousarray(env.lo, dtype=np.float64)
        hi = np.ascontiguousarray(env.hi, dtype=np.float64)
        olo = np.ascontiguousarray(env.obs_lo, dtype=np.float64).reshape(-1)
        ohi = np.ascontiguousarray(env.obs_hi, dtype=np.float64).reshape(-1)
        n = len(env.obs_lo)
        check(self.lib.dpg_upload_env(self.h, len(lo), _ptr(lo), _ptr(hi), n,
                                      _ptr(olo) if n else None, _ptr(ohi) if n else None), self.h)

    def check_pairs(self, x: np.ndarray, node: np.ndarray, prim: np.ndarray, precision: int = 0,
                    contact_band: float = 1e-4) -> ExpandResult:
        """Exact check of the given (node, primitive) pairs; results in input order."""
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, self.nx)
        node = np.ascontiguousarray(node, dtype=np.uint32)
        prim = np.ascontiguousarray(prim, dtype=np.uint32)
        n = len(node)
        es_dtype = np.float64 if precision != 0 else np.float32
        o = dict(verdict=np.empty(n, np.uint8), first_invalid=np.empty(n, np.int16),
                 end_state=np.empty((n, self.nx), es_dtype), min_gap=np.empty(n, np.float32),
                 flags=np.empty(n, np.uint8))
        opts = ExpandOpts(radius=0.0, precision=precision, x_on_device=0, out_on_device=0, mode=0,
                          contact_band=contact_band, ball_band=1e-5)
        out = ExpandOut(capacity=n)
        for k, v in o.items():
            setattr(out, k, _ptr(v))
        check(self.lib.dpg_check_pairs(self.h, C.byref(opts), len(x), _ptr(x), n, _ptr(node), _ptr(prim),
                                       C.byref(out)), self.h)
        res = ExpandResult(o)
        res.update(node=node, prim=prim, n_pairs=n, n_contact_recheck=int(out.n_contact_recheck))
        return res

    def expand(self, x: np.ndarray, radius: float, precision: int = 0, capacity: int | None = None,
               contact_band: float = 1e-4, ball_band: float = 1e-5, outputs=None,
               ball_only: bool = False, reverse: bool = False) -> ExpandResult:
        """Batched expand of the rows of x (N x nx), results in host arrays.
        ball_only: the in-ball (node, prim) pairs without the exact check;
        reverse (with ball_only): the reverse ball, motions keyed on their
        last state (tdb-A*'s reverse search)."""
        x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1, self.nx)
        N = len(x)
        if capacity is None:
            capacity = max(1024, N * 64)
        opts = ExpandOpts(radius=radius, precision=precision, x_on_device=0, out_on_device=0,
                          mode=(1 if ball_only else 0) | (2 if reverse else 0), contact_band=contact_band,
                          ball_band=ball_band)
        while True:
            es_dtype = np.float64 if precision != 0 else np.float32
            o = outputs if outputs is not None else dict(
                node=np.empty(capacity, np.uint32), prim=np.empty(capacity, np.uint32),
                verdict=np.empty(capacity, np.uint8), first_invalid=np.empty(capacity, np.int16),
                end_state=np.empty((capacity, self.nx), es_dtype),
                min_gap=np.empty(capacity, np.float32), flags=np.empty(capacity, np.uint8))
            out = ExpandOut(capacity=capacity)
            for k in ("node", "prim", "verdict", "first_invalid", "end_state", "min_gap", "flags"):
                setattr(out, k, _ptr(o[k]) if o.get(k) is not None else None)
            rc = self.lib.dpg_expand(self.h, C.byref(opts), N, _ptr(x), C.byref(out))
            if rc == _lib.DPG_ERR_CAPACITY and outputs is None:
                capacity = int(out.n_pairs)
                continue
            check(rc, self.h)
            break
        n = int(out.n_pairs)
        res = ExpandResult({k: (v[:n] if v is not None else None) for k, v in o.items()})
        res["n_pairs"] = n
        res["n_scanned"] = int(out.n_scanned)
        res["n_contact_recheck"] = int(out.n_contact_recheck)
        res["n_ball_recheck"] = int(out.n_ball_recheck)
        return res

    def expand_device(self, x_ptr: int, N: int, radius: float, out_ptrs: dict, capacity: int,
                      precision: int = 0, contact_band: float = 1e-4, ball_band: float = 1e-5,
                      ball_only: bool = False):
        """Expand with the nodes and all outputs in device memory (raw device
        pointers); returns the counters.  ball_only: the in-ball pairs
        (node, prim) only."""
        opts = ExpandOpts(radius=radius, precision=precision, x_on_device=1, out_on_device=1,
                          mode=1 if ball_only else 0, contact_band=contact_band, ball_band=ball_band)
        out = ExpandOut(capacity=capacity)
        for k in ("node", "prim", "verdict", "first_invalid", "end_state", "min_gap", "flags"):
            setattr(out, k, C.c_void_p(out_ptrs[k]) if out_ptrs.get(k) else None)
        check(self.lib.dpg_expand(self.h, C.byref(opts), N, C.c_void_p(x_ptr), C.byref(out)), self.h)
        return dict(n_pairs=int(out.n_pairs), n_scanned=int(out.n_scanned),
                    n_contact_recheck=int(out.n_contact_recheck), n_ball_recheck=int(out.n_ball_recheck))

    def lazy_check_device(self, x_ptr: int, N: int, n: int, node_ptr: int, prim_ptr: int, out_ptrs: dict,
                          limit: int, score_ptr: int | None = None, score_stride: int = 1, precision: int = 0,
                          contact_band: float = 1e-4) -> dict:
        """dpg_lazy_check on device arrays: the n candidates (node, prim) of
        the N nodes, ranked per node by score (ascending; None = motion
        order), exact-checked in rank order until each node has `limit`
        valid motions.  out_ptrs: device arrays of n rows (verdict and
        flags required).  Returns the lazy statistics."""
        opts = ExpandOpts(radius=0.0, precision=precision, x_on_device=1, out_on_device=1, mode=0,
                          contact_band=contact_band, ball_band=1e-5)
        out = ExpandOut(capacity=n)
        for k in ("verdict", "first_invalid", "end_state", "min_gap", "flags"):
            setattr(out, k, C.c_void_p(out_ptrs[k]) if out_ptrs.get(k) else None)
        st = LazyStats()
        check(self.lib.dpg_lazy_check(self.h, C.byref(opts), N, C.c_void_p(x_ptr), n, C.c_void_p(node_ptr),
                                      C.c_void_p(prim_ptr), C.c_void_p(score_ptr) if score_ptr else None,
                                      score_stride, limit, C.byref(out), C.byref(st)), self.h)
        return dict(n_checked=int(st.n_checked), n_valid=int(st.n_valid), n_accepted=int(st.n_accepted),
                    rounds=int(st.rounds), max_candidates=int(st.max_candidates),
                    n_contact_recheck=int(out.n_contact_recheck))

    def tuning(self) -> dict:
        t = Tuning()
        check(self.lib.dpg_get_tuning(self.h, C.byref(t)), self.h)
        return {k: getattr(t, k) for k, _ in Tuning._fields_}

    def set_tuning(self, **kw):
        """launch choices (dpg_tuning fields); results never depend on them"""
        t = Tuning(**{**self.tuning(), **kw})
        check(self.lib.dpg_set_tuning(self.h, C.byref(t)), self.h)

    def autotune(self, x_ptr: int, N: int, radius: float, precision: int = 0, reps: int = 3,
                 cache_path: str | None = None) -> dict:
        """dpg_autotune on the N device-resident states at x_ptr: times the
        launch choices, applies the fastest; returns the report."""
        opts = ExpandOpts(radius=radius, precision=precision, x_on_device=1, out_on_device=1, mode=0,
                          contact_band=1e-4, ball_band=1e-5)
        r = TuneReport()
        check(self.lib.dpg_autotune(self.h, C.byref(opts), N, C.c_void_p(x_ptr), reps,
                                    cache_path.encode() if cache_path else None, C.byref(r)), self.h)
        tdict = lambda t: {k: getattr(t, k) for k, _ in Tuning._fields_}
        return {"chosen": tdict(r.chosen), "initial": tdict(r.initial), "ms_chosen": r.ms_chosen,
                "ms_initial": r.ms_initial, "seconds": r.seconds, "candidates": r.candidates,
                "from_cache": bool(r.from_cache), "key": r.key.decode()}

    def timings(self):
        t = (C.c_double * 4)()
        k = self.lib.dpg_last_timings(self.h, t, 4)
        return list(t)[:k]

    def set_abort(self, flag: bool):
        check(self.lib.dpg_set_abort(self.h, 1 if flag else 0), self.h)
