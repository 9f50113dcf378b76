"""ctypes binding of the FP64 oracle (oracle/oracle.c) -- the checker.

Test infrastructure: only the tests, the smoke check and bench.py's CPU
baseline load it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_SO = os.path.join(ORACLE_DIR, "_build", "liboracle.so")


class OrcRobot(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("nx", C.c_int32), ("nu", C.c_int32), ("n_parts", C.c_int32),
        ("dt", C.c_double), ("w", C.c_double * 4), ("box", C.c_double * 2),
        ("hitch", C.c_double), ("wheelbase", C.c_double), ("radius", C.c_double),
        ("mass", C.c_double), ("arm", C.c_double), ("t2t", C.c_double),
        ("inertia", C.c_double * 3), ("ang_gain", C.c_double), ("g", C.c_double),
    ]


class OrcEnv(C.Structure):
    _fields_ = [("dim", C.c_int32), ("lo", C.c_double * 3), ("hi", C.c_double * 3),
                ("n_obs", C.c_int32), ("obs_lo", C.c_void_p), ("obs_hi", C.c_void_p)]


class OrcPrims(C.Structure):
    _fields_ = [("P", C.c_int32), ("len", C.c_void_p), ("soff", C.c_void_p), ("aoff", C.c_void_p),
                ("states", C.c_void_p), ("actions", C.c_void_p)]


class OrcOut(C.Structure):
    _fields_ = [("cap", C.c_int64), ("n_pairs", C.c_int64), ("node", C.c_void_p),
                ("prim", C.c_void_p), ("verdict", C.c_void_p), ("first_invalid", C.c_void_p),
                ("end_state", C.c_void_p), ("min_gap", C.c_void_p), ("n_scanned", C.c_int64)]


_lib = None


def build_oracle(force: bool = False) -> str:
    src = os.path.join(ORACLE_DIR, "oracle.c")
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        subprocess.run(["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-std=c11", "-o",
                        ORACLE_SO + ".tmp", src, "-lm"], check=True)
        os.replace(ORACLE_SO + ".tmp", ORACLE_SO)
    return ORACLE_SO


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build_oracle())
        _lib.orc_robot_default.argtypes = [C.c_int, C.POINTER(OrcRobot)]
        _lib.orc_step.argtypes = [C.POINTER(OrcRobot), C.c_void_p, C.c_void_p, C.c_void_p]
        _lib.orc_distance.argtypes = [C.POINTER(OrcRobot), C.c_void_p, C.c_void_p]
        _lib.orc_distance.restype = C.c_double
        _lib.orc_lower_bound_time.argtypes = [C.POINTER(OrcRobot), C.c_void_p, C.c_void_p]
        _lib.orc_lower_bound_time.restype = C.c_double
        _lib.orc_rollout.argtypes = [C.POINTER(OrcRobot), C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]
        _lib.orc_state_gap.argtypes = [C.POINTER(OrcRobot), C.POINTER(OrcEnv), C.c_void_p, C.c_int]
        _lib.orc_state_gap.restype = C.c_double
        _lib.orc_is_state_valid.argtypes = [C.POINTER(OrcRobot), C.POINTER(OrcEnv), C.c_void_p]
        for f in ("orc_expand",):
            getattr(_lib, f).argtypes = [C.POINTER(OrcRobot), C.POINTER(OrcEnv), C.POINTER(OrcPrims),
                                         C.c_int64, C.c_void_p, C.c_double, C.POINTER(OrcOut)]
        _lib.orc_expand_fast.argtypes = [C.POINTER(OrcRobot), C.POINTER(OrcEnv), C.POINTER(OrcPrims),
                                         C.c_int64, C.c_void_p, C.c_double, C.c_int, C.POINTER(OrcOut)]
        _lib.orc_check_goal.argtypes = [C.POINTER(OrcRobot), C.c_void_p, C.c_int, C.c_void_p,
                                        C.c_double, C.c_int]
        _lib.orc_max_threads.restype = C.c_int
    return _lib


def robot(model) -> OrcRobot:
    """OrcRobot from a workloads.RobotModel (same field meaning)."""
    r = OrcRobot()
    lib().orc_robot_default(model.kind, C.byref(r))
    r.dt = model.dt
    for i in range(4):
        r.w[i] = model.w[i]
    r.box[0], r.box[1] = model.box
    r.hitch, r.wheelbase, r.radius = model.hitch, model.wheelbase, model.radius
    r.mass, r.arm, r.t2t = model.mass, model.arm, model.t2t
    for i in range(3):
        r.inertia[i] = model.inertia[i]
    r.ang_gain, r.g = model.ang_gain, model.g
    return r


def _p(a):
    return C.c_void_p(a.ctypes.data)


class _Keep:
    pass


def env_struct(env):
    k = _Keep()
    k.lo = np.ascontiguousarray(env.obs_lo, dtype=np.float64)
    k.hi = np.ascontiguousarray(env.obs_hi, dtype=np.float64)
    e = OrcEnv()
    e.dim = env.dim
    for i in range(env.dim):
        e.lo[i], e.hi[i] = env.lo[i], env.hi[i]
    e.n_obs = len(k.lo)
    e.obs_lo = _p(k.lo) if len(k.lo) else None
    e.obs_hi = _p(k.hi) if len(k.hi) else None
    return e, k


def prims_struct(prims):
    k = _Keep()
    k.len = np.ascontiguousarray(prims.length, dtype=np.int32)
    k.soff = prims.soff()
    k.aoff = prims.aoff()
    k.st = np.ascontiguousarray(prims.states, dtype=np.float64)
    k.ac = np.ascontiguousarray(prims.actions, dtype=np.float64)
    if k.ac.size == 0:
        k.ac = np.zeros((1, 1))
    p = OrcPrims()
    p.P = len(k.len)
    p.len, p.soff, p.aoff, p.states, p.actions = _p(k.len), _p(k.soff), _p(k.aoff), _p(k.st), _p(k.ac)
    return p, k


def expand(model, prims, env, nodes, radius, fast=False, threads=1, capacity=None):
    """Run the oracle; returns a dict of numpy arrays, node-major order."""
    L = lib()
    r = robot(model)
    e, ke = env_struct(env)
    p, kp = prims_struct(prims)
    x = np.ascontiguousarray(nodes, dtype=np.float64)
    N = len(x)
    cap = capacity if capacity is not None else max(1024, N * 64)
    while True:
        o = dict(node=np.empty(cap, np.uint32), prim=np.empty(cap, np.uint32),
                 verdict=np.empty(cap, np.uint8), first_invalid=np.empty(cap, np.int16),
                 end_state=np.empty((cap, model.nx)), min_gap=np.empty(cap))
        out = OrcOut(cap=cap)
        for k in o:
            setattr(out, k, _p(o[k]))
        if fast:
            rc = L.orc_expand_fast(C.byref(r), C.byref(e), C.byref(p), N, _p(x), radius, threads, C.byref(out))
        else:
            rc = L.orc_expand(C.byref(r), C.byref(e), C.byref(p), N, _p(x), radius, C.byref(out))
        if rc != 0:
            cap = int(out.n_pairs)
            continue
        break
    n = int(out.n_pairs)
    res = {k: v[:n] for k, v in o.items()}
    res["n_pairs"] = n
    res["n_scanned"] = int(out.n_scanned)
    return res


def step(model, x, u):
    r = robot(model)
    x = np.ascontiguousarray(x, dtype=np.float64)
    u = np.ascontiguousarray(u, dtype=np.float64)
    xn = np.empty_like(x)
    lib().orc_step(C.byref(r), _p(x), _p(u), _p(xn))
    return xn


def distance(model, a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return lib().orc_distance(C.byref(robot(model)), _p(a), _p(b))


def lower_bound_time(model, a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return lib().orc_lower_bound_time(C.byref(robot(model)), _p(a), _p(b))


def rollout(model, x0, us):
    us = np.ascontiguousarray(us, dtype=np.float64)
    x0 = np.ascontiguousarray(x0, dtype=np.float64)
    xs = np.empty((len(us) + 1, model.nx))
    lib().orc_rollout(C.byref(robot(model)), _p(x0), _p(us), len(us), _p(xs))
    return xs


def sort_pairs(res, nx):
    """Reorder a result dict by (node, prim)."""
    key = res["node"].astype(np.int64) * (1 << 32) + res["prim"].astype(np.int64)
    order = np.argsort(key, kind="stable")
    out = {}
    for k, v in res.items():
        out[k] = v[order] if isinstance(v, np.ndarray) and len(v) == len(order) else v
    return out


def state_valid(model, env, x):
    """inside the bounds and separated (gap > 0) from every obstacle"""
    L = lib()
    L.orc_is_state_valid.argtypes = [C.POINTER(OrcRobot), C.POINTER(OrcEnv), C.c_void_p]
    L.orc_is_state_valid.restype = C.c_int
    r = robot(model)
    e, ke = env_struct(env)
    x = np.ascontiguousarray(x, dtype=np.float64)
    if not L.orc_is_state_valid(C.byref(r), C.byref(e), _p(x)):
        return False
    return all(L.orc_state_gap(C.byref(r), C.byref(e), _p(x), o) > 0.0 for o in range(e.n_obs))
