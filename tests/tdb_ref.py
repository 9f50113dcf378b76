"""Python restatement of tdb-A*'s check_lazy_trajectory
(src/tdbastar/tdbastar.cpp:314-447, LazyTraj::compute tdbastar.hpp:172-214)
over the oracle's bounds and separating-axis gap -- the checker of
include/dpg_tdb.h (forward and reverse for the translation robots, reverse
for quad2d and the quadrotor)."""
import math

import numpy as np

import oracle_bind as ob
from dynoplan_gb300 import workloads as W


# position and velocity components of the rollout robots (the offset)
_POS = {W.QUAD2D: [0, 1], W.QUAD3D: [0, 1, 2]}
_VEL = {W.QUAD2D: [3, 4], W.QUAD3D: [7, 8, 9]}


def _states(m, prims, p, x, reverse):
    """The motion's states at node x.  Reverse: it ends at the node -- the
    translation robots' position shift (tdbastar.hpp:192-197); for quad2d and
    the quadrotor (db-A*'s transform_primitiveDirectReverse, dbastar.hpp:
    183-201, restated) the last state takes the node's position and velocity,
    velocities move by dv = v_node - v_last and positions by p_node - p_last +
    (t_k - t_last) dv."""
    xs, us = prims.motion(p)
    out = np.array(xs, float)
    if m.kind in _VEL:
        if not reverse:
            raise NotImplementedError("forward transform of the rollout robots: compare with dpg_expand")
        # the canonical trajectory of a rollout robot is its actions rolled out
        # from the stored start (as the library's upload does), not the stored states
        xs = ob.rollout(m, xs[0], us)
        out = np.array(xs, float)
        pc, vc = _POS[m.kind], _VEL[m.kind]
        dv = np.asarray(x, float)[vc] - xs[-1][vc]
        tk = (np.arange(len(xs)) - (len(xs) - 1)) * m.dt
        out[:, pc] += np.asarray(x, float)[pc] - xs[-1][pc] + tk[:, None] * dv[None, :]
        out[:, vc] += dv[None, :]
    elif reverse:
        out[:, :2] += x[:2] - xs[-1, :2]
    else:
        out[:, :2] += x[:2]
    return out


def _in_bounds(env, s):
    return all(env.lo[i] <= s[i] <= env.hi[i] for i in range(env.dim))


def _collides(m, env, s):
    import ctypes as C
    L = ob.lib()
    r = ob.robot(m)
    e, ke = ob.env_struct(env)
    s = np.ascontiguousarray(s, dtype=np.float64)
    return any(L.orc_state_gap(C.byref(r), C.byref(e), s.ctypes.data, o) <= 0.0 for o in range(e.n_obs))


def check(m, prims, env, x, node_g, node, prim, reverse, c_time, c_state, goal, delta):
    out = []
    for n, p in zip(node, prim):
        st = _states(m, prims, int(p), x[n], reverse)
        L = len(st)
        oob = next((k for k in range(L) if not _in_bounds(env, st[k])), L)
        if oob < L:
            out.append((2, oob))
            continue
        col = next((k for k in range(L) if _collides(m, env, st[k])), L)
        if col < L:
            out.append((1, col))
            continue
        v, fi = 0, L
        if len(c_time):
            reaches = ob.distance(m, st[L - 1] if reverse else st[0], goal) <= delta
            g = np.float32(node_g[n])
            for c, (t, cs) in enumerate(zip(c_time, c_state)):
                t_off = np.float32(np.float32(t) - g)
                idx = int(math.floor(float(t_off) / m.dt + 0.5)) if float(t_off) / m.dt >= 0 else \
                    -int(math.floor(-float(t_off) / m.dt + 0.5))
                k = -1
                if reaches and idx >= L - 1:
                    k = L - 1
                if 0 <= idx < L - 1:
                    k = idx
                if k >= 0 and ob.distance(m, st[k], cs) <= delta:
                    v, fi = 3, c
                    break
        out.append((v, fi))
    return np.array(out, np.int64).reshape(-1, 2)


def reverse_ball(m, prims, nodes, radius):
    """tdb-A*'s reverse neighbours (nigh_factory_t with reverse_search,
    include/dynoplan/nigh_custom_spaces.hpp:575-693, queried at
    include/dynoplan/tdbastar/tdbastar.hpp:255): motion p is a neighbour of
    node x when distance(canonical(x), last state of p) <= radius; the
    canonical state zeroes the position, the motion's key keeps its own.
    Returns the sorted (node, prim) keys node * 2^32 + prim."""
    keys = []
    for n, x in enumerate(nodes):
        c = np.array(x, float)
        c[:2] = 0.0
        for p in range(prims.P):
            xs, _ = prims.motion(p)
            if ob.distance(m, c, xs[-1]) <= radius:
                keys.append(n * (1 << 32) + p)
    return np.sort(np.array(keys, np.int64))
