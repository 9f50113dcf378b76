"""Python restatement of the roadmap heuristic (heuristics.cpp:6-42,
109-228; heuristics.hpp:143-182) over the oracle's metric, lower bound and
state validity -- the checker of include/dpg_roadmap.h.  Interpolation:
R^n parts linear, angles along the shorter arc, quaternions by slerp;
edge check: both ends and the bisection midpoints until segments are at
most `resolution` long."""
import heapq
import math

import numpy as np

import oracle_bind as ob
from dynoplan_gb300 import workloads as W

SPEEDS = {W.UNICYCLE1: (0.5, 0.5), W.CAR1: (0.5, 0.5), W.QUAD2D: (2.0, 4.0), W.QUAD3D: (4.0, 8.0)}


def _so2(a, b):
    d = math.fmod(abs(a - b), 2 * math.pi)
    return 2 * math.pi - d if d > math.pi else d


def _dangle(a, b):
    d = math.fmod(b - a + math.pi, 2 * math.pi)
    if d < 0:
        d += 2 * math.pi
    return d - math.pi


def lbt_pr(m, a, b):
    vp, vr = SPEEDS[m.kind]
    if m.kind == W.QUAD3D:
        dq = min(1.0, abs(float(np.dot(a[3:7], b[3:7]))))
        return max(np.linalg.norm(a[:3] - b[:3]) / vp, math.acos(dq) / vr)
    t = max(math.hypot(a[0] - b[0], a[1] - b[1]) / vp, _so2(a[2], b[2]) / vr)
    if m.kind == W.CAR1:
        t = max(t, _so2(a[3], b[3]) / vr)
    return t


def lbt_vel(m, a, b):
    if m.kind == W.QUAD2D:
        return max(math.hypot(a[3] - b[3], a[4] - b[4]) / 4.0, abs(a[5] - b[5]) / 8.0)
    if m.kind == W.QUAD3D:
        return max(np.linalg.norm(a[7:10] - b[7:10]) / 4.0, np.linalg.norm(a[10:13] - b[10:13]) / 8.0)
    return 0.0


def interp(m, a, b, t):
    out = a + t * (b - a)
    if m.kind == W.QUAD3D:
        qa, qb = a[3:7], b[3:7].copy()
        dot = float(np.dot(qa, qb))
        if dot < 0:
            qb, dot = -qb, -dot
        wa, wb = 1 - t, t
        if dot < 0.9995:
            th = math.acos(dot)
            wa, wb = math.sin((1 - t) * th) / math.sin(th), math.sin(t * th) / math.sin(th)
        q = wa * qa + wb * qb
        out[3:7] = q / np.linalg.norm(q)
    else:
        out[2] = a[2] + t * _dangle(a[2], b[2])
        if m.kind == W.CAR1:
            out[3] = a[3] + t * _dangle(a[3], b[3])
    return out


def edge_ok(m, env, a, b, res):
    d = ob.distance(m, a, b)
    depth, seg = 0, d
    while seg > res and depth < 20:
        seg *= 0.5
        depth += 1
    n = 1 << depth
    return all(ob.state_valid(m, env, interp(m, a, b, k / n)) for k in range(n + 1))


def build(m, env, samples, radius, res):
    S = len(samples)
    edges, w = [], []
    for i in range(S):
        for j in range(i + 1, S):
            if ob.distance(m, samples[i], samples[j]) < radius and edge_ok(m, env, samples[i], samples[j], res):
                edges.append((i, j))
                w.append(max(lbt_pr(m, samples[i], samples[j]), lbt_vel(m, samples[i], samples[j])))
    adj = [[] for _ in range(S)]
    for (i, j), wij in zip(edges, w):
        adj[i].append((j, wij))
        adj[j].append((i, wij))
    dist = [float(np.finfo(np.float64).max)] * S
    parent = list(range(S))
    dist[S - 1] = 0.0
    pq = [(0.0, S - 1)]
    while pq:
        d, u = heapq.heappop(pq)
        if d > dist[u]:
            continue
        for v, wv in adj[u]:
            if d + wv < dist[v]:
                dist[v] = d + wv
                parent[v] = u
                heapq.heappush(pq, (dist[v], v))
    return np.array(edges, np.int64).reshape(-1, 2), np.array(w), np.array(dist), np.array(parent)


def heuristic(m, samples, dist, x, goal, connect):
    x0 = np.array(x, float)
    if m.kind == W.QUAD2D:
        x0[3:6] = 0
    if m.kind == W.QUAD3D:
        x0[7:13] = 0
    best = 1e8
    for s, d in zip(samples, dist):
        if ob.distance(m, s, x0) <= connect:
            best = min(best, d + lbt_pr(m, s, x0))
    return max(lbt_vel(m, x, goal), best)
