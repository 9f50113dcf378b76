"""Python restatement of the batched db-A* (include/dpg_search.h) over the FP64
oracle's expansion -- the checker of dpg_search.  Candidates in ascending
motion order (shuffle off), float scores, lowest f then highest g.
Follows dbastar() at src/dbastar/dbastar.cpp:766-920."""
import heapq
import math

import numpy as np

import oracle_bind as ob
from dynoplan_gb300 import workloads as W


def _so2(a, b):
    d = np.fmod(np.abs(a - b), 2 * math.pi)
    return np.where(d > math.pi, 2 * math.pi - d, d)


def distance(m, a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    w = m.w
    if m.kind == W.UNICYCLE1:
        return w[0] * np.hypot(a[..., 0] - b[..., 0], a[..., 1] - b[..., 1]) + w[1] * _so2(a[..., 2], b[..., 2])
    if m.kind == W.CAR1:
        return (w[0] * np.hypot(a[..., 0] - b[..., 0], a[..., 1] - b[..., 1]) + w[1] * _so2(a[..., 2], b[..., 2])
                + w[2] * _so2(a[..., 3], b[..., 3]))
    if m.kind == W.QUAD2D:
        return (w[0] * np.hypot(a[..., 0] - b[..., 0], a[..., 1] - b[..., 1]) + w[1] * _so2(a[..., 2], b[..., 2])
                + w[2] * np.hypot(a[..., 3] - b[..., 3], a[..., 4] - b[..., 4]) + w[3] * np.abs(a[..., 5] - b[..., 5]))
    raise NotImplementedError


def lbt(m, a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    if m.kind == W.UNICYCLE1:
        return np.maximum(np.hypot(a[..., 0] - b[..., 0], a[..., 1] - b[..., 1]) / 0.5, _so2(a[..., 2], b[..., 2]) / 0.5)
    if m.kind == W.CAR1:
        return np.maximum(np.maximum(np.hypot(a[..., 0] - b[..., 0], a[..., 1] - b[..., 1]) / 0.5,
                                     _so2(a[..., 2], b[..., 2]) / 0.5), _so2(a[..., 3], b[..., 3]) / 0.5)
    if m.kind == W.QUAD2D:
        return np.maximum(np.maximum(np.hypot(a[..., 0] - b[..., 0], a[..., 1] - b[..., 1]) / 2.0,
                                     _so2(a[..., 2], b[..., 2]) / 4.0),
                          np.maximum(np.hypot(a[..., 3] - b[..., 3], a[..., 4] - b[..., 4]) / 4.0,
                                     np.abs(a[..., 5] - b[..., 5]) / 8.0))
    raise NotImplementedError


def transformed(m, states, k, x):
    """state k of a primitive (canonical rows `states`) applied at node x"""
    s = states[k].copy()
    pos, vel = ([0, 1], [3, 4]) if m.kind == W.QUAD2D else ([0, 1], [])
    t = k * m.dt
    for i, p in enumerate(pos):
        s[p] += x[p]
        if vel:
            s[p] += t * x[vel[i]]
            s[vel[i]] += x[vel[i]]
    return s


def canonical_table(m, prims):
    if m.kind != W.QUAD2D:
        return [prims.motion(p)[0] for p in range(prims.P)]
    out = []
    for p in range(prims.P):
        xs, us = prims.motion(p)
        out.append(ob.rollout(m, xs[0], us))
    return out


def search(m, prims, env, start, goal, delta, alpha=0.5, batch=1, limit=20, max_expands=100000,
           heuristic=0, dfg=1.0, cdf=1.0, hfun=None, g_at_pop=True):
    """heuristic 0: time lower bound to the goal, -1: blind; hfun(x), when
    given, replaces both (the roadmap heuristic's restatement).  g_at_pop:
    a successor's g counts from its node's g when the batch was popped (the
    GPU search's rule); False reads the node's current g, as the reference's
    one-node loop does -- the same thing when batch = 1."""
    table = canonical_table(m, prims)
    f32 = np.float32
    X = [np.asarray(start, float)]
    g, h, f, parent, motion, inter, version, in_open = [f32(0)], [], [], [-1], [-1], [-1], [0], [True]
    h0 = f32(hfun(start)) if hfun else (f32(lbt(m, start, goal)) if heuristic == 0 else f32(0))
    h.append(h0)
    f.append(f32(g[0] + h0))
    heap = [(f[0], -g[0], 0, 0)]
    expands, status, solution = 0, "EMPTY_QUEUE", -1
    goal_tol = dfg * delta
    nov = (1 - alpha) * delta
    while True:
        if expands >= max_expands:
            status = "MAX_EXPANDS"
            break
        if not heap:
            status = "EMPTY_QUEUE"
            break
        bat = []
        while heap and len(bat) < batch and expands + len(bat) < max_expands:
            ff, mg, i, v = heapq.heappop(heap)
            if not in_open[i] or v != version[i]:
                continue
            in_open[i] = False
            bat.append(i)
        if not bat:
            continue
        done = False
        for i in bat:
            expands += 1
            if distance(m, X[i], goal) < goal_tol:
                solution, done = i, True
                break
        if done:
            status = "SOLVED"
            break
        bx = np.array([X[i] for i in bat])
        gpop = [float(g[i]) for i in bat]  # a successor's g counts from its node's g when popped
        res = ob.expand(m, prims, env, bx, alpha * delta)
        # candidates: valid pairs, node (pop) order, motions ascending
        cands = []
        for b in range(len(bat)):
            sel = (res["node"] == b) & (res["verdict"] == 0)
            for p in np.sort(res["prim"][sel]):
                L = int(prims.length[p])
                xe = transformed(m, table[p], L - 1, bx[b])
                x0 = transformed(m, table[p], 0, bx[b])
                chosen = -1
                for k in range(4):
                    idx = int(np.float32(k + 1) / np.float32(5) * np.float32(L))
                    if idx >= L:
                        continue
                    xi = transformed(m, table[p], idx, bx[b])
                    if distance(m, xi, goal) <= goal_tol:
                        xe, chosen = xi, idx
                        break
                cost = (chosen if chosen != -1 else L - 1) * m.dt
                cands.append((b, int(p), xe, x0, chosen, cost))
        # rounds: every unfinished node, in pop order, visits its next chunk
        # of motions (2 x limit, doubling) until it has `limit` new nodes
        per = [[c for c in cands if c[0] == b] for b in range(len(bat))]
        pos, chunk, n_new = [0] * len(bat), [2 * limit] * len(bat), [0] * len(bat)
        finished = [len(per[b]) == 0 for b in range(len(bat))]
        while not all(finished):
            for b, parent_i in enumerate(bat):
                if finished[b]:
                    continue
                for (cb, p, xe, x0, chosen, cost) in per[b][pos[b]:pos[b] + chunk[b]]:
                    pos[b] += 1
                    hh = f32(hfun(xe)) if hfun else (f32(lbt(m, xe, goal)) if heuristic == 0 else f32(0))
                    gp = gpop[b] if g_at_pop else float(g[parent_i])
                    gg = gp + cost + cdf * float(lbt(m, X[parent_i], x0))
                    nbr = sorted(np.flatnonzero(distance(m, np.array(X), xe[None, :]) <= nov))
                    if not nbr or chosen != -1:
                        X.append(xe)
                        nid = len(X) - 1
                        g.append(f32(gg)); h.append(hh); f.append(f32(f32(gg) + hh))
                        parent.append(parent_i); motion.append(p); inter.append(chosen); version.append(0)
                        in_open.append(True)
                        heapq.heappush(heap, (f[nid], -g[nid], nid, 0))
                        n_new[b] += 1
                    else:
                        for nb in nbr:
                            tent = gg + float(lbt(m, xe, X[nb]))
                            if tent < g[nb]:
                                g[nb] = f32(tent)
                                f[nb] = f32(g[nb] + h[nb])
                                parent[nb], motion[nb], inter[nb] = parent_i, p, -1
                                version[nb] += 1
                                in_open[nb] = True
                                heapq.heappush(heap, (f[nb], -g[nb], nb, version[nb]))
                    if n_new[b] >= limit:
                        break
                if n_new[b] >= limit or pos[b] >= len(per[b]):
                    finished[b] = True
                else:
                    chunk[b] *= 2
    out = {"solved": solution >= 0, "status": status, "expands": expands, "nodes": len(X)}
    if solution >= 0:
        chain = []
        i = solution
        while i != -1:
            chain.append(i)
            i = parent[i]
        chain.reverse()
        cost = 0.0
        for i in chain[1:]:
            L = int(prims.length[motion[i]])
            cost += (inter[i] if inter[i] != -1 else L - 1) * m.dt
        out.update(cost=cost, motions=[motion[i] for i in chain[1:]], g=float(g[solution]))
    return out
