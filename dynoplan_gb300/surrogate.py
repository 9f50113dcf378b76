"""The learned surrogate of the expansion (include/dpg_mlp.h) from Python.

A BF16 MLP scores (node, primitive) pairs with a collision logit and a
cost-to-go; it is trained on labels the exact GPU checker produces.  Device
buffers are torch tensors (plumbing only: every kernel is the library's).
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from . import workloads as W
from ._lib import check

PARAMS = ["W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4", "emb"]
SHAPES = {"W1": (256, 128), "b1": (256,), "W2": (256, 256), "b2": (256,), "W3": (256, 256), "b3": (256,),
          "W4": (16, 256), "b4": (16,)}
NODE_FEAT = 80
CTG_SCALE = 10.0   # cost-to-go targets are seconds / CTG_SCALE


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _ready(t):
    """The library's streams are ordered after the legacy default stream
    only: inputs produced on another torch stream are waited for here."""
    import torch
    s = torch.cuda.current_stream(t.device)
    if s != torch.cuda.default_stream(t.device):
        s.synchronize()


class Surrogate:
    def __init__(self, n_prims: int, max_rows: int = 65536, device: int = 0, seed: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        check(self.lib.dpg_mlp_create(C.byref(h), device, n_prims, max_rows, seed))
        self.h, self.n_prims, self.max_rows = h, n_prims, max_rows

    def close(self):
        if getattr(self, "h", None):
            self.lib.dpg_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def shape(self, name):
        return SHAPES.get(name, (self.n_prims, 16))

    def get(self, name, grad=False) -> np.ndarray:
        i = PARAMS.index(name)
        out = np.empty(self.lib.dpg_mlp_param_size(self.h, i), np.float32)
        check(self.lib.dpg_mlp_get(self.h, i, 1 if grad else 0, out.ctypes.data))
        return out.reshape(self.shape(name))

    def set(self, name, value):
        i = PARAMS.index(name)
        v = np.ascontiguousarray(value, dtype=np.float32).reshape(-1)
        assert v.size == self.lib.dpg_mlp_param_size(self.h, i)
        check(self.lib.dpg_mlp_set(self.h, i, v.ctypes.data))

    def forward(self, node_feat, node, prim, out=None):
        """torch device tensors: node_feat [N x 80] bf16, node/prim [n] int32;
        returns out [n x 2] float32 = (logit, cost-to-go)"""
        import torch
        n = node.numel()
        if out is None:
            out = torch.empty((n, 2), dtype=torch.float32, device=node.device)
        _ready(node)
        check(self.lib.dpg_mlp_forward(self.h, _p(node_feat), _p(node), _p(prim), n, _p(out)))
        return out

    def train_step(self, node_feat, node, prim, target, lr=1e-3, ctg_weight=1.0) -> float:
        loss = C.c_float()
        _ready(node)
        check(self.lib.dpg_mlp_train_step(self.h, _p(node_feat), _p(node), _p(prim), _p(target), node.numel(),
                                          lr, ctg_weight, C.byref(loss)))
        return loss.value

    def set_fused(self, fused: int):
        """forward kernel: 0 the layer-by-layer GEMMs, 1 the fused per-tile
        kernel, 2 the fused warp-specialised kernel (default)"""
        check(self.lib.dpg_mlp_set_fused(self.h, int(fused)))

    def timing(self):
        ms, fl = C.c_double(), C.c_double()
        self.lib.dpg_mlp_last_timing(self.h, C.byref(ms), C.byref(fl))
        return ms.value, fl.value


def node_features(ctx, x_dev, goal=None):
    """[N x 80] bf16 node features (state + occupancy, and the offset to
    `goal` when given) for the context's env"""
    import torch
    N = x_dev.shape[0]
    feat = torch.empty((N, NODE_FEAT), dtype=torch.bfloat16, device=x_dev.device)
    g = None if goal is None else np.ascontiguousarray(goal, dtype=np.float64)
    _ready(x_dev)
    check(_lib.load().dpg_mlp_node_features(ctx.h, _p(x_dev), N, g.ctypes.data if g is not None else None,
                                            _p(feat)), ctx.h)
    return feat


def cost_to_go(model, end_state: np.ndarray, goal: np.ndarray) -> np.ndarray:
    """time lower bound from the transformed end state to the goal position
    (speed 0.5 m/s for the planar robots), in units of CTG_SCALE seconds"""
    d = np.linalg.norm(end_state[:, :2] - goal[None, :2], axis=1)
    return (d / 0.5 / CTG_SCALE).astype(np.float32)


class Dataset:
    """(node features, node index, primitive, [collision, cost-to-go]) on the
    device, drawn from `n_envs` seeded environments of a workload."""

    def __init__(self, node_feat, node, prim, target, n_envs, env_of_node):
        self.node_feat, self.node, self.prim, self.target = node_feat, node, prim, target
        self.n_envs, self.env_of_node = n_envs, env_of_node

    def __len__(self):
        return self.node.numel()


def make_dataset(wl, n_envs: int, nodes_per_env: int, pairs_per_env: int, seed: int, device: int = 0):
    """Labels from the exact checker: every (node, primitive) pair of the ball
    around `nodes_per_env` free-space nodes in each of `n_envs` environments
    like the workload's, checked on the GPU; `pairs_per_env` are kept."""
    import torch

    from . import gpu as G
    cfg = {W.CAR1: (10.0, 10.0, 80, 0.2, 1.5), W.UNICYCLE1: (6.0, 6.0, 30, 0.2, 1.0),
           W.QUAD2D: (8.0, 4.0, 40, 0.2, 1.0)}[wl.robot.kind]
    rng = np.random.default_rng(seed)
    feats, nodes_g, prims, targets, env_of = [], [], [], [], []
    base = 0
    with G.Context(wl.robot, device=device) as ctx:
        ctx.upload_primitives(wl.prims)
        for e in range(n_envs):
            env = W.make_env(cfg[:2], cfg[2], cfg[3], cfg[4], seed=seed * 1000 + e)
            nodes = W.make_nodes(wl.robot, env, nodes_per_env, seed=seed * 1000 + 500 + e)
            goal = W.make_nodes(wl.robot, env, 1, seed=seed * 1000 + 900 + e)[0]
            ctx.upload_env(env)
            res = ctx.expand(nodes, wl.radius, precision=0)
            n = res["n_pairs"]
            keep = rng.choice(n, size=min(pairs_per_env, n), replace=False) if n else np.zeros(0, np.int64)
            x_dev = torch.from_numpy(nodes).to(f"cuda:{device}")
            feats.append(node_features(ctx, x_dev))
            nodes_g.append(res["node"][keep].astype(np.int64) + base)
            prims.append(res["prim"][keep].astype(np.int64))
            coll = (res["verdict"][keep] != 0).astype(np.float32)
            ctg = cost_to_go(wl.robot, res["end_state"][keep].astype(np.float64), goal)
            targets.append(np.stack([coll, ctg], 1))
            env_of.append(np.full(len(nodes), e, np.int32))
            base += len(nodes)
    dev = f"cuda:{device}"
    return Dataset(torch.cat(feats, 0).contiguous(),
                   torch.from_numpy(np.concatenate(nodes_g).astype(np.int32)).to(dev),
                   torch.from_numpy(np.concatenate(prims).astype(np.int32)).to(dev),
                   torch.from_numpy(np.concatenate(targets)).to(dev), n_envs, np.concatenate(env_of))


def search_dataset(robot, prims, problems, opts, nodes_per_env: int = 400, pairs_per_env: int = 20000,
                   ctg_fraction: float = 0.3, radius: float | None = None, device: int = 0, seed: int = 0, log=None):
    """Goal-conditioned labels from completed searches and the exact checker.
      - cost-to-go: for the path s_0..s_n (motions m_1..m_n, durations
        c_1..c_n) of every solved plain search and every i < j <= n, node s_i
        with goal s_j (s_n: the problem's goal) and motion m_{i+1} is
        labelled c_{i+2} + ... + c_j, the time left after the motion, and
        collision 0;
      - collision: `pairs_per_env` of the in-ball pairs of `nodes_per_env`
        free nodes, exact-checked, with the problem's goal (cost-to-go NaN).
    Cost-to-go rows are repeated to make about `ctg_fraction` of the rows.
    problems: list of (env, start, goal).  Returns (Dataset, search results)."""
    import torch

    from . import gpu as G
    from . import search as S
    radius = radius if radius is not None else opts.alpha * opts.delta
    dev = f"cuda:{device}"
    rng = np.random.default_rng(seed)
    feats, results = [], []
    ctg_rows, coll_rows = [], []   # (node row, prim, collision, ctg)
    base = 0

    def add_feats(x, goal):
        nonlocal base
        x_dev = torch.from_numpy(np.ascontiguousarray(x, dtype=np.float64)).to(dev)
        feats.append(node_features(ctx, x_dev, goal))
        base += len(x)
        return base - len(x)

    with G.Context(robot, device=device) as ctx:
        ctx.upload_primitives(prims)
        for i, (env, start, goal) in enumerate(problems):
            ctx.upload_env(env)
            res, motions, states = S.search(ctx, start, goal, opts)
            results.append(res)
            n = len(motions) if res["solved"] else 0
            if n:
                cost = np.array([(int(prims.length[p]) - 1) * robot.dt for p in motions])
                cost[-1] = res["cost"] - cost[:-1].sum()
                for j in range(1, n + 1):
                    r0 = add_feats(states[:j], goal if j == n else states[j])
                    left = np.array([cost[i + 1:j].sum() for i in range(j)])
                    ctg_rows.append(np.stack([r0 + np.arange(j), motions[:j], np.zeros(j), left / CTG_SCALE], 1))
            rand = W.make_nodes(robot, env, nodes_per_env, seed=7000 + 31 * i + seed, vel_sigma=0.5)
            r0 = add_feats(rand, goal)
            exp = ctx.expand(rand, radius, precision=0)
            keep = rng.choice(exp["n_pairs"], size=min(pairs_per_env, exp["n_pairs"]), replace=False)
            coll_rows.append(np.stack([r0 + exp["node"][keep].astype(np.float64), exp["prim"][keep],
                                       (exp["verdict"][keep] != 0), np.full(len(keep), np.nan)], 1))
            if log:
                log(f"problem {i}: {res['status_str']} cost {res['cost']:.2f} in {res['time_ms']:.0f} ms")
    coll = np.concatenate(coll_rows) if coll_rows else np.zeros((0, 4))
    ctg = np.concatenate(ctg_rows) if ctg_rows else np.zeros((0, 4))
    if len(ctg):
        reps = max(1, int(round(ctg_fraction / (1 - ctg_fraction) * len(coll) / len(ctg))))
        ctg = np.repeat(ctg, reps, axis=0)
    rows = np.concatenate([ctg, coll])
    ds = Dataset(torch.cat(feats, 0).contiguous(),
                 torch.from_numpy(rows[:, 0].astype(np.int32)).to(dev),
                 torch.from_numpy(rows[:, 1].astype(np.int32)).to(dev),
                 torch.from_numpy(rows[:, 2:4].astype(np.float32)).to(dev), len(problems), None)
    return ds, results


def train(model: Surrogate, ds: Dataset, epochs: float, batch: int = 65536, lr: float = 2e-3, seed: int = 0,
          ctg_weight: float = 1.0, log=None):
    """Adam over shuffled batches; returns (losses, samples/s, train TFLOP/s)"""
    import torch
    g = torch.Generator(device=ds.node.device).manual_seed(seed)
    n = len(ds)
    steps = max(1, int(math.ceil(epochs * n / batch)))
    losses, dev_ms, flops = [], 0.0, 0.0
    perm = None
    for s in range(steps):
        i0 = (s * batch) % n
        if perm is None or i0 + batch > n:
            perm = torch.randperm(n, generator=g, device=ds.node.device)
            i0 = 0
        idx = perm[i0:i0 + batch]
        lr_s = lr * (0.5 * (1 + math.cos(math.pi * s / steps)))  # cosine decay
        loss = model.train_step(ds.node_feat, ds.node[idx].contiguous(), ds.prim[idx].contiguous(),
                                ds.target[idx].contiguous(), lr=lr_s, ctg_weight=ctg_weight)
        ms, fl = model.timing()
        dev_ms += ms
        flops += fl
        losses.append(loss)
        if log and (s % 50 == 0 or s == steps - 1):
            log(f"step {s}/{steps} loss {loss:.4f}")
    return losses, steps * batch / (dev_ms * 1e-3), flops / (dev_ms * 1e-3) / 1e12
