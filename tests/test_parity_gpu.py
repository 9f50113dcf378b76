"""GPU expansion vs the FP64 oracle, through the C ABI (needs a GB300).

Bars: identical neighbour pairs, verdicts and first-invalid states; end
states within 1e-9 (DPG_FP64, DPG_FP64_STRICT) or 1e-5 relative (DPG_FP32);
see tests/parity_util.py.  Precision 0 = DPG_FP32, 1 = DPG_FP64 (FP32 tests
with FP64 decisions in the bands, FP64 end states), 2 = DPG_FP64_STRICT.
"""
import dataclasses
import os

import numpy as np
import pytest

import oracle_bind as ob
from dynoplan_gb300 import workloads as W
from parity_util import compare

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def gpu(dpg_lib):
    from dynoplan_gb300 import gpu as G
    return G


def run_gpu(G, wl, precision, tuning=None, **kw):
    with G.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        if tuning:
            ctx.set_tuning(**tuning)
        return ctx.expand(wl.nodes, wl.radius, precision=precision, **kw)


@pytest.mark.parametrize("cfg", [1, 2, 3, 5])
@pytest.mark.parametrize("precision", [0, 1, 2])
def test_golden_fixture(gpu, cfg, precision):
    """The committed oracle outputs (tests/golden/oracle_cfg*.npz)."""
    z = np.load(os.path.join(GOLD, f"oracle_cfg{cfg}.npz"))
    kind = int(z["kind"])
    wl = W.Workload("golden", W.robot_model(kind), W.Primitives(z["length"], z["states"], z["actions"]),
                    W.Env(z["env_lo"], z["env_hi"], z["obs_lo"], z["obs_hi"]), z["nodes"],
                    delta=2.0 * float(z["radius"]), alpha=0.5, precision=precision, seed=0)
    res = run_gpu(gpu, wl, precision)
    ora = {k: z[k] for k in ("node", "prim", "verdict", "first_invalid", "end_state", "min_gap")}
    ora["n_pairs"] = len(z["node"])
    compare(kind, res, ora, precision)


@pytest.mark.parametrize("cfg,scale", [(1, 0.1), (2, 0.02), (3, 0.01), (5, 0.01)])
@pytest.mark.parametrize("precision", [0, 1, 2])
def test_parity_seeded(gpu, cfg, scale, precision):
    wl = W.make_workload(cfg, scale=scale, seed=77 + cfg)
    res = run_gpu(gpu, wl, precision)
    ora = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius, fast=True,
                    threads=ob.lib().orc_max_threads())
    assert ora["n_pairs"] > 0
    # the fast baseline carries no min_gap; compare that on the plain oracle below
    compare(wl.robot.kind, res, ora, precision, min_gap=False)


@pytest.mark.parametrize("cfg,scale", [(1, 0.1), (2, 0.02), (2, 0.03), (3, 0.01), (5, 0.01)])
@pytest.mark.parametrize("tuning", [
    {"check_variant": 0}, {"check_variant": 1, "check_blocks_per_sm": 2},
    {"check_variant": 1, "grid_min_nodes": 1 << 30, "pipe_launches": 3}, {"pipe_launches": 1}])
def test_parity_under_tuning(gpu, cfg, scale, tuning):
    """Every launch choice of dpg_set_tuning gives the oracle's results:
    the lockstep check, the slot-parallel check at another occupancy, the
    ball scan without the key grid and another pipeline depth (host outputs)."""
    wl = W.make_workload(cfg, scale=scale, seed=177 + cfg)
    res = run_gpu(gpu, wl, 0, tuning)
    ora = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius)
    compare(wl.robot.kind, res, ora, 0)


@pytest.mark.parametrize("cfg", [1, 2, 3, 5])
def test_min_gap_and_flags(gpu, cfg):
    wl = W.make_workload(cfg, scale=0.005 if cfg != 1 else 0.03, seed=5 + cfg)
    res = run_gpu(gpu, wl, 0)
    ora = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius)
    compare(wl.robot.kind, res, ora, 0)
    assert set(np.unique(res["flags"])) <= {0, 1}


def exact_start_primitives(m, P, steps, seed):
    """Primitives starting exactly at the canonical zero state (no loader
    noise), so the first transformed state is the node's position with
    heading 0."""
    rng = W.Rng(seed)
    lb, ub = np.array(m.u_lb), np.array(m.u_ub)
    states, actions, length = [], [], []
    for p in range(P):
        U = lb + (ub - lb) * rng.uniform((steps, m.nu))
        X = [np.zeros(m.nx)]
        for k in range(steps):
            X.append(W.step(m, X[-1][None], U[k][None])[0])
        states.append(np.array(X))
        actions.append(U)
        length.append(steps + 1)
    return W.Primitives(np.array(length, np.int32), np.concatenate(states), np.concatenate(actions))


@pytest.mark.parametrize("kind", [W.UNICYCLE1, W.CAR1, W.QUAD2D])
def test_contact_band_recheck(gpu, kind):
    """Nodes placed so the robot box touches an obstacle face at the first
    state (gap exactly 0, or within 1e-7 / 3e-5 of it): the FP32 gap falls in
    the band, the pair is recomputed in FP64, and every verdict equals the
    oracle's."""
    m = W.robot_model(kind)
    prims = exact_start_primitives(m, 32, 12, seed=11)
    env = W.Env(np.zeros(2), np.array([8.0, 8.0]), np.array([[4.0, 1.0]]), np.array([[5.0, 7.0]]))
    xs = []
    for dx in (0.0, 1e-7, -1e-7, 3e-5, -3e-5):
        x = np.zeros(m.nx)
        x[0], x[1] = 4.0 - 0.25 + dx, 4.0   # box half length 0.25 along heading 0
        xs.append(x)
    nodes = np.array(xs)
    with gpu.Context(m) as ctx:
        ctx.upload_primitives(prims)
        ctx.upload_env(env)
        res = ctx.expand(nodes, 100.0, precision=0)
    ora = ob.expand(m, prims, env, nodes, 100.0)
    assert ora["n_pairs"] == 5 * 32
    compare(kind, res, ora, 0)
    assert res["n_contact_recheck"] >= 3 * 32
    assert (res["flags"] == 1).sum() == res["n_contact_recheck"]
    assert (res["verdict"][res["node"] == 0] == 1).all()   # touching is contact


def test_edge_cases(gpu):
    m = W.robot_model(W.UNICYCLE1)
    prims = W.make_primitives(m, 40, 0, 12, seed=21)   # some single-state motions
    assert prims.length.min() == 1
    env = W.make_env((6.0, 6.0), 10, 0.2, 1.0, seed=22)
    nodes = W.make_nodes(m, env, 300, seed=23)
    with gpu.Context(m) as ctx:
        ctx.upload_primitives(prims)
        ctx.upload_env(env)
        # no nodes
        assert ctx.expand(nodes[:0], 0.15)["n_pairs"] == 0
        # radius 0: nothing in the ball (starts carry 1e-7 noise)
        assert ctx.expand(nodes, 0.0)["n_pairs"] == 0
        # every pair in the ball
        res = ctx.expand(nodes, 100.0, precision=1)
        assert res["n_pairs"] == 300 * 40
        compare(W.UNICYCLE1, res, ob.expand(m, prims, env, nodes, 100.0), 1)
        # capacity too small: error with the needed count, then retry
        from dynoplan_gb300 import _lib
        with pytest.raises(_lib.DpgError) as e:
            ctx.expand(nodes, 100.0, outputs=dict(
                node=np.empty(10, np.uint32), prim=np.empty(10, np.uint32), verdict=np.empty(10, np.uint8),
                first_invalid=np.empty(10, np.int16), end_state=np.empty((10, 3), np.float32),
                min_gap=np.empty(10, np.float32), flags=np.empty(10, np.uint8)), capacity=10)
        assert e.value.code == _lib.DPG_ERR_CAPACITY
        # abort flag
        ctx.set_abort(True)
        with pytest.raises(_lib.DpgError) as e:
            ctx.expand(nodes, 0.15)
        assert e.value.code == _lib.DPG_ERR_ABORTED
        ctx.set_abort(False)
        assert ctx.expand(nodes, 0.15)["n_pairs"] > 0
    # empty environment: collisions impossible
    env0 = W.Env(np.zeros(2), np.array([6.0, 6.0]), np.zeros((0, 2)), np.zeros((0, 2)))
    with gpu.Context(m) as ctx:
        ctx.upload_primitives(prims)
        ctx.upload_env(env0)
        res = ctx.expand(nodes, 0.15)
        assert DPG_COLLISION_free(res)
        compare(W.UNICYCLE1, res, ob.expand(m, prims, env0, nodes, 0.15), 0)


def DPG_COLLISION_free(res):
    return not (res["verdict"] == 1).any()


def test_bad_arguments(gpu):
    from dynoplan_gb300 import _lib
    m = W.robot_model(W.CAR1)
    with gpu.Context(m) as ctx:
        with pytest.raises(_lib.DpgError) as e:   # expand before upload
            ctx.expand(np.zeros((4, 4)), 0.15)
        assert e.value.code == _lib.DPG_ERR_STATE
        with pytest.raises(_lib.DpgError):        # wrong env dimension
            ctx.upload_env(W.Env(np.zeros(3), np.ones(3), np.zeros((0, 3)), np.zeros((0, 3))))


@pytest.mark.parametrize("cfg,precision", [(1, 1), (1, 2), (2, 0), (3, 0)])
def test_full_size_parity(gpu, cfg, precision):
    """The full workload (config sizes: unicycle1 10,000 nodes x 1,000
    primitives, car1 100,000 x 5,000, quadrotor 50,000 x 5,000), every pair
    against the multi-threaded oracle: identical pairs, verdicts and first
    invalid states, end states within tolerance."""
    wl = W.make_workload(cfg)
    res = run_gpu(gpu, wl, precision)
    ora = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius, fast=True,
                    threads=ob.lib().orc_max_threads())
    assert ora["n_pairs"] > 0
    compare(wl.robot.kind, res, ora, precision, min_gap=False)


def test_full_size_quadrotor_determinism(gpu):
    """quadrotor_v0 at full size: two runs agree bit for bit, and a node
    subset expanded alone gives the same pairs and results."""
    wl = W.make_workload(3)
    with gpu.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        a = ctx.expand(wl.nodes, wl.radius, precision=0)
        b = ctx.expand(wl.nodes, wl.radius, precision=0)
        for k in ("node", "prim", "verdict", "first_invalid", "end_state", "min_gap", "flags"):
            np.testing.assert_array_equal(a[k], b[k])
        sub = wl.nodes[:1500]
        s = ctx.expand(sub, wl.radius, precision=0)
    sel = a["node"] < 1500
    assert sel.sum() == s["n_pairs"]
    key = lambda r, m: np.argsort(r["node"][m].astype(np.int64) * (1 << 32) + r["prim"][m], kind="stable")
    ka, ks = key(a, sel), key(s, np.ones(s["n_pairs"], bool))
    for k in ("node", "prim", "verdict", "first_invalid", "end_state", "min_gap", "flags"):
        np.testing.assert_array_equal(a[k][sel][ka], s[k][ks])


@pytest.mark.parametrize("kind", [W.UNICYCLE1, W.CAR1, W.QUAD3D])
@pytest.mark.parametrize("variant", [0, 1])
def test_obstacle_grid_border_cases(gpu, kind, variant):
    """The obstacle grid that level-1 culling reads: obstacles straddling the
    bounds, lying wholly outside them, and tiny ones; nodes along the
    border so trajectories leave the bounds.  Every result equals the
    oracle's, for both narrow phases."""
    m = W.robot_model(kind)
    dim = 3 if kind == W.QUAD3D else 2
    rng = np.random.default_rng(11 + kind)
    ext = np.array([6.0, 6.0, 3.0][:dim])
    lo = rng.uniform(-1.0, ext + 1.0, (60, dim))
    side = rng.uniform(0.01, 1.2, (60, dim))
    obs_lo, obs_hi = lo - 0.5 * side, lo + 0.5 * side
    env = W.Env(np.zeros(dim), ext, obs_lo, obs_hi)
    nodes = W.make_nodes(m, W.Env(np.zeros(dim), ext, obs_lo[:0], obs_hi[:0]), 600, seed=5)
    nodes[:200, 0] = rng.choice([0.05, ext[0] - 0.05], 200)       # along two edges
    prims = W.make_primitives(m, 60, 5 if dim == 2 else 20, 40 if dim == 2 else 120, seed=3)
    with gpu.Context(m) as ctx:
        ctx.upload_primitives(prims)
        ctx.upload_env(env)
        ctx.set_tuning(check_variant=variant)
        res = ctx.expand(nodes, 0.6)
    ora = ob.expand(m, prims, env, nodes, 0.6)
    assert ora["n_pairs"] > 0 and (ora["verdict"] == 2).any() and (ora["verdict"] == 1).any()
    compare(kind, res, ora, 0)


@pytest.mark.parametrize("cfg,scale,precision", [(2, 0.03, 0), (2, 0.005, 0), (1, 0.3, 1), (1, 0.3, 2), (3, 0.05, 0)])
def test_direct_host_writes(gpu, cfg, scale, precision):
    """Outputs in page-locked host memory, by each host-output path: the
    check kernel writing them itself (DPG_HOST_OUT_DIRECT), one launch with
    range flags (DPG_HOST_OUT_PROGRESS) and the staged launches
    (DPG_HOST_OUT_PIPELINED) give the same rows and the oracle's results;
    small batches (caller's node order) and spatially ordered ones."""
    wl = W.make_workload(cfg, scale=scale, seed=810 + cfg)
    N, nx = wl.nodes.shape
    res = {}
    with gpu.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        n = ctx.expand(wl.nodes, wl.radius, precision=precision)["n_pairs"]
        cap = n + 64
        for direct in (1, 2, 0):
            ctx.set_tuning(host_output=direct)
            pins = {"node": gpu.PinnedArray(cap, np.uint32), "prim": gpu.PinnedArray(cap, np.uint32),
                    "verdict": gpu.PinnedArray(cap, np.uint8), "first_invalid": gpu.PinnedArray(cap, np.int16),
                    "end_state": gpu.PinnedArray((cap, nx), np.float64 if precision else np.float32),
                    "min_gap": gpu.PinnedArray(cap, np.float32), "flags": gpu.PinnedArray(cap, np.uint8)}
            for v in pins.values():
                v.array[...] = 0x5A if v.array.dtype.itemsize == 1 else 7   # stale values must not survive
            r = ctx.expand(wl.nodes, wl.radius, precision=precision, capacity=cap,
                           outputs={k: v.array for k, v in pins.items()})
            res[direct] = {k: (np.array(v) if isinstance(v, np.ndarray) else v) for k, v in r.items()}
            for v in pins.values():
                v.free()
    for k in ("node", "prim", "verdict", "first_invalid", "end_state", "min_gap", "flags"):
        np.testing.assert_array_equal(res[1][k], res[0][k])
        np.testing.assert_array_equal(res[2][k], res[0][k])
    ora = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius, fast=True, threads=ob.lib().orc_max_threads())
    compare(wl.robot.kind, res[1], ora, precision, min_gap=False)


def test_context_reuse_growing_set(gpu):
    """One context through host-buffer expands (the default progress-flag
    path), lazy checks and a larger re-uploaded motion set gives the rows of
    fresh contexts; the host staging buffers that grow with the motion set
    leave the range flags and the lazy counters intact, and a context made
    after it closes works."""
    import torch
    small = W.make_workload(2, scale=0.03, seed=840)
    big = W.make_workload(2, scale=0.03, seed=841, P=2 * small.prims.P)
    keys = ("node", "prim", "verdict", "first_invalid", "end_state", "min_gap")

    def lazy(ctx, wl):
        ball = ctx.expand(wl.nodes, wl.radius, ball_only=True)
        n = ball["n_pairs"]
        dev = "cuda:0"
        x_d = torch.from_numpy(small.nodes).to(dev)
        node_d = torch.from_numpy(ball["node"].view(np.int32)).to(dev)
        prim_d = torch.from_numpy(ball["prim"].view(np.int32)).to(dev)
        outs = {"verdict": torch.empty(n, dtype=torch.uint8, device=dev),
                "first_invalid": torch.empty(n, dtype=torch.int16, device=dev),
                "end_state": torch.empty((n, wl.robot.nx), dtype=torch.float32, device=dev),
                "min_gap": torch.empty(n, dtype=torch.float32, device=dev),
                "flags": torch.zeros(n, dtype=torch.uint8, device=dev)}
        torch.cuda.synchronize()
        st = ctx.lazy_check_device(x_d.data_ptr(), len(small.nodes), n, node_d.data_ptr(), prim_d.data_ptr(),
                                   {k: v.data_ptr() for k, v in outs.items()}, 8)
        assert 0 < st["n_accepted"] <= st["n_valid"] <= st["n_checked"] <= n

    with gpu.Context(small.robot) as ctx:
        assert ctx.tuning()["host_output"] == 2
        ctx.upload_env(small.env)
        ctx.upload_primitives(small.prims)
        r1 = ctx.expand(small.nodes, small.radius)
        lazy(ctx, small)
        ctx.upload_primitives(big.prims)
        r2 = ctx.expand(small.nodes, small.radius)
        lazy(ctx, small)
        r3 = ctx.expand(small.nodes, small.radius)
    f1 = run_gpu(gpu, small, 0)
    f2 = run_gpu(gpu, dataclasses.replace(small, prims=big.prims), 0)
    for k in keys:
        np.testing.assert_array_equal(r1[k], f1[k])
        np.testing.assert_array_equal(r2[k], f2[k])
        np.testing.assert_array_equal(r3[k], f2[k])


@pytest.mark.parametrize("cfg,scale,precision", [(1, 0.3, 1), (2, 0.03, 0), (2, 0.03, 1), (3, 0.01, 0), (5, 0.01, 0)])
def test_min_gap_optional(gpu, cfg, scale, precision):
    """Without the min_gap output the check culls obstacles with the FP64 band
    alone and skips the per-state gap merges: every other output is the same
    as with it, and the oracle's."""
    wl = W.make_workload(cfg, scale=scale, seed=860 + cfg)
    nx = wl.nodes.shape[1]
    with gpu.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        full = ctx.expand(wl.nodes, wl.radius, precision=precision)
        cap = full["n_pairs"] + 64
        o = dict(node=np.empty(cap, np.uint32), prim=np.empty(cap, np.uint32), verdict=np.empty(cap, np.uint8),
                 first_invalid=np.empty(cap, np.int16),
                 end_state=np.empty((cap, nx), np.float64 if precision else np.float32),
                 min_gap=None, flags=np.empty(cap, np.uint8))
        r = ctx.expand(wl.nodes, wl.radius, precision=precision, capacity=cap, outputs=o)
    assert r["n_pairs"] == full["n_pairs"]
    for k in ("node", "prim", "verdict", "first_invalid", "end_state", "flags"):
        np.testing.assert_array_equal(r[k], full[k])
    ora = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius, fast=True, threads=ob.lib().orc_max_threads())
    compare(wl.robot.kind, r, ora, precision, min_gap=False)


@pytest.mark.parametrize("n_obs", [32, 33, 96, 97, 128, 129, 300])
def test_obstacle_counts_around_mask_words(gpu, n_obs):
    """Obstacle counts at the edges of the candidate bitmask words (32 a word,
    culling up to 128, every obstacle tested above that): the results equal
    the oracle's for both narrow phases, with and without min_gap."""
    m = W.robot_model(W.CAR1)
    env = W.make_env((10.0, 10.0), n_obs, 0.1, 0.6, seed=900 + n_obs)
    nodes = W.make_nodes(m, env, 2500, seed=901)
    prims = W.make_primitives(m, 80, 5, 60, seed=902)
    ora = ob.expand(m, prims, env, nodes, 0.5)   # the reference oracle (min_gap included)
    assert (ora["verdict"] == 1).any() and (ora["verdict"] == 0).any()
    with gpu.Context(m) as ctx:
        ctx.upload_primitives(prims)
        ctx.upload_env(env)
        for variant in (0, 1):
            ctx.set_tuning(check_variant=variant)
            res = ctx.expand(nodes, 0.5)
            compare(W.CAR1, res, ora, 0)
            cap = res["n_pairs"] + 64
            o = dict(node=np.empty(cap, np.uint32), prim=np.empty(cap, np.uint32), verdict=np.empty(cap, np.uint8),
                     first_invalid=np.empty(cap, np.int16), end_state=np.empty((cap, 4), np.float32),
                     min_gap=None, flags=np.empty(cap, np.uint8))
            r2 = ctx.expand(nodes, 0.5, capacity=cap, outputs=o)
            compare(W.CAR1, r2, ora, 0, min_gap=False)
