"""The key-grid ball scan (batches of >= 2048 nodes for robots whose kept
key has one or two components) against the all-primitive scan (batches
under 2048 nodes) and the oracle (needs a GB300).

Bar: the same pairs with bit-identical check outputs, and the same number
of FP64 ball re-tests, whichever scan found them.
"""
import dataclasses
import math

import numpy as np
import pytest

import oracle_bind as ob
from dynoplan_gb300 import workloads as W
from parity_util import compare, sort_by_pair

pytestmark = pytest.mark.gpu

SPLIT = 1024  # under the 2048-node batch size of the grid scan
KEYS = ("node", "prim", "verdict", "first_invalid", "end_state", "min_gap", "flags")


@pytest.fixture(scope="module")
def gpu(dpg_lib):
    from dynoplan_gb300 import gpu as G
    return G


def expand_both(G, robot, prims, env, nodes, radius, precision):
    """(one call over all nodes, calls of SPLIT nodes with node ids shifted)"""
    assert len(nodes) >= 2048
    with G.Context(robot) as ctx:
        ctx.upload_primitives(prims)
        ctx.upload_env(env)
        whole = ctx.expand(nodes, radius, precision=precision)
        parts = []
        for s in range(0, len(nodes), SPLIT):
            r = ctx.expand(nodes[s:s + SPLIT], radius, precision=precision)
            r["node"] = r["node"] + s
            parts.append(r)
    split = {k: np.concatenate([r[k] for r in parts]) for k in KEYS}
    split["n_pairs"] = sum(r["n_pairs"] for r in parts)
    split["n_ball_recheck"] = sum(r["n_ball_recheck"] for r in parts)
    return whole, split


def assert_same(a, b):
    assert a["n_pairs"] == b["n_pairs"], (a["n_pairs"], b["n_pairs"])
    assert a["n_ball_recheck"] == b["n_ball_recheck"]
    a, b = sort_by_pair(a), sort_by_pair(b)
    for k in KEYS:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


@pytest.mark.parametrize("cfg,P,N", [(1, 1000, 4096), (2, 2000, 6000), (5, 3000, 5000)])
@pytest.mark.parametrize("precision", [0, 1])
def test_grid_matches_full_scan_and_oracle(gpu, cfg, P, N, precision):
    wl = W.make_workload(cfg, seed=300 + cfg, P=P, N=N)
    whole, split = expand_both(gpu, wl.robot, wl.prims, wl.env, wl.nodes, wl.radius, precision)
    assert whole["n_pairs"] > 0
    assert_same(whole, split)
    ora = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius, fast=True,
                    threads=ob.lib().orc_max_threads())
    compare(wl.robot.kind, whole, ora, precision, min_gap=False)


def test_grid_linear_rate_component(gpu):
    """quad2d with a rate weight large enough that the grid's linear
    component (the angular rate) culls cells."""
    wl = W.make_workload(5, seed=311, P=3000, N=4000)
    robot = dataclasses.replace(wl.robot, w=(1.0, 0.5, 0.2, 2.0))
    whole, split = expand_both(gpu, robot, wl.prims, wl.env, wl.nodes, 0.4, 0)
    assert whole["n_pairs"] > 0
    assert_same(whole, split)


def test_grid_seam_and_wide_ranges(gpu):
    """car1 nodes on and around the +-pi seam of both angles; then a weight
    so small that the range spans the whole circle."""
    wl = W.make_workload(2, seed=312, P=2500, N=3000)
    nodes = wl.nodes.copy()
    eps = np.array([0.0, 1e-7, -1e-7, 1e-3, -1e-3, 0.05, -0.05, 0.2])
    seam = np.concatenate([math.pi + eps, -math.pi + eps])
    nodes[:, 2] = seam[np.arange(len(nodes)) % len(seam)]
    nodes[::2, 3] = seam[(np.arange(len(nodes)) // 3)[::2] % len(seam)]
    whole, split = expand_both(gpu, wl.robot, wl.prims, wl.env, nodes, wl.radius, 0)
    assert whole["n_pairs"] > 0
    assert_same(whole, split)
    robot = dataclasses.replace(wl.robot, w=(1.0, 1e-6, 0.5, 0.0))
    whole, split = expand_both(gpu, robot, wl.prims, wl.env, nodes, wl.radius, 0)
    assert_same(whole, split)


def test_grid_large_primitive_set(gpu):
    """More primitives than the grid scan counts in shared memory (12,288):
    the counts go through global atomics."""
    wl = W.make_workload(1, seed=313, P=13000, N=2500)
    whole, split = expand_both(gpu, wl.robot, wl.prims, wl.env, wl.nodes, wl.radius, 0)
    assert whole["n_pairs"] > 0
    assert_same(whole, split)


def test_clustered_batch_order(gpu):
    """5,000 car1 nodes inside one or two cells of the spatial-order grid (the
    stable tile sort must rank thousands of nodes per cell): the same results
    as batches under 2048 nodes, and two calls agree bit for bit."""
    wl = W.make_workload(2, seed=314, P=2000, N=5000)
    rng = np.random.default_rng(314)
    nodes = wl.nodes.copy()
    c = 0.5 * (wl.env.lo[:2] + wl.env.hi[:2])
    nodes[:, :2] = c + rng.uniform(-0.05, 0.05, (len(nodes), 2))
    whole, split = expand_both(gpu, wl.robot, wl.prims, wl.env, nodes, wl.radius, 0)
    assert whole["n_pairs"] > 0
    assert_same(whole, split)
    again, _ = expand_both(gpu, wl.robot, wl.prims, wl.env, nodes, wl.radius, 0)
    for k in KEYS:
        np.testing.assert_array_equal(whole[k], again[k], err_msg=k)
