"""tdb-A*'s pair checks (include/dpg_tdb.h): forward and reverse verdicts
and the constraint test against tests/tdb_ref.py; the forward transform of
the rollout robots against the regular FP64 check, their reverse against
the restatement."""
import numpy as np
import pytest

from dynoplan_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg,reverse", [(1, False), (1, True), (2, False), (2, True)])
def test_tdb_checks_match_restatement(dpg_lib, cfg, reverse):
    import tdb_ref
    from dynoplan_gb300 import gpu as G
    from dynoplan_gb300 import tdb as T
    wl = W.make_workload(cfg, scale=0.02, seed=40 + cfg)
    m = wl.robot
    rng = np.random.default_rng(cfg + 10 * reverse)
    N = len(wl.nodes)
    n = 3000
    node = rng.integers(0, N, n)
    prim = rng.integers(0, wl.prims.P, n)
    node_g = rng.uniform(0, 5, N).astype(np.float32)
    goal = wl.nodes[0]
    delta = 0.3
    with G.Context(m) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        v0, fi0, _ = T.check_pairs(ctx, wl.nodes, node, prim, reverse=reverse)
        # constraints taken from states of valid pairs, so that some pairs violate them
        valid = np.flatnonzero(v0 == 0)
        assert len(valid) > 20
        pick = rng.choice(valid, 12, replace=False)
        c_time, c_state = [], []
        for i in pick:
            st = tdb_ref._states(m, wl.prims, int(prim[i]), wl.nodes[node[i]], reverse)
            k = int(rng.integers(0, len(st)))
            c_time.append(float(node_g[node[i]]) + k * m.dt + float(rng.uniform(-0.02, 0.02)))
            c_state.append(st[k] + rng.normal(0, 0.05, m.nx))
        c_time, c_state = np.array(c_time), np.array(c_state)
        v, fi, end = T.check_pairs(ctx, wl.nodes, node, prim, reverse=reverse, node_g=node_g, c_time=c_time,
                                   c_state=c_state, goal=goal, delta=delta)
    ref = tdb_ref.check(m, wl.prims, wl.env, wl.nodes, node_g, node, prim, reverse, c_time, c_state, goal, delta)
    assert np.array_equal(v.astype(np.int64), ref[:, 0])
    assert np.array_equal(fi.astype(np.int64), ref[:, 1])
    assert (v == T.CONSTRAINT_VIOLATION).sum() >= 12
    assert np.array_equal(v0[v != T.CONSTRAINT_VIOLATION], v[v != T.CONSTRAINT_VIOLATION])


@pytest.mark.parametrize("cfg", [3, 5])
def test_tdb_forward_rollout_robots_match_check_pairs(dpg_lib, cfg):
    from dynoplan_gb300 import gpu as G
    from dynoplan_gb300 import tdb as T
    wl = W.make_workload(cfg, scale=0.01, seed=60 + cfg)
    with G.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        r = ctx.expand(wl.nodes, wl.radius, precision=1)
        v, fi, end = T.check_pairs(ctx, wl.nodes, r["node"], r["prim"])
    assert r["n_pairs"] > 0
    assert np.array_equal(v, r["verdict"])
    assert np.array_equal(fi, r["first_invalid"].astype(np.int32))
    assert np.allclose(end, r["end_state"], rtol=0, atol=1e-9)


@pytest.mark.parametrize("cfg", [3, 5])
def test_tdb_reverse_rollout_robots_match_restatement(dpg_lib, cfg):
    """Reverse pairs of the rollout robots (quadrotor, quad2d): the motion
    ends at the node with the node's position and velocity; verdicts, first
    invalid states and end states against the FP64 restatement."""
    import tdb_ref
    from dynoplan_gb300 import gpu as G
    from dynoplan_gb300 import tdb as T
    wl = W.make_workload(cfg, scale=0.01, seed=70 + cfg)
    m = wl.robot
    rng = np.random.default_rng(cfg)
    n = 160
    node = rng.integers(0, len(wl.nodes), n).astype(np.uint32)
    prim = rng.integers(0, wl.prims.P, n).astype(np.uint32)
    with G.Context(m) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        v, fi, end = T.check_pairs(ctx, wl.nodes, node, prim, reverse=True)
    ref = tdb_ref.check(m, wl.prims, wl.env, wl.nodes, np.zeros(len(wl.nodes), np.float32), node, prim, True,
                        [], [], None, 0.0)
    assert np.array_equal(v.astype(np.int64), ref[:, 0])
    assert np.array_equal(fi.astype(np.int64), ref[:, 1])
    assert len(set(v.tolist())) >= 2, "the sample must hold more than one verdict"
    for i in range(n):
        st = tdb_ref._states(m, wl.prims, int(prim[i]), wl.nodes[node[i]], True)
        L = len(st)
        k = fi[i] if v[i] == 2 else L - 1   # DPG_OUT_OF_BOUNDS: the end state is the first state out
        assert np.allclose(end[i], st[k], rtol=0, atol=1e-9)
        assert np.allclose(st[L - 1][:2], wl.nodes[node[i]][:2], atol=1e-9)   # it ends at the node


@pytest.mark.parametrize("cfg", [1, 2])
def test_reverse_ball_matches_restatement(dpg_lib, cfg):
    """The reverse ball (DPG_MODE_REVERSE): motions keyed on their last
    state against the node's canonical state; identical pair sets to the
    restatement over the oracle's metric, for a small and a spatially
    ordered batch, and its pairs check like tdb-A*'s reverse pairs."""
    import tdb_ref
    from dynoplan_gb300 import gpu as G
    from dynoplan_gb300 import tdb as T
    wl = W.make_workload(cfg, scale=0.03, seed=70 + cfg)
    m = wl.robot
    radius = 0.6   # the last states lie away from the origin: a wider ball than the forward one
    for nodes in (wl.nodes[:150], np.concatenate([wl.nodes] * (1 + 2100 // len(wl.nodes)))[:2100]):
        with G.Context(m) as ctx:
            ctx.upload_primitives(wl.prims)
            ctx.upload_env(wl.env)
            r = ctx.expand(nodes, radius, ball_only=True, reverse=True)
            got = np.sort(r["node"].astype(np.int64) * (1 << 32) + r["prim"].astype(np.int64))
            if len(nodes) <= 150:
                v, fi, _ = T.check_pairs(ctx, nodes, r["node"], r["prim"], reverse=True)
        ref = tdb_ref.reverse_ball(m, wl.prims, nodes[:150] if len(nodes) > 150 else nodes, radius)
        if len(nodes) > 150:
            got = got[got < 150 * (1 << 32)]
        else:
            refc = tdb_ref.check(m, wl.prims, wl.env, nodes, np.zeros(len(nodes), np.float32), r["node"], r["prim"],
                                 True, np.zeros(0), np.zeros((0, m.nx)), nodes[0], 0.3)
            assert np.array_equal(v.astype(np.int64), refc[:, 0]) and np.array_equal(fi.astype(np.int64), refc[:, 1])
        assert len(ref) > 0
        np.testing.assert_array_equal(got, ref)


def test_reverse_ball_refused_for_rollout_robots(dpg_lib):
    from dynoplan_gb300 import gpu as G
    from dynoplan_gb300._lib import DpgError
    wl = W.make_workload(5, scale=0.005)
    with G.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        with pytest.raises(DpgError):
            ctx.expand(wl.nodes, 0.5, ball_only=True, reverse=True)
