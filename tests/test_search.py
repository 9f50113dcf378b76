"""dpg_search (batched db-A* over the GPU expansion) against its FP64 oracle
restatement (tests/search_ref.py): same termination, expansions, explored
nodes, solution motions and cost, for batch sizes 1 (the reference's
one-node-per-iteration order) and 8."""
import numpy as np
import pytest

from dynoplan_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def problem(kind, seed, P=300, n_obs=20, extent=(6.0, 6.0)):
    m = W.robot_model(kind)
    steps = {W.UNICYCLE1: (5, 30), W.CAR1: (5, 30), W.QUAD2D: (20, 60)}[kind]
    prims = W.make_primitives(m, P, steps[0], steps[1], seed=seed)
    env = W.make_env(extent, n_obs, 0.2, 1.0, seed=seed + 1)
    se = W.make_nodes(m, env, 2, seed=seed + 2, vel_sigma=0.0)
    return m, prims, env, se[0], se[1]


@pytest.mark.parametrize("kind,seed,batch", [(W.UNICYCLE1, 1, 1), (W.UNICYCLE1, 2, 8), (W.CAR1, 3, 1),
                                              (W.CAR1, 4, 8)])
def test_search_matches_oracle(dpg_lib, kind, seed, batch):
    import search_ref
    from dynoplan_gb300 import gpu as G
    from dynoplan_gb300 import search as S
    m, prims, env, start, goal = problem(kind, seed)
    delta = 0.5
    with G.Context(m) as ctx:
        ctx.upload_primitives(prims)
        ctx.upload_env(env)
        res, motions, states = S.search(ctx, start, goal, S.options(delta, batch=batch, max_expands=400,
                                                                    precision=1))
    ref = search_ref.search(m, prims, env, start, goal, delta, batch=batch, max_expands=400)
    assert res["status_str"] == ref["status"]
    assert res["expands"] == ref["expands"]
    assert res["nodes"] == ref["nodes"]
    if ref["solved"]:
        assert list(motions) == ref["motions"]
        assert res["cost"] == pytest.approx(ref["cost"], abs=1e-9)
        np.testing.assert_allclose(states[0], start)


def test_search_solves_and_path_is_valid(dpg_lib):
    """A solved run: consecutive node states jump by at most delta, the last
    state is within delta of the goal, and every used motion is exactly
    valid at its node (re-checked through dpg_check_pairs)."""
    from dynoplan_gb300 import gpu as G
    from dynoplan_gb300 import search as S
    import search_ref
    m, prims, env, start, goal = problem(W.UNICYCLE1, 7, P=400, n_obs=10)
    delta = 0.6
    with G.Context(m) as ctx:
        ctx.upload_primitives(prims)
        ctx.upload_env(env)
        res, motions, states = S.search(ctx, start, goal, S.options(delta, batch=16, max_expands=20000))
        assert res["solved"], res
        chk = ctx.check_pairs(states[:-1], np.arange(len(motions)), motions)
        assert (chk["verdict"] == 0).all()
    table = search_ref.canonical_table(m, prims)
    for i, p in enumerate(motions):
        x_end = search_ref.transformed(m, table[p], int(prims.length[p]) - 1, states[i])
        assert search_ref.distance(m, x_end, states[i + 1]) <= delta + 1e-9 or i == len(motions) - 1
    assert search_ref.distance(m, states[-1], goal) < delta
