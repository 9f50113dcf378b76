"""The roadmap heuristic (include/dpg_roadmap.h) against its Python
restatement over the oracle (tests/roadmap_ref.py): state validity, the
edge set and weights, Dijkstra distances, h on random states."""
import numpy as np
import pytest

from dynoplan_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg", [1, 2, 5, 3])
def test_roadmap_matches_restatement(dpg_lib, cfg):
    import roadmap_ref as ref
    import oracle_bind as ob
    from dynoplan_gb300 import gpu as G
    from dynoplan_gb300 import roadmap as RM
    c = W.CONFIGS[cfg]
    m = W.robot_model(c["kind"])
    env = W.make_env(c["extent"], c["n_obs"], c["side"][0], c["side"][1], seed=300 + cfg)
    with G.Context(m) as ctx:
        ctx.upload_env(env)
        # validity on random states (some in collision, some out of bounds)
        rng = np.random.default_rng(cfg)
        pd = 3 if m.kind == W.QUAD3D else 2
        x = np.zeros((400, m.nx))
        x[:, :pd] = env.lo - 0.2 + (env.hi - env.lo + 0.4) * rng.random((400, pd))
        if m.kind == W.QUAD3D:
            q = rng.normal(size=(400, 4))
            x[:, 3:7] = q / np.linalg.norm(q, axis=1, keepdims=True)
        else:
            x[:, 2:m.nx] = rng.uniform(-np.pi, np.pi, (400, m.nx - 2))
        got = RM.states_valid(ctx, x)
        want = np.array([ob.state_valid(m, env, xi) for xi in x])
        assert np.array_equal(got, want) and 0 < got.sum() < len(got)
        # roadmap over free samples
        S = 60
        samples = RM.sample_free(ctx, m, env, S, 2000, seed=cfg)
        assert len(samples) == S
        radius, res = (2.0, 0.25) if m.kind != W.QUAD3D else (2.5, 0.3)
        rm = RM.Roadmap(ctx, samples, radius, res)
        ij, w = rm.edges()
        rij, rw, rdist, rpar = ref.build(m, env, samples, radius, res)
        assert len(ij) > 0
        assert np.array_equal(ij.astype(np.int64), rij)
        assert np.allclose(w, rw, rtol=1e-12, atol=0)
        dist, par = rm.distances()
        fin = rdist < 1e300
        assert np.array_equal(dist < 1e300, fin)
        assert np.allclose(dist[fin], rdist[fin], rtol=1e-9, atol=1e-12)
        # parents: a shortest-path tree (ties may pick another parent)
        wd = {(int(a), int(b)): v for (a, b), v in zip(ij, w)}
        for v in np.flatnonzero(fin):
            if v == S - 1:
                continue
            p = int(par[v])
            e = wd.get((min(p, v), max(p, v)))
            assert e is not None and abs(dist[p] + e - dist[v]) <= 1e-9 * max(1.0, dist[v])
        # h on random free states
        goal = samples[-1]
        q = RM.sample_free(ctx, m, env, 50, 2000, seed=100 + cfg)
        if m.kind == W.QUAD2D:
            q[:, 3:6] = rng.normal(0, 0.5, (len(q), 3))
        h = rm.heuristic(q, goal, connect_radius=1.0)
        hr = np.array([ref.heuristic(m, samples, rdist, xi, goal, 1.0) for xi in q])
        assert np.allclose(h, hr, rtol=1e-9, atol=1e-12)
        rm.close()


@pytest.mark.parametrize("kind,seed,batch", [(W.UNICYCLE1, 11, 1), (W.CAR1, 12, 4)])
def test_search_with_roadmap_heuristic_matches_restatement(dpg_lib, kind, seed, batch):
    """dpg_search with DPG_HEU_ROADMAP against search_ref with the roadmap
    restatement as its heuristic: same expansions, nodes and solution"""
    import roadmap_ref
    import search_ref
    from dynoplan_gb300 import gpu as G
    from dynoplan_gb300 import roadmap as RM
    from dynoplan_gb300 import search as S
    from test_search import problem
    m, prims, env, start, goal = problem(kind, seed)
    delta = 0.5
    with G.Context(m) as ctx:
        ctx.upload_primitives(prims)
        ctx.upload_env(env)
        mid = RM.sample_free(ctx, m, env, 80, 3000, seed=seed)
        samples = np.concatenate([start[None], mid, goal[None]])
        rm = RM.Roadmap(ctx, samples, 1.5, 0.25)
        dist, _ = rm.distances()
        res, motions, _ = S.search(ctx, start, goal, S.options(delta, batch=batch, max_expands=300, precision=1,
                                                               heuristic=S.HEU_ROADMAP, roadmap=rm,
                                                               connect_radius_h=1.0))
        rm.close()
    hfun = lambda x: roadmap_ref.heuristic(m, samples, dist, x, goal, 1.0)
    ref = search_ref.search(m, prims, env, start, goal, delta, batch=batch, max_expands=300, hfun=hfun)
    assert res["status_str"] == ref["status"]
    assert res["expands"] == ref["expands"]
    assert res["nodes"] == ref["nodes"]
    if ref["solved"]:
        assert list(motions) == ref["motions"]
