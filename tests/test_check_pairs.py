"""dpg_check_pairs (exact check of an explicit pair list, results in input
order) and the ball-only mode of dpg_expand, against the oracle."""
import numpy as np
import pytest

import oracle_bind as ob
from dynoplan_gb300 import workloads as W
from parity_util import compare

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu(dpg_lib):
    from dynoplan_gb300 import gpu as G
    return G


@pytest.mark.parametrize("cfg,scale", [(1, 0.05), (2, 0.02), (3, 0.01), (5, 0.01)])
@pytest.mark.parametrize("precision", [0, 1])
def test_check_pairs_matches_oracle(gpu, cfg, scale, precision):
    wl = W.make_workload(cfg, scale=scale, seed=40 + cfg)
    ora = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius)
    rng = np.random.default_rng(cfg)
    # a shuffled subset with repeats, and pairs outside the ball (the check
    # does not care about the ball)
    idx = rng.integers(0, ora["n_pairs"], size=max(1, ora["n_pairs"] // 2))
    node = ora["node"][idx]
    prim = ora["prim"][idx]
    extra_node = rng.integers(0, len(wl.nodes), 200).astype(np.uint32)
    extra_prim = rng.integers(0, wl.prims.P, 200).astype(np.uint32)
    node = np.concatenate([node, extra_node])
    prim = np.concatenate([prim, extra_prim])
    with gpu.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        got = ctx.check_pairs(wl.nodes, node, prim, precision=precision)
        ball = ctx.expand(wl.nodes, wl.radius, ball_only=True)
    # the oracle on the same explicit list (pair by pair)
    ref = {k: [] for k in ("verdict", "first_invalid", "end_state", "min_gap")}
    import ctypes as C
    r = ob.robot(wl.robot)
    e, ke = ob.env_struct(wl.env)
    p, kp = ob.prims_struct(wl.prims)
    xs = np.empty((int(wl.prims.length.max()), wl.robot.nx))
    for n_, p_ in zip(node, prim):
        fi, es, mg = C.c_int16(), np.empty(wl.robot.nx), C.c_double()
        x = np.ascontiguousarray(wl.nodes[n_])
        ob.lib().orc_check_pair.argtypes = [C.POINTER(ob.OrcRobot), C.POINTER(ob.OrcEnv), C.POINTER(ob.OrcPrims),
                                            C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_int16), C.c_void_p,
                                            C.POINTER(C.c_double)]
        v = ob.lib().orc_check_pair(C.byref(r), C.byref(e), C.byref(p), x.ctypes.data, int(p_), xs.ctypes.data,
                                    C.byref(fi), es.ctypes.data, C.byref(mg))
        ref["verdict"].append(v)
        ref["first_invalid"].append(fi.value)
        ref["end_state"].append(es)
        ref["min_gap"].append(mg.value)
    ref = {k: np.array(v) for k, v in ref.items()}
    ref.update(node=node, prim=prim, n_pairs=len(node))
    ref["verdict"] = ref["verdict"].astype(np.uint8)
    ref["first_invalid"] = ref["first_invalid"].astype(np.int16)
    # results are in input order: compare row by row (no sort)
    np.testing.assert_array_equal(got["verdict"], ref["verdict"])
    np.testing.assert_array_equal(got["first_invalid"], ref["first_invalid"])
    compare(wl.robot.kind, got, ref, precision)
    # ball-only mode gives exactly the oracle's pair set
    key = lambda n, q: np.sort(n.astype(np.int64) * (1 << 32) + q.astype(np.int64))
    np.testing.assert_array_equal(key(ball["node"], ball["prim"]), key(ora["node"], ora["prim"]))
