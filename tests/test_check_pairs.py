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


def test_check_pairs_rejects_out_of_range_indices(gpu):
    """A node index >= N or a primitive index >= P is refused with
    DPG_ERR_ARG: host lists before any copy, device lists by the kernels
    that group the pairs (they skip such pairs and count them); the in-range
    pairs of the same call are untouched memory-wise, and the context stays
    usable."""
    import ctypes as C

    import torch

    from dynoplan_gb300 import _lib
    wl = W.make_workload(2, scale=0.01, seed=77)
    N, P = len(wl.nodes), wl.prims.P
    good_n = np.arange(8, dtype=np.uint32) % N
    good_p = np.arange(8, dtype=np.uint32) % P
    with gpu.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        for bad_n, bad_p in ((N, 0), (0, P), (2 ** 31, 2 ** 32 - 1)):
            node = np.r_[good_n, np.uint32(bad_n)].astype(np.uint32)
            prim = np.r_[good_p, np.uint32(bad_p)].astype(np.uint32)
            with pytest.raises(_lib.DpgError) as e:
                ctx.check_pairs(wl.nodes, node, prim)
            assert e.value.code == _lib.DPG_ERR_ARG
            # the same lists in device memory
            x_d = torch.from_numpy(wl.nodes).cuda()
            n_d = torch.from_numpy(node.view(np.int32)).cuda()
            p_d = torch.from_numpy(prim.view(np.int32)).cuda()
            verdict = torch.zeros(len(node), dtype=torch.uint8, device="cuda")
            opts = _lib.ExpandOpts(radius=0.0, precision=0, x_on_device=1, out_on_device=1, mode=0,
                                   contact_band=1e-4, ball_band=1e-5)
            out = _lib.ExpandOut(capacity=len(node))
            out.verdict = C.c_void_p(verdict.data_ptr())
            torch.cuda.synchronize()
            rc = ctx.lib.dpg_check_pairs(ctx.h, C.byref(opts), N, C.c_void_p(x_d.data_ptr()), len(node),
                                         C.c_void_p(n_d.data_ptr()), C.c_void_p(p_d.data_ptr()), C.byref(out))
            assert rc == _lib.DPG_ERR_ARG
        # still usable, and the good pairs agree with a clean call
        ok = ctx.check_pairs(wl.nodes, good_n, good_p)
        assert ok["n_pairs"] == 8
