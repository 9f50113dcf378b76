"""dpg_lazy_check against the oracle: candidates of a ball-only expand,
ranked by a score (or motion order), checked lazily until each node has
`limit` valid motions.  Bars: the accepted set of every node is exactly
the first `limit` oracle-valid candidates in rank order; every checked
candidate's verdict and first invalid state equal the oracle's and its end
state is within the parity tolerance (tests/parity_util.py); every
candidate a node needs in the reference loop's order is checked."""
import numpy as np
import pytest

import oracle_bind as ob
from dynoplan_gb300 import workloads as W
from lazy_ref import lazy_accept
from parity_util import compare

pytestmark = pytest.mark.gpu


def run_lazy(wl, precision, limit, score_kind, seed):
    import torch

    from dynoplan_gb300 import _lib
    from dynoplan_gb300 import gpu as G
    with G.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        ball = ctx.expand(wl.nodes, wl.radius, ball_only=True)
        n = ball["n_pairs"]
        rng = np.random.default_rng(seed)
        score = None
        if score_kind == "random":
            score = rng.standard_normal(n).astype(np.float32)
            score[rng.random(n) < 0.05] = np.nan          # unscored candidates rank last
            score[rng.random(n) < 0.05] = 0.5             # ties broken by primitive index
        dev = "cuda:0"
        x_d = torch.from_numpy(wl.nodes).to(dev)
        node_d = torch.from_numpy(ball["node"].view(np.int32)).to(dev)
        prim_d = torch.from_numpy(ball["prim"].view(np.int32)).to(dev)
        sc_d = torch.from_numpy(np.stack([score, np.zeros_like(score)], 1)).to(dev) if score is not None else None
        es_t = torch.float64 if precision else torch.float32
        outs = {"verdict": torch.empty(n, dtype=torch.uint8, device=dev),
                "first_invalid": torch.empty(n, dtype=torch.int16, device=dev),
                "end_state": torch.empty((n, wl.robot.nx), dtype=es_t, device=dev),
                "min_gap": torch.empty(n, dtype=torch.float32, device=dev),
                "flags": torch.full((n,), 0x7f, dtype=torch.uint8, device=dev)}
        torch.cuda.synchronize()
        st = ctx.lazy_check_device(x_d.data_ptr(), len(wl.nodes), n, node_d.data_ptr(), prim_d.data_ptr(),
                                   {k: v.data_ptr() for k, v in outs.items()}, limit,
                                   score_ptr=sc_d.data_ptr() if sc_d is not None else None, score_stride=2,
                                   precision=precision)
        got = {k: v.cpu().numpy() for k, v in outs.items()}
    return ball, score, got, st, _lib


@pytest.mark.parametrize("cfg,scale,precision,limit,score_kind", [
    (2, 0.02, 0, 20, "random"), (2, 0.02, 0, 20, None), (3, 0.01, 0, 10, "random"),
    (1, 0.1, 1, 20, "random"), (5, 0.01, 0, 5, None), (2, 0.01, 0, 100000, "random")])
def test_lazy_matches_oracle(cfg, scale, precision, limit, score_kind):
    wl = W.make_workload(cfg, scale=scale, seed=300 + cfg)
    ball, score, got, st, _lib = run_lazy(wl, precision, limit, score_kind, seed=cfg)
    ora = ob.expand(wl.robot, wl.prims, wl.env, wl.nodes, wl.radius, fast=True, threads=ob.lib().orc_max_threads())
    # oracle results in the candidate order of the ball stage
    key = lambda nd, pr: nd.astype(np.int64) * (1 << 32) + pr.astype(np.int64)
    ko, kb = key(ora["node"], ora["prim"]), key(ball["node"], ball["prim"])
    oi = np.argsort(ko)
    pos = oi[np.searchsorted(ko[oi], kb)]
    np.testing.assert_array_equal(ko[pos], kb)             # same candidate set
    valid = ora["verdict"][pos] == 0
    accepted, needed = lazy_accept(ball["node"], ball["prim"], valid, score, limit)
    checked = got["verdict"] != _lib.DPG_UNCHECKED
    np.testing.assert_array_equal((got["flags"] & _lib.DPG_FLAG_ACCEPTED) != 0, accepted)
    assert checked[needed].all()
    assert st["n_checked"] == int(checked.sum())
    assert st["n_accepted"] == int(accepted.sum())
    assert st["n_valid"] == int((got["verdict"] == 0).sum())
    assert ((got["flags"] & ~np.uint8(3)) == 0).all()
    sel = np.flatnonzero(checked)
    sub = {"node": ball["node"][sel], "prim": ball["prim"][sel], "n_pairs": len(sel),
           **{k: got[k][sel] for k in ("verdict", "first_invalid", "end_state")}}
    ref = {"node": ora["node"][pos[sel]], "prim": ora["prim"][pos[sel]], "n_pairs": len(sel),
           **{k: ora[k][pos[sel]] for k in ("verdict", "first_invalid", "end_state")}}
    compare(wl.robot.kind, sub, ref, precision, min_gap=False)
    if limit >= st["max_candidates"]:
        assert checked.all()                               # nothing to skip
    # nothing beyond what the reference loop needs, except the last round's
    # overshoot: at most ceil((limit - valid) * f) - 1 extra per node (f <= 16)
    assert int((checked & ~needed).sum()) <= 16 * limit * len(np.unique(ball["node"]))


def test_lazy_rejects_bad_input():
    import torch

    from dynoplan_gb300 import _lib
    from dynoplan_gb300 import gpu as G
    wl = W.make_workload(2, scale=0.01, seed=9)
    N = len(wl.nodes)
    with G.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        x_d = torch.from_numpy(wl.nodes).cuda()
        node = torch.tensor([0, 1, N], dtype=torch.int32, device="cuda")
        prim = torch.tensor([0, 1, 2], dtype=torch.int32, device="cuda")
        outs = {"verdict": torch.empty(3, dtype=torch.uint8, device="cuda"),
                "flags": torch.empty(3, dtype=torch.uint8, device="cuda")}
        ptrs = {k: v.data_ptr() for k, v in outs.items()}
        torch.cuda.synchronize()
        with pytest.raises(_lib.DpgError) as e:       # node index out of range
            ctx.lazy_check_device(x_d.data_ptr(), N, 3, node.data_ptr(), prim.data_ptr(), ptrs, 20)
        assert e.value.code == _lib.DPG_ERR_ARG
        node[2] = 0
        with pytest.raises(_lib.DpgError) as e:       # limit must be >= 1
            ctx.lazy_check_device(x_d.data_ptr(), N, 3, node.data_ptr(), prim.data_ptr(), ptrs, 0)
        assert e.value.code == _lib.DPG_ERR_ARG
        st = ctx.lazy_check_device(x_d.data_ptr(), N, 3, node.data_ptr(), prim.data_ptr(), ptrs, 1)
        assert st["n_checked"] >= 2


def test_per_node_drop_in_counts():
    """The plain drop-in bench helper (one dpg_expand per node) checks the
    same pairs as one batched call."""
    import ctypes as C

    from dynoplan_gb300 import _lib
    from dynoplan_gb300 import gpu as G
    wl = W.make_workload(2, scale=0.01, seed=12)
    lib = _lib.load()
    with G.Context(wl.robot) as ctx:
        ctx.upload_primitives(wl.prims)
        ctx.upload_env(wl.env)
        batched = ctx.expand(wl.nodes[:200], wl.radius)["n_pairs"]
        opts = _lib.ExpandOpts(radius=wl.radius, precision=0, x_on_device=0, out_on_device=0, mode=0,
                               contact_band=1e-4, ball_band=1e-5)
        xs = np.ascontiguousarray(wl.nodes[:200])
        pairs, secs = C.c_int64(), C.c_double()
        _lib.check(lib.dpg_bench_per_node_expand(ctx.h, C.byref(opts), 200, wl.robot.nx, xs.ctypes.data,
                                                 C.byref(pairs), C.byref(secs)), ctx.h)
    assert pairs.value == batched and secs.value > 0
