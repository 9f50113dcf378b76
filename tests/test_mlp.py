"""The surrogate MLP's tensor-core kernels: forward outputs and every
parameter gradient against the FP64 numpy restatement (tests/mlp_ref.py),
then a short training run on exact-checker labels that must beat the plain
method (random order of lazy checks) on held-out environments.

Tolerances: forward outputs |d| <= 2e-3 * (1 + |y|); gradients relative L2
error <= 2e-2 per parameter (FP32 accumulation order, rare bf16 rounding
flips of pre-activation gradients)."""
import numpy as np
import pytest

from dynoplan_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _random_params(rng, P):
    p = {"W1": rng.normal(0, 1 / np.sqrt(96), (256, 128)), "b1": rng.normal(0, 0.1, 256),
         "W2": rng.normal(0, 1 / 16, (256, 256)), "b2": rng.normal(0, 0.1, 256),
         "W3": rng.normal(0, 1 / 16, (256, 256)), "b3": rng.normal(0, 0.1, 256),
         "W4": np.zeros((16, 256)), "b4": np.zeros(16), "emb": rng.normal(0, 0.5, (P, 16))}
    p["W4"][:2] = rng.normal(0, 1 / 16, (2, 256))
    p["b4"][:2] = rng.normal(0, 0.1, 2)
    p["W1"][:, 96:] = 0.0
    return {k: v.astype(np.float32) for k, v in p.items()}


@pytest.mark.parametrize("B", [300, 4096])
def test_forward_and_gradients_match_numpy(dpg_lib, B):
    torch = pytest.importorskip("torch")
    import mlp_ref
    from dynoplan_gb300.surrogate import Surrogate
    rng = np.random.default_rng(B)
    P, N = 50, 200
    params = _random_params(rng, P)
    feat = rng.normal(0, 1, (N, 80)).astype(np.float32)
    feat[:, 16:] = (rng.random((N, 64)) < 0.3)
    node = rng.integers(0, N, B)
    prim = rng.integers(0, P, B)
    target = np.stack([(rng.random(B) < 0.4).astype(np.float32), rng.random(B).astype(np.float32)], 1)
    s = Surrogate(P, max_rows=max(B, 1024), seed=1)
    for k, v in params.items():
        s.set(k, v)
    dev = "cuda:0"
    feat_d = torch.from_numpy(feat).to(dev).to(torch.bfloat16)
    node_d = torch.from_numpy(node.astype(np.int32)).to(dev)
    prim_d = torch.from_numpy(prim.astype(np.int32)).to(dev)
    tgt_d = torch.from_numpy(target).to(dev)
    out = s.forward(feat_d, node_d, prim_d).cpu().numpy()
    ref_out, ref_loss, ref_g = mlp_ref.forward_backward(params, feat_d.float().cpu().numpy(), node, prim, target, 1.0)
    assert np.all(np.abs(out - ref_out) <= 2e-3 * (1 + np.abs(ref_out)))
    loss = s.train_step(feat_d, node_d, prim_d, tgt_d, lr=0.0, ctg_weight=1.0)
    assert loss == pytest.approx(ref_loss, rel=1e-3)
    for k in ("W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4", "emb"):
        g = s.get(k, grad=True).astype(np.float64)
        r = ref_g[k]
        if k == "W4":
            g, r = g[:2], r[:2]
        if k == "b4":
            g, r = g[:2], r[:2]
        err = np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-12)
        assert err <= 2e-2, (k, err)
    # lr = 0 leaves the weights unchanged
    np.testing.assert_array_equal(s.get("W2"), params["W2"])
    s.close()


def _checks_to_k_valid(order_keys, node, valid, k):
    """mean number of exact checks per node until k valid pairs are found
    (or the node's list is exhausted), visiting pairs in ascending key order"""
    total, nodes = 0, 0
    order = np.lexsort((order_keys, node))
    node_s, valid_s = node[order], valid[order]
    starts = np.flatnonzero(np.r_[True, node_s[1:] != node_s[:-1]])
    ends = np.r_[starts[1:], len(node_s)]
    for a, b in zip(starts, ends):
        c = np.cumsum(valid_s[a:b])
        hit = np.searchsorted(c, k)
        total += min(hit + 1, b - a)
        nodes += 1
    return total / max(nodes, 1)


def test_training_beats_random_order_on_held_out_envs(dpg_lib):
    """Trained on exact labels from 16 car1 environments, the surrogate's
    order finds 5 valid expansions per node with fewer exact checks than the
    shuffled order Expander::expand_lazy uses, on 4 unseen environments."""
    torch = pytest.importorskip("torch")
    from dynoplan_gb300 import surrogate as S
    wl = W.make_workload(2, scale=0.2, seed=3)   # 1000 car1 primitives
    train = S.make_dataset(wl, n_envs=16, nodes_per_env=1500, pairs_per_env=20000, seed=11)
    test = S.make_dataset(wl, n_envs=4, nodes_per_env=600, pairs_per_env=10 ** 9, seed=99)
    m = S.Surrogate(wl.prims.P, max_rows=16384, seed=0)
    losses, rate, tflops = S.train(m, train, epochs=6, batch=16384, lr=3e-3)
    assert np.mean(losses[-5:]) < 0.8 * np.mean(losses[:5])
    out = m.forward(test.node_feat, test.node, test.prim).cpu().numpy()
    valid = (test.target[:, 0].cpu().numpy() == 0)
    node = test.node.cpu().numpy()
    rng = np.random.default_rng(0)
    mlp_checks = _checks_to_k_valid(out[:, 0], node, valid, 5)   # ascending collision logit
    rnd = np.mean([_checks_to_k_valid(rng.random(len(node)), node, valid, 5) for _ in range(3)])
    assert mlp_checks < 0.9 * rnd, (mlp_checks, rnd)
    m.close()


@pytest.mark.parametrize("B", [1, 129, 5000, 300000])
def test_fused_forward_matches_layer_by_layer(dpg_lib, B):
    """the persistent fused forward (one CTA per SM walking 128-row tiles,
    several tiles per CTA at the largest size) against the layer-by-layer
    GEMMs: same bf16 operands and FP32 accumulation order"""
    torch = pytest.importorskip("torch")
    from dynoplan_gb300.surrogate import Surrogate
    rng = np.random.default_rng(B + 7)
    P, N = 64, 1000
    params = _random_params(rng, P)
    feat = rng.normal(0, 1, (N, 80)).astype(np.float32)
    feat[:, 16:] = (rng.random((N, 64)) < 0.3)
    dev = "cuda:0"
    feat_d = torch.from_numpy(feat).to(dev).to(torch.bfloat16)
    node_d = torch.from_numpy(rng.integers(0, N, B).astype(np.int32)).to(dev)
    prim_d = torch.from_numpy(rng.integers(0, P, B).astype(np.int32)).to(dev)
    s = Surrogate(P, max_rows=65536, seed=2)
    for k, v in params.items():
        s.set(k, v)
    s.set_fused(0)
    ref = s.forward(feat_d, node_d, prim_d).cpu().numpy()
    for kind in (1, 2):   # one CTA per tile walk; warp-specialised with overlapped epilogues
        s.set_fused(kind)
        out = s.forward(feat_d, node_d, prim_d).cpu().numpy()
        assert out.shape == (B, 2) and np.isfinite(out).all()
        assert np.abs(out - ref).max() <= 1e-3 * (1 + np.abs(ref).max())
