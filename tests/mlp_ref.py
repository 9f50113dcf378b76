"""FP64 numpy restatement of the surrogate MLP's forward and backward pass,
with bf16 rounding at the same points as the GPU kernels (inputs, weights,
hidden activations, loss gradient, pre-activation gradients).  Test
infrastructure: the checker of dynoplan_gb300's MLP kernels."""
import numpy as np


def bf16(x):
    """round to the nearest bfloat16 (ties to even), returned as float64"""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


GELU_A, GELU_B = np.sqrt(2.0 / np.pi), 0.044715


def gelu(z):
    """tanh form of GELU (Hendrycks & Gimpel 2016)"""
    return 0.5 * z * (1.0 + np.tanh(GELU_A * (z + GELU_B * z ** 3)))


def gelu_grad(z):
    t = np.tanh(GELU_A * (z + GELU_B * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * GELU_A * (1.0 + 3.0 * GELU_B * z * z)


def assemble(node_feat, emb, node, prim):
    B = len(node)
    X = np.zeros((B, 128))
    X[:, :80] = bf16(node_feat)[node]
    X[:, 80:96] = bf16(emb)[prim]
    return X


def forward_backward(p, node_feat, node, prim, target, ctg_weight):
    """p: dict of FP32 parameters (W1 256x128, b1, W2, b2, W3, b3, W4 16x256, b4,
    emb P x 16).  Returns (outputs [B x 2], loss, grads dict)."""
    W = [bf16(p["W1"]), bf16(p["W2"]), bf16(p["W3"]), bf16(p["W4"])]
    b = [p["b1"].astype(np.float64), p["b2"].astype(np.float64), p["b3"].astype(np.float64),
         p["b4"].astype(np.float64)]
    X = assemble(node_feat, p["emb"], node, prim)
    B = len(node)
    Z, H = [], [X]
    for l in range(3):
        z = H[-1] @ W[l].T + b[l]
        Z.append(z)
        H.append(bf16(gelu(z)))
    out = H[3] @ W[3].T + b[3]
    lg, ct = out[:, 0], out[:, 1]
    y, t = target[:, 0].astype(np.float64), target[:, 1].astype(np.float64)
    sp = np.where(lg > 20, lg, np.log1p(np.exp(np.minimum(lg, 20))))
    loss = np.mean(sp - y * lg + 0.5 * ctg_weight * (ct - t) ** 2)
    dY = np.zeros((B, 16))
    dY[:, 0] = bf16((1 / (1 + np.exp(-lg)) - y) / B)
    dY[:, 1] = bf16(ctg_weight * (ct - t) / B)
    g = {"W4": dY.T @ H[3], "b4": dY.sum(0)}
    dZ = bf16((dY @ W[3]) * gelu_grad(Z[2]))
    for l in (2, 1, 0):
        g[f"W{l + 1}"] = dZ.T @ H[l]
        g[f"b{l + 1}"] = dZ.sum(0)
        dH = dZ @ W[l]
        if l > 0:
            dZ = bf16(dH * gelu_grad(Z[l - 1]))
    demb = np.zeros_like(p["emb"], dtype=np.float64)
    np.add.at(demb, prim, dH[:, 80:96])
    g["emb"] = demb
    return out[:, :2], loss, g
