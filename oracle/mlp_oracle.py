"""NumPy reference of the potential-surrogate MLP (test infrastructure only).

Network: 3 -> 256 -> 256 -> 256 -> 256 -> 1 with SiLU activations,
    z1 = W1 u + b1, h_k = silu(z_k), z_{k+1} = W_{k+1} h_k + b_{k+1}, out = w5 . h4 + b5,
with u = x / length_scale and Phi(x) = phi_scale * out(u). The acceleration is
-grad_x Phi = -(phi_scale / length_scale) grad_u out.

Training loss on a batch of B points with potential and gradient targets:
    L = (alpha / B) sum (out - phi_t)^2 + (beta / B) sum |grad_u out - g_t|^2
(targets already in network units). ``loss_and_grads`` returns the exact
gradient of L with respect to every parameter, including the second-order
terms that the gradient-matching part needs (the derivative of grad_u out with
respect to the weights); a test checks it against central differences. Used to
check the GPU training and inference kernels.
"""

from __future__ import annotations

import numpy as np

HIDDEN = 256
NAMES = ("W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4", "w5", "b5")


def init_params(seed: int = 0, dtype=np.float64) -> dict:
    rng = np.random.default_rng(seed)

    def lin(nout, nin):
        return rng.normal(0.0, np.sqrt(2.0 / nin), (nout, nin)).astype(dtype)

    p = {
        "W1": lin(HIDDEN, 3), "b1": np.zeros(HIDDEN, dtype),
        "W2": lin(HIDDEN, HIDDEN), "b2": np.zeros(HIDDEN, dtype),
        "W3": lin(HIDDEN, HIDDEN), "b3": np.zeros(HIDDEN, dtype),
        "W4": lin(HIDDEN, HIDDEN), "b4": np.zeros(HIDDEN, dtype),
        "w5": (rng.normal(0.0, np.sqrt(1.0 / HIDDEN), HIDDEN)).astype(dtype), "b5": np.zeros(1, dtype),
    }
    return p


def sig(z):
    return 1.0 / (1.0 + np.exp(-z))


def silu(z):
    return z * sig(z)


def dsilu(z):
    s = sig(z)
    return s * (1.0 + z * (1.0 - s))


def d2silu(z):
    s = sig(z)
    return s * (1.0 - s) * (2.0 + z * (1.0 - 2.0 * s))


def forward(p: dict, u: np.ndarray):
    """Returns out (B,), grad_u out (B, 3) and the cache for training."""
    z1 = u @ p["W1"].T + p["b1"]
    h1 = silu(z1)
    z2 = h1 @ p["W2"].T + p["b2"]
    h2 = silu(z2)
    z3 = h2 @ p["W3"].T + p["b3"]
    h3 = silu(z3)
    z4 = h3 @ p["W4"].T + p["b4"]
    h4 = silu(z4)
    out = h4 @ p["w5"] + p["b5"][0]
    # input gradient (backward pass)
    d4 = dsilu(z4) * p["w5"]
    u3 = d4 @ p["W4"]
    d3 = dsilu(z3) * u3
    u2 = d3 @ p["W3"]
    d2 = dsilu(z2) * u2
    u1 = d2 @ p["W2"]
    d1 = dsilu(z1) * u1
    g = d1 @ p["W1"]
    cache = dict(u=u, z1=z1, h1=h1, z2=z2, h2=h2, z3=z3, h3=h3, z4=z4, h4=h4, d1=d1, d2=d2, d3=d3, d4=d4,
                 u1=u1, u2=u2, u3=u3)
    return out, g, cache


def loss_and_grads(p: dict, u, phi_t, g_t, alpha: float, beta: float, w=None):
    """Loss 1/B sum_b w_b [alpha (out_b - phi_t,b)^2 + beta |g_b - g_t,b|^2] (w_b = 1
    when w is None) and its exact gradient with respect to every parameter."""
    B = len(u)
    w = np.ones(B) if w is None else np.asarray(w, np.float64)
    out, g, c = forward(p, u)
    rphi = out - phi_t
    rg = g - g_t
    L = alpha * np.sum(w * rphi**2) / B + beta * np.sum(w[:, None] * rg**2) / B
    Pb = 2.0 * alpha * w * rphi / B          # dL/dout
    Eb = 2.0 * beta * w[:, None] * rg / B    # dL/dg
    gr = {k: np.zeros_like(v) for k, v in p.items()}
    # ---- through the input-gradient (backward) graph
    gr["W1"] += c["d1"].T @ Eb
    Db1 = Eb @ p["W1"].T
    Ub1 = dsilu(c["z1"]) * Db1
    Zb1 = d2silu(c["z1"]) * c["u1"] * Db1
    gr["W2"] += c["d2"].T @ Ub1
    Db2 = Ub1 @ p["W2"].T
    Ub2 = dsilu(c["z2"]) * Db2
    Zb2 = d2silu(c["z2"]) * c["u2"] * Db2
    gr["W3"] += c["d3"].T @ Ub2
    Db3 = Ub2 @ p["W3"].T
    Ub3 = dsilu(c["z3"]) * Db3
    Zb3 = d2silu(c["z3"]) * c["u3"] * Db3
    gr["W4"] += c["d4"].T @ Ub3
    Db4 = Ub3 @ p["W4"].T
    gr["w5"] += np.sum(dsilu(c["z4"]) * Db4, axis=0)
    Zb4 = d2silu(c["z4"]) * p["w5"] * Db4
    # ---- through the forward graph (potential term and the z-dependence above)
    gr["w5"] += c["h4"].T @ Pb
    gr["b5"] += np.sum(Pb, keepdims=True)
    Zb4 = Zb4 + dsilu(c["z4"]) * np.outer(Pb, p["w5"])
    gr["W4"] += Zb4.T @ c["h3"]
    gr["b4"] += Zb4.sum(0)
    Zb3 = Zb3 + dsilu(c["z3"]) * (Zb4 @ p["W4"])
    gr["W3"] += Zb3.T @ c["h2"]
    gr["b3"] += Zb3.sum(0)
    Zb2 = Zb2 + dsilu(c["z2"]) * (Zb3 @ p["W3"])
    gr["W2"] += Zb2.T @ c["h1"]
    gr["b2"] += Zb2.sum(0)
    Zb1 = Zb1 + dsilu(c["z1"]) * (Zb2 @ p["W2"])
    gr["W1"] += Zb1.T @ c["u"]
    gr["b1"] += Zb1.sum(0)
    return L, gr


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round float values to bfloat16 (round to nearest even), returned as float32."""
    f = np.asarray(a, np.float32)
    bits = f.view(np.uint32).astype(np.uint64)
    rounding = ((bits >> 16) & 1) + 0x7FFF
    out = ((bits + rounding) >> 16 << 16).astype(np.uint32)
    return out.view(np.float32)


def forward_bf16(p: dict, u: np.ndarray):
    """The inference numerics: BF16 weights and BF16 activations entering every
    256x256 product, FP32 accumulation; the 3->256 and 256->1 layers in FP32.
    Returns (out, grad_u out) as float64."""
    f32 = np.float32
    W = {k: bf16_round(p[k]).astype(f32) for k in ("W2", "W3", "W4")}
    z1 = (u.astype(f32) @ p["W1"].astype(f32).T + p["b1"].astype(f32))
    h1 = bf16_round(silu(z1))
    z2 = h1 @ W["W2"].T + p["b2"].astype(f32)
    h2 = bf16_round(silu(z2))
    z3 = h2 @ W["W3"].T + p["b3"].astype(f32)
    h3 = bf16_round(silu(z3))
    z4 = h3 @ W["W4"].T + p["b4"].astype(f32)
    h4 = silu(z4)
    out = h4 @ p["w5"].astype(f32) + f32(p["b5"][0])
    d4 = bf16_round(dsilu(z4) * p["w5"].astype(f32))
    d3 = bf16_round(dsilu(z3) * (d4 @ W["W4"]))
    d2 = bf16_round(dsilu(z2) * (d3 @ W["W3"]))
    d1 = dsilu(z1) * (d2 @ W["W2"])
    g = d1 @ p["W1"].astype(f32)
    return out.astype(np.float64), g.astype(np.float64)
