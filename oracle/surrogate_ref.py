"""CPU restatement of the learned surrogate's network (test infrastructure:
only tests/ import this module; the product path never does).

The surrogate has no counterpart in the reference (it is a new component on
top of the Warren1995 engine, Engines/Warren1995.py:50-92); this module is
its FP64 oracle. Its backward pass is pinned by central finite differences
of its own forward pass (tests/test_surrogate_oracle.py), and the GPU
kernels (pyphasefield_gb300/csrc/surrogate.cu) are checked against it.

`bf16=True` rounds every operand the GPU feeds to its BF16 tensor-core GEMMs
to bfloat16 (round to nearest even) at the same places, so the remaining
difference to the GPU is FP32-vs-FP64 accumulation only; `bf16=False` is the
exact FP64 network.

Layouts follow the library: tokens t = (sample, patch row, patch col),
patch columns k = (channel, py, px), fields [b][ch][H][W], weights W[out][in],
depthwise weights [C][9] with tap (dy + 1) * 3 + (dx + 1).
"""
from __future__ import annotations

import numpy as np
from scipy.special import erf


def bf16(x):
    """float64 -> float32 -> bfloat16 (round to nearest even) -> float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32)).view(np.uint32).astype(np.uint64)
    r = ((a + 0x7FFF + ((a >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _id(x):
    return np.asarray(x, dtype=np.float64)


def patches(f, P):
    """fields [B, 2, H, W] -> [B * (H/P) * (W/P), 2 P P]."""
    B, ch, H, W = f.shape
    gh, gw = H // P, W // P
    x = f.reshape(B, ch, gh, P, gw, P).transpose(0, 2, 4, 1, 3, 5)
    return x.reshape(B * gh * gw, ch * P * P)


def unpatch(x, B, H, W, P):
    gh, gw = H // P, W // P
    return x.reshape(B, gh, gw, 2, P, P).transpose(0, 3, 1, 4, 2, 5).reshape(B, 2, H, W)


def gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2 * np.pi)


def dwconv(y, w, b, B, gh, gw):
    """Depthwise 3x3 over the token grid, zero padding; y [T, C]."""
    C = y.shape[1]
    g = np.pad(y.reshape(B, gh, gw, C), ((0, 0), (1, 1), (1, 1), (0, 0)))
    h = np.broadcast_to(b, (B, gh, gw, C)).copy()
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            h += w[:, (dy + 1) * 3 + (dx + 1)] * g[:, 1 + dy:1 + dy + gh, 1 + dx:1 + dx + gw]
    return h.reshape(-1, C)


def dwconv_bwd(dh, y, w, B, gh, gw):
    """Gradients of dwconv: (dy, dw, db)."""
    C = y.shape[1]
    d = dh.reshape(B, gh, gw, C)
    g = np.pad(y.reshape(B, gh, gw, C), ((0, 0), (1, 1), (1, 1), (0, 0)))
    dgp = np.zeros_like(g)
    dw = np.zeros_like(w)
    for dy in (-1, 0, 1):
        for dx in (-1, 0, 1):
            tap = (dy + 1) * 3 + (dx + 1)
            sl = (slice(None), slice(1 + dy, 1 + dy + gh), slice(1 + dx, 1 + dx + gw))
            dw[:, tap] = (d * g[sl]).sum(axis=(0, 1, 2))
            dgp[sl] += d * w[:, tap]
    return dgp[:, 1:-1, 1:-1].reshape(-1, C), dw, d.sum(axis=(0, 1, 2))


def normalise(f, norm):
    o0, s0, o1, s1 = norm
    out = np.array(f, dtype=np.float64)
    out[:, 0] = (out[:, 0] - o0) * s0
    out[:, 1] = (out[:, 1] - o1) * s1
    return out


def forward(params, f_old, P, L, norm, bf16_ops=True):
    """Returns (out [T, 2PP], cache)."""
    q = bf16 if bf16_ops else _id
    B, _, H, W = f_old.shape
    gh, gw = H // P, W // P
    X = q(patches(normalise(f_old, norm), P))
    y = X @ q(params["w_in"]).T + params["b_in"]
    cache = {"X": X, "ys": [y], "hs": [], "pres": [], "acts": []}
    for l in range(L):
        h = dwconv(y, params[f"dw{l}"], params[f"bdw{l}"], B, gh, gw)
        pre = q(h) @ q(params[f"w1_{l}"]).T + params[f"b1_{l}"]
        act = q(gelu(pre))
        y = y + act @ q(params[f"w2_{l}"]).T + params[f"b2_{l}"]
        cache["hs"].append(h)
        cache["pres"].append(pre)
        cache["acts"].append(act)
        cache["ys"].append(y)
    out = q(y) @ q(params["w_out"]).T + params["b_out"]
    return out, cache


def target(f_old, f_new, P, scale):
    d = np.array(f_new, dtype=np.float64) - f_old
    d[:, 0] *= scale[0]
    d[:, 1] *= scale[1]
    return patches(d, P)


def loss_and_grads(params, f_old, f_new, P, L, norm, scale, bf16_ops=True):
    """MSE on the normalised change and the gradient of every parameter."""
    q = bf16 if bf16_ops else _id
    B, _, H, W = f_old.shape
    gh, gw = H // P, W // P
    out, c = forward(params, f_old, P, L, norm, bf16_ops)
    d = out - target(f_old, f_new, P, scale)
    loss = float((d * d).mean())
    dout = q(2.0 * d / d.size)
    g = {}
    yL = q(c["ys"][L])
    g["w_out"] = dout.T @ yL
    g["b_out"] = dout.sum(0)
    dy = dout @ q(params["w_out"])
    for l in reversed(range(L)):
        dyb = q(dy)
        g[f"w2_{l}"] = dyb.T @ c["acts"][l]
        g[f"b2_{l}"] = dy.sum(0)
        dpre = q((dyb @ q(params[f"w2_{l}"])) * gelu_grad(c["pres"][l]))
        g[f"w1_{l}"] = dpre.T @ q(c["hs"][l])
        g[f"b1_{l}"] = dpre.sum(0)
        dh = dpre @ q(params[f"w1_{l}"])
        ddy, g[f"dw{l}"], g[f"bdw{l}"] = dwconv_bwd(dh, c["ys"][l], params[f"dw{l}"], B, gh, gw)
        dy = dy + ddy
    dyb = q(dy)
    g["w_in"] = dyb.T @ c["X"]
    g["b_in"] = dyb.sum(0)
    return loss, g, out


def param_shapes(P, C, E, L):
    K = 2 * P * P
    s = {"w_in": (C, K), "b_in": (C,), "w_out": (K, C), "b_out": (K,)}
    for l in range(L):
        s.update({f"dw{l}": (C, 9), f"bdw{l}": (C,), f"w1_{l}": (E, C), f"b1_{l}": (E,),
                  f"w2_{l}": (C, E), f"b2_{l}": (C,)})
    return s


def random_params(P, C, E, L, rng, scale=1.0):
    p = {}
    for k, shp in param_shapes(P, C, E, L).items():
        fan = shp[1] if len(shp) == 2 else 1
        p[k] = rng.normal(0, scale / np.sqrt(fan), shp)
    return p
