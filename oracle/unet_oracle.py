"""CPU oracle (test infrastructure) for the learned surrogate: a float64 numpy
forward and backward pass of the U-Net that ``fingering_dynamics_gb300.surrogate``
trains with its own CUDA kernels.  Only tests import it.  There is no
reference counterpart (the reference has no learned component); the
gradients of this oracle are pinned by finite differences in
``tests/test_unet_oracle.py``.

Layout: activations NHWC, weights ``[Cout][3][3][Cin]``, "same" padding with
zeros, stride 1.  The network (channels c1..c4, input channels padded to 16):

    e1 = G(conv(G(conv(x, c1)), c1))                       H x W
    e2 = G(conv(G(conv(pool(e1), c2)), c2))                H/2
    e3 = G(conv(G(conv(pool(e2), c3)), c3))                H/4
    e4 = G(conv(G(conv(pool(e3), c4)), c4))                H/8
    d3 = G(conv(G(conv([up(e4), e3], c3)), c3))            H/4
    d2 = G(conv(G(conv([up(d3), e2], c2)), c2))            H/2
    d1 = G(conv(G(conv([up(d2), e1], c1)), c1))            H x W
    out = conv(d1, 16);  prediction = x[..., :3] + out[..., :3]

G = GELU (tanh form), pool = 2x2 mean, up = nearest 2x, [a, b] = channel
concatenation.  Loss = sum over fluid pixels and the 3 predicted channels of
(prediction - target)^2 / (3 * fluid pixels).
"""
from __future__ import annotations

import numpy as np

GELU_C = np.sqrt(2.0 / np.pi)

# (name, input channels key, output channels key) in forward order; the keys
# are resolved against the level widths by layer_shapes()
LAYERS = ("enc1a", "enc1b", "enc2a", "enc2b", "enc3a", "enc3b", "enc4a", "enc4b",
          "dec3a", "dec3b", "dec2a", "dec2b", "dec1a", "dec1b", "out")


def layer_shapes(c=(32, 64, 128, 256), cin=16, cout=16):
    c1, c2, c3, c4 = c
    return {"enc1a": (cin, c1), "enc1b": (c1, c1), "enc2a": (c1, c2), "enc2b": (c2, c2),
            "enc3a": (c2, c3), "enc3b": (c3, c3), "enc4a": (c3, c4), "enc4b": (c4, c4),
            "dec3a": (c4 + c3, c3), "dec3b": (c3, c3), "dec2a": (c3 + c2, c2), "dec2b": (c2, c2),
            "dec1a": (c2 + c1, c1), "dec1b": (c1, c1), "out": (c1, cout)}


def gelu(z):
    return 0.5 * z * (1.0 + np.tanh(GELU_C * (z + 0.044715 * z ** 3)))


def gelu_grad(z):
    u = GELU_C * (z + 0.044715 * z ** 3)
    t = np.tanh(u)
    du = GELU_C * (1.0 + 3 * 0.044715 * z ** 2)
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * du


def _shift(x, dy, dx):
    """x[n, y + dy, x + dx, :] with zeros outside."""
    N, H, W, C = x.shape
    out = np.zeros_like(x)
    ys, yd = (slice(dy, H), slice(0, H - dy)) if dy >= 0 else (slice(0, H + dy), slice(-dy, H))
    xs, xd = (slice(dx, W), slice(0, W - dx)) if dx >= 0 else (slice(0, W + dx), slice(-dx, W))
    out[:, yd, xd, :] = x[:, ys, xs, :]
    return out


def conv3x3(x, w, b=None):
    """out[n,y,x,co] = sum_{ky,kx,ci} x[n, y+ky-1, x+kx-1, ci] w[co,ky,kx,ci] (+ b[co])."""
    out = np.zeros(x.shape[:3] + (w.shape[0],))
    for ky in range(3):
        for kx in range(3):
            out += _shift(x, ky - 1, kx - 1) @ w[:, ky, kx, :].T
    if b is not None:
        out += b
    return out


def conv3x3_dgrad(dz, w):
    dx = np.zeros(dz.shape[:3] + (w.shape[3],))
    for ky in range(3):
        for kx in range(3):
            dx += _shift(dz @ w[:, ky, kx, :], 1 - ky, 1 - kx)
    return dx


def conv3x3_wgrad(x, dz):
    Co, Ci = dz.shape[3], x.shape[3]
    dw = np.zeros((Co, 3, 3, Ci))
    dzf = dz.reshape(-1, Co)
    for ky in range(3):
        for kx in range(3):
            dw[:, ky, kx, :] = dzf.T @ _shift(x, ky - 1, kx - 1).reshape(-1, Ci)
    return dw


def pool(x):
    N, H, W, C = x.shape
    return x.reshape(N, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4))


def pool_grad(dy):
    return np.repeat(np.repeat(dy, 2, axis=1), 2, axis=2) * 0.25


def up(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up_grad(dy):
    N, H, W, C = dy.shape
    return dy.reshape(N, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def init_params(c=(32, 64, 128, 256), seed=0, cin=16, cout=16):
    """He-style initialisation; the output layer starts at zero (so the
    initial network predicts no change)."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, (ci, co) in layer_shapes(c, cin, cout).items():
        std = np.sqrt(2.0 / (9 * ci))
        p[name + ".w"] = rng.normal(0.0, std, (co, 3, 3, ci)) * (0.0 if name == "out" else 1.0)
        p[name + ".b"] = np.zeros(co)
    return p


def forward(p, x):
    """Returns (prediction (N,H,W,3), cache)."""
    cache = {"x": x}

    def block(name, inp):
        z = conv3x3(inp, p[name + ".w"], p[name + ".b"])
        cache[name] = (inp, z)
        return gelu(z)

    e1 = block("enc1b", block("enc1a", x))
    e2 = block("enc2b", block("enc2a", pool(e1)))
    e3 = block("enc3b", block("enc3a", pool(e2)))
    e4 = block("enc4b", block("enc4a", pool(e3)))
    d3 = block("dec3b", block("dec3a", np.concatenate([up(e4), e3], axis=3)))
    d2 = block("dec2b", block("dec2a", np.concatenate([up(d3), e2], axis=3)))
    d1 = block("dec1b", block("dec1a", np.concatenate([up(d2), e1], axis=3)))
    out = conv3x3(d1, p["out.w"], p["out.b"])
    cache["out"] = (d1, out)
    cache["widths"] = (e1.shape[3], e2.shape[3], e3.shape[3], e4.shape[3])
    return x[..., :3] + out[..., :3], cache


def loss_and_grad_out(pred, target, fluid):
    """Masked mean squared error and its gradient w.r.t. the prediction."""
    m = fluid[..., None].astype(np.float64)
    n = 3.0 * max(float(m.sum()), 1.0)
    d = (pred - target) * m
    return float(np.sum(d * d) / n), 2.0 * d / n


def backward(p, cache, dpred):
    """Gradients of the loss w.r.t. every parameter, given dL/dprediction."""
    g = {}
    c1, c2, c3, c4 = cache["widths"]
    N, H, W, _ = dpred.shape
    dout = np.zeros((N, H, W, p["out.w"].shape[0]))
    dout[..., :3] = dpred
    d1, _ = cache["out"]
    g["out.w"] = conv3x3_wgrad(d1, dout)
    g["out.b"] = dout.sum(axis=(0, 1, 2))
    dd1 = conv3x3_dgrad(dout, p["out.w"])

    def block_back(name, dy):
        inp, z = cache[name]
        dz = dy * gelu_grad(z)
        g[name + ".w"] = conv3x3_wgrad(inp, dz)
        g[name + ".b"] = dz.sum(axis=(0, 1, 2))
        return conv3x3_dgrad(dz, p[name + ".w"])

    du1 = block_back("dec1a", block_back("dec1b", dd1))
    dd2, de1 = up_grad(du1[..., :c2]), du1[..., c2:]
    du2 = block_back("dec2a", block_back("dec2b", dd2))
    dd3, de2 = up_grad(du2[..., :c3]), du2[..., c3:]
    du3 = block_back("dec3a", block_back("dec3b", dd3))
    de4, de3 = up_grad(du3[..., :c4]), du3[..., c4:]
    dp3 = block_back("enc4a", block_back("enc4b", de4))
    de3 = de3 + pool_grad(dp3)
    dp2 = block_back("enc3a", block_back("enc3b", de3))
    de2 = de2 + pool_grad(dp2)
    dp1 = block_back("enc2a", block_back("enc2b", de2))
    de1 = de1 + pool_grad(dp1)
    block_back("enc1a", block_back("enc1b", de1))
    return g


def adamw_step(w, g, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8, wd=1e-2):
    """Decoupled weight decay Adam (Loshchilov & Hutter), in place; step >= 1."""
    m[...] = b1 * m + (1 - b1) * g
    v[...] = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    w[...] = w - lr * (mh / (np.sqrt(vh) + eps) + wd * w)
