"""The surrogate's CPU oracle (oracle/unet_oracle.py) pinned by finite
differences: its analytic gradients equal central differences of its loss."""
import numpy as np

from oracle import unet_oracle as U


def _setup(seed=0):
    rng = np.random.default_rng(seed)
    c = (3, 4, 5, 6)
    p = U.init_params(c, seed=seed, cin=4, cout=4)
    p["out.w"] = rng.normal(0, 0.1, p["out.w"].shape)  # non-zero so every path carries gradient
    for k in p:
        if k.endswith(".b"):
            p[k] = rng.normal(0, 0.1, p[k].shape)
    x = rng.normal(0, 1, (2, 8, 16, 4))
    t = rng.normal(0, 1, (2, 8, 16, 3))
    fluid = rng.random((2, 8, 16)) > 0.2
    return p, x, t, fluid


def _loss(p, x, t, fluid):
    pred, _ = U.forward(p, x)
    return U.loss_and_grad_out(pred, t, fluid)[0]


def test_gradients_match_finite_differences():
    p, x, t, fluid = _setup()
    pred, cache = U.forward(p, x)
    _, dpred = U.loss_and_grad_out(pred, t, fluid)
    g = U.backward(p, cache, dpred)
    rng = np.random.default_rng(1)
    h = 1e-6
    for name in U.LAYERS:
        for suffix in (".w", ".b"):
            k = name + suffix
            for _ in range(3):
                idx = tuple(rng.integers(0, s) for s in p[k].shape)
                old = p[k][idx]
                p[k][idx] = old + h
                lp = _loss(p, x, t, fluid)
                p[k][idx] = old - h
                lm = _loss(p, x, t, fluid)
                p[k][idx] = old
                fd = (lp - lm) / (2 * h)
                assert abs(fd - g[k][idx]) <= 1e-6 + 1e-5 * abs(fd), (k, idx, fd, g[k][idx])


def test_conv_dgrad_is_adjoint():
    rng = np.random.default_rng(3)
    x = rng.normal(size=(2, 5, 7, 3))
    w = rng.normal(size=(4, 3, 3, 3))
    dz = rng.normal(size=(2, 5, 7, 4))
    # <conv(x), dz> == <x, dgrad(dz)> and == <w, wgrad(x, dz)>
    lhs = np.sum(U.conv3x3(x, w) * dz)
    assert np.isclose(lhs, np.sum(x * U.conv3x3_dgrad(dz, w)))
    assert np.isclose(lhs, np.sum(w * U.conv3x3_wgrad(x, dz)))


def test_zero_output_layer_predicts_persistence():
    p = U.init_params((4, 4, 4, 4), seed=0, cin=4, cout=4)
    x = np.random.default_rng(0).normal(size=(1, 8, 8, 4))
    pred, _ = U.forward(p, x)
    assert np.array_equal(pred, x[..., :3])
