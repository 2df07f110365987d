"""Learned surrogate: its CUDA kernels against the numpy oracle
(oracle/unet_oracle.py), the whole network's gradients against the oracle's,
and training on batched-LBM trajectories beating persistence on held-out
geometries."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

from oracle import unet_oracle as U  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from fingering_dynamics_gb300 import build
    build.build()


def _bf(a):
    """Round to bfloat16 (as numpy float64) and the device tensor."""
    t = torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(torch.bfloat16)
    return t.float().double().numpy(), t.cuda()


def _call(name, *args):
    from fingering_dynamics_gb300 import _lib as L
    L.call(name, *args)


def _p(t):
    import ctypes as C
    return C.c_void_p(t.data_ptr()) if t is not None else None


@pytest.mark.parametrize("cin,cout,act", [(16, 32, 1), (32, 16, 0), (48, 64, 1), (64, 96, 0), (96, 32, 1)])
def test_conv_forward_matches_oracle(cin, cout, act):
    rng = np.random.default_rng(cin + cout)
    N, H, W = 2, 8, 24
    xh, x = _bf(rng.normal(size=(N, H, W, cin)))
    wh, w = _bf(rng.normal(0, 0.2, size=(cout, 3, 3, cin)))
    b = rng.normal(0, 0.1, cout).astype(np.float32)
    bd = torch.from_numpy(b).cuda()
    z = torch.empty((N, H, W, cout), dtype=torch.bfloat16, device="cuda")
    y = torch.empty_like(z)
    _call("sg_conv3x3", _p(x), N, H, W, cin, _p(w), _p(bd), cout, act, _p(z), _p(y), None)
    torch.cuda.synchronize()
    zr = U.conv3x3(xh, wh, b.astype(np.float64))
    yr = U.gelu(zr) if act else zr
    scale = np.abs(zr).max()
    assert np.abs(z.float().cpu().numpy() - zr).max() <= 1e-2 * scale
    assert np.abs(y.float().cpu().numpy() - yr).max() <= 1e-2 * scale


@pytest.mark.parametrize("n,h,w,cin,cout,splits", [(2, 3, 128, 16, 32, 0), (1, 4, 128, 32, 16, 0),
                                                   (1, 2, 256, 64, 64, 0), (2, 2, 128, 96, 32, 3),
                                                   (1, 3, 128, 128, 144, 0), (1, 2, 128, 384, 128, 5),
                                                   (1, 2, 128, 32, 32, 7), (1, 2, 128, 64, 96, 0)])
def test_tcgen05_weight_gradient_matches_oracle(n, h, w, cin, cout, splits):
    """The tcgen05 weight gradient (MN-major operand boxes, one kernel row of
    taps per CTA, FP32 partials added in a fixed order) against the oracle and
    against the warp-level kernel; covers both assignments of M (output
    channels, input channels), tiles that end inside the 128 rows (144 = 128 +
    16, 96), 16 to 128 channels on N and more splits than chunks."""
    rng = np.random.default_rng(11 + cin + cout)
    xh, x = _bf(rng.normal(size=(n, h, w, cin)))
    dzh, dz = _bf(rng.normal(size=(n, h, w, cout)))
    from fingering_dynamics_gb300 import _lib as L
    nparts = max(int(L.lib().sg_wgrad_partial_floats(n, h, w, cin, cout)), 8 * cout * 9 * cin)
    part = torch.empty(nparts, dtype=torch.float32, device="cuda")
    dw = torch.empty((cout, 3, 3, cin), dtype=torch.float32, device="cuda")
    dw2 = torch.empty_like(dw)
    _call("sg_conv3x3_wgrad_tc", _p(x), _p(dz), n, h, w, cin, cout, _p(dw), _p(part), part.numel(), splits, None)
    _call("sg_conv3x3_wgrad", _p(x), _p(dz), n, h, w, cin, cout, _p(dw2), _p(part), part.numel(), 0, None)
    torch.cuda.synchronize()
    assert _tc_status() == 0
    dwr = U.conv3x3_wgrad(xh, dzh)
    scale = np.abs(dwr).max()
    assert np.abs(dw.cpu().numpy() - dwr).max() <= 1e-4 * scale
    assert np.abs(dw.cpu().numpy() - dw2.cpu().numpy()).max() <= 1e-4 * scale


@pytest.mark.parametrize("cin,cout", [(16, 32), (32, 16), (64, 64), (96, 32)])
def test_conv_gradients_match_oracle(cin, cout):
    """Weight gradient (FP32, deterministic split-K) and data gradient (the
    forward kernel on flipped weights)."""
    rng = np.random.default_rng(7 + cin)
    N, H, W = 2, 8, 40
    xh, x = _bf(rng.normal(size=(N, H, W, cin)))
    dzh, dz = _bf(rng.normal(size=(N, H, W, cout)))
    wh, w = _bf(rng.normal(0, 0.2, size=(cout, 3, 3, cin)))
    from fingering_dynamics_gb300 import _lib as L
    nparts = L.lib().sg_wgrad_partial_floats(N, H, W, cin, cout)
    part = torch.empty(max(int(nparts), 4 * cout * 9 * cin), dtype=torch.float32, device="cuda")
    dw = torch.empty((cout, 3, 3, cin), dtype=torch.float32, device="cuda")
    dw2 = torch.empty_like(dw)
    _call("sg_conv3x3_wgrad", _p(x), _p(dz), N, H, W, cin, cout, _p(dw), _p(part), part.numel(), 0, None)
    _call("sg_conv3x3_wgrad", _p(x), _p(dz), N, H, W, cin, cout, _p(dw2), _p(part), part.numel(), 3, None)
    wt = torch.empty((cin, 3, 3, cout), dtype=torch.bfloat16, device="cuda")
    _call("sg_flip_weights", _p(w), cin, cout, _p(wt), None)
    dx = torch.empty((N, H, W, cin), dtype=torch.bfloat16, device="cuda")
    _call("sg_conv3x3", _p(dz), N, H, W, cout, _p(wt), None, cin, 0, None, _p(dx), None)
    torch.cuda.synchronize()
    dwr = U.conv3x3_wgrad(xh, dzh)
    assert np.abs(dw.cpu().numpy() - dwr).max() <= 1e-4 * np.abs(dwr).max()
    assert np.abs(dw2.cpu().numpy() - dwr).max() <= 1e-4 * np.abs(dwr).max()
    dxr = U.conv3x3_dgrad(dzh, wh)
    assert np.abs(dx.float().cpu().numpy() - dxr).max() <= 1e-2 * np.abs(dxr).max()


@pytest.mark.parametrize("conv,W", [("auto", 32), ("tma", 128), ("tma_ws", 128)])
def test_network_gradients_match_oracle(conv, W):
    """Loss and every layer's gradients against the oracle; with conv="tma"
    the forward and data-gradient convolutions of the full-width level run on
    the TMA-fed kernel (the narrower levels fall back to the tcgen05 one)."""
    from fingering_dynamics_gb300.surrogate import UNet
    widths = (16, 16, 32, 32)
    net = UNet(widths, seed=3, conv=conv)
    rng = np.random.default_rng(5)
    # a non-zero output layer so that every layer carries gradient
    net.w["out"] = torch.from_numpy(rng.normal(0, 0.05, net.w["out"].shape).astype(np.float32)).cuda()
    for n in net.b:
        net.b[n] = torch.from_numpy(rng.normal(0, 0.05, net.b[n].shape).astype(np.float32)).cuda()
    net.w16 = {n: t.to(torch.bfloat16) for n, t in net.w.items()}
    N, H = 2, 16
    x = rng.normal(size=(N, H, W, 16))
    x[..., 3] = (rng.random((N, H, W)) < 0.2)
    x[..., 4:] = 0
    xn = x.copy()
    xn[..., :3] += rng.normal(0, 0.3, size=(N, H, W, 3))
    xh, xd = _bf(x)
    xnh, xnd = _bf(xn)
    loss = net.loss_grad(xd.contiguous(), xnd.contiguous())
    torch.cuda.synchronize()
    params = {}
    for n in net.w:
        params[n + ".w"] = net.w16[n].float().double().cpu().numpy()
        params[n + ".b"] = net.b[n].double().cpu().numpy()
    pred, cache = U.forward(params, xh)
    lref, dpred = U.loss_and_grad_out(pred, xnh[..., :3], xh[..., 3] == 0)
    g = U.backward(params, cache, dpred)
    assert abs(float(loss) - lref) <= 2e-2 * lref
    for n in net.w:
        for got, ref in ((net.gw[n].double().cpu().numpy(), g[n + ".w"]), (net.gb[n].double().cpu().numpy(),
                                                                           g[n + ".b"])):
            err = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-30)
            cos = float(np.sum(got * ref) / max(np.linalg.norm(got) * np.linalg.norm(ref), 1e-30))
            assert err <= 6e-2 and cos >= 0.998, (n, err, cos)


def test_adamw_matches_oracle():
    from fingering_dynamics_gb300 import _lib as L  # noqa: F401
    rng = np.random.default_rng(1)
    n = 1000
    w = rng.normal(size=n)
    m = np.zeros(n)
    v = np.zeros(n)
    wd, md, vd = (torch.from_numpy(a.astype(np.float32)).cuda() for a in (w, m, v))
    w16 = torch.empty(n, dtype=torch.bfloat16, device="cuda")
    for step in range(1, 4):
        g = rng.normal(size=n)
        gd = torch.from_numpy(g.astype(np.float32)).cuda()
        _call("sg_adamw", _p(wd), _p(w16), _p(gd), _p(md), _p(vd), n, 1e-3, 0.9, 0.999, 1e-8, 1e-2, step, None)
        U.adamw_step(w, g.astype(np.float32).astype(np.float64), m, v, step)
    torch.cuda.synchronize()
    assert np.abs(wd.double().cpu().numpy() - w).max() <= 1e-6
    assert torch.equal(w16, wd.to(torch.bfloat16))


def test_training_beats_persistence_on_held_out_geometries():
    """Trajectories of a small batched ensemble (jump of 100 iterations);
    members 0..5 train, 6..7 (other geometries) evaluate."""
    from fingering_dynamics_gb300.ensemble import ensemble_specs
    from fingering_dynamics_gb300.surrogate import UNet, evaluate, generate_trajectories, train
    specs = ensemble_specs(8, seed=11, sizes_w=(128,), sizes_h=(64,))
    frames, finite = generate_trajectories(specs, n_frames=8, jump=100)
    assert bool(finite.all())
    net = UNet((16, 32, 32, 64), seed=0)
    before = evaluate(net, frames[6:])
    assert abs(before["gain"] - 1.0) < 1e-6           # zero output layer: persistence
    hist = train(net, frames[:6], steps=150, batch=8, lr=2e-3, log_every=50)
    after = evaluate(net, frames[6:])
    assert hist[-1][1] < hist[0][1]
    assert after["gain"] > 1.0, after                 # the network beats "no change" on unseen geometries


def test_rollout_judge_accepts_or_falls_back():
    from fingering_dynamics_gb300.ensemble import ensemble_specs
    from fingering_dynamics_gb300.lattice import Lattice
    from fingering_dynamics_gb300.surrogate import UNet, rollout
    prm, g = ensemble_specs(1, seed=4, sizes_w=(128,), sizes_h=(64,))[0].build()
    lat = Lattice(prm, g, dtype="f32")
    lat.step(200)
    net = UNet((16, 32, 32, 64), seed=0)   # untrained: persistence
    recs = rollout(net, lat, jumps_per_check=2, checks=2, jump=50, tol=0.02)
    assert len(recs) == 2
    assert lat.iteration == 200 + 2 * 3 * 50
    assert bool(torch.isfinite(lat.psi).all())
    for r in recs:
        assert r["accepted"] == (abs(r["sat_lbm"] - r["sat_surrogate"]) <= 0.02 * r["sat_lbm"])


def _tc_status(clear=True):
    import ctypes as C
    from fingering_dynamics_gb300 import _lib as L
    v = C.c_uint(0)
    L.call("sg_tc_status", C.byref(v), int(clear))
    return v.value


@pytest.mark.parametrize("n,h,w,cin,cout,act", [(1, 8, 16, 16, 16, 0), (2, 8, 40, 32, 32, 1), (2, 16, 24, 64, 64, 1),
                                                (1, 8, 16, 96, 32, 0), (2, 8, 32, 256, 128, 1),
                                                # widths that are multiples of 128: the halo-tile kernel
                                                (1, 4, 128, 16, 32, 1), (2, 3, 128, 32, 64, 0),
                                                (1, 2, 256, 64, 64, 1), (1, 3, 128, 96, 32, 1),
                                                (1, 2, 128, 16, 16, 0)])
def test_tcgen05_conv_matches_oracle(n, h, w, cin, cout, act):
    """The tcgen05 / TMEM convolution against the oracle and against the
    warp-level tensor-core kernel (same inputs; both accumulate in FP32)."""
    rng = np.random.default_rng(cin * 7 + cout)
    xh, x = _bf(rng.normal(size=(n, h, w, cin)))
    wh, wt = _bf(rng.normal(0, 0.2, size=(cout, 3, 3, cin)))
    b = rng.normal(0, 0.1, cout).astype(np.float32)
    bd = torch.from_numpy(b).cuda()
    outs = {}
    for name in ("sg_conv3x3_tc", "sg_conv3x3"):
        z = torch.zeros((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
        y = torch.zeros_like(z)
        _call(name, _p(x), n, h, w, cin, _p(wt), _p(bd), cout, act, _p(z), _p(y), None)
        torch.cuda.synchronize()
        outs[name] = (z.float().cpu().numpy(), y.float().cpu().numpy())
    assert _tc_status() == 0
    zr = U.conv3x3(xh, wh, b.astype(np.float64))
    yr = U.gelu(zr) if act else zr
    scale = np.abs(zr).max()
    ztc, ytc = outs["sg_conv3x3_tc"]
    assert np.abs(ztc - zr).max() <= 1e-2 * scale
    assert np.abs(ytc - yr).max() <= 1e-2 * scale
    # the two tensor-core paths round their FP32 sums to the same bfloat16 almost everywhere
    assert np.mean(ztc != outs["sg_conv3x3"][0]) < 0.02


@pytest.mark.parametrize("n,h,w,cin,cout,act", [(1, 4, 128, 16, 32, 1), (2, 3, 128, 32, 64, 0), (1, 2, 256, 64, 64, 1),
                                                (1, 3, 128, 96, 32, 1), (1, 2, 128, 16, 16, 0),
                                                (2, 4, 128, 128, 128, 1), (1, 8, 256, 384, 128, 0),
                                                (1, 4, 256, 32, 96, 1)])
@pytest.mark.parametrize("kernel", ["sg_conv3x3_tma", "sg_conv3x3_tma_ws"])
def test_tma_conv_matches_oracle(kernel, n, h, w, cin, cout, act):
    """The TMA-fed tcgen05 convolution (tensor-map boxes into a ring of
    stages, zero fill as the padding) against the oracle and against the
    halo-tile tcgen05 kernel; covers 1, 2 and 4 rows per tile, 2, 3 and 4
    stages, and 16 to 128 output channels per tile."""
    rng = np.random.default_rng(cin * 11 + cout + h)
    xh, x = _bf(rng.normal(size=(n, h, w, cin)))
    wh, wt = _bf(rng.normal(0, 0.2, size=(cout, 3, 3, cin)))
    b = rng.normal(0, 0.1, cout).astype(np.float32)
    bd = torch.from_numpy(b).cuda()
    outs = {}
    for name in (kernel, "sg_conv3x3_tc"):
        z = torch.zeros((n, h, w, cout), dtype=torch.bfloat16, device="cuda")
        y = torch.zeros_like(z)
        _call(name, _p(x), n, h, w, cin, _p(wt), _p(bd), cout, act, _p(z), _p(y), None)
        torch.cuda.synchronize()
        outs[name] = (z.float().cpu().numpy(), y.float().cpu().numpy())
    assert _tc_status() == 0
    zr = U.conv3x3(xh, wh, b.astype(np.float64))
    yr = U.gelu(zr) if act else zr
    scale = np.abs(zr).max()
    zt, yt = outs[kernel]
    assert np.abs(zt - zr).max() <= 1e-2 * scale
    assert np.abs(yt - yr).max() <= 1e-2 * scale
    # the same products summed in another order: the bfloat16 results agree almost everywhere
    assert np.mean(zt != outs["sg_conv3x3_tc"][0]) < 0.05


def test_accelerated_ensemble_runs_to_the_horizon():
    """The accelerated ensemble (batched jumps, batched LBM judge, exact
    restore and plain fallback) reaches the same iteration as the plain
    batched run, with finite states; an untrained network (persistence) is
    mostly rejected by the judge."""
    from fingering_dynamics_gb300.ensemble import ensemble_specs
    from fingering_dynamics_gb300.surrogate import UNet, accelerated_ensemble
    members = [s.build() for s in ensemble_specs(4, seed=21, sizes_w=(128,), sizes_h=(64,))]
    net = UNet((16, 32, 32, 64), seed=0)
    r = accelerated_ensemble(net, members, rounds=2, jumps_per_check=2, jump=50)
    assert r["horizon_iterations"] == 2 * 3 * 50
    assert r["member_rounds"] == 8 and 0 <= r["accepted_rounds"] <= 8
    assert np.isfinite(r["final_saturation_rel_error_mean"]) and r["plain_s"] > 0 and r["accelerated_s"] > 0
