"""Learned surrogate: a convolutional U-Net that advances (psi, u_x, u_y) by a
fixed number of lattice steps (a "jump") given the solid mask, trained on
trajectories of the batched LBM with this package's own CUDA kernels
(include/fdsurrogate.h: tensor-core implicit-GEMM convolutions, forward and
data gradient on tcgen05 with the accumulator in tensor memory or on
warp-level MMA, whichever is faster for the shape, weight gradient on
warp-level MMA, and the training elementwise kernels), and a rollout
driver that uses the plain LBM as its judge and fallback.

The reference has no learned component.  Network (widths c1..c4, 3x3 convs,
GELU, 2x2 mean pooling, nearest upsampling, skip concatenation):

    e1 = G(conv(G(conv(x, c1)), c1))                       H x W
    e2 = G(conv(G(conv(pool(e1), c2)), c2))                H/2
    e3 = G(conv(G(conv(pool(e2), c3)), c3))                H/4
    e4 = G(conv(G(conv(pool(e3), c4)), c4))                H/8
    d3 = G(conv(G(conv([up(e4), e3], c3)), c3))            H/4
    d2 = G(conv(G(conv([up(d3), e2], c2)), c2))            H/2
    d1 = G(conv(G(conv([up(d2), e1], c1)), c1))            H x W
    out = conv(d1, 16);  prediction = x[..., :3] + out[..., :3]

A frame is NHWC bfloat16 with 16 channels: psi, u_x / U, u_y / U, solid (1 on
solid cells), zeros; U = ``VELOCITY_SCALE``.  The output layer starts at
zero, so the untrained network predicts "no change" (persistence).
"""
from __future__ import annotations

import ctypes as C
import math
import time

import numpy as np
import torch

from . import _lib as L

VELOCITY_SCALE = 0.01
FRAME_CHANNELS = 16
LAYERS = ("enc1a", "enc1b", "enc2a", "enc2b", "enc3a", "enc3b", "enc4a", "enc4b",
          "dec3a", "dec3b", "dec2a", "dec2b", "dec1a", "dec1b", "out")


def layer_shapes(c=(32, 64, 128, 256), cin=FRAME_CHANNELS, cout=FRAME_CHANNELS):
    c1, c2, c3, c4 = c
    return {"enc1a": (cin, c1), "enc1b": (c1, c1), "enc2a": (c1, c2), "enc2b": (c2, c2),
            "enc3a": (c2, c3), "enc3b": (c3, c3), "enc4a": (c3, c4), "enc4b": (c4, c4),
            "dec3a": (c4 + c3, c3), "dec3b": (c3, c3), "dec2a": (c3 + c2, c2), "dec2b": (c2, c2),
            "dec1a": (c2 + c1, c1), "dec1b": (c1, c1), "out": (c1, cout)}


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _s():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def frame_from_fields(psi, ux, uy, solid) -> torch.Tensor:
    """(H, W) device tensors -> one frame (H, W, 16) bfloat16."""
    H, W = psi.shape
    fr = torch.zeros((H, W, FRAME_CHANNELS), dtype=torch.float32, device=psi.device)
    fl = ~solid
    fr[..., 0] = psi.float()
    fr[..., 1] = torch.where(fl, ux.float(), 0) / VELOCITY_SCALE
    fr[..., 2] = torch.where(fl, uy.float(), 0) / VELOCITY_SCALE
    fr[..., 3] = solid.float()
    return fr.to(torch.bfloat16)


def expand(frames4: torch.Tensor) -> torch.Tensor:
    """Frames stored with their 4 live channels -> the network's 16 channels."""
    return torch.nn.functional.pad(frames4, (0, FRAME_CHANNELS - frames4.shape[-1])).contiguous()


def fields_from_frame(fr: torch.Tensor):
    """One frame -> (psi, ux, uy) float32 (H, W) tensors."""
    f = fr.float()
    return f[..., 0], f[..., 1] * VELOCITY_SCALE, f[..., 2] * VELOCITY_SCALE


class UNet:
    """The network, its FP32 master weights, bfloat16 copies, AdamW moments and
    activation buffers (allocated per batch shape)."""

    def __init__(self, widths=(32, 64, 128, 256), seed: int = 0, device="cuda", params: dict | None = None,
                 conv: str = "auto"):
        """``conv`` selects the forward and data-gradient convolution kernel:
        "tcgen05" (fifth-generation tensor cores, accumulator in tensor
        memory), "tma" (the same fed by tensor-map boxes from one thread;
        images whose width is a multiple of 128, the others fall back to
        "tcgen05"), "tma_ws" (its persistent warp-specialised form, same
        shapes), "mma" (warp-level tensor-core instructions) or "auto" (all
        that take the shape timed once per convolution shape at first use, the
        fastest kept).  The weight gradient runs on the tcgen05 kernel at widths
        that are multiples of 128 for every choice but "mma" ("auto": the faster
        of the two per shape), else on the warp-level kernel."""
        if conv not in ("tcgen05", "tma", "tma_ws", "mma", "auto"):
            raise ValueError("conv must be 'tcgen05', 'tma', 'tma_ws', 'mma' or 'auto'")
        self.conv = conv
        self.conv_choice = {}  # (N, H, W, Cin, Cout) -> kernel name, filled by "auto"
        self.widths = tuple(widths)
        self.shapes = layer_shapes(self.widths)
        self.device = torch.device(device)
        rng = np.random.default_rng(seed)
        self.w, self.b = {}, {}
        for name, (ci, co) in self.shapes.items():
            if params is not None:
                w = np.asarray(params[name + ".w"], np.float32)
                b = np.asarray(params[name + ".b"], np.float32)
            else:
                std = math.sqrt(2.0 / (9 * ci))
                w = (rng.normal(0.0, std, (co, 3, 3, ci)) * (0.0 if name == "out" else 1.0)).astype(np.float32)
                b = np.zeros(co, np.float32)
            self.w[name] = torch.from_numpy(w).to(self.device).contiguous()
            self.b[name] = torch.from_numpy(b).to(self.device).contiguous()
        self.w16 = {n: t.to(torch.bfloat16) for n, t in self.w.items()}
        self.wt16 = {n: torch.empty((ci, 3, 3, co), dtype=torch.bfloat16, device=self.device)
                     for n, (ci, co) in self.shapes.items()}
        self.gw = {n: torch.zeros_like(t) for n, t in self.w.items()}
        self.gb = {n: torch.zeros_like(t) for n, t in self.b.items()}
        self.mw = {n: torch.zeros_like(t) for n, t in self.w.items()}
        self.vw = {n: torch.zeros_like(t) for n, t in self.w.items()}
        self.mb = {n: torch.zeros_like(t) for n, t in self.b.items()}
        self.vb = {n: torch.zeros_like(t) for n, t in self.b.items()}
        self.steps = 0
        self._buf = {}
        self._flipped = False

    @property
    def n_params(self) -> int:
        return sum(t.numel() for t in self.w.values()) + sum(t.numel() for t in self.b.values())

    def flops_forward(self, N, H, W) -> float:
        """Multiply-adds x 2 of the convolutions of one forward pass."""
        f, lvl = 0.0, {"1": 1, "2": 2, "3": 4, "4": 8}
        for name, (ci, co) in self.shapes.items():
            d = 1 if name == "out" else lvl[name[3]]
            f += 2.0 * 9 * ci * co * N * (H // d) * (W // d)
        return f

    def state_dict(self) -> dict:
        out = {}
        for n in LAYERS:
            out[n + ".w"] = self.w[n].cpu().numpy()
            out[n + ".b"] = self.b[n].cpu().numpy()
        return out

    # ------------------------------------------------------------------
    def _buffers(self, N, H, W):
        key = (N, H, W)
        if key in self._buf:
            return self._buf[key]
        if H % 8 or W % 8:
            raise ValueError("frame height and width must be multiples of 8")
        c1, c2, c3, c4 = self.widths
        dev, bf = self.device, torch.bfloat16
        lv = {1: (H, W), 2: (H // 2, W // 2), 3: (H // 4, W // 4), 4: (H // 8, W // 8)}

        def t(level, ch):
            h, w = lv[level]
            return torch.empty((N, h, w, ch), dtype=bf, device=dev)

        level = {"enc1a": 1, "enc1b": 1, "enc2a": 2, "enc2b": 2, "enc3a": 3, "enc3b": 3, "enc4a": 4, "enc4b": 4,
                 "dec3a": 3, "dec3b": 3, "dec2a": 2, "dec2b": 2, "dec1a": 1, "dec1b": 1, "out": 1}
        B = {"level": level, "lv": lv}
        for name, (ci, co) in self.shapes.items():
            B["z." + name] = t(level[name], co)
            B["y." + name] = t(level[name], co)
            B["dy." + name] = t(level[name], co)
            B["dz." + name] = t(level[name], co)
            B["dx." + name] = t(level[name], ci)
        B["p1"], B["p2"], B["p3"] = t(2, c1), t(3, c2), t(4, c3)
        B["u3"], B["u2"], B["u1"] = t(3, c4 + c3), t(2, c3 + c2), t(1, c2 + c1)
        B["de1"], B["de2"], B["de3"] = t(1, c1), t(2, c2), t(3, c3)
        wp = max(L.lib().sg_wgrad_partial_floats(N, *lv[level[n]], ci, co) for n, (ci, co) in self.shapes.items())
        B["wpart"] = torch.empty(int(wp), dtype=torch.float32, device=dev)
        B["bpart"] = torch.empty(int(L.lib().sg_bias_partial_floats(max(c1, c2, c3, c4, FRAME_CHANNELS))),
                                 dtype=torch.float32, device=dev)
        B["lpart"] = torch.empty(2 * L.lib().sg_loss_blocks(), dtype=torch.float32, device=dev)
        self._buf[key] = B
        return B

    _KERNELS = {"mma": "sg_conv3x3", "tcgen05": "sg_conv3x3_tc", "tma": "sg_conv3x3_tma",
                "tma_ws": "sg_conv3x3_tma_ws"}

    @staticmethod
    def _takes(kernel, w, ci, co):
        """Whether a kernel takes the shape (the TMA-fed ones: widths that are
        multiples of 128, channel counts that are multiples of 16)."""
        return not kernel.startswith("tma") or (w % 128 == 0 and ci % 16 == 0 and co % 16 == 0)

    def _run_conv(self, x, N, h, w, ci, wt, bias, co, act, z, y):
        """One 3x3 convolution with the kernel chosen for its shape."""
        key = (N, h, w, ci, co)
        args = (_p(x), N, h, w, ci, _p(wt), _p(bias), co, act, _p(z), _p(y), _s())
        if self.conv != "auto":
            k = self.conv if self._takes(self.conv, w, ci, co) else "tcgen05"
            fn = self._KERNELS[k]
        elif key in self.conv_choice:
            fn = self.conv_choice[key]
        else:  # time each kernel that takes the shape once on the real operands; the last call's result stands
            best = None
            for k, fn in self._KERNELS.items():
                if not self._takes(k, w, ci, co):
                    continue
                L.call(fn, *args)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(2):
                    L.call(fn, *args)
                e1.record()
                e1.synchronize()
                t = e0.elapsed_time(e1)
                if best is None or t < best[0]:
                    best = (t, fn)
            fn = self.conv_choice[key] = best[1]
        L.call(fn, *args)

    _WGRAD = {"mma": "sg_conv3x3_wgrad", "tcgen05": "sg_conv3x3_wgrad_tc"}

    def _run_wgrad(self, inp, dz, N, h, w, ci, co, gw, part):
        """Weight gradient of one layer: the tcgen05 kernel (widths that are
        multiples of 128) or the warp-level one; with conv="auto" both are timed
        once per shape and the faster kept (their FP32 sums differ in the last
        bits only)."""
        key = ("wgrad", N, h, w, ci, co)
        args = (_p(inp), _p(dz), N, h, w, ci, co, _p(gw), _p(part), part.numel(), 0, _s())
        ok_tc = w % 128 == 0
        if self.conv == "mma" or not ok_tc:
            fn = self._WGRAD["mma"]
        elif self.conv != "auto":
            fn = self._WGRAD["tcgen05"]
        elif key in self.conv_choice:
            fn = self.conv_choice[key]
        else:
            best = None
            for fn in self._WGRAD.values():
                L.call(fn, *args)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(2):
                    L.call(fn, *args)
                e1.record()
                e1.synchronize()
                t = e0.elapsed_time(e1)
                if best is None or t < best[0]:
                    best = (t, fn)
            fn = self.conv_choice[key] = best[1]
        L.call(fn, *args)

    def _conv(self, name, x, B, act=True):
        ci, co = self.shapes[name]
        N, h, w, c = x.shape
        assert c == ci, (name, c, ci)
        self._run_conv(x, N, h, w, ci, self.w16[name], self.b[name], co, 1 if act else 0,
                       B["z." + name] if act else None, B["y." + name])
        return B["y." + name]

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        """x: (N, H, W, 16) bfloat16 frames -> out (N, H, W, 16) bfloat16 (the
        prediction is x[..., :3] + out[..., :3])."""
        N, H, W, _ = x.shape
        B = self._buffers(N, H, W)
        c1, c2, c3, c4 = self.widths
        lv = B["lv"]
        s = _s()
        self._x = x
        e1 = self._conv("enc1b", self._conv("enc1a", x, B), B)
        L.call("sg_pool2", _p(e1), N, H, W, c1, _p(B["p1"]), s)
        e2 = self._conv("enc2b", self._conv("enc2a", B["p1"], B), B)
        L.call("sg_pool2", _p(e2), N, *lv[2], c2, _p(B["p2"]), s)
        e3 = self._conv("enc3b", self._conv("enc3a", B["p2"], B), B)
        L.call("sg_pool2", _p(e3), N, *lv[3], c3, _p(B["p3"]), s)
        e4 = self._conv("enc4b", self._conv("enc4a", B["p3"], B), B)
        L.call("sg_up2", _p(e4), N, *lv[4], c4, _p(B["u3"]), c4 + c3, 0, s)
        L.call("sg_copy_channels", _p(e3), N * lv[3][0] * lv[3][1], c3, _p(B["u3"]), c4 + c3, c4, s)
        d3 = self._conv("dec3b", self._conv("dec3a", B["u3"], B), B)
        L.call("sg_up2", _p(d3), N, *lv[3], c3, _p(B["u2"]), c3 + c2, 0, s)
        L.call("sg_copy_channels", _p(e2), N * lv[2][0] * lv[2][1], c2, _p(B["u2"]), c3 + c2, c3, s)
        d2 = self._conv("dec2b", self._conv("dec2a", B["u2"], B), B)
        L.call("sg_up2", _p(d2), N, *lv[2], c2, _p(B["u1"]), c2 + c1, 0, s)
        L.call("sg_copy_channels", _p(e1), N * H * W, c1, _p(B["u1"]), c2 + c1, c2, s)
        d1 = self._conv("dec1b", self._conv("dec1a", B["u1"], B), B)
        return self._conv("out", d1, B, act=False)

    def predict(self, x: torch.Tensor) -> torch.Tensor:
        """Frames one jump later: x[..., :3] + out[..., :3], other channels of x."""
        out = self.forward(x)
        y = x.clone()
        y[..., :3] = (x[..., :3].float() + out[..., :3].float()).to(torch.bfloat16)
        return y

    # ------------------------------------------------------------------
    def _flip_all(self):
        s = _s()
        for name, (ci, co) in self.shapes.items():
            L.call("sg_flip_weights", _p(self.w16[name]), ci, co, _p(self.wt16[name]), s)
        self._flipped = True

    def _layer_back(self, name, inp, dz, B, need_dx=True):
        """Weight / bias gradients of layer `name` from dz; returns dx."""
        ci, co = self.shapes[name]
        N, h, w, _ = inp.shape
        s = _s()
        self._run_wgrad(inp, dz, N, h, w, ci, co, self.gw[name], B["wpart"])
        L.call("sg_bias_grad", _p(dz), N * h * w, co, _p(self.gb[name]), _p(B["bpart"]), s)
        if not need_dx:
            return None
        dx = B["dx." + name]
        self._run_conv(dz, N, h, w, co, self.wt16[name], None, ci, 0, None, dx)
        return dx

    def _gelu_back(self, name, dy, B):
        dz = B["dz." + name]
        L.call("sg_gelu_bwd", _p(dy), _p(B["z." + name]), dy.numel(), _p(dz), _s())
        return dz

    def _block_back(self, name, inp, dy, B, need_dx=True):
        return self._layer_back(name, inp, self._gelu_back(name, dy, B), B, need_dx)

    def backward(self, dout: torch.Tensor):
        """Gradients (self.gw, self.gb) of the loss whose gradient w.r.t. the
        output of the last forward() is dout."""
        if not self._flipped:
            self._flip_all()
        x = self._x
        N, H, W, _ = x.shape
        B = self._buffers(N, H, W)
        lv = B["lv"]
        c1, c2, c3, c4 = self.widths
        s = _s()
        y = lambda n: B["y." + n]
        dd1 = self._layer_back("out", y("dec1b"), dout, B)
        du1 = self._block_back("dec1a", B["u1"], self._block_back("dec1b", y("dec1a"), dd1, B), B)
        dd2 = B["dy.dec2b"]
        L.call("sg_up2_bwd", _p(du1), N, *lv[2], c2 + c1, 0, c2, _p(dd2), s)
        du2 = self._block_back("dec2a", B["u2"], self._block_back("dec2b", y("dec2a"), dd2, B), B)
        dd3 = B["dy.dec3b"]
        L.call("sg_up2_bwd", _p(du2), N, *lv[3], c3 + c2, 0, c3, _p(dd3), s)
        du3 = self._block_back("dec3a", B["u3"], self._block_back("dec3b", y("dec3a"), dd3, B), B)
        de4 = B["dy.enc4b"]
        L.call("sg_up2_bwd", _p(du3), N, *lv[4], c4 + c3, 0, c4, _p(de4), s)
        dp3 = self._block_back("enc4a", B["p3"], self._block_back("enc4b", y("enc4a"), de4, B), B)
        de3 = B["de3"]
        L.call("sg_pool2_bwd", _p(dp3), N, *lv[3], c3, _p(de3), s)
        L.call("sg_add_channels", _p(du3), N * lv[3][0] * lv[3][1], c4 + c3, c4, c3, _p(de3), s)
        dp2 = self._block_back("enc3a", B["p2"], self._block_back("enc3b", y("enc3a"), de3, B), B)
        de2 = B["de2"]
        L.call("sg_pool2_bwd", _p(dp2), N, *lv[2], c2, _p(de2), s)
        L.call("sg_add_channels", _p(du2), N * lv[2][0] * lv[2][1], c3 + c2, c3, c2, _p(de2), s)
        dp1 = self._block_back("enc2a", B["p1"], self._block_back("enc2b", y("enc2a"), de2, B), B)
        de1 = B["de1"]
        L.call("sg_pool2_bwd", _p(dp1), N, H, W, c1, _p(de1), s)
        L.call("sg_add_channels", _p(du1), N * H * W, c2 + c1, c2, c1, _p(de1), s)
        self._block_back("enc1a", x, self._block_back("enc1b", y("enc1a"), de1, B), B, need_dx=False)

    def loss_grad(self, x: torch.Tensor, xn: torch.Tensor) -> torch.Tensor:
        """Forward, masked MSE of the prediction against xn, backward.
        Returns the loss as a 0-d device tensor (no host sync)."""
        N, H, W, Cc = x.shape
        out = self.forward(x)
        B = self._buffers(N, H, W)
        count = max(float((x[..., 3] == 0).sum().item()), 1.0)
        dout = B["dy.out"]
        L.call("sg_masked_mse", _p(x), _p(out), _p(xn), N * H * W, Cc, _p(dout), _p(B["lpart"]),
               C.c_float(1.0 / (3.0 * count)), _s())
        self.backward(dout)
        lp = B["lpart"].view(-1, 2)
        return lp[:, 0].sum() / (3.0 * count)

    def adamw(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=1e-2):
        self.steps += 1
        s = _s()
        for n in LAYERS:
            L.call("sg_adamw", _p(self.w[n]), _p(self.w16[n]), _p(self.gw[n]), _p(self.mw[n]), _p(self.vw[n]),
                   self.w[n].numel(), lr, beta1, beta2, eps, weight_decay, self.steps, s)
            L.call("sg_adamw", _p(self.b[n]), None, _p(self.gb[n]), _p(self.mb[n]), _p(self.vb[n]),
                   self.b[n].numel(), lr, beta1, beta2, eps, 0.0, self.steps, s)
        self._flipped = False


# ----------------------------------------------------------------------------
# data: trajectories of the batched LBM
# ----------------------------------------------------------------------------
def member_frame(lat) -> torch.Tensor:
    """Frame of the next iteration of a fused-mode lattice (Lattice.peek)."""
    lat.peek()
    return frame_from_fields(lat.psi, lat.ux, lat.uy, ~lat.fluid)


def generate_trajectories(specs, n_frames: int, jump: int = 200, dtype: str = "f32", warmup: int = 0):
    """Advance an ensemble of members (MemberSpec) with the batched LBM and
    record a frame of every member every `jump` iterations.  Returns frames
    (members, n_frames, H, W, 4) bfloat16 on the GPU (the four live channels;
    ``expand`` makes network inputs; all members share one lattice size) and
    the members' finite flags."""
    from .ensemble import Ensemble
    ens = Ensemble([s.build() for s in specs], dtype=dtype)
    if warmup:
        ens.step(warmup)
    H, W = ens.lattices[0].H, ens.lattices[0].W
    frames = torch.empty((len(specs), n_frames, H, W, 4), dtype=torch.bfloat16, device=ens.lattices[0].device)
    for k in range(n_frames):
        if k:
            ens.step(jump)
        torch.cuda.current_stream().wait_stream(ens.stream)
        for m, lat in enumerate(ens.lattices):
            frames[m, k] = member_frame(lat)[..., :4]
    # per member, in the storage type (an FP32 copy of every frame would double the footprint)
    finite = torch.stack([torch.isfinite(frames[m]).all() for m in range(len(specs))])
    ens.close()
    return frames, finite


def train(net: UNet, frames: torch.Tensor, steps: int, batch: int = 32, lr: float = 1e-3, seed: int = 0,
          log_every: int = 0, lr_end: float | None = None):
    """AdamW on random (frame k, frame k+1) pairs of `frames`
    (members, n_frames, H, W, 4); the learning rate follows a cosine from
    `lr` to `lr_end` (constant if None).  Returns the loss history (host
    floats)."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    M, F = frames.shape[:2]
    hist = []
    for it in range(steps):
        if lr_end is not None and steps > 1:
            rate = lr_end + 0.5 * (lr - lr_end) * (1.0 + math.cos(math.pi * it / (steps - 1)))
        else:
            rate = lr
        mi = torch.randint(0, M, (batch,), generator=g)
        fi = torch.randint(0, F - 1, (batch,), generator=g)
        x = expand(frames[mi, fi])
        xn = expand(frames[mi, fi + 1])
        loss = net.loss_grad(x, xn)
        net.adamw(lr=rate)
        if log_every and (it % log_every == 0 or it == steps - 1):
            hist.append((it, float(loss.item())))
    return hist


def evaluate(net: UNet, frames: torch.Tensor, batch: int = 16) -> dict:
    """Masked MSE of the network and of persistence (no change) over every
    consecutive pair of `frames`."""
    M, F = frames.shape[:2]
    se_net = se_per = cnt = 0.0
    pairs = [(m, k) for m in range(M) for k in range(F - 1)]
    for i in range(0, len(pairs), batch):
        mi = torch.tensor([p[0] for p in pairs[i:i + batch]])
        fi = torch.tensor([p[1] for p in pairs[i:i + batch]])
        x = expand(frames[mi, fi])
        xn = expand(frames[mi, fi + 1])
        pred = net.predict(x).float()[..., :3]
        tgt = xn.float()[..., :3]
        fl = (x[..., 3] == 0).unsqueeze(-1).float()
        se_net += float((((pred - tgt) ** 2) * fl).sum())
        se_per += float((((x.float()[..., :3] - tgt) ** 2) * fl).sum())
        cnt += float(fl.sum()) * 3
    return {"mse_net": se_net / cnt, "mse_persistence": se_per / cnt, "gain": se_per / max(se_net, 1e-30)}


def rollout_saturation_error(net: UNet, frames: torch.Tensor, start: int = 0, jumps: int = 5,
                             batch: int = 16) -> list[dict]:
    """Autoregressive surrogate rollout from frame `start` of every member of
    `frames` (held-out LBM trajectories): per jump, the relative saturation
    error against the LBM frame of the same iteration (mean and max over
    members)."""
    M = frames.shape[0]
    jumps = min(jumps, frames.shape[1] - 1 - start)
    errs = [[] for _ in range(jumps)]
    for i in range(0, M, batch):
        x = expand(frames[i:i + batch, start])
        fluid = x[..., 3] == 0
        for j in range(jumps):
            x = net.predict(x)
            sp = (((x[..., 0].float() > 0) & fluid).sum(dim=(1, 2)).float() / fluid.sum(dim=(1, 2)).float())
            tr = frames[i:i + batch, start + j + 1, ..., 0].float()
            st = (((tr > 0) & fluid).sum(dim=(1, 2)).float() / fluid.sum(dim=(1, 2)).float())
            errs[j] += ((sp - st).abs() / st.clamp_min(1e-12)).tolist()
    return [{"jump": j + 1, "mean": float(np.mean(e)), "max": float(np.max(e))} for j, e in enumerate(errs)]


# ----------------------------------------------------------------------------
# rollout with the LBM as judge
# ----------------------------------------------------------------------------
def saturation(psi, fluid) -> float:
    return float(((psi > 0) & fluid).sum().item() / max(int(fluid.sum().item()), 1))


def rollout(net: UNet, lat, jumps_per_check: int = 5, checks: int = 4, jump: int = 200, tol: float = 0.02):
    """Advance a reference-mode Lattice by surrogate jumps, judged by the LBM.

    Each round: `jumps_per_check` surrogate jumps from the current state, the
    lattice restarted from the equilibrium of the predicted fields (density
    kept from the last LBM state), then `jump` LBM iterations as the judge.
    The round is accepted if the judged saturation is within `tol` (relative)
    of the surrogate's prediction for the same iteration (one more jump);
    otherwise the lattice falls back to plain LBM from the round's start.
    Returns per-round records and timings."""
    fluid = lat.fluid
    solid = ~fluid
    records = []
    for r in range(checks):
        start_it = lat.iteration
        t0 = time.perf_counter()
        saved = {k: getattr(lat, k).clone() for k in ("psi", "ux", "uy", "rho")}
        x = frame_from_fields(lat.psi, lat.ux, lat.uy, solid).unsqueeze(0).contiguous()  # (1, H, W, 16)
        for _ in range(jumps_per_check):
            x = net.predict(x)
        psi, ux, uy = fields_from_frame(x[0])
        nxt = net.predict(x)
        psi_next, _, _ = fields_from_frame(nxt[0])
        torch.cuda.synchronize()
        t_sur = time.perf_counter() - t0
        lat.restart_from_fields(torch.where(fluid, psi, lat.params.psi_wall), ux, uy, rho=lat.rho,
                                iteration=start_it + jumps_per_check * jump)
        t1 = time.perf_counter()
        lat.step(jump)
        torch.cuda.synchronize()
        t_judge = time.perf_counter() - t1
        s_lbm = saturation(lat.psi, fluid)
        s_sur = saturation(psi_next, fluid)
        ok = bool(np.isfinite(s_lbm)) and abs(s_lbm - s_sur) <= tol * max(s_lbm, 1e-12)
        rec = {"round": r, "start": start_it, "accepted": ok, "sat_lbm": s_lbm, "sat_surrogate": s_sur,
               "t_surrogate_s": t_sur, "t_judge_s": t_judge}
        if not ok:  # fall back: plain LBM from the round's start
            lat.restart_from_fields(saved["psi"], saved["ux"], saved["uy"], rho=saved["rho"], iteration=start_it)
            t2 = time.perf_counter()
            lat.step((jumps_per_check + 1) * jump)
            torch.cuda.synchronize()
            rec["t_fallback_s"] = time.perf_counter() - t2
        records.append(rec)
    return records


def accelerated_ensemble(net: UNet, members, rounds: int, jumps_per_check: int = 5, jump: int = 200,
                         tol: float = 0.02, dtype: str = "f32", restart: str = "regularised") -> dict:
    """The surrogate-accelerated ensemble against the plain batched LBM over
    the same horizon, rounds x (jumps_per_check + 1) x jump iterations.

    Plain: one batched ensemble of the members.  Accelerated, per round: one
    batched forward per jump for all members, every lattice restarted from
    the equilibrium of its predicted fields, `jump` batched LBM iterations as
    the judge (one batch over all members, built once: its CUDA graph is
    captured once); a member whose judged saturation misses the surrogate's
    own prediction for that iteration by more than `tol` (relative) is put
    back to its state at the round's start (exactly) and advanced by plain
    batched LBM instead.  Returns wall times, final saturations and
    acceptance.  ``restart``: "regularised" (equilibrium plus the first-order
    non-equilibrium part of the predicted flow, fd_add_nonequilibrium) or
    "equilibrium".  The plain run is advanced round by round, so each round's
    plain saturations are known: the record gives, for the member-rounds the
    judge accepted, the saturation error against the plain run at the end of
    the round (how well the judge's self-consistency test tracks the truth)."""
    from .ensemble import Ensemble
    from .lattice import Lattice

    if restart not in ("regularised", "equilibrium"):
        raise ValueError("restart must be 'regularised' or 'equilibrium'")
    span = (jumps_per_check + 1) * jump
    horizon = rounds * span

    def batch(lats):
        """A batch over `lats` whose strips give about one tile per resident
        CTA (8..64 rows): a small batch of few members would otherwise march
        few long strips, one iteration taking a whole strip's time."""
        sms = torch.cuda.get_device_properties(lats[0].device).multi_processor_count
        band_rows = sum(-(-lat.W // 128) * lat.H for lat in lats)
        rows = int(min(64, max(8, -(-band_rows // (5 * sms)))))
        return Ensemble.from_lattices(lats, rows_per_strip=rows, band_width=128)

    def advance(lats, n, ens=None):
        """n iterations of every lattice (reference mode in and out) in one
        batch: `ens` (a batch over exactly these lattices) or a new one."""
        own = ens is None
        if own:
            ens = batch(lats)
        for lat in lats:
            lat.enter_fused()
        ens.step(n - 1)
        if own:
            ens.close()
        for lat in lats:
            lat.exit_fused()

    def sats(lats):  # saturations of all lattices, one host synchronisation
        v = torch.stack([((lat.psi > 0) & lat.fluid).sum().double() / lat.fluid.sum().clamp(min=1).double()
                         for lat in lats])
        return v.tolist()

    plain = [Lattice(p, g, dtype=dtype) for p, g in members]
    plain_batch = batch(plain)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sat_plain_rounds = []
    for _ in range(rounds):
        advance(plain, span, plain_batch)
        sat_plain_rounds.append(sats(plain))
    torch.cuda.synchronize()
    t_plain = time.perf_counter() - t0
    plain_batch.close()
    sat_plain = sat_plain_rounds[-1]
    del plain
    torch.cuda.empty_cache()

    lats = [Lattice(p, g, dtype=dtype) for p, g in members]
    accepted = 0
    phase = {"network": 0.0, "restart": 0.0, "judge": 0.0, "replay": 0.0, "checkpoint": 0.0}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tick = t0

    def lap(name):  # wall time per phase (one device synchronisation per phase)
        nonlocal tick
        torch.cuda.synchronize()
        now = time.perf_counter()
        phase[name] += now - tick
        tick = now

    judge = None  # the batch over all members, built at the first judge
    accepted_err = []  # saturation error against the plain run of accepted member-rounds, at the round's end
    for rnd in range(rounds):
        ck = [lat.checkpoint() for lat in lats]
        lap("checkpoint")
        x = torch.stack([frame_from_fields(lat.psi, lat.ux, lat.uy, ~lat.fluid) for lat in lats]).contiguous()
        for _ in range(jumps_per_check):
            x = net.predict(x)
        nxt = net.predict(x)
        fl = nxt[..., 3] == 0
        sat_sur = (((nxt[..., 0].float() > 0) & fl).sum(dim=(1, 2)).float() / fl.sum(dim=(1, 2)).float()).tolist()
        lap("network")
        for m, lat in enumerate(lats):
            psi, ux, uy = fields_from_frame(x[m])
            lat.restart_from_fields(torch.where(lat.fluid, psi, lat.params.psi_wall), ux, uy, rho=lat.rho,
                                    iteration=lat.iteration + jumps_per_check * jump,
                                    regularised=restart == "regularised")
        lap("restart")
        if judge is None:
            judge = batch(lats)
        advance(lats, jump, judge)
        rejected = []
        for m, s_lbm in enumerate(sats(lats)):
            if np.isfinite(s_lbm) and abs(s_lbm - sat_sur[m]) <= tol * max(s_lbm, 1e-12):
                accepted += 1
                sp = sat_plain_rounds[rnd][m]
                if np.isfinite(sp) and sp > 0:
                    accepted_err.append(abs(s_lbm - sp) / sp)
            else:
                rejected.append(m)
        lap("judge")
        for m in rejected:
            lats[m].restore(ck[m])
        if rejected:
            advance([lats[m] for m in rejected], span)
        lap("replay")
    if judge is not None:
        judge.close()
    torch.cuda.synchronize()
    t_acc = time.perf_counter() - t0
    sat_acc = sats(lats)
    # members whose plain run stayed finite with some invading fluid (a member that diverges in the plain
    # LBM has no reference to compare with)
    ok = [m for m, p in enumerate(sat_plain) if np.isfinite(p) and p > 0]
    rel = [abs(sat_acc[m] - sat_plain[m]) / sat_plain[m] for m in ok]
    return {"members": len(members), "rounds": rounds, "horizon_iterations": horizon,
            "plain_s": t_plain, "accelerated_s": t_acc, "speedup": t_plain / t_acc,
            "accelerated_phase_s": {k: round(v, 4) for k, v in phase.items()},
            "accepted_rounds": accepted, "member_rounds": rounds * len(members),
            "members_compared": len(ok), "restart": restart,
            "final_saturation_rel_error_mean": float(np.mean(rel)) if rel else None,
            "final_saturation_rel_error_max": float(np.max(rel)) if rel else None,
            "accepted_vs_plain_rel_error_mean": float(np.mean(accepted_err)) if accepted_err else None,
            "accepted_vs_plain_rel_error_max": float(np.max(accepted_err)) if accepted_err else None}


def breakthrough_race(net: UNet, members, max_rounds: int, jumps_per_check: int = 5, jump: int = 200,
                      tol: float = 0.02, dtype: str = "f32", restart: str = "regularised") -> dict:
    """Plain batched LBM against the surrogate-accelerated ensemble, each run
    until every member has broken through (invading fluid within five columns
    of the outlet: fd_diag.breakthrough) or `max_rounds` rounds of
    (jumps_per_check + 1) x jump iterations have passed.  Each round of the
    accelerated run is a round of accelerated_ensemble (jumps, restart, LBM
    judge, plain replay of rejected members).  Breakthrough is checked at the
    end of every round in both runs.  Returns per member the iteration and the
    wall time of breakthrough in either run, and the wall time until the last
    member that broke through in the plain run broke through in each."""
    from .ensemble import Ensemble
    from .lattice import Lattice

    span = (jumps_per_check + 1) * jump

    def batch(lats):
        sms = torch.cuda.get_device_properties(lats[0].device).multi_processor_count
        band_rows = sum(-(-lat.W // 128) * lat.H for lat in lats)
        rows = int(min(64, max(8, -(-band_rows // (5 * sms)))))
        return Ensemble.from_lattices(lats, rows_per_strip=rows, band_width=128)

    def advance(lats, n, ens):
        for lat in lats:
            lat.enter_fused()
        ens.step(n - 1)
        for lat in lats:
            lat.exit_fused()

    def through(lats):
        return [bool(lat.diagnostics()["breakthrough"]) for lat in lats]

    n = len(members)
    res = {}
    for mode in ("plain", "accelerated"):
        lats = [Lattice(p, g, dtype=dtype) for p, g in members]
        # the batch puts its lattices into the fused state: the accelerated run builds it after its first
        # restart (checkpoints and restarts need the reference state)
        ens = batch(lats) if mode == "plain" else None
        hit_it = [None] * n
        hit_s = [None] * n
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rounds = 0
        for rounds in range(1, max_rounds + 1):
            if mode == "plain":
                advance(lats, span, ens)
            else:
                ck = [lat.checkpoint() for lat in lats]
                x = torch.stack([frame_from_fields(lat.psi, lat.ux, lat.uy, ~lat.fluid) for lat in lats]).contiguous()
                for _ in range(jumps_per_check):
                    x = net.predict(x)
                nxt = net.predict(x)
                fl = nxt[..., 3] == 0
                sat_sur = (((nxt[..., 0].float() > 0) & fl).sum(dim=(1, 2)).float()
                           / fl.sum(dim=(1, 2)).float()).tolist()
                for m, lat in enumerate(lats):
                    psi, ux, uy = fields_from_frame(x[m])
                    lat.restart_from_fields(torch.where(lat.fluid, psi, lat.params.psi_wall), ux, uy, rho=lat.rho,
                                            iteration=lat.iteration + jumps_per_check * jump,
                                            regularised=restart == "regularised")
                if ens is None:
                    ens = batch(lats)
                advance(lats, jump, ens)
                sat_lbm = [float(((lat.psi > 0) & lat.fluid).sum() / lat.fluid.sum().clamp(min=1)) for lat in lats]
                rejected = [m for m in range(n) if not (np.isfinite(sat_lbm[m]) and abs(sat_lbm[m] - sat_sur[m])
                                                        <= tol * max(sat_lbm[m], 1e-12))]
                for m in rejected:
                    lats[m].restore(ck[m])
                if rejected:
                    sub = [lats[m] for m in rejected]
                    tmp = batch(sub)
                    advance(sub, span, tmp)
                    tmp.close()
            flags = through(lats)
            now = time.perf_counter() - t0
            for m in range(n):
                if flags[m] and hit_it[m] is None:
                    hit_it[m], hit_s[m] = rounds * span, now
            if all(h is not None for h in hit_it):
                break
        if ens is not None:
            ens.close()
        res[mode] = {"breakthrough_iteration": hit_it, "breakthrough_s": hit_s, "rounds": rounds}
        del lats
        torch.cuda.empty_cache()
    both = [m for m in range(n) if res["plain"]["breakthrough_s"][m] is not None
            and res["accelerated"]["breakthrough_s"][m] is not None]
    out = {"members": n, "span_iterations": span, "max_rounds": max_rounds, "restart": restart,
           "plain": res["plain"], "accelerated": res["accelerated"],
           "members_through_plain": sum(h is not None for h in res["plain"]["breakthrough_s"]),
           "members_through_accelerated": sum(h is not None for h in res["accelerated"]["breakthrough_s"]),
           "members_through_both": len(both)}
    if both:
        tp = max(res["plain"]["breakthrough_s"][m] for m in both)
        ta = max(res["accelerated"]["breakthrough_s"][m] for m in both)
        out["time_to_last_breakthrough_plain_s"] = tp
        out["time_to_last_breakthrough_accelerated_s"] = ta
        out["breakthrough_speedup"] = tp / ta
        it_err = [abs(res["accelerated"]["breakthrough_iteration"][m] - res["plain"]["breakthrough_iteration"][m])
                  / res["plain"]["breakthrough_iteration"][m] for m in both]
        out["breakthrough_iteration_rel_error_mean"] = float(np.mean(it_err))
    return out
