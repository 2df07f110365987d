"""The reference's step API on a GB300: ``Compute``, ``stream``,
``bottom_top_wall`` and ``Bounce_back`` with the reference's names, argument
meanings and in-place conventions, each function one CUDA kernel.

The reference keeps its parameters as module globals (fingering_periodic.py:
15-44, fingering.py:16-50) and its state as numpy arrays on a ``Compute``
object.  Here the state is torch tensors on the GPU:

* ``f``, ``g``: (9, H, W); ``psi``, ``nabla_psix``, ``nabla_psiy``,
  ``nabla_psi2``: (H, W) - as in the reference;
* ``rho``, ``ux``, ``uy``, ``p``, ``mu``, ``mix_tau``: read as 1-D tensors over
  fluid cells in row-major order (the reference's ``array[mask]`` layout) and
  stored on the full grid; assigning a 1-D tensor scatters it back;
* ``F``, ``feq``, ``geq``: (9, n_fluid), filled by the driver loop as in the
  reference.

The modules :mod:`fingering_dynamics_gb300.fingering_periodic` and
:mod:`fingering_dynamics_gb300.fingering` expose these under the reference's
module names with the reference's default globals; ``Compute`` reads the
globals of its module when it is constructed.  With dtype float64 every
kernel reproduces the reference's arithmetic bit for bit, so the reference's
own loop body, run against these objects, gives the reference's numbers.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .geometry import SOLID_BIT, circle_link_bits, rect_link_bits

_FD_DTYPE = {torch.float64: L.FD_F64, torch.float32: L.FD_F32}


def _vp(t: torch.Tensor):
    return C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _params(H, W, variant, flags=0, tau=0.8, eta_n=0.1, M=1.0, a=0.0, kappa=0.0, gamma=0.0, psi_wall=0.0,
            outlet_coef=2 / 3):
    return L.fd_params(H, W, variant, flags, tau, eta_n, M, a, kappa, gamma, psi_wall, outlet_coef)


class ComputeBase:
    """State and per-function kernels of one lattice (fingering_periodic.py:47-324).

    Subclasses set ``_globals`` (a function returning the module's globals)
    and ``_variant`` (0 periodic, 1 walls).
    """

    _variant = L.FD_VARIANT_PERIODIC
    _globals = staticmethod(lambda: {})

    def __init__(self, mask, dtype=torch.float64, device="cuda"):
        gl = self._globals()
        H, W = int(gl["H"]), int(gl["W"])
        walls = self._variant == L.FD_VARIANT_WALLS
        self._dtype = dtype
        self._fd = _FD_DTYPE[dtype]
        self._dev = torch.empty(0, device=device).device  # concrete index, e.g. cuda:0
        self.mask = np.asarray(mask, dtype=bool)
        if self.mask.shape != (H, W):
            raise ValueError(f"mask shape {self.mask.shape} does not match H, W = {H}, {W}")
        self.block_mask = np.logical_not(self.mask)
        self._mask_t = torch.from_numpy(self.mask).to(self._dev)
        self._n_fluid = int(self.mask.sum())
        word = np.where(self.block_mask, SOLID_BIT, 0).astype(np.uint16)
        self._word = torch.from_numpy(word.view(np.int16)).to(self._dev)
        self.gamma = float(gl["gamma"])
        self._prm = _params(H, W, self._variant, 3 if walls else 0, float(gl["tau"]), float(gl["Eta_n"]),
                            float(gl["M"]), float(gl["a"]), float(gl["kappa"]), self.gamma,
                            float(gl["psi_wall"]), 1.5 if walls else 2 / 3)
        self.H, self.W = H, W
        # initial psi and rho (fingering_periodic.py:90-103, fingering.py:95-107)
        psi0 = np.full((H, W), -1.0)
        psi0[:, :5] = 1.0
        if walls:
            # fingering.py:106-107 draws from numpy's global generator (seed it for
            # reproducible runs, as the reference's own caller would)
            my_number = np.random.randint(0, 1, size=(H, W)) * 2 - 1.0
            rho0 = np.ones((H, W)) + np.random.rand(H, W) * 0.001 * my_number
        else:
            rho0 = np.ones((H, W)) * float(gl.get("rho0", 1.0))
        d = self._dev
        self.f = torch.zeros((9, H, W), dtype=dtype, device=d)
        self.g = torch.zeros((9, H, W), dtype=dtype, device=d)
        self.psi = torch.zeros((H, W), dtype=dtype, device=d)
        self.nabla_psix = torch.zeros((H, W), dtype=dtype, device=d)
        self.nabla_psiy = torch.zeros((H, W), dtype=dtype, device=d)
        self.nabla_psi2 = torch.zeros((H, W), dtype=dtype, device=d)
        self._full = {n: torch.zeros((H, W), dtype=dtype, device=d) for n in ("rho", "ux", "uy", "p", "mu", "mix_tau")}
        self.F = torch.zeros((9, self._n_fluid), dtype=dtype, device=d)
        self.feq = torch.zeros((9, self._n_fluid), dtype=dtype, device=d)
        self.geq = torch.zeros((9, self._n_fluid), dtype=dtype, device=d)
        psi0_d = torch.from_numpy(psi0).to(d)
        rho0_d = torch.from_numpy(np.ascontiguousarray(rho0)).to(d)
        L.call("fd_compute_init", C.byref(self._prm), self._fd, _vp(self._word), _vp(psi0_d), _vp(rho0_d),
               C.byref(self._fields()), _stream())
        torch.cuda.current_stream().synchronize()

    # -- compacted fluid fields ------------------------------------------------
    def _fields(self) -> L.fd_fields:
        fu = self._full
        return L.fd_fields(self.f.data_ptr(), self.g.data_ptr(), self.psi.data_ptr(), self.nabla_psix.data_ptr(),
                           self.nabla_psiy.data_ptr(), self.nabla_psi2.data_ptr(), fu["rho"].data_ptr(),
                           fu["ux"].data_ptr(), fu["uy"].data_ptr(), fu["p"].data_ptr(), fu["mu"].data_ptr(),
                           fu["mix_tau"].data_ptr())

    def _check_layout(self):
        for t in (self.f, self.g, self.psi, self.nabla_psix, self.nabla_psiy, self.nabla_psi2):
            if not t.is_contiguous() or t.device != self._dev or t.dtype != self._dtype:
                raise ValueError("Compute arrays must stay contiguous tensors of the lattice's dtype and device")

    def _masked_get(self, name):
        return self._full[name][self._mask_t]

    def _masked_set(self, name, value):
        v = torch.as_tensor(value, dtype=self._dtype, device=self._dev)
        if v.shape != (self._n_fluid,):
            raise ValueError(f"{name} must have shape ({self._n_fluid},)")
        self._full[name][self._mask_t] = v

    rho = property(lambda s: s._masked_get("rho"), lambda s, v: s._masked_set("rho", v))
    ux = property(lambda s: s._masked_get("ux"), lambda s, v: s._masked_set("ux", v))
    uy = property(lambda s: s._masked_get("uy"), lambda s, v: s._masked_set("uy", v))
    p = property(lambda s: s._masked_get("p"), lambda s, v: s._masked_set("p", v))
    mu = property(lambda s: s._masked_get("mu"), lambda s, v: s._masked_set("mu", v))
    mix_tau = property(lambda s: s._masked_get("mix_tau"), lambda s, v: s._masked_set("mix_tau", v))

    def _field(self, name, masked=True):
        self._check_layout()
        out = torch.zeros((self.H, self.W), dtype=self._dtype, device=self._dev)
        L.call("fd_field", C.byref(self._prm), self._fd, L.FIELDS[name], _vp(self._word), C.byref(self._fields()),
               _vp(out), _stream())
        return out[self._mask_t] if masked else out

    def _term(self, term, j):
        self._check_layout()
        out = torch.zeros((self.H, self.W), dtype=self._dtype, device=self._dev)
        L.call("fd_collision_term", C.byref(self._prm), self._fd, L.TERMS[term], int(j), _vp(self._word),
               C.byref(self._fields()), _vp(out), _stream())
        return out[self._mask_t]

    # -- the reference's methods -------------------------------------------------
    def getP(self):            # fingering_periodic.py:123-124
        return self._field("p")

    def getUx(self):           # fingering_periodic.py:126-132
        return self._field("ux")

    def getUy(self):           # fingering_periodic.py:134-139
        return self._field("uy")

    def getMu(self):           # fingering_periodic.py:141-144
        return self._field("mu")

    def getMu_plain(self):     # fingering_periodic.py:146-149
        return self._field("mu_plain", masked=False)

    def getRho(self):          # fingering_periodic.py:151-152
        return self._field("rho")

    def getfeq(self, n):       # fingering_periodic.py:171-181
        return self._term("feq", n)

    def getgeq(self, n):       # fingering_periodic.py:183-192
        return self._term("geq", n)

    def getLarge_F(self, n):   # fingering_periodic.py:194-199
        return self._term("large_F", n)

    # getA0 / getA1_8 / getB0 / getB1_8 (fingering_periodic.py:155-169) are the
    # sub-expressions of getfeq / getgeq; they are evaluated inside those kernels.

    def getMix_tau(self):      # fingering_periodic.py:201-208
        return self._field("mix_tau")

    def udpatePsi(self):       # fingering_periodic.py:210-212
        self.psi.copy_(self._field("psi", masked=False))

    def getNabla_psix(self):   # fingering_periodic.py:214-226
        return self._field("npx", masked=False)

    def getNabla_psiy(self):   # fingering_periodic.py:228-240
        return self._field("npy", masked=False)

    def getNabla_psi2(self):   # fingering_periodic.py:242-256
        return self._field("np2", masked=False)

    def getF(self, i):
        """fingering_periodic.py:258-260; the forcing and equilibrium are
        evaluated from the current fields (the reference reads the F[i] and
        feq[i] its loop stored from the same fields just before)."""
        return self._term("F", i)

    def getG(self, i):         # fingering_periodic.py:262-264
        return self._term("G", i)

    def _zou_he(self, fn):
        self._check_layout()
        side = torch.empty((6, self.H), dtype=self._dtype, device=self._dev)
        ux = torch.from_numpy(self._inlet_ux()).to(self._dev)
        L.call("fd_boundary_fields", C.byref(self._prm), self._fd, _vp(self._word), _vp(self.psi),
               _vp(self.nabla_psi2), _vp(side), _stream())
        L.call(fn, C.byref(self._prm), self._fd, _vp(self.f), _vp(self.g), _vp(side), _vp(ux), _stream())
        torch.cuda.current_stream().synchronize()

    def zou_he_boundary_inlet(self):    # fingering_periodic.py:268-302 / fingering.py:298-364
        self._zou_he("fd_zou_he_inlet")

    def zou_he_boundary_outlet(self):   # fingering_periodic.py:305-324 / fingering.py:369-390
        self._zou_he("fd_zou_he_outlet")

    def _inlet_ux(self):
        gl = self._globals()
        H, u0 = self.H, float(gl["u0"])
        if self._variant == L.FD_VARIANT_WALLS:
            return np.full(H, u0)
        temp = np.array([i * 3 / (H / 2) for i in range(int(-H / 2), int(H / 2))])
        return u0 * np.exp(- (temp ** 2) / 2)


def _shape_params(f: torch.Tensor) -> L.fd_params:
    if f.dim() != 3 or f.shape[0] != 9:
        raise ValueError("populations must be (9, H, W) tensors")
    return _params(int(f.shape[1]), int(f.shape[2]), L.FD_VARIANT_PERIODIC)


def stream(f: torch.Tensor, g: torch.Tensor):
    """fingering_periodic.py:327-343: shift every population plane by its
    lattice velocity, periodic in x and y, in place."""
    prm = _shape_params(f)
    fd = _FD_DTYPE[f.dtype]
    sf, sg = f.clone(), g.clone()
    L.call("fd_stream", C.byref(prm), fd, _vp(sf), _vp(sg), _vp(f), _vp(g), _stream())
    torch.cuda.current_stream().synchronize()


def bottom_top_wall(f_behind, g_behind, f, g):
    """fingering.py:432-451 on (9, rows, cols) views (the reference passes
    ``f[:, 1:-1]``, i.e. rows 1..H-2)."""
    for t in (g_behind, f, g):
        if t.shape != f_behind.shape or t.stride() != f_behind.stride():
            raise ValueError("bottom_top_wall: all four views must share shape and strides")
    if f_behind.stride(2) != 1:
        raise ValueError("bottom_top_wall: the last axis must be contiguous")
    L.call("fd_bottom_top_wall", _FD_DTYPE[f.dtype], int(f.shape[1]), int(f.shape[2]), int(f.stride(0)),
           int(f.stride(1)), _vp(f_behind), _vp(g_behind), _vp(f), _vp(g), _stream())
    torch.cuda.current_stream().synchronize()


class Bounce_back:
    """bounce_back.py:5-167: half-way bounce-back from the reference's mask
    lists, applied on the GPU through link bits."""

    def __init__(self, H, W):
        self.H = H
        self.W = W
        self._cache = {}

    def _apply(self, key, keep, make_bits, f_behind, g_behind, f, g):
        # the cache holds the caller's mask objects too, so an id() in a key
        # can never be reused by a different object while the entry exists
        if key not in self._cache:
            bits = make_bits().astype(np.uint16)
            self._cache[key] = (keep, torch.from_numpy(bits.view(np.int16)).to(f.device))
        prm = _shape_params(f)
        L.call("fd_bounce_back", C.byref(prm), _FD_DTYPE[f.dtype], _vp(self._cache[key][1]), _vp(f_behind),
               _vp(g_behind), _vp(f), _vp(g), _stream())
        torch.cuda.current_stream().synchronize()

    def halfway_bounceback_rec(self, corner_list, f_behind, g_behind, f, g):     # bounce_back.py:25-86
        H, W = f.shape[1], f.shape[2]
        key = ("rec", H, W, tuple(tuple(sorted(c.items())) for c in corner_list))
        self._apply(key, None, lambda: rect_link_bits(corner_list, H, W), f_behind, g_behind, f, g)

    def halfway_bounceback_circle(self, side_list, concave_list, convex_list, f_behind, g_behind, f, g):
        """bounce_back.py:89-167."""
        masks = (*side_list, *concave_list, *convex_list)
        key = ("circle", tuple(id(m) for m in masks))
        self._apply(key, masks, lambda: circle_link_bits(side_list, concave_list, convex_list), f_behind, g_behind,
                    f, g)
