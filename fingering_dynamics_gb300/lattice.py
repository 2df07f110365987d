"""GPU lattice state and stepping.

:class:`Lattice` owns one simulation's device buffers and drives the CUDA
kernels through the C ABI.  It offers two equivalent ways to advance:

* :meth:`Lattice.step_reference` runs the reference's loop body
  (fingering_periodic.py:454-479 / fingering.py:558-585) one function at a
  time, each function one kernel.
* :meth:`Lattice.step` / :meth:`Lattice.advance` use the fused kernel, one
  launch per iteration.

Device layout (all torch tensors on one GPU):

* ``pop[0]``, ``pop[1]``: (18, H, W) population buffers, f planes then g
  planes.  In *reference* mode ``pop[cur]`` holds the pre-collision
  populations of the current iteration (the reference's ``f``/``g``); in
  *fused* mode it holds the post-collision populations whose streaming is
  pending.  Switching modes costs one collision or one
  stream + bounce-back + Zou-He + macroscopic update; no buffer is copied.
* ``side[0]``, ``side[1]``: (6, H) psi_x, psi_y, mu at columns 0 and W-1.
* ``psi``, ``npx``, ``npy``, ``np2``, ``rho``, ``ux``, ``uy``, ``p``, ``mu``,
  ``mix_tau``: (H, W) fields, current in reference mode.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L
from .geometry import Geometry
from .params import LBMParams

# name -> (reference-layout torch dtype, reference-layout fd dtype, packed storage or None)
#   f64        FP64 everywhere; the fused kernel reproduces the reference bit for bit
#   f32        FP32 reference-order kernels; fused kernel in deviation form, FP32 storage
#   f16 / bf16 as f32, fused storage of f deviations and g_1..g_8 in FP16 / BF16 (g_0 FP32),
#              stochastic rounding by default (``rounding="nearest"`` for round to nearest even)
#   f32-exact  FP32 with the reference's operand order in the fused kernel too
DTYPES = {
    "f64": (torch.float64, L.FD_F64, None),
    "f32": (torch.float32, L.FD_F32, (L.FD_F32, 0, 0)),
    "f16": (torch.float32, L.FD_F32, (L.FD_F16, 0, 0)),
    "bf16": (torch.float32, L.FD_F32, (L.FD_BF16, 0, 0)),
    "f32-exact": (torch.float32, L.FD_F32, None),
}
FIELD_NAMES = ("psi", "npx", "npy", "np2", "rho", "ux", "uy", "p", "mu", "mix_tau")


def make_fd_params(prm: LBMParams) -> L.fd_params:
    flags = ((L.FD_INIT_MU if prm.init_mu else 0) | (L.FD_INIT_UY if prm.init_uy else 0)
             | (L.FD_OUTLET_PRESSURE if prm.outlet == "pressure" else 0))
    return L.fd_params(prm.H, prm.W, prm.variant_id, flags, prm.tau, prm.eta_n, prm.M, prm.a, prm.kappa,
                       prm.gamma, prm.psi_wall, prm.outlet_coef, prm.force_x, prm.force_y)


def _ptr(t: torch.Tensor | None):
    return None if t is None else C.c_void_p(t.data_ptr())


class Lattice:
    """One two-phase D2Q9 simulation resident on a GPU."""

    def __init__(self, params: LBMParams, geometry: Geometry, dtype: str = "f64", device="cuda",
                 rho0: np.ndarray | None = None, psi0: np.ndarray | None = None, rounding: str = "stochastic",
                 seed: int = 0):
        """``rounding`` / ``seed``: rounding of the FP16/BF16 stores of the
        fused step (include/fdlbm.h ``fd_storage``); the step at iteration k
        uses seed + k, so a run is reproducible and a resumed run continues
        bit for bit."""
        if dtype not in DTYPES:
            raise ValueError(f"dtype must be one of {sorted(DTYPES)}")
        if (geometry.H, geometry.W) != (params.H, params.W):
            raise ValueError("geometry and params disagree on the lattice size")
        self.params = params
        self.geometry = geometry
        self.dtype = dtype
        self.tdtype, self.fd_dtype, packed = DTYPES[dtype]
        if rounding not in L.ROUNDING:
            raise ValueError(f"rounding must be one of {sorted(L.ROUNDING)}")
        self.rounding = rounding
        self.seed = int(seed) & 0xFFFFFFFF
        self.storage = None if packed is None else L.fd_storage(*packed, L.ROUNDING[rounding], 0)
        if torch.device(device).type != "cuda":
            raise ValueError("Lattice runs on a CUDA device only")
        self.device = torch.empty(0, device=device).device  # concrete index, e.g. cuda:0
        H, W = params.H, params.W
        self.H, self.W = H, W
        self.prm = make_fd_params(params)
        dev, td = self.device, self.tdtype
        self.mask = torch.from_numpy(np.ascontiguousarray(geometry.mask_word).view(np.int16)).to(dev)
        self.fluid = torch.from_numpy(~geometry.solid).to(dev)
        self.inlet_ux = torch.from_numpy(np.ascontiguousarray(params.inlet_ux, np.float64)).to(dev)
        self.pop = [torch.zeros((18, H, W), dtype=td, device=dev) for _ in range(2)]
        self.side = [torch.zeros((6, H), dtype=td, device=dev) for _ in range(2)]
        self.cur = 0
        self.scur = 0
        self.ppop = None   # packed buffers, allocated on first entry into fused mode
        self.pcur = 0
        for n in FIELD_NAMES:
            setattr(self, n, torch.zeros((H, W), dtype=td, device=dev))
        psi0 = params.initial_psi(geometry.solid) if psi0 is None else np.asarray(psi0, np.float64)
        psi0_d = torch.from_numpy(np.ascontiguousarray(psi0, np.float64)).to(dev)
        rho0_d = None if rho0 is None else torch.from_numpy(np.ascontiguousarray(rho0, np.float64)).to(dev)
        self.mode = "reference"
        self.iteration = 0
        L.call("fd_compute_init", C.byref(self.prm), self.fd_dtype, _ptr(self.mask), _ptr(psi0_d), _ptr(rho0_d),
               C.byref(self.fields()), self._stream())
        self._keep = (psi0_d, rho0_d)  # alive until the init kernels ran
        torch.cuda.current_stream(self.device).synchronize()
        self._keep = None

    # ------------------------------------------------------------------
    @property
    def f(self) -> torch.Tensor:
        return self.pop[self.cur][:9]

    @property
    def g(self) -> torch.Tensor:
        return self.pop[self.cur][9:]

    def _stream(self):
        return C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)

    def fields(self, pop: torch.Tensor | None = None) -> L.fd_fields:
        p = self.pop[self.cur] if pop is None else pop
        return L.fd_fields(p.data_ptr(), p[9:].data_ptr(), *(getattr(self, n).data_ptr() for n in
                                                              ("psi", "npx", "npy", "np2", "rho", "ux", "uy", "p",
                                                               "mu", "mix_tau")))

    # ------------------------------------------------------------------
    # reference-order pieces (each one kernel)
    # ------------------------------------------------------------------
    def _require(self, mode):
        if self.mode != mode:
            raise RuntimeError(f"lattice is in {self.mode} mode, this call needs {mode} mode")

    def collide(self):
        """fingering_periodic.py:455-460 in place on the current populations."""
        self._require("reference")
        L.call("fd_collide", C.byref(self.prm), self.fd_dtype, _ptr(self.mask), C.byref(self.fields()), self._stream())

    def boundary_fields(self, out: torch.Tensor):
        L.call("fd_boundary_fields", C.byref(self.prm), self.fd_dtype, _ptr(self.mask), _ptr(self.psi), _ptr(self.np2),
               _ptr(out), self._stream())

    def _finish_from(self, src: torch.Tensor, side: torch.Tensor, dst: torch.Tensor):
        """stream + bounce-back + Zou-He + macroscopic update of a pending
        iteration: ``src`` holds post-collision populations (also the
        reference's f_behind snapshot), ``dst`` receives the new ones."""
        s = self._stream()
        prm = C.byref(self.prm)
        L.call("fd_stream", prm, self.fd_dtype, _ptr(src), _ptr(src[9:]), _ptr(dst), _ptr(dst[9:]), s)
        L.call("fd_bounce_back", prm, self.fd_dtype, _ptr(self.mask), _ptr(src), _ptr(src[9:]), _ptr(dst),
               _ptr(dst[9:]), s)
        L.call("fd_zou_he_inlet", prm, self.fd_dtype, _ptr(dst), _ptr(dst[9:]), _ptr(side), _ptr(self.inlet_ux), s)
        L.call("fd_zou_he_outlet", prm, self.fd_dtype, _ptr(dst), _ptr(dst[9:]), _ptr(side), _ptr(self.inlet_ux), s)
        fl = C.byref(self.fields(dst))
        L.call("fd_update_rho_psi", prm, self.fd_dtype, _ptr(self.mask), fl, s)
        L.call("fd_update_macros", prm, self.fd_dtype, _ptr(self.mask), fl, s)

    def step_reference(self, n: int = 1):
        """n iterations of the loop body, one kernel per reference function."""
        self._require("reference")
        for _ in range(n):
            self.collide()
            self.boundary_fields(self.side[self.scur])
            src, dst = self.pop[self.cur], self.pop[1 - self.cur]
            self._finish_from(src, self.side[self.scur], dst)
            self.cur = 1 - self.cur
            self.iteration += 1

    # ------------------------------------------------------------------
    # fused path
    # ------------------------------------------------------------------
    def enter_fused(self):
        """Collide the current iteration and keep the result as fused state."""
        if self.mode == "fused":
            return
        self.boundary_fields(self.side[self.scur])
        self.collide()
        if self.storage is not None:
            if self.ppop is None:
                nbytes = L.lib().fd_packed_bytes(self.H, self.W, C.byref(self.storage))
                if not nbytes:
                    raise L.FDError(-1, "fd_packed_bytes", "invalid storage")
                self.ppop = [torch.empty(nbytes, dtype=torch.uint8, device=self.device) for _ in range(2)]
            L.call("fd_pack", C.byref(self.prm), self.fd_dtype, _ptr(self.pop[self.cur]), C.byref(self.storage),
                   _ptr(self.ppop[self.pcur]), self._stream())
        self.mode = "fused"

    def advance(self, n: int, rows_per_warp: int = 0):
        """n fused kernels (n more collisions); stays in fused mode."""
        self._require("fused")
        if n <= 0:
            return
        sa, sb = self.side[self.scur], self.side[1 - self.scur]
        if self.storage is None:
            a, b = self.pop[self.cur], self.pop[1 - self.cur]
            L.call("fd_fused_step", C.byref(self.prm), self.fd_dtype, _ptr(self.mask), _ptr(self.inlet_ux), _ptr(a),
                   _ptr(b), _ptr(sa), _ptr(sb), int(n), int(rows_per_warp), self._stream())
            if n % 2:
                self.cur = 1 - self.cur
        else:
            a, b = self.ppop[self.pcur], self.ppop[1 - self.pcur]
            self.storage.seed = self.step_seed()
            L.call("fd_fused_step_packed", C.byref(self.prm), C.byref(self.storage), _ptr(self.mask),
                   _ptr(self.inlet_ux), _ptr(a), _ptr(b), _ptr(sa), _ptr(sb), int(n), int(rows_per_warp),
                   self._stream())
            if n % 2:
                self.pcur = 1 - self.pcur
        if n % 2:
            self.scur = 1 - self.scur
        self.iteration += n

    def advance_host(self, host_in: torch.Tensor, host_out: torch.Tensor | None = None, n: int = 1,
                     chunk_rows: int = 0):
        """n fused iterations of a state held in host memory: ``host_in`` holds
        the packed bytes of :meth:`current_buffer` (as written by
        :meth:`download_populations`); they are uploaded, advanced and the
        result downloaded into ``host_out`` (default ``host_in``, in place) by
        one pipelined call (fd_fused_step_packed_host), the copies of both
        directions overlapping each other and the kernels.  The device state
        follows as after :meth:`advance`.  Asynchronous on the lattice's
        stream; pinned host tensors are needed for the overlap."""
        self._require("fused")
        if self.storage is None:
            raise ValueError("advance_host needs packed storage (dtype f32, f16 or bf16)")
        if n <= 0:
            return
        host_out = host_in if host_out is None else host_out
        nbytes = self.ppop[self.pcur].numel()
        for t in (host_in, host_out):
            if t.device.type != "cpu" or t.dtype != torch.uint8 or t.numel() != nbytes or not t.is_contiguous():
                raise ValueError(f"host buffers must be contiguous uint8 CPU tensors of {nbytes} bytes")
        a, b = self.ppop[self.pcur], self.ppop[1 - self.pcur]
        sa, sb = self.side[self.scur], self.side[1 - self.scur]
        self.storage.seed = self.step_seed()
        L.call("fd_fused_step_packed_host", C.byref(self.prm), C.byref(self.storage), _ptr(self.mask),
               _ptr(self.inlet_ux), _ptr(host_in), _ptr(host_out), _ptr(a), _ptr(b), _ptr(sa), _ptr(sb), int(n),
               int(chunk_rows), self._stream())
        if n % 2:
            self.pcur = 1 - self.pcur
            self.scur = 1 - self.scur
        self.iteration += n

    def peek(self):
        """Fields of the next iteration (psi, rho, ux, uy, ... in the field
        tensors) without leaving fused mode: the pending packed state is
        unpacked into the reference-layout buffers, which the fused state does
        not use, and finished there.  The state itself is not touched, so a
        lattice that is a member of an ensemble can be read between batched
        steps."""
        self._require("fused")
        if self.storage is None:
            raise ValueError("peek needs packed storage (dtype f32, f16 or bf16)")
        L.call("fd_unpack", C.byref(self.prm), C.byref(self.storage), _ptr(self.ppop[self.pcur]), self.fd_dtype,
               _ptr(self.pop[self.cur]), self._stream())
        self._finish_from(self.pop[self.cur], self.side[self.scur], self.pop[1 - self.cur])

    def restart_from_fields(self, psi, ux, uy, rho=None, iteration: int | None = None,
                            regularised: bool = False):
        """Replace the state by the equilibrium of the given fields ((H, W)
        device tensors or arrays): populations f = feq(rho, u, psi, mu(psi)),
        g = geq, as Compute.__init__ builds them (fingering_periodic.py:
        100-121) but with the given velocity (FD_INIT_VELOCITY); with
        ``regularised`` also the first-order non-equilibrium part of the
        flow's velocity gradients (fd_add_nonequilibrium).  Leaves the
        lattice in reference mode at ``iteration`` (default: unchanged)."""
        dev, td = self.device, self.tdtype
        self.mode = "reference"
        self.ux.copy_(torch.as_tensor(ux, device=dev, dtype=td))
        self.uy.copy_(torch.as_tensor(uy, device=dev, dtype=td))
        psi_d = torch.as_tensor(psi, device=dev).to(torch.float64).contiguous()
        rho_d = None if rho is None else torch.as_tensor(rho, device=dev).to(torch.float64).contiguous()
        prm = L.fd_params.from_buffer_copy(self.prm)
        prm.flags |= L.FD_INIT_MU | L.FD_INIT_VELOCITY
        # psi_d / rho_d were allocated on this stream, so the caching allocator
        # reuses their memory only for work ordered after the init kernels
        L.call("fd_compute_init", C.byref(prm), self.fd_dtype, _ptr(self.mask), _ptr(psi_d), _ptr(rho_d),
               C.byref(self.fields()), self._stream())
        if regularised:
            L.call("fd_add_nonequilibrium", C.byref(prm), self.fd_dtype, _ptr(self.mask), C.byref(self.fields()),
                   self._stream())
        if iteration is not None:
            self.iteration = int(iteration)

    def checkpoint(self) -> dict:
        """In-memory copy of a reference-mode state (populations, boundary
        values, fields, iteration) for :meth:`restore`."""
        self._require("reference")
        ck = {"pop": self.pop[self.cur].clone(), "side": self.side[self.scur].clone(), "iteration": self.iteration}
        for n in FIELD_NAMES:
            ck[n] = getattr(self, n).clone()
        return ck

    def restore(self, ck: dict):
        """Return to a state taken by :meth:`checkpoint` (reference mode)."""
        self.mode = "reference"
        self.pop[self.cur].copy_(ck["pop"])
        self.side[self.scur].copy_(ck["side"])
        for n in FIELD_NAMES:
            getattr(self, n).copy_(ck[n])
        self.iteration = ck["iteration"]

    def check_finite(self, clear: bool = True):
        """Raise FloatingPointError if a packed fused step met a non-finite
        density or psi since the status was last cleared, as the reference's
        numpy step does under np.seterr(all='raise') (fingering_periodic.py:
        496); the device status word is shared by every lattice on the device.
        Synchronous."""
        v = C.c_uint(0)
        L.call("fd_device_status", C.byref(v), int(bool(clear)))
        if v.value & L.FD_STATUS_NONFINITE:
            raise FloatingPointError("a fused step met a non-finite density or psi")

    def step_seed(self) -> int:
        """Stochastic-rounding seed of the next fused launch."""
        return (self.seed + self.iteration) & 0xFFFFFFFF

    def exit_fused(self):
        """Finish the pending iteration; the fields become current."""
        if self.mode == "reference":
            return
        if self.storage is not None:
            L.call("fd_unpack", C.byref(self.prm), C.byref(self.storage), _ptr(self.ppop[self.pcur]), self.fd_dtype,
                   _ptr(self.pop[self.cur]), self._stream())
        src, dst = self.pop[self.cur], self.pop[1 - self.cur]
        self._finish_from(src, self.side[self.scur], dst)
        self.cur = 1 - self.cur
        self.mode = "reference"
        self.iteration += 1

    def step(self, n: int = 1, rows_per_warp: int = 0):
        """n iterations of the loop body through the fused kernel."""
        if n <= 0:
            return
        if self.mode == "reference":
            self.enter_fused()
            self.advance(n - 1, rows_per_warp)
            self.exit_fused()
        else:
            self.advance(n, rows_per_warp)

    # ------------------------------------------------------------------
    # diagnostics
    # ------------------------------------------------------------------
    def diagnostics(self) -> dict:
        """FP64 colour masses, saturation, finger tip and breakthrough of the
        current state (either mode); see include/fdlbm.h ``fd_diag``."""
        if not hasattr(self, "_diag_scratch"):
            nbytes = L.lib().fd_diag_scratch_bytes()
            self._diag_scratch = torch.empty(nbytes, dtype=torch.uint8, device=self.device)
            self._diag_out = torch.empty(C.sizeof(L.fd_diag), dtype=torch.uint8, device=self.device)
        packed = self.mode == "fused" and self.storage is not None
        buf = self.current_buffer()
        L.call("fd_diagnostics", C.byref(self.prm), self.fd_dtype, C.byref(self.storage) if packed else None,
               _ptr(buf), _ptr(self.mask), _ptr(self._diag_scratch), _ptr(self._diag_out), self._stream())
        host = self._diag_out.cpu().numpy().tobytes()
        return L.fd_diag.from_buffer_copy(host).as_dict()

    # ------------------------------------------------------------------
    # checkpoint / resume
    # ------------------------------------------------------------------
    def save_snapshot(self, path: str):
        """Write the complete state to ``path`` (.npz): mode, iteration, the
        current population buffer (reference layout or packed bytes), the
        current boundary-value buffer and, in reference mode, the macroscopic
        fields.  :meth:`load_snapshot` restores it exactly, so a resumed run
        continues bit for bit."""
        torch.cuda.current_stream(self.device).synchronize()
        rec = {"mode": np.array(self.mode), "iteration": np.array(self.iteration), "dtype": np.array(self.dtype),
               "H": np.array(self.H), "W": np.array(self.W), "mask_word": self.geometry.mask_word,
               "state": self.current_buffer().cpu().numpy(), "side": self.side[self.scur].cpu().numpy(),
               "rounding": np.array(self.rounding), "seed": np.array(self.seed, dtype=np.uint32)}
        if self.mode == "reference":
            for n in FIELD_NAMES:
                rec[n] = getattr(self, n).cpu().numpy()
        np.savez(path, **rec)

    def load_snapshot(self, path: str):
        """Restore a state written by :meth:`save_snapshot` into this lattice
        (same size, dtype and geometry)."""
        with np.load(path, allow_pickle=False) as z:
            if (int(z["H"]), int(z["W"]), str(z["dtype"])) != (self.H, self.W, self.dtype):
                raise ValueError("snapshot was written by a lattice of another size or dtype")
            if not np.array_equal(z["mask_word"], self.geometry.mask_word):
                raise ValueError("snapshot was written for another geometry")
            mode = str(z["mode"])
            if mode == "fused" and self.storage is not None and self.ppop is None:
                self.mode = "reference"
                self.enter_fused()  # allocates the packed buffers
            self.mode = mode
            self.iteration = int(z["iteration"])
            if "seed" in z.files:  # the stochastic-rounding stream continues where it stopped
                self.seed = int(z["seed"])
                self.rounding = str(z["rounding"])
                if self.storage is not None:
                    self.storage.rounding = L.ROUNDING[self.rounding]
            self.current_buffer().copy_(torch.from_numpy(z["state"]))
            self.side[self.scur].copy_(torch.from_numpy(z["side"]))
            if mode == "reference":
                for n in FIELD_NAMES:
                    getattr(self, n).copy_(torch.from_numpy(z[n]))
        torch.cuda.current_stream(self.device).synchronize()

    def macroscopic(self) -> dict:
        """psi, u_x, u_y (numpy, (H, W), NaN-free: 0 on solid cells for u) of
        the current iteration; leaves the lattice in the mode it was in."""
        fused = self.mode == "fused"
        if fused:
            self.exit_fused()
        torch.cuda.current_stream(self.device).synchronize()
        fluid = self.fluid
        out = {"psi": self.psi.double().cpu().numpy(),
               "ux": torch.where(fluid, self.ux, 0).double().cpu().numpy(),
               "uy": torch.where(fluid, self.uy, 0).double().cpu().numpy()}
        if fused:
            self.enter_fused()
        return out

    # ------------------------------------------------------------------
    # host buffers
    # ------------------------------------------------------------------
    def current_buffer(self) -> torch.Tensor:
        """The device buffer that holds the state: (18, H, W) populations, or
        the packed bytes in fused mode with packed storage."""
        if self.mode == "fused" and self.storage is not None:
            return self.ppop[self.pcur]
        return self.pop[self.cur]

    def upload_populations(self, host: torch.Tensor):
        """Copy the state buffer from host memory (same shape and dtype as
        :meth:`current_buffer`; asynchronous when ``host`` is pinned)."""
        self.current_buffer().copy_(host, non_blocking=True)

    def download_populations(self, host: torch.Tensor):
        """Copy the state buffer into host memory."""
        host.copy_(self.current_buffer(), non_blocking=True)

    # ------------------------------------------------------------------
    def state(self) -> dict:
        """Host copies of the reference-layout state (reference mode)."""
        self._require("reference")
        torch.cuda.current_stream(self.device).synchronize()
        out = {"f": self.f.double().cpu().numpy(), "g": self.g.double().cpu().numpy()}
        solid = self.geometry.solid
        for n in FIELD_NAMES:
            a = getattr(self, n).double().cpu().numpy()
            if n in ("rho", "ux", "uy", "p", "mu", "mix_tau"):
                a = np.where(solid, np.nan, a)
            out[n] = a
        return out
