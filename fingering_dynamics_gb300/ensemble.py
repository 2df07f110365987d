"""Batched ensembles: many independent lattices advanced together.

Each member is a :class:`~fingering_dynamics_gb300.lattice.Lattice` in fused
mode with packed storage; :class:`Ensemble` hands their buffers to the C
batch (``fd_batch_*``), which advances every member one iteration per
persistent launch over a tile table and replays the iteration loop from a CUDA
graph.  :meth:`Ensemble.autotune` picks the tile shape (band width and rows
per strip) by timing the candidates on the ensemble itself.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, replace

import numpy as np
import torch

from . import _lib as L
from .geometry import build_geometry, random_blocks
from .lattice import Lattice
from .params import LBMParams, from_relaxation_times, walls_reference_params

DEFAULT_CANDIDATES = ((128, 16), (128, 32), (128, 64), (64, 32), (64, 64), (256, 16), (256, 32))


@dataclass
class MemberSpec:
    """One seeded ensemble member.

    family "spec" (and "config", the same parameterisation over narrower
    porosity and inlet ranges): lattice parameters from relaxation times
    (tau_def = 1.0, tau_inv from the viscosity ratio), interfacial tension
    ``sigma``, psi_wall from the contact angle through the droplet calibration
    table and the reference's mobility rule.  family "stable": the
    constants of fingering.py:16-50 with the viscosity ratio, psi_wall and inlet
    speed of this member.  The reference model diverges within tens of steps
    for much of the "spec" ranges on dense random obstacles (tau_inv -> 0.525,
    mobility ~1e2-1e3 from the rule at small sigma); "stable" runs thousands.
    """
    H: int
    W: int
    porosity: float
    viscosity_ratio: float
    contact_angle_deg: float
    sigma: float
    u_in: float
    seed: int
    family: str = "stable"
    psi_wall: float = -1.0

    def params(self, tau_def: float = 1.0, variant: str = "walls") -> LBMParams:
        if self.family == "stable":
            prm = walls_reference_params().with_size(self.H, self.W)
            return replace(prm, M=self.viscosity_ratio, psi_wall=self.psi_wall, u0=self.u_in,
                           inlet_ux=np.full(self.H, self.u_in))
        tau_inv = 0.5 + (tau_def - 0.5) / self.viscosity_ratio
        return from_relaxation_times(self.H, self.W, tau_inv, tau_def, self.sigma, self.contact_angle_deg,
                                     self.u_in, variant=variant)

    def build(self, tau_def: float = 1.0, variant: str = "walls"):
        prm = self.params(tau_def, variant)
        rmax = max(3, min(14, self.H // 12))
        rects, circles = random_blocks(self.H, self.W, self.porosity, min(6, rmax), rmax, self.seed,
                                       x_margin=min(32, self.W // 8))
        return prm, build_geometry(self.H, self.W, rects=rects, circles=circles, walls=variant == "walls")


def ensemble_specs(n: int, seed: int, sizes_w=(256, 512, 1024, 2048), sizes_h=(128, 256, 512),
                   porosity=None, ratio=None, angle=(30.0, 150.0), sigma=(1e-4, 1e-3),
                   u_in=None, family: str = "stable", psi_wall=(-1.0, -0.5)) -> list[MemberSpec]:
    """n members drawn from a seeded generator: sizes uniform over the given
    widths x heights, porosity uniform, viscosity ratio and interfacial
    tension log-uniform, contact angle, psi_wall and inlet speed uniform.

    Family "spec" defaults to the ranges of the benchmark configuration
    (viscosity ratio 2..20, porosity 0.6..0.85, inlet 0.005..0.02).  Family
    "config" keeps that configuration's viscosity-ratio, contact-angle and
    interfacial-tension ranges and narrows porosity (0.70..0.85) and inlet speed (0.003..0.010), the two
    ranges whose upper / lower ends the Darcy argument below rules out;
    members that still diverge are quarantined by the batch
    (Ensemble.member_status).  Family
    "stable" defaults to viscosity ratio 2..5, porosity 0.70..0.85 and inlet
    0.003..0.010: the medium must carry the imposed flux with density
    differences of order 3 u nu L / k (Darcy), and denser or faster members
    diverge within a few thousand steps (with either outlet rule); on the
    96-member draw of seed 2024 none of these diverges within 6000 steps,
    against 35 of 96 with the configuration's porosity and inlet ranges."""
    if family not in ("spec", "config", "stable"):
        raise ValueError(f"unknown ensemble family {family!r}")
    if ratio is None:
        ratio = (2.0, 20.0) if family in ("spec", "config") else (2.0, 5.0)
    if porosity is None:
        porosity = (0.6, 0.85) if family == "spec" else (0.70, 0.85)
    if u_in is None:
        u_in = (0.005, 0.02) if family == "spec" else (0.003, 0.010)
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        lr = rng.uniform(math.log(ratio[0]), math.log(ratio[1]))
        ls = rng.uniform(math.log(sigma[0]), math.log(sigma[1]))
        out.append(MemberSpec(H=int(rng.choice(sizes_h)), W=int(rng.choice(sizes_w)),
                              porosity=float(rng.uniform(*porosity)), viscosity_ratio=float(math.exp(lr)),
                              contact_angle_deg=float(rng.uniform(*angle)), sigma=float(math.exp(ls)),
                              u_in=float(rng.uniform(*u_in)), seed=int(rng.integers(0, 2 ** 31)), family=family,
                              psi_wall=float(rng.uniform(*psi_wall))))
    return out


def tile_count(sizes, band_width: int, rows_per_strip: int) -> int:
    """Tiles per iteration of a batch of lattices of the given (H, W) sizes:
    bands of `band_width` cells times strips of at most `rows_per_strip` rows."""
    return sum(-(-W // band_width) * -(-H // min(rows_per_strip, H)) for H, W in sizes)


def round_filling_rows(sizes, band_width: int, grid: int, max_rounds: int = 8, min_fill: float = 0.9) -> list:
    """For each round count r = 1 .. max_rounds of a persistent grid of `grid`
    CTAs, the shortest strips (>= 16 rows) whose tiles fit in r rounds, kept
    when they need all r rounds and fill at least `min_fill` of them."""
    hmax = max(H for H, _ in sizes)
    out = []
    for r in range(1, max_rounds + 1):
        rows = next((h for h in range(16, hmax + 1) if tile_count(sizes, band_width, h) <= r * grid), None)
        if rows is None:
            continue
        t = tile_count(sizes, band_width, rows)
        if t > (r - 1) * grid and t >= min_fill * r * grid:
            out.append(rows)
    return out


class Ensemble:
    """Independent lattices advanced by one batched launch per iteration."""

    def __init__(self, members, dtype: str = "f32", rows_per_strip: int = 32, band_width: int = 128,
                 device="cuda", rounding: str = "stochastic"):
        """members: (LBMParams, Geometry) or (LBMParams, Geometry, initial psi) tuples.
        ``rounding``: FP16/BF16 store rounding (stochastic by default); member
        k's stochastic-rounding seed is k, its steps use seed + iteration as
        they would when advanced alone."""
        lattices = [Lattice(m[0], m[1], dtype=dtype, device=device, psi0=m[2] if len(m) > 2 else None,
                            rounding=rounding, seed=k)
                    for k, m in enumerate(members)]
        self._attach(lattices, rows_per_strip, band_width)

    @classmethod
    def from_lattices(cls, lattices, rows_per_strip: int = 32, band_width: int = 128) -> "Ensemble":
        """A batch over existing lattices (same packed storage type), in their
        current state: lattices in reference mode enter the fused state here."""
        ens = cls.__new__(cls)
        ens._batch = C.c_void_p()
        ens._attach(list(lattices), rows_per_strip, band_width)
        return ens

    def _attach(self, lattices, rows_per_strip, band_width):
        self.lattices = lattices
        for lat in self.lattices:
            if lat.storage is None:
                raise ValueError("ensembles use packed storage: dtype f32, f16 or bf16")
            lat.enter_fused()
        self.device = self.lattices[0].device
        self.stream = torch.cuda.Stream(device=self.device)
        n = len(self.lattices)
        arr = (L.fd_instance * n)()
        for k, lat in enumerate(self.lattices):
            arr[k] = L.fd_instance(lat.prm, lat.mask.data_ptr(), lat.inlet_ux.data_ptr(),
                                   lat.ppop[lat.pcur].data_ptr(), lat.ppop[1 - lat.pcur].data_ptr(),
                                   lat.side[lat.scur].data_ptr(), lat.side[1 - lat.scur].data_ptr(),
                                   lat.step_seed())
        self._inst = arr
        self._batch = C.c_void_p()
        L.call("fd_batch_create", arr, n, C.byref(self.lattices[0].storage), int(rows_per_strip), int(band_width),
               C.byref(self._batch))
        self.config = (int(band_width), int(rows_per_strip))
        self.cells = sum(lat.H * lat.W for lat in self.lattices)

    @property
    def tiles(self) -> int:
        return L.lib().fd_batch_tiles(self._batch)

    def configure(self, band_width: int, rows_per_strip: int):
        L.call("fd_batch_configure", self._batch, int(rows_per_strip), int(band_width))
        self.config = (int(band_width), int(rows_per_strip))

    def step(self, n: int, use_graph: bool = True):
        """Advance every member n iterations."""
        if n <= 0:
            return
        cur = torch.cuda.current_stream(self.device)
        self.stream.wait_stream(cur)
        L.call("fd_batch_step", self._batch, int(n), int(bool(use_graph)), C.c_void_p(self.stream.cuda_stream))
        cur.wait_stream(self.stream)
        if n % 2:
            for lat in self.lattices:
                lat.pcur ^= 1
                lat.scur ^= 1
        for lat in self.lattices:
            lat.iteration += n

    def time_steps(self, n: int, use_graph: bool = True) -> float:
        """Seconds for n iterations (CUDA events on the batch stream)."""
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(self.device)
        e0.record(self.stream)
        L.call("fd_batch_step", self._batch, int(n), int(bool(use_graph)), C.c_void_p(self.stream.cuda_stream))
        e1.record(self.stream)
        torch.cuda.synchronize(self.device)
        if n % 2:
            for lat in self.lattices:
                lat.pcur ^= 1
                lat.scur ^= 1
        for lat in self.lattices:
            lat.iteration += n
        return e0.elapsed_time(e1) / 1e3

    def _live_sizes(self) -> list:
        """(H, W) of the members the batch still steps (not flagged non-finite)."""
        return [(lat.H, lat.W) for lat, q in zip(self.lattices, self.member_status()) if not q]

    def tiles_for(self, band_width: int, rows_per_strip: int) -> int:
        """Tiles per iteration of the shape (as fd_batch builds them: members
        flagged non-finite are left out)."""
        return tile_count(self._live_sizes(), band_width, rows_per_strip)

    def wave_candidates(self, bands=(64, 128, 256), max_rounds: int = 8, min_fill: float = 0.9) -> list:
        """Shapes whose tile count just fits a whole number of rounds of the
        persistent grid (every CTA takes one tile at a time): for each band
        width and round count r, the shortest strips whose tiles fit in r
        rounds, kept when they fill at least `min_fill` of them.  A tile count
        just over a whole number of rounds leaves a last round in which a few
        CTAs run while the others wait (up to a fifth of the launch)."""
        keep = self.config
        sizes = self._live_sizes()
        out = []
        for band in bands:
            self.configure(band, 64)
            grid = int(L.lib().fd_batch_grid(self._batch))
            if grid > 0:
                out += [(band, rows) for rows in round_filling_rows(sizes, band, grid, max_rounds, min_fill)]
        if keep is not None:
            self.configure(*keep)
        return sorted(set(out))

    def autotune(self, candidates=None, steps: int = 20) -> dict:
        """Time every (band width, rows per strip) candidate on this ensemble
        and keep the fastest; returns {candidate: MLUPS}.  Default candidates:
        a fixed set plus the shapes that fill whole rounds of the grid."""
        if candidates is None:
            candidates = sorted(set(DEFAULT_CANDIDATES) | set(self.wave_candidates()))
        res = {}
        for band, rows in candidates:
            self.configure(band, rows)
            self.time_steps(2)
            t = self.time_steps(steps)
            res[(band, rows)] = self.cells * steps / t / 1e6
        best = max(res, key=res.get)
        self.configure(*best)
        return res

    def diagnostics(self) -> list[dict]:
        return [lat.diagnostics() for lat in self.lattices]

    def member_status(self, clear: bool = False) -> list[bool]:
        """True for every member that met a non-finite density or psi and is
        quarantined: the batch skips its tiles from then on while the others
        keep stepping (include/fdlbm.h fd_batch_member_status).  ``clear``
        releases every member afterwards (restore their states first)."""
        n = len(self.lattices)
        out = (C.c_uint32 * n)()
        r = L.lib().fd_batch_member_status(self._batch, out, int(bool(clear)))
        if r not in (L.FD_OK, L.FD_ERR_NONFINITE):
            raise L.FDError(r, "fd_batch_member_status", L.lib().fd_last_error().decode(errors="replace"))
        return [bool(v) for v in out]

    def close(self):
        if self._batch:
            L.lib().fd_batch_destroy(self._batch)
            self._batch = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
