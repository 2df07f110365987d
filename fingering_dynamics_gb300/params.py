"""Model parameters of the two-phase free-energy D2Q9 LBM.

The reference keeps its parameters as module constants derived from physical
inputs (fingering_periodic.py:15-44, fingering.py:16-50) and reads them as
globals at call time.  Here they live in one dataclass, :class:`LBMParams`,
which is also what the C ABI's ``fd_params`` struct is filled from.

Two constructors restate the reference's derivations:

* :func:`periodic_reference_params` - fingering_periodic.py:15-44
* :func:`walls_reference_params` - fingering.py:16-50

and :func:`from_relaxation_times` builds the same parameter set from lattice
quantities (tau of each fluid, interfacial tension, contact angle, inlet
speed), which is how synthetic workloads are specified.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace

import numpy as np

VARIANT_PERIODIC = 0   # fingering_periodic.py: periodic in y, Gaussian inlet, outlet coefficient 2/3
VARIANT_WALLS = 1      # fingering.py: psi_wall ghost rows, wall rows 1 and H-2, plug inlet, corners, 1.5
VARIANT_PERIODIC_XY = 2  # extension: periodic in x and y, body force, no inlet / outlet

_VARIANTS = {"periodic": VARIANT_PERIODIC, "walls": VARIANT_WALLS, "periodic_xy": VARIANT_PERIODIC_XY}


@dataclass
class LBMParams:
    """Lattice-unit parameters of one simulation.

    Field names follow the reference's globals: ``tau`` is the constant
    relaxation time of the order-parameter populations g
    (fingering_periodic.py:26); ``eta_n`` and ``M`` define the harmonic mix
    of kinematic viscosities that gives the f relaxation time
    (fingering_periodic.py:201-208); ``a`` and ``kappa`` are the free-energy
    coefficients (fingering_periodic.py:38-39); ``gamma`` is the mobility in
    the g equilibrium (fingering_periodic.py:163-169); ``psi_wall`` is the
    order parameter written into solid cells (fingering_periodic.py:18,93).
    """
    H: int
    W: int
    variant: str = "periodic"
    tau: float = 1 / (3.0 - math.sqrt(3))
    eta_n: float = 0.0
    M: float = 20.0
    a: float = 0.0
    kappa: float = 0.0
    gamma: float = 0.0
    psi_wall: float = -0.5
    u0: float = 0.0
    outlet_coef: float = 2 / 3
    inlet: str = "gaussian"           # "gaussian" (fingering_periodic.py:270-271) or "plug" (fingering.py:299)
    slab: int = 5                     # psi = +1 on columns [0, slab) at start (fingering_periodic.py:91)
    init_mu: bool = False             # fingering.py:122 computes mu before the equilibria
    init_uy: bool = False             # fingering.py:123 computes u_y (with f = 0) before the equilibria
    inlet_ux: np.ndarray | None = field(default=None, repr=False)
    force_x: float = 0.0              # body force per unit mass, variant "periodic_xy" only
    force_y: float = 0.0
    outlet: str = "velocity"          # "velocity" (the reference's) or "pressure" (rho = 1; an extension)

    def __post_init__(self):
        if self.variant not in _VARIANTS:
            raise ValueError(f"variant must be one of {sorted(_VARIANTS)}")
        if self.outlet not in ("velocity", "pressure"):
            raise ValueError("outlet must be 'velocity' or 'pressure'")
        if self.inlet_ux is None:
            self.inlet_ux = inlet_profile(self.H, self.u0, self.inlet)
        self.inlet_ux = np.ascontiguousarray(self.inlet_ux, dtype=np.float64)
        if self.inlet_ux.shape != (self.H,):
            raise ValueError("inlet_ux must have shape (H,)")

    @property
    def variant_id(self) -> int:
        return _VARIANTS[self.variant]

    def with_size(self, H: int, W: int) -> "LBMParams":
        return replace(self, H=H, W=W, inlet_ux=inlet_profile(H, self.u0, self.inlet))

    def initial_psi(self, solid: np.ndarray) -> np.ndarray:
        """psi = -1, +1 on the inlet slab, psi_wall on solid (fingering_periodic.py:90-93)."""
        psi = np.full((self.H, self.W), -1.0)
        psi[:, :self.slab] = 1.0
        psi[np.asarray(solid, bool)] = self.psi_wall
        return psi


def inlet_profile(H: int, u0: float, kind: str) -> np.ndarray:
    """Inlet u_x per row.

    ``gaussian``: fingering_periodic.py:270-271, evaluated with numpy exactly
    as the reference does (H even).  ``plug``: the constant u0 of
    fingering.py:299.
    """
    if kind == "plug":
        return np.full(H, float(u0))
    if kind == "gaussian":
        if H % 2:
            raise ValueError("the Gaussian inlet profile of the periodic variant needs an even H")
        temp = np.array([i * 3 / (H / 2) for i in range(int(-H / 2), int(H / 2))])
        return u0 * np.exp(- (temp ** 2) / 2)
    raise ValueError(f"unknown inlet profile {kind!r}")


def _derived(tau, C_W, Ca, Eta, R_Nu, rho0, R_sigma, C_rho, xi, u0_rule):
    v0 = (tau - 0.5) / 3
    C_t = v0 / R_Nu * (C_W ** 2)
    Eta_n = Eta / (C_rho * (C_W ** 2) / C_t)
    sigma = R_sigma * (C_t ** 2) / (C_rho * (C_W ** 3))
    u0 = u0_rule(Ca, sigma, rho0, v0, Eta_n)
    kappa = 0.75 * sigma * xi
    a = - 2.0 * kappa / (xi ** 2)
    return Eta_n, sigma, u0, kappa, a


def periodic_reference_params(H: int = 400, W: int = 400, psi_wall: float = -0.5, Pe: float = 15,
                              M: float = 20.0) -> LBMParams:
    """The constant chain of fingering_periodic.py:15-44."""
    tau = 1 / (3.0 - math.sqrt(3))
    Eta_n, sigma, u0, kappa, a = _derived(
        tau, 1.5 * 10 ** (-7), 2.0 * 7.33 * 10 ** (-3), 0.001, 0.001 / 1000, 1.0, 0.045,
        1.0 * 10 ** 3, 2.0, lambda Ca, s, r0, v0, En: Ca * s / (r0 * v0))
    gamma = u0 * 20 / ((-a * Pe) * (tau - 0.5))
    return LBMParams(H=H, W=W, variant="periodic", tau=tau, eta_n=Eta_n, M=M, a=a, kappa=kappa,
                     gamma=gamma, psi_wall=psi_wall, u0=u0, outlet_coef=2 / 3, inlet="gaussian",
                     slab=5)


def walls_reference_params(H: int = 380, W: int = 380, psi_wall: float = -1.0, Pe: float = 400,
                           M: float = 20.0) -> LBMParams:
    """The constant chain of fingering.py:16-50 (gamma uses H, fingering.py:43)."""
    tau = 1 / (3.0 - math.sqrt(3))
    v0 = (tau - 0.5) / 3
    R_Nu = 0.001 / 1000
    C_W = 1.5 * (10 ** (-7))
    C_rho = 1000
    C_t = (v0 / R_Nu) * (C_W ** 2)
    Eta_n = 0.001 * C_t / (C_rho * (C_W ** 2))
    sigma = 0.045 * (C_t ** 2) / (C_rho * (C_W ** 3))
    u0 = 3.0 * 7.33 * (10 ** (-3)) * sigma / Eta_n
    kappa = 0.75 * 2.0 * sigma
    a = - 2.0 * kappa / (2.0 ** 2)
    gamma = u0 * H / ((-a * Pe) * (tau - 0.5))
    return LBMParams(H=H, W=W, variant="walls", tau=tau, eta_n=Eta_n, M=M, a=a, kappa=kappa,
                     gamma=gamma, psi_wall=psi_wall, u0=u0, outlet_coef=1.5, inlet="plug",
                     slab=5, init_mu=True, init_uy=True)


def periodic_xy_params(H: int = 128, W: int = 256, tau_inv: float = 0.6, tau_def: float = 1.0, sigma: float = 1e-3,
                       contact_angle_deg: float = 60.0, force_x: float = 1e-5, gamma: float = 1.0, slab: int = 32,
                       xi: float = 2.0, tau_g: float | None = None) -> LBMParams:
    """The fully periodic, body-force-driven configuration (an extension with
    no reference counterpart: the reference always has a Zou-He inlet and
    outlet and no body force).  Viscosities from the relaxation times as in
    :func:`from_relaxation_times`; kappa, a from sigma (fingering_periodic.py:
    37-39); psi_wall from the contact-angle calibration; the mobility gamma is
    given directly (the reference's rule needs an inlet speed); invading fluid
    on x < slab."""
    from .calibration import psi_wall_for_angle
    tau = (1 / (3.0 - math.sqrt(3))) if tau_g is None else tau_g
    eta_n = (tau_inv - 0.5) / 3.0
    M = (tau_def - 0.5) / (tau_inv - 0.5)
    kappa = 0.75 * sigma * xi
    a = -2.0 * kappa / (xi ** 2)
    return LBMParams(H=H, W=W, variant="periodic_xy", tau=tau, eta_n=eta_n, M=M, a=a, kappa=kappa, gamma=gamma,
                     psi_wall=psi_wall_for_angle(contact_angle_deg), u0=0.0, outlet_coef=2 / 3, inlet="plug",
                     slab=slab, force_x=force_x, force_y=0.0)


def from_relaxation_times(H: int, W: int, tau_inv: float, tau_def: float, sigma: float,
                          contact_angle_deg: float, u_in: float, variant: str = "walls",
                          Pe: float = 15.0, mobility_length: float = 20.0, xi: float = 2.0,
                          tau_g: float | None = None, angle_map: str = "calibrated") -> LBMParams:
    """Parameters from lattice quantities.

    * ``tau_inv`` / ``tau_def``: f relaxation times of the invading (psi=+1)
      and defending (psi=-1) fluid at rho=1.  With the mixing rule of
      fingering_periodic.py:201-208, psi=+1 gives tau = 3*Eta_n + 0.5 and
      psi=-1 gives 3*M*Eta_n + 0.5, so Eta_n = (tau_inv-0.5)/3 and
      M = (tau_def-0.5)/(tau_inv-0.5).
    * ``sigma``: interfacial tension; kappa = 0.75*sigma*xi, a = -2*kappa/xi^2
      (fingering_periodic.py:37-39).
    * mobility: the reference's rule gamma = u0*L/((-a*Pe)*(tau-0.5))
      (fingering_periodic.py:40) with L = ``mobility_length``.
    * contact angle: psi_wall from the droplet calibration table
      (fingering_dynamics_gb300.calibration; theta measured through the
      invading fluid).  The reference sets psi_wall directly and carries no
      angle formula.  ``angle_map="cos"`` uses psi_wall = cos(theta) instead.
    """
    tau = (1 / (3.0 - math.sqrt(3))) if tau_g is None else tau_g
    eta_n = (tau_inv - 0.5) / 3.0
    M = (tau_def - 0.5) / (tau_inv - 0.5)
    kappa = 0.75 * sigma * xi
    a = -2.0 * kappa / (xi ** 2)
    gamma = u_in * mobility_length / ((-a * Pe) * (tau - 0.5))
    if angle_map == "cos":
        psi_wall = math.cos(math.radians(contact_angle_deg))
    else:
        from .calibration import psi_wall_for_angle
        psi_wall = psi_wall_for_angle(contact_angle_deg)
    if variant == "walls":
        return LBMParams(H=H, W=W, variant="walls", tau=tau, eta_n=eta_n, M=M, a=a, kappa=kappa,
                         gamma=gamma, psi_wall=psi_wall, u0=u_in, outlet_coef=1.5, inlet="plug",
                         slab=5, init_mu=True, init_uy=True)
    return LBMParams(H=H, W=W, variant="periodic", tau=tau, eta_n=eta_n, M=M, a=a, kappa=kappa,
                     gamma=gamma, psi_wall=psi_wall, u0=u_in, outlet_coef=2 / 3, inlet="gaussian",
                     slab=5)
