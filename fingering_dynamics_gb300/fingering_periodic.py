"""GB300 drop-in for the step API of lattice_boltzmann/fingering_periodic.py.

Same names as the reference module: ``Compute`` (fingering_periodic.py:47-324),
``stream`` (327-343), ``bottom_top_wall`` (354-366) and the module globals
the step reads (fingering_periodic.py:15-44).  ``Compute`` reads this module's
globals when it is constructed, so a driver sets ``H``, ``W``, ``psi_wall``,
... on this module exactly as it would on the reference's.  Arrays are torch
tensors on the GPU (see :mod:`fingering_dynamics_gb300.compute`).
"""
from . import compute as _compute
from .params import periodic_reference_params as _defaults

_d = _defaults()
H = 400
W = 400
MAX_T = 4000
rho0 = 1.0
psi_wall = _d.psi_wall
tau = _d.tau
Eta_n = _d.eta_n
M = _d.M
a = _d.a
kappa = _d.kappa
gamma = _d.gamma
u0 = _d.u0
del _d


class Compute(_compute.ComputeBase):
    """fingering_periodic.py:47-324 (periodic in y, Gaussian inlet, outlet 2/3)."""

    _variant = 0
    _globals = staticmethod(lambda: globals())


stream = _compute.stream
bottom_top_wall = _compute.bottom_top_wall
