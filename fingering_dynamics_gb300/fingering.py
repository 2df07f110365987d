"""GB300 drop-in for the step API of lattice_boltzmann/fingering.py (walls at
the bottom and top): ``Compute`` (fingering.py:53-390), ``stream``
(393-419), ``bottom_top_wall`` (432-451) and the module globals the step reads
(fingering.py:16-50).  ``Compute`` reads this module's globals when it is
constructed; its initial density is drawn from numpy's global generator as
fingering.py:106-107 does.
"""
from . import compute as _compute
from .params import walls_reference_params as _defaults

_d = _defaults()
H = 380
W = 380
MAX_T = 1000
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
    """fingering.py:53-390 (psi_wall ghost rows, plug inlet, corner nodes, outlet 1.5)."""

    _variant = 1
    _globals = staticmethod(lambda: globals())


stream = _compute.stream
bottom_top_wall = _compute.bottom_top_wall
