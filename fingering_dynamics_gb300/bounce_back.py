"""GB300 drop-in for lattice_boltzmann/bounce_back.py (class ``Bounce_back``)."""
from .compute import Bounce_back  # noqa: F401
