"""Drop-in for lattice_boltzmann/create_block.py (class ``Createblock``)."""
from .geometry import Createblock  # noqa: F401
