"""GB300-native direct-minimisation energy-and-gradient path of jrystal.

The modules keep jrystal's public names and signatures (``pw``, ``energy``,
``potential``, ``kinetic``, ``occupation``, ``hamiltonian``, ``grid``,
``crystal``, ``ewald``, ``entropy``, ``braket``, ``pseudopotential``, ``sbt``)
over a C-ABI CUDA library of
hand-written sm_103a kernels (``libjrystal_gb300.so``).
"""
__version__ = "0.1.0"

from . import (band, braket, calc, crystal, energy, entropy, ewald, grid, hamiltonian,  # noqa
               kinetic, occupation, potential, pseudopotential, pw, sbt, utils, workloads, xc)
from .crystal import Crystal  # noqa: F401
from ._ops import get_precision, set_precision  # noqa: F401
