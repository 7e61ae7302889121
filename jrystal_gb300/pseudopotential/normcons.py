"""Norm-conserving pseudopotential for plane waves
(jrystal/pseudopotential/normcons.py): the local and nonlocal functions
under one name."""
from .beta import beta_sbt_grid  # noqa: F401
from .local import energy_local, hamiltonian_local, potential_local_reciprocal  # noqa: F401
from .nloc import (energy_nonlocal, hamiltonian_matrix, hamiltonian_nonlocal,  # noqa: F401
                   hamiltonian_trace, potential_nonlocal_psi_reciprocal, projector_table)
