"""Norm-conserving pseudopotentials (jrystal/pseudopotential): UPF reader,
containers, numerical spherical Bessel transform, real spherical harmonics,
the local V_loc(G) table and the beta-projector rows.  The tables are built
once on the host, as the reference builds them, and handed to the device
plan (PlaneWavePlan.set_pseudopotential), whose kernels evaluate the local
and nonlocal energy and gradient terms."""
from . import beta, dataclass, load, local, nloc, normcons, sbt, spherical  # noqa: F401
from .dataclass import NormConservingPseudopotential, Pseudopotential  # noqa: F401

__all__ = ["dataclass", "Pseudopotential", "NormConservingPseudopotential", "local", "load",
           "spherical", "beta", "normcons", "nloc", "sbt"]
