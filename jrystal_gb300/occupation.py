"""Occupations (jrystal/_src/occupation.py): the fixed uniform and gamma
forms used by the direct-minimisation path.  The learnable forms
(idempotent, simplex projector) are not part of the implemented path."""
from __future__ import annotations

from typing import Optional

import torch

from ._ops import real_dtype


def uniform(num_k: int, num_electrons: int, spin: int = 0, num_bands: Optional[int] = None,
            spin_restricted: bool = True) -> torch.Tensor:
  """1/K on the occupied bands of each spin channel (occupation.py:147-190)."""
  num_bands = num_electrons if num_bands is None else num_bands
  occ = torch.zeros((2, num_k, num_bands), dtype=real_dtype(), device="cuda")
  occ[0, :, :(num_electrons + spin) // 2] = 1 / num_k
  occ[1, :, :(num_electrons - spin) // 2] = 1 / num_k
  return occ.sum(0, keepdim=True) if spin_restricted else occ


def gamma(num_k: int, num_electrons: int, spin: int = 0, num_bands: Optional[int] = None,
          spin_restricted: bool = True) -> torch.Tensor:
  """Electrons at the first k-point only (occupation.py:193-237)."""
  num_bands = num_electrons if num_bands is None else num_bands
  occ = torch.zeros((2, num_k, num_bands), dtype=real_dtype(), device="cuda")
  occ[0, 0, :(num_electrons + spin) // 2] = 1
  occ[1, 0, :(num_electrons - spin) // 2] = 1
  return occ.sum(0, keepdim=True) if spin_restricted else occ


_LEARNABLE = ("idempotent", "simplex-projector")


def param_init(key, num_bands: int, num_electrons: int, num_kpts: int, spin: int = 0,
               method: str = "simplex-projector", spin_restricted: bool = True):
  """occupation.py:240-258 for the fixed methods."""
  if method == "uniform":
    return uniform(num_kpts, num_electrons, spin, num_bands, spin_restricted)
  if method == "gamma":
    return gamma(num_kpts, num_electrons, spin, num_bands, spin_restricted)
  if method in _LEARNABLE:
    raise NotImplementedError(f"learnable occupation {method!r} is outside the implemented path")
  raise ValueError(f"Invalid method: {method}")


def occupation(params, num_kpts: int, num_electrons: Optional[int] = None, spin: int = 0,
               method: str = "simplex-projector", spin_restricted: bool = True):
  """Fixed occupations pass through without gradient (occupation.py:261-278)."""
  if method in ("uniform", "gamma"):
    return params.detach() if isinstance(params, torch.Tensor) else params
  if method in _LEARNABLE:
    raise NotImplementedError(f"learnable occupation {method!r} is outside the implemented path")
  raise ValueError(f"Invalid method: {method}")
