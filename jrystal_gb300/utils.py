"""Array utilities (jrystal/_src/utils.py)."""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from ._ops import as_tensor, fftn, safe_real  # noqa: F401
from .grid import fft_factor  # noqa: F401


def absolute_square(array: torch.Tensor) -> torch.Tensor:
  """|z|^2 (utils.py:108-130)."""
  return torch.real(torch.conj(array) * array) if torch.is_complex(array) else array * array


def volume(cell_vectors) -> float:
  """|det(cell)| (utils.py:133-158)."""
  return float(abs(np.linalg.det(np.asarray(cell_vectors if not isinstance(cell_vectors, torch.Tensor)
                                          else cell_vectors.cpu(), dtype=np.float64))))


def wave_to_density(wave_grid: torch.Tensor, occupation=None) -> torch.Tensor:
  """|psi|^2, reduced with the occupation over (kpt, band) (utils.py:161-197)."""
  dens = absolute_square(wave_grid)
  if occupation is not None:
    occ = as_tensor(occupation, dens.dtype)
    if occ.shape != dens.shape[:3]:
      raise ValueError(f"wave_grid's shape ({tuple(wave_grid.shape)}) and occupation's shape "
                       f"({tuple(occ.shape)}) cannot align.")
    dens = torch.einsum("skb...,skb->s...", dens, occ)
  return dens


def wave_to_density_reciprocal(wave_grid: torch.Tensor, occupation=None) -> torch.Tensor:
  """FFT of wave_to_density (utils.py:200-224)."""
  return fftn(wave_to_density(wave_grid, occupation))


def expand_coefficient(coeff_compact: torch.Tensor, mask) -> torch.Tensor:
  """(s,k,g,b) sphere coefficients -> (s,k,b,x,y,z) grid (utils.py:257-281)."""
  mask_t = as_tensor(mask, torch.bool)
  c = torch.swapaxes(coeff_compact, -1, -2)
  out = torch.zeros(c.shape[:-1] + tuple(mask_t.shape), dtype=c.dtype, device=c.device)
  idx = torch.nonzero(mask_t.reshape(-1), as_tuple=False).reshape(-1)
  out.reshape(c.shape[:-1] + (-1,))[..., idx] = c
  return out


def squeeze_coefficient(coeff: torch.Tensor, mask) -> torch.Tensor:
  """(s,k,b,x,y,z) -> (s,k,g,b) at the mask's positions (utils.py:284-308)."""
  mask_t = as_tensor(mask, torch.bool)
  idx = torch.nonzero(mask_t.reshape(-1), as_tuple=False).reshape(-1)
  c = coeff.reshape(coeff.shape[:-3] + (-1,))[..., idx]
  return torch.swapaxes(c, -1, -2)


def check_spin_number(num_electrons: int, spin: int) -> None:
  """utils.py:311-328."""
  if num_electrons % 2 != spin % 2:
    raise ValueError("spin number is not valid for the system. ")
