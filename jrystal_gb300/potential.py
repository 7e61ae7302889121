"""Potentials (jrystal/_src/potential.py)."""
from __future__ import annotations

import numpy as np
import torch

from ._ops import as_tensor, fftn, ifftn
from .xc import xc_density


def _g2(g):
  return torch.sum(g * g, dim=-1)


def hartree_reciprocal(density_grid_reciprocal, g_vector_grid, kohn_sham=False):
  """4 pi rho(G)/|G|^2, 0 at G=0, halved unless kohn_sham (potential.py:24-77)."""
  g = as_tensor(g_vector_grid)
  rho_g = as_tensor(density_grid_reciprocal)
  if rho_g.dim() != g.shape[-1] + 1:
    raise ValueError("density_grid_reciprocal must contains spin axis")
  rho_g = torch.sum(rho_g, dim=0)
  g2 = _g2(g).clone()
  g2[0, 0, 0] = 1.0
  out = rho_g / g2
  out[0, 0, 0] = 0
  out = out * 4 * np.pi
  if kohn_sham:
    out = out.detach()
  else:
    out = out / 2
  return out


def hartree(density_grid_reciprocal, g_vector_grid, kohn_sham=False):
  """Real-space Hartree potential (potential.py:80-118)."""
  rho_g = as_tensor(density_grid_reciprocal)
  return ifftn(hartree_reciprocal(rho_g, g_vector_grid, kohn_sham))


def external_reciprocal(position, charge, g_vector_grid, vol):
  """-(4 pi N/vol) sum_a Z_a exp(-i G.R_a)/(|G|^2 + 1e-10), 0 at G=0 (potential.py:121-166)."""
  g = as_tensor(g_vector_grid)
  pos = as_tensor(position, g.dtype)
  z = as_tensor(charge, g.dtype)
  n = float(np.prod(g.shape[:-1]))
  si = torch.exp(-1j * (g @ pos.T))
  vi = z / (_g2(g)[..., None] + 1e-10)
  vi[0, 0, 0] = 0
  vi = vi * 4 * np.pi
  return -torch.sum(vi * si, dim=-1) * n / vol


def external(position, charge, g_vector_grid, vol):
  """potential.py:169-200."""
  return ifftn(external_reciprocal(position, charge, g_vector_grid, vol))


def effective(density_grid, position, charge, g_vector_grid, vol, split=False,
              xc_type="lda_x", kohn_sham=False):
  """V_H + V_ext + v_xc (potential.py:203-279); split returns the parts."""
  rho = as_tensor(density_grid)
  if rho.dim() == 3:
    rho = rho[None]
  rho_g = fftn(rho)
  v_h = ifftn(hartree_reciprocal(rho_g, g_vector_grid, kohn_sham))
  v_e = ifftn(external_reciprocal(position, charge, g_vector_grid, vol))
  v_xc = xc_density(rho, g_vector_grid, kohn_sham, xc_type)
  if split:
    return v_h, v_e, v_xc
  return v_h[None] + v_e[None] + v_xc
