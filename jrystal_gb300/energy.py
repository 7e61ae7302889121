"""Energy terms (jrystal/_src/energy.py) on dense grids.  The optimiser
loop uses the fused sphere path of :mod:`jrystal_gb300.engine` instead."""
from __future__ import annotations

import numpy as np
import torch

from . import braket, potential, pw
from ._ops import as_tensor, fftn, safe_real, to_numpy
from .ewald import ewald_coulomb_repulsion
from .grid import translation_vectors
from .utils import absolute_square, wave_to_density
from .xc import xc_density


def hartree(density_grid_reciprocal, g_vector_grid, vol, kohn_sham=False):
  """energy.py:29-82."""
  rho_g = as_tensor(density_grid_reciprocal)
  g = as_tensor(g_vector_grid)
  if rho_g.dim() != g.shape[-1] + 1:
    raise AssertionError("density_grid_reciprocal must contains spin axis")
  v = potential.hartree_reciprocal(rho_g, g, kohn_sham)[None]
  return safe_real(braket.reciprocal_braket(v, rho_g, vol))


def external(density_grid_reciprocal, position, charge, g_vector_grid, vol):
  """energy.py:85-135."""
  rho_g = as_tensor(density_grid_reciprocal)
  g = as_tensor(g_vector_grid)
  if rho_g.dim() != g.shape[-1] + 1:
    raise AssertionError("density_grid_reciprocal must contains spin axis")
  v = potential.external_reciprocal(position, charge, g, vol)[None]
  return safe_real(braket.reciprocal_braket(v, rho_g, vol))


def kinetic(g_vector_grid, kpts, coeff_grid, occupation=None):
  """1/2 sum |G+k|^2 |c|^2 (energy.py:138-182)."""
  g = as_tensor(g_vector_grid)
  k = as_tensor(kpts, g.dtype)
  c = as_tensor(coeff_grid)
  ek = torch.sum((g[None] + k[:, None, None, None, :])**2, dim=-1)    # (k,x,y,z)
  e = torch.einsum("kxyz,skbxyz->skb", ek.to(absolute_square(c).dtype), absolute_square(c))
  if occupation is not None:
    return torch.sum(e * as_tensor(occupation, e.dtype)) / 2
  return e / 2


def xc_energy(density_grid, g_vector_grid, vol, xc_type, kohn_sham=False):
  """sum eps_xc(rho) rho vol/N (energy.py:185-211)."""
  rho = as_tensor(density_grid)
  if rho.dim() != 4:
    raise AssertionError("density_grid must contains spin axis")
  num = float(np.prod(rho.shape[-3:]))
  if not kohn_sham:
    # gradient v_xc (LDA and PBE) through the library's potential
    from .xc import xc_energy_grad
    return xc_energy_grad(rho, g_vector_grid, vol, xc_type)
  e = xc_density(rho, g_vector_grid, kohn_sham, xc_type)
  return torch.sum(e * rho) * vol / num


def nuclear_repulsion(position, charge, cell_vectors, g_vector_grid, vol, ewald_eta,
                      ewald_cutoff):
  """Ewald nuclear repulsion, FP64 on the device (energy.py:214-243)."""
  return ewald_coulomb_repulsion(position, charge, g_vector_grid, vol, ewald_eta,
                                 translation_vectors(to_numpy(cell_vectors), ewald_cutoff),
                                 cell_vectors=cell_vectors, ewald_cutoff=ewald_cutoff)


def total_energy(coefficient, position, charge, g_vector_grid, kpts, vol, occupation=None,
                 kohn_sham=False, xc="lda_x", split=False):
  """Kinetic + external + Hartree + xc, no Ewald (energy.py:246-307)."""
  c = as_tensor(coefficient)
  wave = pw.wave_grid(c, vol)
  if occupation is None:
    occupation = torch.ones(c.shape[:3], dtype=wave.real.dtype, device=c.device)
  rho = wave_to_density(wave, occupation)
  rho_g = fftn(rho)
  e_kin = kinetic(g_vector_grid, kpts, c, occupation)
  e_ext = external(rho_g, position, charge, g_vector_grid, vol)
  e_har = hartree(rho_g, g_vector_grid, vol, kohn_sham)
  e_xc = xc_energy(rho, g_vector_grid, vol, xc, kohn_sham)
  if split:
    return e_kin, e_ext, e_har, e_xc
  return e_kin + e_ext + e_har + e_xc


def band_energy(coefficient, position, charge, g_vector_grid, kpts, vol, occupation,
                kohn_sham=False, xc_type="lda_x"):
  """<psi|T + V_eff|psi> per state (energy.py:310-365)."""
  c = as_tensor(coefficient)
  rho_sum = pw.density_grid(c, vol, occupation)
  rho_band = pw.density_grid(c, vol)
  v_eff = potential.effective(rho_sum, position, charge, g_vector_grid, vol, split=False,
                              xc_type=xc_type, kohn_sham=kohn_sham)
  num = float(np.prod(rho_band.shape[-3:]))
  e_eff = torch.einsum("skbxyz,sxyz->skb", rho_band.to(v_eff.dtype), v_eff) * vol / num
  e_kin = kinetic(g_vector_grid, kpts, c)
  return safe_real(e_eff + e_kin)
