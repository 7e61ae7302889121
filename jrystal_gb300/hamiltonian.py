"""Kohn-Sham Hamiltonian in the band basis (jrystal/_src/hamiltonian.py)."""
from __future__ import annotations

import torch

from . import braket, potential, pw
from ._ops import as_tensor
from .kinetic import kinetic_operator


def _parts(band_coefficient, positions, charges, effictive_density_grid, g_vector_grid, kpts, vol,
           xc, kohn_sham, diagonal):
  v_eff = potential.effective(effictive_density_grid, positions, charges, g_vector_grid, vol,
                              False, xc, kohn_sham)
  c = as_tensor(band_coefficient)
  wave = pw.wave_grid(c, vol)
  if v_eff.dim() == 4 and v_eff.shape[0] == 1:
    v_eff = v_eff[0]
  f_eff = braket.expectation(wave, v_eff.to(wave.dtype), vol, diagonal=diagonal, mode="real")
  t_kin = kinetic_operator(g_vector_grid, kpts)
  f_kin = braket.expectation(c, t_kin.to(c.dtype), vol, diagonal=diagonal, mode="kinetic")
  return f_eff + f_kin


def hamiltonian_matrix_trace(band_coefficient, positions, charges, effictive_density_grid,
                             g_vector_grid, kpts, vol, xc="lda_x", kohn_sham=True,
                             keep_kpts_axis=False):
  """sum_i <psi_i|T + V_eff|psi_i> (hamiltonian.py:105-168)."""
  tr = _parts(band_coefficient, positions, charges, effictive_density_grid, g_vector_grid, kpts,
              vol, xc, kohn_sham, True).real
  return torch.sum(tr, dim=(1, 2)) if keep_kpts_axis else torch.sum(tr)


def hamiltonian_matrix(band_coefficient, positions, charges, effictive_density_grid,
                       g_vector_grid, kpts, vol, xc="lda_x", kohn_sham=True):
  """Full H_ij = <psi_i|T + V_eff|psi_j> per (spin, kpt) (hamiltonian.py:171-240);
  jrystal obtains the same matrix as the complex Hessian of the trace."""
  return _parts(band_coefficient, positions, charges, effictive_density_grid, g_vector_grid, kpts,
                vol, xc, kohn_sham, False)
