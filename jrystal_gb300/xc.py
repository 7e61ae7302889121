"""LDA exchange-correlation on the grid (jrystal/_src/xc.py:222-253, LDA
branch: jax_xc ``lda_x`` and ``lda_c_vwn`` unpolarised, '+'-separated)."""
from __future__ import annotations

import torch

from ._ops import as_tensor, lda


def xc_density(density_grid, g_vector_grid=None, kohn_sham: bool = False, xc_type: str = "lda_x"):
  """eps_xc(rho) of shape (x,y,z) (kohn_sham=False) or v_xc of shape
  (1,x,y,z) (kohn_sham=True), as jrystal returns them."""
  rho = as_tensor(density_grid)
  if "gga" in xc_type:
    raise NotImplementedError("GGA functionals are outside the implemented LDA path")
  if rho.dim() == 4 and rho.shape[0] != 1:
    raise NotImplementedError("spin-polarised LDA is not implemented")
  r = rho[0] if rho.dim() == 4 else rho
  out = lda(r.detach(), xc_type, kohn_sham)
  return out[None] if kohn_sham else out
