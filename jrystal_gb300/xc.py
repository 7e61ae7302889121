"""Exchange-correlation on the grid (jrystal/_src/xc.py:222-253): jax_xc
``lda_x`` / ``lda_c_vwn`` and ``gga_x_pbe`` / ``gga_c_pbe``, unpolarised,
'+'-separated (LDA and PBE terms are not mixed, as in jrystal)."""
from __future__ import annotations

import torch

from ._ops import as_tensor, lda


def xc_density(density_grid, g_vector_grid=None, kohn_sham: bool = False, xc_type: str = "lda_x"):
  """eps_xc(rho) of shape (x,y,z) (kohn_sham=False) or v_xc of shape
  (1,x,y,z) (kohn_sham=True), as jrystal returns them."""
  rho = as_tensor(density_grid)
  if rho.dim() == 4 and rho.shape[0] != 1:
    raise NotImplementedError("spin-polarised LDA is not implemented")
  r = rho[0] if rho.dim() == 4 else rho
  if "gga" in xc_type:
    # PBE needs grad rho: the library's grid path on a plan of this G grid
    if g_vector_grid is None:
      raise ValueError("GGA functionals need g_vector_grid")
    from .plans import field_plan
    from ._ops import get_precision
    plan = field_plan(g_vector_grid, xc_type, get_precision())
    out = plan.potential(r.detach(), kohn_sham=kohn_sham)[2]
    return out[None] if kohn_sham else out
  out = lda(r.detach(), xc_type, kohn_sham)
  return out[None] if kohn_sham else out
