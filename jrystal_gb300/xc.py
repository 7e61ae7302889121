"""Exchange-correlation on the grid (jrystal/_src/xc.py:222-253): jax_xc
``lda_x`` / ``lda_c_vwn`` (unpolarised and spin-polarised) and ``gga_x_pbe``
/ ``gga_c_pbe`` (unpolarised), '+'-separated (LDA and PBE terms are not
mixed, as in jrystal)."""
from __future__ import annotations

import torch

from ._ops import as_tensor, lda, lda_eps, lda_eps_pol, lda_pol_raw


def xc_density(density_grid, g_vector_grid=None, kohn_sham: bool = False, xc_type: str = "lda_x"):
  """eps_xc(rho) of shape (x,y,z) (kohn_sham=False) or v_xc of shape
  (S,x,y,z) (kohn_sham=True), as jrystal returns them; a (2,x,y,z) density
  is spin-polarised (LDA only; the Kohn-Sham form is vxc_lda's
  eps + rho_s d eps/d rho_s, xc.py:109-124).  Gradients: the LDA
  eps carries its elementwise derivative; v_xc is taken at a stopped
  density (jrystal/_src/xc.py:234-235, 247-248); the PBE eps has no
  vector-Jacobian product here (energy.xc_energy, whose gradient is v_xc,
  has one), so a density that requires grad is refused there."""
  rho = as_tensor(density_grid)
  if rho.dim() == 4 and rho.shape[0] == 2:
    if "gga" in xc_type:
      raise NotImplementedError("spin-polarised PBE is not implemented")
    return lda_pol_raw(rho.detach(), xc_type, 1) if kohn_sham else lda_eps_pol(rho, xc_type)
  if rho.dim() == 4 and rho.shape[0] != 1:
    raise ValueError("density_grid must have 1 or 2 spin channels")
  r = rho[0] if rho.dim() == 4 else rho
  if "gga" in xc_type:
    # PBE needs grad rho: the library's grid path on a plan of this G grid
    if g_vector_grid is None:
      raise ValueError("GGA functionals need g_vector_grid")
    from .plans import field_plan
    from ._ops import get_precision
    if not kohn_sham and r.requires_grad and torch.is_grad_enabled():
      raise NotImplementedError(
        "the PBE energy density has no gradient here; differentiate energy.xc_energy instead")
    plan = field_plan(g_vector_grid, xc_type, get_precision())
    out = plan.potential(r.detach(), kohn_sham=kohn_sham)[2]
    return out[None] if kohn_sham else out
  if kohn_sham:
    return lda(r, xc_type, True)[None]
  return lda_eps(r, xc_type)


class _XcEnergy(torch.autograd.Function):
  """E_xc = vol/N sum eps_xc(rho) rho with d E_xc / d rho = vol/N v_xc(rho)
  (the Kohn-Sham potential is the functional derivative, LDA and PBE)."""

  @staticmethod
  def forward(ctx, rho, g_vector_grid, vol, xc_type):
    r = rho.detach()
    num = float(r[0].numel())
    eps = xc_density(r, g_vector_grid, False, xc_type)
    ctx.save_for_backward(r)
    ctx.args = (g_vector_grid, float(vol) / num, xc_type)
    return torch.sum(eps * r.sum(0)) * (float(vol) / num)

  @staticmethod
  def backward(ctx, g):
    (r,) = ctx.saved_tensors
    gv, scale, xc_type = ctx.args
    # the functional derivative per channel: d(eps rho)/d rho_s
    v = lda_pol_raw(r, xc_type, 2) if r.shape[0] == 2 else xc_density(r, gv, True, xc_type)
    return g * v * scale, None, None, None


def xc_energy_grad(rho, g_vector_grid, vol, xc_type):
  """Differentiable non-Kohn-Sham exchange-correlation energy of rho (S,x,y,z)."""
  return _XcEnergy.apply(rho, g_vector_grid, vol, xc_type)
