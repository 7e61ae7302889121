"""torch.autograd binding of the fused energy/gradient entry point."""
from __future__ import annotations

import torch


class DirectMinimizationEnergy(torch.autograd.Function):
  """total energy (kinetic + external + Hartree + xc) of the parameters
  {w_re, w_im}; backward uses the hand-written adjoint of jrg_energy_grad.
  Parameters are real, so the torch and jax cotangent conventions agree."""

  @staticmethod
  def forward(ctx, w_re, w_im, plan, occupation):
    e, gr, gi = plan.energy_and_grad(w_re.detach().contiguous(), w_im.detach().contiguous(),
                                     occupation)
    ctx.save_for_backward(gr, gi)
    return e[4].clone()

  @staticmethod
  def backward(ctx, grad_out):
    gr, gi = ctx.saved_tensors
    return grad_out * gr, grad_out * gi, None, None


def total_energy(w_re, w_im, plan, occupation):
  return DirectMinimizationEnergy.apply(w_re, w_im, plan, occupation)
