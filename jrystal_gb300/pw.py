"""Plane-wave map (jrystal/_src/pw.py): parameters, orthonormal
coefficients, wave functions and densities on the FFT grid."""
from __future__ import annotations

from typing import Optional

import numpy as np
import torch

from . import plans
from ._ops import as_tensor, fftn, get_precision, ifftn, precision_of, real_dtype, to_numpy
from .grid import g_vectors
from .utils import absolute_square, expand_coefficient, volume


def _generator(key):
  if isinstance(key, torch.Generator):
    return key
  g = torch.Generator(device="cuda")
  g.manual_seed(int(np.asarray(key).reshape(-1)[-1]) if not isinstance(key, int) else key)
  return g


def param_init(key, num_bands: int, num_kpts: int, freq_mask, spin_restricted: bool = True,
               sharding=None) -> dict:
  """Raw parameters {'w_re','w_im'} of shape (spin, kpt, num_g, band), uniform
  in [0, 1) as jrystal draws them (pw.py:29-91, unitary_module.py:84-124).
  ``key`` is an integer seed or a torch.Generator (jax keys are not available)."""
  if sharding is not None:
    raise NotImplementedError("sharding: one GPU per process (pass None)")
  num_spin = 1 if spin_restricted else 2
  num_g = int(np.sum(to_numpy(freq_mask)))
  shape = (num_spin, num_kpts, num_g, num_bands)
  gen = _generator(key)
  dt = real_dtype()
  return {"w_re": torch.rand(shape, generator=gen, device="cuda", dtype=dt),
          "w_im": torch.rand(shape, generator=gen, device="cuda", dtype=dt)}


def _params(pw_param):
  if isinstance(pw_param, dict):
    return as_tensor(pw_param["w_re"]), as_tensor(pw_param["w_im"])
  if isinstance(pw_param, (tuple, list)):
    return as_tensor(pw_param[0]), as_tensor(pw_param[1])
  w = as_tensor(pw_param)
  if torch.is_complex(w):
    return w.real.contiguous(), w.imag.contiguous()
  return w, torch.zeros_like(w)


class _Coeff(torch.autograd.Function):
  """Cholesky QR of the parameters on the device; backward: the library's
  vector-Jacobian product of the map (jrg_coeff_adjoint)."""

  @staticmethod
  def forward(ctx, w_re, w_im, plan):
    w_re, w_im = w_re.detach().contiguous(), w_im.detach().contiguous()
    ctx.save_for_backward(w_re, w_im)
    ctx.plan = plan
    return plan.coeff(w_re, w_im)

  @staticmethod
  def backward(ctx, g):
    w_re, w_im = ctx.saved_tensors
    gr, gi = ctx.plan.coeff_adjoint(w_re, w_im, g)
    return gr, gi, None


def coeff_sphere(pw_param, freq_mask) -> torch.Tensor:
  """Orthonormal sphere coefficients (spin, kpt, num_g, band), Cholesky QR on
  the device (equal to the QR of unitary_module.py:74-80 up to a phase per
  band), differentiable with respect to the parameters."""
  w_re, w_im = _params(pw_param)
  prec = precision_of(w_re)
  w_im = w_im.to(w_re.dtype)
  s, k, g, b = w_re.shape
  plan = plans.mask_plan(to_numpy(freq_mask),
                         k, b, s, prec)
  return _Coeff.apply(w_re, w_im, plan)


def coeff(pw_param, freq_mask, sharding=None) -> torch.Tensor:
  """Orthonormal coefficients on the grid, (spin, kpt, band, x, y, z) (pw.py:94-137)."""
  if sharding is not None:
    raise NotImplementedError("sharding: one GPU per process (pass None)")
  return expand_coefficient(coeff_sphere(pw_param, freq_mask), freq_mask)


def wave_grid(coeff, vol) -> torch.Tensor:
  """IFFT_3(c) * N / sqrt(vol) (pw.py:140-211)."""
  c = as_tensor(coeff)
  n = float(np.prod(c.shape[-3:]))
  return ifftn(c) * (n / np.sqrt(float(vol)))


def density_grid(coeff, vol, occupation=None) -> torch.Tensor:
  """sum_kb f |psi|^2 -> (spin, x, y, z), or per band without occupation (pw.py:214-284)."""
  dens = absolute_square(wave_grid(coeff, vol))
  if occupation is not None:
    occ = as_tensor(occupation, dens.dtype)
    if occ.shape != dens.shape[:3]:
      raise ValueError("Occupation should have a leading dimension that is the same as coeff. "
                       f"Got occupation shape: {tuple(occ.shape)}, coeff shape: {tuple(dens.shape)}")
    dens = torch.einsum("skb...,skb->s...", dens, occ)
  return dens


def density_grid_reciprocal(coeff, vol, occupation=None) -> torch.Tensor:
  """Unnormalised FFT of density_grid (pw.py:287-334)."""
  return fftn(density_grid(coeff, vol, occupation))


def density_from_sphere(coeff_sphere_, freq_mask, occupation) -> torch.Tensor:
  """Occupation-weighted density straight from sphere coefficients (fused
  scatter + FFT + |psi|^2 kernels); the vol factor is not applied, so the
  result equals density_grid(expand_coefficient(c), 1.0, occupation)."""
  c = as_tensor(coeff_sphere_)
  s, k, g, b = c.shape
  plan = plans.mask_plan(to_numpy(freq_mask),
                         k, b, s, precision_of(c))
  return plan.density(c.contiguous(), occupation) * plan.vol


def wave_r(r, coeff, cell_vectors, g_vector_grid=None) -> torch.Tensor:
  """Direct O(G) evaluation at one point (pw.py:337-379)."""
  c = as_tensor(coeff)
  r = as_tensor(r, real_dtype(precision_of(c)))
  if tuple(r.shape) != (3,):
    raise ValueError("r must have shape (3,)")
  vol = volume(cell_vectors)
  if g_vector_grid is None:
    g_vector_grid = g_vectors(to_numpy(cell_vectors), c.shape[-3:])
  g = as_tensor(g_vector_grid, r.dtype)
  phase = torch.exp(1j * (g @ r))
  return torch.einsum("...xyz,xyz->...", c, phase.to(c.dtype)) / np.sqrt(vol)
