"""Occupations (jrystal/_src/occupation.py): the fixed uniform and gamma
forms and the learnable simplex-projector and idempotent forms.

The learnable maps act on (S, K, B) numbers; they are evaluated with torch
on the plan's device and differentiated by torch autograd (the occupation
gradient dE/df comes from jrg_energy_grad_bands)."""
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


def simplex_projector_init(num_bands: int, num_kpts: int, device=None) -> dict:
  """occupation.py:281-291: evenly spaced logits (i - n/2) / 10."""
  n = num_bands * num_kpts
  p = ((torch.arange(n, dtype=torch.float64, device=device or "cuda") - n // 2) * 0.1)
  p = p.reshape(num_kpts, num_bands)
  return {"param_up": p.clone(), "param_down": p.clone()}


def proj(x: torch.Tensor, total) -> torch.Tensor:
  """occupation.py:294-343: projection of x in [0,1]^n onto sum(x) = total,
  0 <= x <= 1, by a uniform shift clipped at 0 (push down) or 1 (push up);
  the shift is found from the sorted values (differentiable as jax's is)."""
  n = x.shape[0]
  ar = torch.arange(n, dtype=x.dtype, device=x.device)
  total = torch.as_tensor(total, dtype=x.dtype, device=x.device)
  xsum = x.sum()

  def first_true(mask):
    return torch.argmax(mask.to(torch.int32))

  def pushdown():
    xs, _ = torch.sort(x)
    cs = torch.cumsum(xs, 0)
    rho = (xsum - total - cs) / (n - ar - 1)
    k = first_true(xs > rho)
    lam = torch.where(k == 0, (xsum - total) / n, (xsum - total - cs[k - 1]) / (n - k))
    return torch.clamp(x - lam, min=0.0)

  def pushup():
    xs, _ = torch.sort(x, descending=True)
    cs = torch.cumsum(xs, 0)
    rho = (xsum - total + (ar + 1 - cs)) / (n - ar - 1)
    k = first_true(xs - rho < 1.0)
    lam = torch.where(k == 0, (total - xsum) / n, (total - xsum - (k - cs[k - 1])) / (n - k))
    return torch.clamp(x + lam, max=1.0)

  return torch.where(xsum <= total, pushup(), pushdown())


def simplex_projector(params: dict, num_electrons: int, spin: int = 0,
                      spin_restricted: bool = True) -> torch.Tensor:
  """occupation.py:346-375: sigmoid of the logits projected onto the
  electron-count constraint per spin channel, divided by K."""
  num_kpts, num_bands = params["param_up"].shape
  out = []
  for key, m in (("param_up", (num_electrons + spin) // 2), ("param_down", (num_electrons - spin) // 2)):
    x = torch.sigmoid(params[key]).reshape(-1)
    out.append((proj(x, m * num_kpts) / num_kpts).reshape(num_kpts, num_bands))
  occ = torch.stack(out)
  return occ.sum(0, keepdim=True) if spin_restricted else occ


def idempotent_param_init(key, num_bands: int, num_electrons: int, num_kpts: int, spin: int = 0,
                          spin_restricted: bool = True, device=None) -> dict:
  """occupation.py:27-82: real weights of a (B K) x (n K) orthogonal matrix,
  uniform [0, 1) from the seed ``key`` (an int or a torch.Generator)."""
  gen = key if isinstance(key, torch.Generator) else torch.Generator(device=device or "cuda").manual_seed(int(key))
  dev = gen.device
  n_up, n_down = (num_electrons + spin) // 2, (num_electrons - spin) // 2
  up = {"w_re": torch.rand((num_bands * num_kpts, n_up * num_kpts), generator=gen, device=dev,
                           dtype=torch.float64)}
  if spin_restricted:
    return {"param_up": up, "param_down": up}
  down = {"w_re": torch.rand((num_bands * num_kpts, n_down * num_kpts), generator=gen, device=dev,
                             dtype=torch.float64)}
  return {"param_up": up, "param_down": down}


def idempotent(params: dict, num_kpts: int, spin_restricted: bool = True) -> torch.Tensor:
  """occupation.py:85-144: occupations = row sums of squares of the reduced-QR
  orthogonal factor of each channel's weights, reshaped (K, B), divided by K."""
  def o(p):
    u = torch.linalg.qr(p["w_re"], mode="reduced")[0]
    occ = (u * u).sum(1)
    return occ.reshape(num_kpts, -1)
  up, down = o(params["param_up"]), o(params["param_down"])
  if spin_restricted:
    return (up + down)[None] / num_kpts
  return torch.stack([up, down]) / num_kpts


def param_init(key, num_bands: int, num_electrons: int, num_kpts: int, spin: int = 0,
               method: str = "simplex-projector", spin_restricted: bool = True):
  """occupation.py:240-258."""
  if method == "idempotent":
    return idempotent_param_init(key, num_bands, num_electrons, num_kpts, spin, spin_restricted)
  if method == "uniform":
    return uniform(num_kpts, num_electrons, spin, num_bands, spin_restricted)
  if method == "gamma":
    return gamma(num_kpts, num_electrons, spin, num_bands, spin_restricted)
  if method == "simplex-projector":
    return simplex_projector_init(num_bands, num_kpts)
  raise ValueError(f"Invalid method: {method}")


def occupation(params, num_kpts: int, num_electrons: Optional[int] = None, spin: int = 0,
               method: str = "simplex-projector", spin_restricted: bool = True):
  """occupation.py:261-278; fixed occupations pass through without gradient."""
  if method == "idempotent":
    return idempotent(params, num_kpts, spin_restricted)
  if method in ("uniform", "gamma"):
    return params.detach() if isinstance(params, torch.Tensor) else params
  if method == "simplex-projector":
    return simplex_projector(params, num_electrons, spin, spin_restricted)
  raise ValueError(f"Invalid method: {method}")
