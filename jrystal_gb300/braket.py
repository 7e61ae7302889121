"""Inner products (jrystal/_src/braket.py)."""
from __future__ import annotations

import numpy as np
import torch

from ._ops import as_tensor


def reciprocal_braket(bra, ket, vol):
  """Parseval-weighted reciprocal inner product, real part (braket.py:27-72)."""
  bra, ket = as_tensor(bra), as_tensor(ket)
  if tuple(bra.shape[-3:]) != tuple(ket.shape[-3:]):
    raise ValueError(f"bra and ket shape are not aligned. Got {tuple(bra.shape)} and "
                     f"{tuple(ket.shape)}.")
  num = float(np.prod(bra.shape))
  prod = torch.sum(torch.conj(bra) * ket) if torch.is_complex(bra) else torch.sum(bra * ket)
  return torch.real(prod) / num * (vol / num)


def real_braket(bra, ket, vol):
  """Real-space inner product (braket.py:75-114)."""
  bra, ket = as_tensor(bra), as_tensor(ket)
  if tuple(bra.shape) != tuple(ket.shape):
    raise ValueError(f"bra and ket shape are not aligned. Got {tuple(bra.shape)} and "
                     f"{tuple(ket.shape)}.")
  num = float(np.prod(bra.shape))
  return torch.sum(bra * ket) * vol / num


def expectation(bra, hamiltonian, vol, ket=None, diagonal=False, mode="real"):
  """<psi_i|H|psi_j> for a diagonal operator on the grid (braket.py:117-206)."""
  bra = as_tensor(bra)
  ket = bra if ket is None else as_tensor(ket)
  h = as_tensor(hamiltonian)
  if bra.dim() != 6 or h.dim() not in (3, 4):
    raise ValueError("bra must be (spin, kpt, band, x, y, z) and the operator 3- or 4-dimensional")
  num = float(np.prod(bra.shape[-3:]))
  factor = {"reciprocal": vol / num / num, "real": vol / num, "kinetic": 1.0}
  if mode not in factor:
    raise ValueError(f"Argument 'mode' must be one of 'real', 'reciprocal', or 'kinetic'. Got {mode}")
  hb = (h[None, None, None] if h.dim() == 3 else h[None, :, None]) * ket
  cb = torch.conj(bra) if torch.is_complex(bra) else bra
  if diagonal:
    out = torch.einsum("skbxyz,skbxyz->skb", cb, hb)
  else:
    out = torch.einsum("skixyz,skjxyz->skij", cb, hb)
  return out * factor[mode]
