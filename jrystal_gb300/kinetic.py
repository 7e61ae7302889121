"""Kinetic operator |G+k|^2/2 (jrystal/_src/kinetic.py:21-44)."""
import torch

from ._ops import as_tensor


def kinetic_operator(g_vector_grid, kpts=None):
  g = as_tensor(g_vector_grid)
  k = torch.zeros((1, 3), dtype=g.dtype, device=g.device) if kpts is None else as_tensor(kpts, g.dtype)
  return torch.sum((g[None] + k[:, None, None, None, :])**2, dim=-1) / 2
