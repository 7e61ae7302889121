"""Fermi-Dirac entropy of occupations (jrystal/_src/entropy.py:19-54)."""
import torch

from ._ops import as_tensor


def fermi_dirac(occupation, eps: float = 1e-8):
  occ = as_tensor(occupation)
  num_spin, num_k, _ = occ.shape
  top = (3 - num_spin) / num_k
  return -torch.sum(occ * torch.log(eps + occ) + (top - occ) * torch.log(eps + top - occ))
