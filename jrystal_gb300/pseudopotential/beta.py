"""Beta functions in reciprocal space (jrystal/pseudopotential/beta.py:26-120).

  beta_l(|G+k|) = int beta(r) j_l(|G+k| r) r^2 dr

through the numerical spherical Bessel transform on g = linspace(1e-4,
kmax, 2 n_r) and a not-a-knot cubic spline in g, evaluated at |G+k|.  As in
the reference, kmax is the largest |G+k| over the whole FFT grid and all the
k-points of the call, so the spline nodes (hence the values, to rounding)
match the reference's for the same grid and k-points.
"""
from __future__ import annotations

from typing import List, Optional

import numpy as np
from scipy.interpolate import CubicSpline

from .sbt import sbt


def max_gk_radius(g_vector_grid, kpts=None) -> float:
  """max |G + k| over the grid and the k-points."""
  g = np.asarray(g_vector_grid, dtype=np.float64).reshape(-1, 3)
  ks = np.zeros((1, 3)) if kpts is None else np.asarray(kpts, dtype=np.float64).reshape(-1, 3)
  return float(max(np.sqrt(np.max(np.sum((g + k) ** 2, axis=-1))) for k in ks))


def beta_sbt_radius(r_grid, nonlocal_beta_grid, nonlocal_angular_momentum, radius,
                    kmax: float) -> np.ndarray:
  """beta_i(radius) of one atom: [beta, *radius.shape]."""
  r = np.asarray(r_grid, dtype=np.float64)
  b = np.asarray(nonlocal_beta_grid, dtype=np.float64)
  if len(nonlocal_angular_momentum) != b.shape[0] or r.shape[0] != b.shape[1]:
    raise ValueError("beta grid, angular momenta and r grid do not match")
  if r[0] == 0:
    r, b = r[1:], b[:, 1:]
  k, bk = sbt(r, b, l=[int(x) for x in nonlocal_angular_momentum], kmax=kmax)
  return CubicSpline(k, bk, axis=1)(np.asarray(radius, dtype=np.float64))


def _beta_sbt_single_atom(r_grid, nonlocal_beta_grid, nonlocal_angular_momentum, g_vector_grid,
                          kpts=None) -> np.ndarray:
  """[kpt, beta, x, y, z] (beta.py:26-86)."""
  g = np.asarray(g_vector_grid, dtype=np.float64)
  ks = np.zeros((1, 3)) if kpts is None else np.asarray(kpts, dtype=np.float64).reshape(-1, 3)
  radius = np.sqrt(np.sum((ks[:, None, None, None, :] + g[None]) ** 2, axis=-1))
  out = beta_sbt_radius(r_grid, nonlocal_beta_grid, nonlocal_angular_momentum, radius,
                        float(np.max(radius)))
  return np.swapaxes(out, 0, 1)


def beta_sbt_grid(r_grid: List, nonlocal_beta_grid: List, nonlocal_angular_momentum: List,
                  g_vector_grid, kpts: Optional[np.ndarray] = None) -> List[np.ndarray]:
  """One [kpt, beta, x, y, z] array per atom (beta.py:89-120)."""
  return [_beta_sbt_single_atom(r, b, l, g_vector_grid, kpts)
          for r, b, l in zip(r_grid, nonlocal_beta_grid, nonlocal_angular_momentum)]
