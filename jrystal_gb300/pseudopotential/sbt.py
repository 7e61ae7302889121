"""Numerical spherical Bessel transform (jrystal/sbt/sbt_numerical.py:13-81).

  S_l[f](g) = sum_i f(r_i) j_l(g r_i) r_i^2 dr_i

on the output grid g = linspace(1e-4, kmax, 2 len(r)), with dr_i = r_{i+1} - r_i
(0 for the last point) unless ``delta_r`` is given.  This is the quadrature
the reference's pseudopotential tables are built from; the table values
therefore carry the same discretisation.
"""
from __future__ import annotations

from typing import Optional, Sequence, Tuple, Union

import numpy as np
from scipy.special import spherical_jn


def sbt(r_grid, f_grid, l: Union[int, Sequence[int]], kmax: float,
        delta_r: Optional[np.ndarray] = None) -> Tuple[np.ndarray, np.ndarray]:
  """(g grid, transforms [f, g]); ``l`` is one order for every row of
  ``f_grid`` or one order per row."""
  r = np.asarray(r_grid, dtype=np.float64)
  if delta_r is None:
    dr = np.zeros_like(r)
    dr[:-1] = r[1:] - r[:-1]
  else:
    dr = np.asarray(delta_r, dtype=np.float64)
  g = np.linspace(0.0001, kmax, len(r) * 2)
  gr = g[:, None] * r[None, :]
  f = np.asarray(f_grid, dtype=np.float64)
  w = r * r * dr
  if hasattr(l, "__len__"):
    if f.ndim != 2 or f.shape[0] != len(l):
      raise ValueError("The length of l must be the same as the batch dimension of f_grid")
    out = np.stack([spherical_jn(int(li), gr) @ (fi * w) for li, fi in zip(l, f)])
  elif isinstance(l, (int, np.integer)):
    f = np.atleast_2d(f)
    out = (f * w) @ spherical_jn(int(l), gr).T
  else:
    raise ValueError("'l' must be a integer or a list of int")
  return g, out
