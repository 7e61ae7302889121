"""Ewald nuclear repulsion, FP64 on the device (jrystal/_src/ewald.py:21-86)."""
from __future__ import annotations

import numpy as np

from . import plans
from ._ops import to_numpy


def _cell_from_g(g_vector_grid):
  g = to_numpy(g_vector_grid)
  b = np.stack([g[1, 0, 0], g[0, 1, 0], g[0, 0, 1]])   # fftfreq index 1 on each axis
  return 2 * np.pi * np.linalg.inv(b).T


def ewald_coulomb_repulsion(positions, charges, g_vector_grid, vol, ewald_eta, ewald_grid,
                            cell_vectors=None, ewald_cutoff=None) -> float:
  """Real-space erfc sum over the translations, reciprocal sum over the FFT
  G grid (as |S(G)|^2), self and background terms.  ``ewald_grid`` must be
  the grid of grid.translation_vectors (n^3 translations)."""
  g = to_numpy(g_vector_grid)
  cell = _cell_from_g(g) if cell_vectors is None else to_numpy(cell_vectors).astype(np.float64)
  n = int(round(np.cbrt(to_numpy(ewald_grid).reshape(-1, 3).shape[0])))
  s2 = float(np.linalg.norm(np.sum(cell, axis=0))**2)
  if ewald_cutoff is None or int(np.ceil(ewald_cutoff / s2)) != n:
    ewald_cutoff = (n - 0.5) * s2                 # same translation count n
  grid = g.shape[:3]
  mask = np.zeros(grid, dtype=bool)
  mask[0, 0, 0] = True
  plan = plans.get_plan(cell, to_numpy(positions).astype(np.float64).reshape(-1, 3),
                        to_numpy(charges).astype(np.float64).reshape(-1), grid, mask,
                        np.zeros((1, 3)), 1, 1, 64)
  return plan.ewald(float(ewald_eta), float(ewald_cutoff))
