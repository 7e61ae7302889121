"""Cache of device plans for the jrystal-compatible functional API."""
from __future__ import annotations

import hashlib

import numpy as np

from .engine import PlaneWavePlan

_CACHE = {}
_MAX = 8


def _key(*parts):
  h = hashlib.sha1()
  for p in parts:
    a = np.ascontiguousarray(np.asarray(p))
    h.update(str(a.dtype).encode())
    h.update(str(a.shape).encode())
    h.update(a.tobytes())
  return h.hexdigest()


def get_plan(cell, positions, charges, grid, mask, kpts, num_band, num_spin, precision,
             xc="lda_x+lda_c_vwn") -> PlaneWavePlan:
  key = _key(cell, positions, charges, grid, mask, kpts, num_band, num_spin, precision,
             np.frombuffer(xc.encode(), dtype=np.uint8))
  plan = _CACHE.get(key)
  if plan is None:
    if len(_CACHE) >= _MAX:
      _CACHE.pop(next(iter(_CACHE))).close()
    plan = PlaneWavePlan(cell, positions, charges, grid, mask, kpts, num_band, num_spin, precision,
                         xc)
    _CACHE[key] = plan
  return plan


def mask_plan(mask, num_kpt, num_band, num_spin, precision) -> PlaneWavePlan:
  """Plan for geometry-free work on a sphere (orthonormalisation, density)."""
  mask = np.asarray(mask, dtype=bool)
  cell = np.diag(np.asarray(mask.shape, dtype=np.float64))
  return get_plan(cell, np.zeros((0, 3)), np.zeros(0), mask.shape, mask, np.zeros((num_kpt, 3)),
                  num_band, num_spin, precision)


def field_plan(g_vector_grid, xc, precision) -> PlaneWavePlan:
  """Plan for grid-only work (potentials, PBE fields) on the cell whose G
  grid is given: the reciprocal vectors are the G vectors of the FFT indices
  (1,0,0), (0,1,0), (0,0,1), and the cell follows as 2 pi B^{-T}."""
  g = np.asarray(g_vector_grid, dtype=np.float64)
  grid = g.shape[:3]
  recip = np.stack([g[1, 0, 0], g[0, 1, 0], g[0, 0, 1]])
  cell = 2.0 * np.pi * np.linalg.inv(recip).T
  mask = np.zeros(grid, dtype=bool)
  mask[0, 0, 0] = True
  return get_plan(cell, np.zeros((0, 3)), np.zeros(0), grid, mask, np.zeros((1, 3)), 1, 1,
                  precision, xc)


def clear():
  for p in _CACHE.values():
    p.close()
  _CACHE.clear()
