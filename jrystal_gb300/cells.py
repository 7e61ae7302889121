"""Random strained cells for trajectory generation and held-out evaluation:
Si diamond (a = 10.26 bohr), C diamond (a = 6.74 bohr) and Al FCC (a = 7.65
bohr, one atom, Z = 13), each lattice vector scaled by U(-3%, +3%)."""
from __future__ import annotations

import numpy as np

from . import grid as _grid
from .workloads import Workload

KINDS = ("si", "c", "al")


def strained_cell(rng, kind=None, grids=(24, 27, 32, 36, 48), bands=(8, 16), kgrid=(2, 2, 2),
                  precision=32, name=None) -> Workload:
  kind = kind or KINDS[rng.integers(0, 3)]
  a = {"si": 10.26, "c": 6.74, "al": 7.65}[kind]
  cell = np.array([[0, a / 2, a / 2], [a / 2, 0, a / 2], [a / 2, a / 2, 0]])
  cell = cell * (1 + rng.uniform(-0.03, 0.03, size=(3, 1)))
  if kind == "al":
    frac, z = np.zeros((1, 3)), np.array([13.0])
  else:
    frac = np.array([[0, 0, 0], [0.25, 0.25, 0.25]])
    z = np.full(2, 14.0 if kind == "si" else 6.0)
  n = int(grids[rng.integers(0, len(grids))])
  nb = int(rng.integers(bands[0], bands[1] + 1))
  return Workload(name or f"{kind}_{n}_{nb}", cell, frac @ cell, z, (n, n, n), kgrid, nb, nb // 2,
                  precision, seed=int(rng.integers(0, 2**31 - 1)))
