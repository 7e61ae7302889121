"""Host-side grids: G/R vectors, Monkhorst-Pack k-points, frequency masks and
Ewald translations (jrystal/_src/grid.py).  These run once per geometry on
the host, as in jrystal."""
from __future__ import annotations

import numpy as np

from .const import CUFFT_FACTORS


def fft_factor(n: int) -> int:
  """Smallest tabulated FFT size >= n (jrystal/_src/utils.py:227-254)."""
  if n > 2048:
    raise ValueError(f"The grid number {n} is too large!")
  for v in CUFFT_FACTORS:
    if v >= n:
      return v
  raise ValueError(n)


def proper_grid_size(grid_sizes):
  """jrystal/_src/grid.py:181-210."""
  if hasattr(grid_sizes, "__len__"):
    g = np.array(grid_sizes)
  else:
    try:
      g = np.ones(3, dtype=int) * int(grid_sizes)
    except Exception:
      raise TypeError("mesh should be a scalar, tuple, list or np.array.")
  return np.array([fft_factor(int(i)) for i in g])


def _vector_grid(basis, grid_sizes, normalize=False):
  dim = len(grid_sizes)
  basis = np.asarray(basis, dtype=np.float64)
  out = 0.
  for i in range(dim):
    shape = tuple(grid_sizes[i] if a == i else 1 for a in range(dim)) + (dim,)
    freq = np.fft.fftfreq(grid_sizes[i], 1 if normalize else 1 / grid_sizes[i])
    out = out + np.reshape(np.outer(freq, basis[i]), shape)
  return out


def reciprocal_vectors(cell_vectors):
  return 2 * np.pi * np.linalg.inv(np.asarray(cell_vectors, dtype=np.float64)).T


def g_vectors(cell_vectors, grid_sizes):
  """G vectors in fftfreq order, shape (*grid, 3) (jrystal/_src/grid.py:122-149)."""
  return _vector_grid(reciprocal_vectors(cell_vectors), [int(g) for g in grid_sizes])


def r_vectors(cell_vectors, grid_sizes):
  """jrystal/_src/grid.py:152-178."""
  return _vector_grid(cell_vectors, [int(g) for g in grid_sizes], normalize=True)


def monkhorst_pack(size):
  """Fractional Monkhorst-Pack points (i + 1/2)/n - 1/2, row-major order."""
  size = np.asarray(size)
  idx = np.indices(size).transpose((1, 2, 3, 0)).reshape((-1, 3))
  return (idx + 0.5) / size - 0.5


def k_vectors(cell_vectors, grid_sizes):
  """Cartesian Monkhorst-Pack k-points (jrystal/_src/grid.py:239-262)."""
  return monkhorst_pack(grid_sizes) @ reciprocal_vectors(cell_vectors)


def spherical_mask(cell_vectors, grid_sizes, cutoff_energy):
  """|G|^2/2 <= E_cut (jrystal/_src/grid.py:265-293)."""
  g = g_vectors(cell_vectors, grid_sizes)
  return np.linalg.norm(g, axis=-1)**2 <= cutoff_energy * 2


def cubic_mask(grid_sizes):
  """jrystal/_src/grid.py:296-325."""
  masks = []
  for size in grid_sizes:
    g_max = (size - 1) // 2
    lo, hi = -g_max // 2, g_max // 2
    m = np.ones((size,), dtype=bool)
    m[hi + 1:lo] = False
    masks.append(m)
  return np.einsum("i,j,k->ijk", *masks)


def estimate_max_cutoff_energy(cell_vectors, mask):
  """jrystal/_src/grid.py:328-348."""
  g = g_vectors(cell_vectors, mask.shape)
  return float(np.max(np.linalg.norm(g, axis=-1)**2 / 2 * mask))


def translation_vectors(cell_vectors, cutoff=1e4):
  """Ewald translations (jrystal/_src/grid.py:213-236)."""
  cell_vectors = np.asarray(cell_vectors, dtype=np.float64)
  n = int(np.ceil(cutoff / np.linalg.norm(np.sum(cell_vectors, axis=0))**2))
  return np.reshape(_vector_grid(cell_vectors, [n, n, n]), [-1, 3])


def alias_free_cutoff(cell_vectors, n):
  """Cutoff of the largest alias-free sphere on an n^3 grid:
  1/2 (R/2)^2 with R = (n/2) 2 pi / max_i |a_i|, lowered by one part in 1e9
  so that a G shell lying exactly on that radius is excluded whatever the
  rounding of |G|^2 (Si2 48^3: 5029, Si8 64^3: 17071, Si64 96^3: 57747)."""
  r = (n / 2) * 2 * np.pi / np.max(np.linalg.norm(np.asarray(cell_vectors), axis=1))
  return 0.5 * (r / 2)**2 * (1 - 1e-9)
