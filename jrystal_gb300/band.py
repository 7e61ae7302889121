"""k-point paths for band structures (jrystal/_src/band/k_path.py:27-62).

jrystal delegates to ASE's ``Cell.bandpath(path, npoints)``
(ase.dft.kpoints, Setyawan-Curtarolo special points).  ASE is not a
dependency here; this module restates the part the band driver uses:

* the special points of the face-centred cubic, body-centred cubic and
  simple cubic lattices, given in the conventional cubic frame in units of
  2 pi / a (G = Gamma);
* a path string such as ``"LGXL"`` or ``"GXWKGLUWLK,UX"`` (a comma starts a
  disconnected segment);
* ``num`` points distributed over the segments in proportion to their
  Cartesian lengths, both ends of each connected path included, the jump
  across a comma given no points.

Point placement along the path may differ from ASE's by rounding; the band
energies at any given k-point do not depend on it.
"""
from __future__ import annotations

from typing import Dict

import numpy as np

# special points in units of 2 pi / a, conventional cubic frame
_SPECIAL = {
  "fcc": {"G": (0, 0, 0), "X": (0, 1, 0), "W": (0.5, 1, 0), "K": (0.75, 0.75, 0),
          "L": (0.5, 0.5, 0.5), "U": (0.25, 1, 0.25)},
  "bcc": {"G": (0, 0, 0), "H": (0, 0, 1), "N": (0.5, 0.5, 0), "P": (0.5, 0.5, 0.5)},
  "cubic": {"G": (0, 0, 0), "X": (0, 0.5, 0), "M": (0.5, 0.5, 0), "R": (0.5, 0.5, 0.5)},
}
_DEFAULT_PATH = {"fcc": "GXWKGLUWLK,UX", "bcc": "GHNGPH,PN", "cubic": "GXMGRX,MR"}


def lattice_frame(cell_vectors):
  """(lattice name, conventional constant a, orthonormal frame rows e_1..e_3)
  of a cubic-family cell given as rows a_1..a_3 (bohr)."""
  a = np.asarray(cell_vectors, dtype=np.float64)
  lens = np.linalg.norm(a, axis=1)
  if not np.allclose(lens, lens[0], rtol=1e-6):
    raise NotImplementedError("k paths: only cubic, fcc and bcc cells are supported")
  cosang = np.array([a[1] @ a[2], a[0] @ a[2], a[0] @ a[1]]) / lens[0] ** 2
  if np.allclose(cosang, 0.0, atol=1e-6):
    return "cubic", lens[0], a / lens[0]
  if np.allclose(cosang, 0.5, atol=1e-6):                  # fcc primitive, 60 degrees
    conv = lens[0] * np.sqrt(2.0)
    e = np.stack([a[1] + a[2] - a[0], a[0] + a[2] - a[1], a[0] + a[1] - a[2]]) / conv
    return "fcc", conv, e
  if np.allclose(np.abs(cosang), 1.0 / 3.0, atol=1e-6):    # bcc primitive, 109.47 degrees
    conv = lens[0] * 2.0 / np.sqrt(3.0)
    e = np.stack([a[1] + a[2], a[0] + a[2], a[0] + a[1]]) / conv
    return "bcc", conv, e
  raise NotImplementedError("k paths: only cubic, fcc and bcc cells are supported")


def special_points(cell_vectors) -> Dict[str, np.ndarray]:
  """Cartesian special points (1/bohr) of the cell's lattice."""
  name, conv, e = lattice_frame(cell_vectors)
  return {k: (2 * np.pi / conv) * (np.asarray(v, dtype=np.float64) @ e)
          for k, v in _SPECIAL[name].items()}


def _segments(path: str):
  out = []
  for part in path.replace(" ", "").split(","):
    labels, i = [], 0
    while i < len(part):
      lab = part[i]
      i += 1
      while i < len(part) and part[i].isdigit():      # labels such as "X1"
        lab += part[i]
        i += 1
      labels.append(lab)
    if labels:
      out.append(labels)
  return out


def get_k_path(cell_vectors, path=None, num: int = 60, fractional: bool = False) -> np.ndarray:
  """k-points along ``path`` (jrystal/_src/band/k_path.py:27-62): Cartesian
  (1/bohr) by default, or fractional coordinates in the reciprocal basis."""
  cell = np.asarray(cell_vectors, dtype=np.float64)
  name, _, _ = lattice_frame(cell)
  pts = special_points(cell)
  segs = _segments(path or _DEFAULT_PATH[name])
  for s in segs:
    for lab in s:
      if lab not in pts:
        raise ValueError(f"unknown special point {lab!r} for a {name} lattice")
  legs = []                                   # (start, end, length)
  for s in segs:
    for p, q in zip(s[:-1], s[1:]):
      legs.append((pts[p], pts[q], float(np.linalg.norm(pts[q] - pts[p]))))
  total = sum(L for _, _, L in legs)
  nends = len(segs)                           # one closing point per connected path
  if num < nends + len(legs):
    raise ValueError("num is too small for this path")
  # points per leg (excluding the leg's end point), proportional to length
  free = num - nends
  raw = np.array([L / total * free if total > 0 else free / len(legs) for _, _, L in legs])
  cnt = np.maximum(1, np.floor(raw).astype(int))
  while cnt.sum() < free:
    cnt[np.argmax(raw - cnt)] += 1
  while cnt.sum() > free:
    cnt[np.argmax(cnt - raw)] -= 1
  kpts, li = [], 0
  for s in segs:
    for _ in range(len(s) - 1):
      a, b, _ = legs[li]
      for t in np.arange(cnt[li]) / cnt[li]:
        kpts.append(a + t * (b - a))
      li += 1
    kpts.append(pts[s[-1]])
  kpts = np.array(kpts)
  if fractional:
    return kpts @ cell.T / (2 * np.pi)
  return kpts
