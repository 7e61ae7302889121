"""Named benchmark cells: all-electron silicon in the FCC primitive cell (2
atoms), the conventional cubic cell (8 atoms) and a 2x2x2 supercell (64
atoms), LDA (Slater + VWN), plane-wave sphere = the largest alias-free
sphere of the FFT grid, fixed uniform occupation of the lowest bands."""
from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import grid as _grid


@dataclass
class Workload:
  name: str
  cell: np.ndarray
  positions: np.ndarray
  charges: np.ndarray
  grid_sizes: tuple
  kgrid: tuple
  num_band: int
  num_occ: int                 # doubly occupied bands
  precision: int               # 32 or 64
  seed: int
  lr: float = 1e-2
  steps: int = 200
  xc: str = "lda_x+lda_c_vwn"
  gamma_plus_mp: bool = False  # prepend the Gamma point to the MP grid

  @property
  def cutoff(self):
    return _grid.alias_free_cutoff(self.cell, min(self.grid_sizes))

  @property
  def mask(self):
    return _grid.spherical_mask(self.cell, self.grid_sizes, self.cutoff)

  @property
  def kpts(self):
    k = _grid.k_vectors(self.cell, self.kgrid)
    if self.gamma_plus_mp:
      k = np.concatenate([np.zeros((1, 3)), k])
    return k

  @property
  def num_kpt(self):
    return int(np.prod(self.kgrid)) + (1 if self.gamma_plus_mp else 0)

  @property
  def occupation(self):
    """Uniform occupation 2/K on the lowest num_occ bands (jrystal's
    occupation.uniform with 2*num_occ electrons, spin restricted)."""
    occ = np.zeros((1, self.num_kpt, self.num_band))
    occ[:, :, :self.num_occ] = 2.0 / self.num_kpt
    return occ

  def init_params(self, seed: Optional[int] = None):
    """w_re, w_im ~ N(0, 1) of shape (1, K, n_g, B)."""
    rng = np.random.default_rng(self.seed if seed is None else seed)
    ng = int(self.mask.sum())
    shape = (1, self.num_kpt, ng, self.num_band)
    dt = np.float64 if self.precision == 64 else np.float32
    return rng.standard_normal(shape).astype(dt), rng.standard_normal(shape).astype(dt)


def _diamond_basis():
  base = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
  return np.concatenate([base, base + 0.25])


def si2_fcc(precision=64):
  """Si diamond primitive cell, a = 10.26 bohr, 48^3, MP 2x2x2, 8 bands (4 occupied)."""
  a = 10.26
  cell = np.array([[0, a / 2, a / 2], [a / 2, 0, a / 2], [a / 2, a / 2, 0]])
  pos = np.array([[0, 0, 0], [0.25, 0.25, 0.25]]) @ cell
  return Workload("si2_fcc_48", cell, pos, np.full(2, 14.0), (48, 48, 48), (2, 2, 2), 8, 4,
                  precision, seed=0, lr=1e-2, steps=200)


def si8_cubic(precision=32):
  """Si 8-atom conventional cubic cell, a = 10.26 bohr, 64^3, MP 3x3x3, 24 bands (16 occupied)."""
  a = 10.26
  cell = np.eye(3) * a
  pos = _diamond_basis() @ cell
  return Workload("si8_cubic_64", cell, pos, np.full(8, 14.0), (64, 64, 64), (3, 3, 3), 24, 16,
                  precision, seed=1, lr=1e-2, steps=200)


def si64_supercell(precision=32):
  """Si 64-atom 2x2x2 supercell, a = 20.52 bohr, atoms displaced N(0, 0.02) (seed 4),
  96^3, Gamma + MP 2x2x2, 160 bands (128 occupied)."""
  a = 10.26
  base = _diamond_basis()
  frac = np.concatenate([(base + np.array(s)) / 2 for s in np.ndindex(2, 2, 2)])
  cell = np.eye(3) * 2 * a
  rng = np.random.default_rng(4)
  pos = frac @ cell + rng.normal(0.0, 0.02, size=(64, 3))
  return Workload("si64_supercell_96", cell, pos, np.full(64, 14.0), (96, 96, 96), (2, 2, 2), 160,
                  128, precision, seed=4, lr=1e-2, steps=200, gamma_plus_mp=True)


WORKLOADS = {"si2_fcc_48": si2_fcc, "si8_cubic_64": si8_cubic, "si64_supercell_96": si64_supercell}


def model_pseudopotential(wl: Workload, z_valence: int = 4):
  """Tables of an analytic norm-conserving model pseudopotential on every atom
  of ``wl`` (the timed norm-conserving variant of a workload; the model is not
  fitted to silicon): local V(r) = -z erf(r / 0.8) / r and two Gaussian
  projectors beta_l(r) = r^l exp(-(r / 0.9)^2), l = 0, 1, with D = diag(0.8,
  1.6) Ha, on a logarithmic radial mesh.  Returns (V_loc(G) grid, projector
  table [K, 4 atoms, G]) for PlaneWavePlan.set_pseudopotential."""
  from math import erf
  from .pseudopotential import local, nloc
  r = 1e-3 * np.exp(0.025 * np.arange(450))
  vloc = -z_valence * np.array([erf(x / 0.8) for x in r]) / r
  betas = np.stack([np.exp(-(r / 0.9) ** 2), r * np.exp(-(r / 0.9) ** 2)])
  nat = wl.positions.shape[0]
  g = _grid.g_vectors(wl.cell, wl.grid_sizes)
  vol = float(abs(np.linalg.det(wl.cell)))
  v = local.potential_local_reciprocal(wl.positions, g, [r] * nat, [vloc] * nat, [z_valence] * nat, vol)
  table = nloc.projector_table(wl.positions, g, wl.kpts, wl.mask, [r] * nat, [betas] * nat,
                               [np.array([0, 1])] * nat, [np.diag([0.8, 1.6])] * nat)
  return v, table
