"""Small seeded test systems built with the oracle's host setup functions."""
import os

import numpy as np

from oracle import restatement as R

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def fcc_si(a=10.26):
  cell = np.array([[0, a / 2, a / 2], [a / 2, 0, a / 2], [a / 2, a / 2, 0]], dtype=np.float64)
  frac = np.array([[0, 0, 0], [0.25, 0.25, 0.25]])
  return cell, frac @ cell, np.array([14.0, 14.0])


def cubic_si8(a=10.26):
  cell = np.eye(3) * a
  base = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
  frac = np.concatenate([base, base + 0.25])
  return cell, frac @ cell, np.full(8, 14.0)


def diamond():
  c = R.read_xyz(os.path.join(GOLDEN, "diamond.xyz"))
  return c.cell_vectors, c.positions, np.asarray(c.charges, dtype=np.float64)


def make_system(kind="diamond", grid=(12, 12, 12), kgrid=(2, 1, 1), nb=4, nocc=2,
                mask="sphere", xc="lda_x+lda_c_vwn"):
  if kind == "diamond":
    cell, pos, chg = diamond()
  elif kind == "si2":
    cell, pos, chg = fcc_si()
  elif kind == "si8":
    cell, pos, chg = cubic_si8()
  else:
    raise ValueError(kind)
  grid = tuple(grid)
  if mask == "sphere":
    ecut = R.alias_free_cutoff(cell, min(grid))
    m = R.spherical_mask(cell, grid, ecut)
  else:
    m = R.cubic_mask(grid)
  kpts = R.k_vectors(cell, kgrid)
  K = kpts.shape[0]
  occ = R.uniform_occupation(K, 2 * nocc, num_bands=nb)
  return R.System(cell, pos, chg, grid, m, kpts, occ, xc)


def random_params(sysm, seed=0, ns=1, dtype=np.float64):
  rng = np.random.default_rng(seed)
  shape = (ns, sysm.kpts.shape[0], int(sysm.mask.sum()), sysm.occupation.shape[-1])
  return rng.normal(size=shape).astype(dtype), rng.normal(size=shape).astype(dtype)


def nc_tables(sysm, symbols, upf_dir, kpts=None):
  """Norm-conserving pseudopotential tables of a system from the UPF files in
  ``upf_dir``: (container, V_loc(G) grid, dense projector rows
  [k, beta, m, x, y, z], sphere projector table [k, J, G])."""
  from types import SimpleNamespace
  from jrystal_gb300.pseudopotential import NormConservingPseudopotential, local, nloc
  crystal = SimpleNamespace(symbols=list(symbols), positions=sysm.positions, charges=sysm.charges)
  pp = NormConservingPseudopotential.create(crystal, upf_dir)
  g = sysm.g_vector_grid
  k = sysm.kpts if kpts is None else kpts
  vloc = local.potential_local_reciprocal(sysm.positions, g, pp.r_grid, pp.local_potential_grid,
                                          pp.local_potential_charge, sysm.vol)
  dense = nloc.potential_nonlocal_psi_reciprocal(sysm.positions, g, k, pp.r_grid,
                                                 pp.nonlocal_beta_grid,
                                                 pp.nonlocal_angular_momentum,
                                                 pp.nonlocal_d_matrix)
  table = nloc.projector_table(sysm.positions, g, k, sysm.mask, pp.r_grid, pp.nonlocal_beta_grid,
                               pp.nonlocal_angular_momentum, pp.nonlocal_d_matrix)
  return pp, vloc, dense, table


def with_pseudopotential(sysm, vloc, dense, nelec_per_band_pairs=None):
  """A copy of the oracle system with the pseudopotential tables attached."""
  import dataclasses
  return dataclasses.replace(sysm, v_local=vloc, proj=dense)
