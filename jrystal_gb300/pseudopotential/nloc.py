"""Nonlocal (beta-projector) part of the norm-conserving pseudopotential
(jrystal/pseudopotential/nloc.py).

The projector rows follow potential_nonlocal_psi_reciprocal (nloc.py:42-139):
for atom a, beta b1 and m,

  P[k, (a,b1,m), G] = 4 pi i^{l_b1} exp(-i (G+k).R_a)
                      sum_b2 S[b1,b2] Y_{l_b2, m}(G+k) beta_b2(|G+k|),

S = V sqrt(lambda + 0j) from eigh(D) = V diag(lambda) V^T (eigenvalues in
ascending order), Y the real harmonics padded to 2 l_max + 1 values of m.
F = sum_G c P (c not conjugated) and H_nl = F^H F / vol per band pair
(nloc.py:143-157), so the energy is sum_b f_b / vol sum_{a,b2,m}
|lambda_b2| |x_{a,b2,m}|^2 with x the unmixed projections: for a diagonal D
with entries not in ascending order (the bundled Ge, Ga and As files) the
eigenvalues are paired with other betas than their own, and a negative
D entry counts with its absolute value.  These formulas are kept as they are
here, so results match the reference's for the same files.

projector_table() evaluates the same rows on the plane-wave sphere only and
drops rows that vanish identically (m beyond 2 l + 1); this is the table the
device plan contracts with (jrg_plan_set_pseudopotential).
"""
from __future__ import annotations

from typing import List, Optional

import numpy as np
import torch

from .. import braket
from .._ops import as_tensor, fftn, ifftn
from ..kinetic import kinetic_operator
from .. import potential as _potential
from .. import pw as _pw
from ..utils import wave_to_density
from ..xc import xc_density
from .beta import beta_sbt_radius, max_gk_radius
from .local import energy_local, hamiltonian_local
from .spherical import batch_sph_harm_real, cartesian_to_spherical


def _real_harmonics(gk: np.ndarray, l_max: int) -> np.ndarray:
  """[l, *gk.shape[:-1], 2 l_max + 1] real harmonics of the directions of gk."""
  sph = cartesian_to_spherical(gk)
  theta, phi = sph[..., 1], sph[..., 2]
  y = np.zeros((l_max + 1,) + gk.shape[:-1] + (2 * l_max + 1,), dtype=np.float64)
  for l in range(l_max + 1):
    y[l, ..., :2 * l + 1] = batch_sph_harm_real(l, theta, phi)
  return y


def _atom_rows(pos, gk, y_lm, angmom, dmat, beta_gk) -> np.ndarray:
  """[kpt, beta, m, *points] rows of one atom (nloc.py:108-133).
  gk: [kpt, *points, 3]; y_lm: [l, kpt, *points, M]; beta_gk: [kpt, beta, *points]."""
  angmom = np.asarray(angmom, dtype=np.int64)
  eigval, eigvec = np.linalg.eigh(np.asarray(dmat, dtype=np.float64))
  dsqrt = eigvec * np.sqrt(eigval + 0j)
  y_a = y_lm[angmom]                                        # [b2, kpt, *pts, M]
  y_a = np.moveaxis(y_a, -1, 2)                             # [b2, kpt, M, *pts]
  t = y_a * np.swapaxes(beta_gk, 0, 1)[:, :, None]          # [b2, kpt, M, *pts]
  out = np.tensordot(dsqrt, t, axes=([1], [0]))             # [b1, kpt, M, *pts]
  out = np.swapaxes(out, 0, 1)                              # [kpt, b1, M, *pts]
  sf = np.exp(-1j * (gk @ np.asarray(pos, dtype=np.float64)))   # [kpt, *pts]
  out = out * sf[:, None, None]
  phase = (1j ** angmom).reshape((1, -1, 1) + (1,) * (out.ndim - 3))
  return out * phase * 4 * np.pi


def potential_nonlocal_psi_reciprocal(position, g_vector_grid, kpts, r_grid, nonlocal_beta_grid,
                                      nonlocal_angular_momentum, nonlocal_d_matrix,
                                      beta_gk: Optional[List[np.ndarray]] = None,
                                      fourier_transform_method: str = "sbt",
                                      concat: bool = True):
  """Dense rows <beta_i | G+k>: [kpt, beta, m, x, y, z] (per atom when not
  concat) (nloc.py:42-139)."""
  if fourier_transform_method != "sbt":
    raise NotImplementedError("only fourier_transform_method='sbt' is implemented")
  if len(nonlocal_beta_grid) != len(nonlocal_angular_momentum):
    raise ValueError("one beta grid per atom is required")
  g = np.asarray(g_vector_grid, dtype=np.float64)
  ks = np.asarray(kpts, dtype=np.float64).reshape(-1, 3)
  gk = ks[:, None, None, None, :] + g[None]
  l_max = int(np.max(np.hstack(nonlocal_angular_momentum)))
  y_lm = _real_harmonics(gk, l_max)
  kmax = max_gk_radius(g, ks)
  radius = np.sqrt(np.sum(gk * gk, axis=-1))
  pos = np.asarray(position, dtype=np.float64).reshape(-1, 3)
  out = []
  for a in range(pos.shape[0]):
    if beta_gk is not None:
      bgk = np.asarray(beta_gk[a])
    else:
      bgk = np.swapaxes(beta_sbt_radius(r_grid[a], nonlocal_beta_grid[a],
                                        nonlocal_angular_momentum[a], radius, kmax), 0, 1)
    out.append(_atom_rows(pos[a], gk, y_lm, nonlocal_angular_momentum[a], nonlocal_d_matrix[a],
                          bgk))
  return np.concatenate(out, axis=1) if concat else out


def projector_table(positions, g_vector_grid, kpts, freq_mask, r_grid, nonlocal_beta_grid,
                    nonlocal_angular_momentum, nonlocal_d_matrix, kmax: Optional[float] = None
                    ) -> np.ndarray:
  """[kpt, J, G] rows of potential_nonlocal_psi_reciprocal on the sphere
  points of ``freq_mask`` (row-major mask order), identically-zero rows
  dropped.  ``kmax`` (default: max |G+k| over the grid and ``kpts``) sets the
  spline nodes of the beta transforms."""
  g = np.asarray(g_vector_grid, dtype=np.float64)
  ks = np.asarray(kpts, dtype=np.float64).reshape(-1, 3)
  mask = np.asarray(freq_mask, dtype=bool)
  gs = g[mask]                                            # [G, 3]
  gk = ks[:, None, :] + gs[None]                          # [kpt, G, 3]
  if kmax is None:
    kmax = max_gk_radius(g, ks)
  l_max = int(np.max(np.hstack(nonlocal_angular_momentum)))
  y_lm = _real_harmonics(gk, l_max)
  radius = np.sqrt(np.sum(gk * gk, axis=-1))
  pos = np.asarray(positions, dtype=np.float64).reshape(-1, 3)
  rows = []
  for a in range(pos.shape[0]):
    bgk = np.swapaxes(beta_sbt_radius(r_grid[a], nonlocal_beta_grid[a],
                                      nonlocal_angular_momentum[a], radius, kmax), 0, 1)
    ra = _atom_rows(pos[a], gk, y_lm, nonlocal_angular_momentum[a], nonlocal_d_matrix[a], bgk)
    ra = ra.reshape(ks.shape[0], -1, gs.shape[0])         # [kpt, beta*M, G]
    keep = np.any(ra != 0, axis=(0, 2))
    rows.append(ra[:, keep])
  if not rows:
    return np.zeros((ks.shape[0], 0, gs.shape[0]), dtype=np.complex128)
  return np.ascontiguousarray(np.concatenate(rows, axis=1))


def hamiltonian_nonlocal(pw_coefficients, potential_nl_psi_reciprocal, vol) -> torch.Tensor:
  """H_nl[s,k,b1,b2] = sum_j conj(F_b1j) F_b2j / vol, F = sum_G c P
  (nloc.py:143-157)."""
  c = as_tensor(pw_coefficients)
  p = as_tensor(potential_nl_psi_reciprocal, c.dtype)
  f = torch.einsum("skbxyz,kjmxyz->skbjm", c, p)
  return torch.einsum("skbjm,skcjm->skbc", torch.conj(f), f) / vol


def energy_nonlocal(pw_coefficients, potential_nl_psi_reciprocal, vol, occupation=None):
  """sum_{s,k,b} f_skb H_nl[s,k,b,b] (nloc.py:238-248)."""
  h = hamiltonian_nonlocal(pw_coefficients, potential_nl_psi_reciprocal, vol)
  d = torch.diagonal(h, dim1=-2, dim2=-1)
  occ = as_tensor(occupation, d.real.dtype) if occupation is not None else torch.ones_like(d.real)
  return torch.sum(d * occ).real


def _hartree_xc(hamiltonian_density_grid, g_vector_grid, xc, kohn_sham):
  """V_H and v_xc of the fixed density (nloc.py:213-222)."""
  rho = as_tensor(hamiltonian_density_grid)
  v_h = ifftn(_potential.hartree_reciprocal(fftn(rho), g_vector_grid, kohn_sham=kohn_sham))
  v_xc = xc_density(rho, g_vector_grid, kohn_sham=kohn_sham, xc_type=xc)
  return v_h, v_xc


def hamiltonian_matrix(coefficient, hamiltonian_density_grid, potential_local_grid_reciprocal,
                       potential_nl_psi_reciprocal, g_vector_grid, kpts, vol, xc: str = "lda_x",
                       kohn_sham: bool = True) -> torch.Tensor:
  """H_ij = <psi_i| T + v_loc + V_nl + V_H + v_xc |psi_j> (nloc.py:160-235)."""
  c = as_tensor(coefficient)
  wave = _pw.wave_grid(c, vol)
  ext_nloc = hamiltonian_nonlocal(c, potential_nl_psi_reciprocal, vol)
  ext_loc = hamiltonian_local(wave, potential_local_grid_reciprocal, vol)
  v_h, v_xc = _hartree_xc(hamiltonian_density_grid, g_vector_grid, xc, kohn_sham)
  v_s = v_h + v_xc
  if v_s.dim() == 4 and v_s.shape[0] == 1:
    v_s = v_s[0]
  h_s = braket.expectation(wave, v_s.to(wave.dtype), vol, diagonal=False, mode="real")
  t_kin = kinetic_operator(g_vector_grid, kpts)
  h_kin = braket.expectation(c, t_kin.to(c.dtype), vol, diagonal=False, mode="kinetic")
  return ext_nloc + ext_loc + h_s + h_kin


def hamiltonian_trace(coefficient, hamiltonian_density_grid, potential_local_grid_reciprocal,
                      potential_nl_psi_reciprocal, g_vector_grid, kpts, vol, xc: str = "lda_x",
                      kohn_sham: bool = True) -> torch.Tensor:
  """sum_i <psi_i| H |psi_i> with unit occupations (nloc.py:251-303)."""
  c = as_tensor(coefficient)
  wave = _pw.wave_grid(c, vol)
  occ = torch.ones(wave.shape[:3], dtype=wave.real.dtype, device=wave.device)
  dens = wave_to_density(wave, occ)
  e_nl = energy_nonlocal(c, potential_nl_psi_reciprocal, vol, occ)
  e_loc = energy_local(fftn(dens), potential_local_grid_reciprocal, vol)
  v_h, v_xc = _hartree_xc(hamiltonian_density_grid, g_vector_grid, xc, kohn_sham)
  if v_h.dim() == 4 and v_h.shape[0] == 1:
    v_h = v_h[0]
  if v_xc.dim() == 4 and v_xc.shape[0] == 1:
    v_xc = v_xc[0]
  har = braket.expectation(wave, v_h.to(wave.dtype), vol, diagonal=True, mode="real")
  exc = braket.expectation(wave, v_xc.to(wave.dtype), vol, diagonal=True, mode="real")
  t_kin = kinetic_operator(g_vector_grid, kpts)
  kin = braket.expectation(c, t_kin.to(c.dtype), vol, diagonal=True, mode="kinetic")
  return (e_nl + e_loc + torch.sum(har + exc) + torch.sum(kin)).real
