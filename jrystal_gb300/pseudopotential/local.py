"""Local part of the norm-conserving pseudopotential
(jrystal/pseudopotential/local.py:32-187).

  V_loc(G) = N / vol sum_a exp(-i G.R_a) [ 4 pi S_0[v_a + z_a / r](|G|)
                                          - 4 pi z_a / |G|^2 ],   V_loc(0) = 0,

with S_0 the numerical l = 0 spherical Bessel transform (kmax = max |G| of
the grid) interpolated by a not-a-knot cubic spline, z_a the valence charge
and v_a the radial local potential in Hartree.  The table replaces the
all-electron Coulomb table of the device plan (same N / vol normalisation),
so the external energy and potential of every entry point become the
reference's energy_local and ifftn(V_loc).
"""
from __future__ import annotations

import numpy as np
import torch
from scipy.interpolate import CubicSpline

from .. import braket
from .._ops import as_tensor, ifftn
from .sbt import sbt


def potential_local_reciprocal(positions, g_vector_grid, r_grid, local_potential_grid,
                               local_potential_charge, vol, fourier_transform_method: str = "sbt"
                               ) -> np.ndarray:
  """Complex (x, y, z) V_loc(G) (local.py:32-132)."""
  if fourier_transform_method != "sbt":
    if fourier_transform_method == "fft":
      raise NotImplementedError("fourier_transform_method='fft' is not implemented; use 'sbt'")
    raise ValueError(f"Invalid fourier transform method: {fourier_transform_method}."
                     "Can only be 'sbt' or 'fft'.")
  g = np.asarray(g_vector_grid, dtype=np.float64)
  pos = np.asarray(positions, dtype=np.float64).reshape(-1, 3)
  gr = np.sqrt(np.sum(g * g, axis=-1))
  n = float(np.prod(g.shape[:-1]))
  kmax = float(np.max(gr))
  zs = np.asarray(local_potential_charge, dtype=np.float64)
  g_safe = gr.copy()
  g_safe[0, 0, 0] = 1e10
  out = np.zeros(g.shape[:-1], dtype=np.complex128)
  for a, (r, v, z) in enumerate(zip(r_grid, local_potential_grid, zs)):
    r = np.asarray(r, dtype=np.float64)
    vp = np.asarray(v, dtype=np.float64) + z / r
    kk, fk = sbt(r, vp[None], l=0, kmax=kmax)
    v1 = CubicSpline(kk, fk[0])(gr) * 4 * np.pi
    va = v1 - 4 * np.pi * z / g_safe ** 2
    va[0, 0, 0] = 0.0
    out += va * np.exp(-1j * (g @ pos[a]))
  return out * n / vol


def hamiltonian_local(wave_grid, potential_local_grid_reciprocal, vol) -> torch.Tensor:
  """<psi_i| v_loc |psi_j> with v_loc = ifftn(V_loc(G)) (local.py:135-160)."""
  v = ifftn(as_tensor(potential_local_grid_reciprocal))
  return braket.expectation(wave_grid, v, vol, diagonal=False, mode="real")


def energy_local(reciprocal_density_grid, potential_local_grid_reciprocal, vol) -> torch.Tensor:
  """reciprocal_braket(V_loc, rho(G), vol) (local.py:163-187)."""
  return braket.reciprocal_braket(potential_local_grid_reciprocal, reciprocal_density_grid, vol)
