"""Spherical coordinates and real spherical harmonics
(jrystal/pseudopotential/spherical.py:28-101).

Conventions of the reference: ``cartesian_to_spherical`` returns
(r, theta = azimuth in [0, 2 pi), phi = polar angle), with r = eps at the
origin (so the origin maps to phi = pi/2, theta = 0).  Complex harmonics
Y_l^m carry the Condon-Shortley phase (scipy's sph_harm_y); the real form
per m in -l..l is

  m > 0:  sqrt2 (-1)^m Re Y_l^m,   m < 0:  sqrt2 (-1)^m Im((-1)^m conj Y_l^m),
  m = 0:  Re Y_l^0.

The associated Legendre functions come from the standard upward recurrence
in l at fixed m (P_m^m = (-1)^m (2m-1)!! (1-x^2)^{m/2},
P_{m+1}^m = x (2m+1) P_m^m, (l-m) P_l^m = x (2l-1) P_{l-1}^m - (l+m-1) P_{l-2}^m).
"""
from __future__ import annotations

from math import factorial

import numpy as np


def cartesian_to_spherical(x, eps: float = 1e-10) -> np.ndarray:
  x = np.asarray(x, dtype=np.float64)
  r = np.linalg.norm(x, axis=-1)
  r = np.where(r == 0.0, eps, r)
  phi = np.arccos(np.clip(x[..., 2] / r, -1.0, 1.0))
  theta = np.mod(np.arctan2(x[..., 1], x[..., 0]) + 2 * np.pi, 2 * np.pi)
  return np.stack((r, theta, phi), axis=-1)


def assoc_legendre(l: int, m: int, x) -> np.ndarray:
  """P_l^m(x) for 0 <= m <= l, Condon-Shortley phase included."""
  x = np.asarray(x, dtype=np.float64)
  s = np.sqrt(np.maximum(0.0, (1.0 - x) * (1.0 + x)))
  pmm = np.ones_like(x)
  odd = 1.0
  for _ in range(m):
    pmm = -pmm * odd * s
    odd += 2.0
  if l == m:
    return pmm
  p1 = x * (2 * m + 1) * pmm
  if l == m + 1:
    return p1
  p0 = pmm
  for ll in range(m + 2, l + 1):
    p0, p1 = p1, (x * (2 * ll - 1) * p1 - (ll + m - 1) * p0) / (ll - m)
  return p1


def sph_harm(l: int, m: int, polar, azimuth) -> np.ndarray:
  """Complex Y_l^m(polar, azimuth) with the Condon-Shortley phase."""
  am = abs(m)
  norm = np.sqrt((2 * l + 1) / (4 * np.pi) * factorial(l - am) / factorial(l + am))
  y = norm * assoc_legendre(l, am, np.cos(polar)) * np.exp(1j * am * np.asarray(azimuth))
  return (-1) ** am * np.conj(y) if m < 0 else y


def batch_sph_harm(l: int, theta, phi) -> np.ndarray:
  """Complex Y_{l,m}, m = -l..l on the last axis (theta azimuth, phi polar)."""
  return np.stack([sph_harm(l, m, phi, theta) for m in range(-l, l + 1)], axis=-1)


def batch_sph_harm_real(l: int, theta, phi) -> np.ndarray:
  """Real harmonics of order l, m = -l..l on the last axis
  (spherical.py:69-86)."""
  y = batch_sph_harm(l, theta, phi)
  m = np.arange(-l, l + 1)
  sgn = (-1.0) ** m
  y2 = np.conj(y) * sgn
  out = np.where(m >= 0, y.real * np.sqrt(2) * sgn, y2.imag * np.sqrt(2) * sgn)
  out[..., l] = y[..., l].real
  return out
