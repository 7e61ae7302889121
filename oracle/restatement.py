"""FP64 NumPy restatement of jrystal's direct-minimisation path.

TEST INFRASTRUCTURE ONLY: the oracle the CUDA library is checked against.
Product code never imports this module.

Array conventions follow jrystal: parameters ``w_re``/``w_im`` of shape
(spin, kpt, num_g, band); dense coefficient grids (spin, kpt, band, x, y, z);
densities (spin, x, y, z); G vectors in fftfreq order.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

try:  # multi-threaded FFTs for the timed CPU baseline; same transform as np.fft
  import scipy.fft as _sfft
except ImportError:  # pragma: no cover
  _sfft = None

# worker threads of the oracle's FFTs (the CPU baseline raises it)
FFT_WORKERS = 1


def _fftn(x, axes=(-3, -2, -1)):
  if _sfft is not None:
    return _sfft.fftn(x, axes=axes, workers=FFT_WORKERS)
  return np.fft.fftn(x, axes=axes)


def _ifftn(x, axes=(-3, -2, -1)):
  if _sfft is not None:
    return _sfft.ifftn(x, axes=axes, workers=FFT_WORKERS)
  return np.fft.ifftn(x, axes=axes)


# jrystal/_src/const.py:18 (the Angstrom->Bohr factor jrystal applies on read).
ANGSTROM2BOHR = 1.8897259886

_SYMBOLS = (
  "X H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co "
  "Ni Cu Zn Ga Ge As Se Br Kr Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te "
  "I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu Hf Ta W Re Os Ir "
  "Pt Au Hg Tl Pb Bi Po At Rn"
).split()
ATOMIC_NUMBER = {s: i for i, s in enumerate(_SYMBOLS) if i > 0}


# --------------------------------------------------------------------------
# crystal / geometry   (jrystal/_src/crystal.py:124-152, utils.py:133-158)
# --------------------------------------------------------------------------
@dataclass
class Crystal:
  charges: np.ndarray
  positions: np.ndarray       # bohr
  cell_vectors: np.ndarray    # bohr, rows are lattice vectors
  spin: int = 0
  symbols: list = field(default_factory=list)

  @property
  def vol(self):
    return abs(np.linalg.det(self.cell_vectors))

  @property
  def scaled_positions(self):
    return self.positions @ np.linalg.inv(self.cell_vectors).T

  @property
  def reciprocal_vectors(self):
    return 2 * np.pi * np.linalg.inv(self.cell_vectors).T

  @property
  def num_electron(self):
    return int(np.sum(self.charges))


def read_xyz(path: str, spin: Optional[int] = None) -> Crystal:
  """Extended-xyz reader (Lattice="..." header, species + Cartesian Å).

  Follows ``Crystal.create_from_file`` (jrystal/_src/crystal.py:124-152):
  positions and cell in Å times ANGSTROM2BOHR; spin defaults to the parity
  of the electron count (crystal.py:143-145).
  """
  with open(path) as f:
    lines = [ln.rstrip("\n") for ln in f]
  nat = int(lines[0].split()[0])
  header = lines[1]
  i = header.index('Lattice="') + len('Lattice="')
  j = header.index('"', i)
  cell = np.array([float(v) for v in header[i:j].split()]).reshape(3, 3)
  symbols, pos = [], []
  for ln in lines[2:2 + nat]:
    parts = ln.split()
    symbols.append(parts[0])
    pos.append([float(v) for v in parts[1:4]])
  charges = np.array([ATOMIC_NUMBER[s] for s in symbols])
  positions = np.array(pos) * ANGSTROM2BOHR
  cell = cell * ANGSTROM2BOHR
  if spin is None:
    spin = int(np.sum(charges)) % 2
  return Crystal(charges, positions, cell, spin, symbols)


# --------------------------------------------------------------------------
# grids   (jrystal/_src/grid.py, utils.py:227-254)
# --------------------------------------------------------------------------
def fft_sizes(limit: int = 2048):
  """7-smooth sizes up to ``limit`` (the table jrystal/_src/const.py:265)."""
  out = set()
  p2 = 1
  while p2 <= limit:
    p3 = p2
    while p3 <= limit:
      p5 = p3
      while p5 <= limit:
        p7 = p5
        while p7 <= limit:
          out.add(p7)
          p7 *= 7
        p5 *= 5
      p3 *= 3
    p2 *= 2
  return sorted(out)


def fft_factor(n: int) -> int:
  """jrystal/_src/utils.py:227-254."""
  if n > 2048:
    raise ValueError(f"The grid number {n} is too large!")
  for v in fft_sizes():
    if v >= n:
      return v
  raise ValueError(n)


def proper_grid_size(grid_sizes):
  """jrystal/_src/grid.py:181-210."""
  if hasattr(grid_sizes, "__len__"):
    g = np.array(grid_sizes)
  else:
    g = np.ones(3, dtype=int) * int(grid_sizes)
  return np.array([fft_factor(int(i)) for i in g])


def _vector_grid(basis, grid_sizes, normalize=False):
  """jrystal/_src/grid.py:93-119 (fftfreq-ordered lattice combination)."""
  dim = len(grid_sizes)
  out = 0.
  for i in range(dim):
    shape = tuple(grid_sizes[i] if a == i else 1 for a in range(dim)) + (dim,)
    freq = np.fft.fftfreq(grid_sizes[i], 1 if normalize else 1 / grid_sizes[i])
    out = out + np.reshape(np.outer(freq, basis[i]), shape)
  return out


def g_vectors(cell_vectors, grid_sizes):
  """jrystal/_src/grid.py:122-149."""
  b = 2 * np.pi * np.linalg.inv(cell_vectors).T
  return _vector_grid(b, list(grid_sizes))


def r_vectors(cell_vectors, grid_sizes):
  """jrystal/_src/grid.py:152-178."""
  return _vector_grid(np.asarray(cell_vectors), list(grid_sizes), True)


def monkhorst_pack(size):
  """ase.dft.kpoints.monkhorst_pack: fractional (i + 1/2)/n - 1/2."""
  size = np.asarray(size)
  idx = np.indices(size).transpose((1, 2, 3, 0)).reshape((-1, 3))
  return (idx + 0.5) / size - 0.5


def k_vectors(cell_vectors, grid_sizes):
  """jrystal/_src/grid.py:239-262."""
  b = 2 * np.pi * np.linalg.inv(cell_vectors).T
  return monkhorst_pack(grid_sizes) @ b


def spherical_mask(cell_vectors, grid_sizes, cutoff_energy):
  """jrystal/_src/grid.py:265-293."""
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


def translation_vectors(cell_vectors, cutoff=1e4):
  """jrystal/_src/grid.py:213-236."""
  n = int(np.ceil(cutoff / np.linalg.norm(np.sum(cell_vectors, axis=0))**2))
  grid = _vector_grid(np.asarray(cell_vectors), [n, n, n])
  return np.reshape(grid, [-1, 3])


def alias_free_cutoff(cell_vectors, n):
  """Largest alias-free sphere for an n^3 grid: 1/2 (R/2)^2 with
  R = (n/2) 2pi / max|a_i| (the cutoff convention of the benchmark cells)."""
  r = (n / 2) * 2 * np.pi / np.max(np.linalg.norm(cell_vectors, axis=1))
  return 0.5 * (r / 2)**2 * (1 - 1e-9)


# --------------------------------------------------------------------------
# plane-wave map   (jrystal/_src/pw.py, unitary_module.py, utils.py)
# --------------------------------------------------------------------------
def unitary_householder(w_re, w_im):
  """Reduced QR of W = w_re + i w_im over (num_g, band): unitary_module.py:64-80."""
  w = np.asarray(w_re) + 1j * np.asarray(w_im)
  q, _ = np.linalg.qr(w, mode="reduced")
  return q


def cholesky_qr(w_re, w_im):
  """Q = W R^{-1} with R^H R = W^H W (R upper, positive diagonal).

  Equal to the Householder Q of unitary_module.py:74-80 up to a unit-modulus
  phase per column, which every energy term is invariant to.
  """
  w = np.asarray(w_re) + 1j * np.asarray(w_im)
  s = np.einsum("...gi,...gj->...ij", w.conj(), w)
  low = np.linalg.cholesky(s)                # s = L L^H
  r = np.swapaxes(low.conj(), -1, -2)        # R = L^H
  rinv = np.linalg.inv(r)
  return w @ rinv, r


def expand_coefficient(coeff_compact, mask):
  """jrystal/_src/utils.py:257-281: (s,k,g,b) -> (s,k,b,x,y,z)."""
  c = np.swapaxes(coeff_compact, -1, -2)
  out = np.zeros(c.shape[:-1] + mask.shape, dtype=c.dtype)
  out[..., mask] = c
  return out


def squeeze_coefficient(coeff, mask):
  """jrystal/_src/utils.py:284-308: (s,k,b,x,y,z) -> (s,k,g,b)."""
  return np.swapaxes(coeff[..., mask], -1, -2)


def coeff(w_re, w_im, mask):
  """jrystal/_src/pw.py:94-137 (dense grid of orthonormal coefficients)."""
  return expand_coefficient(unitary_householder(w_re, w_im), mask)


def wave_grid(coeff_dense, vol):
  """jrystal/_src/pw.py:140-211: IFFT_3 * N / sqrt(vol)."""
  n = np.prod(coeff_dense.shape[-3:])
  return _ifftn(coeff_dense) * n / np.sqrt(vol)


def wave_r(r, coeff_dense, cell_vectors, g_vector_grid=None):
  """jrystal/_src/pw.py:337-379: direct O(G) evaluation at one point."""
  vol = abs(np.linalg.det(cell_vectors))
  if g_vector_grid is None:
    g_vector_grid = g_vectors(cell_vectors, coeff_dense.shape[-3:])
  phase = np.exp(1j * g_vector_grid @ r)
  return np.einsum("...xyz,xyz->...", coeff_dense, phase) / np.sqrt(vol)


def wave_to_density(wave, occupation=None):
  """jrystal/_src/utils.py:161-197."""
  dens = np.real(np.conj(wave) * wave)
  if occupation is not None:
    dens = np.einsum("skb...,skb->s...", dens, occupation)
  return dens


def density_grid(coeff_dense, vol, occupation=None):
  """jrystal/_src/pw.py:214-284."""
  return wave_to_density(wave_grid(coeff_dense, vol), occupation)


def density_grid_reciprocal(coeff_dense, vol, occupation=None):
  """jrystal/_src/pw.py:287-334 (unnormalised forward FFT)."""
  return _fftn(density_grid(coeff_dense, vol, occupation))


# --------------------------------------------------------------------------
# occupations, entropy   (jrystal/_src/occupation.py, entropy.py)
# --------------------------------------------------------------------------
def uniform_occupation(num_k, num_electrons, spin=0, num_bands=None,
                       spin_restricted=True):
  """jrystal/_src/occupation.py:147-190."""
  num_bands = num_electrons if num_bands is None else num_bands
  occ = np.zeros([2, num_k, num_bands])
  occ[0, :, :(num_electrons + spin) // 2] = 1 / num_k
  occ[1, :, :(num_electrons - spin) // 2] = 1 / num_k
  if spin_restricted:
    return np.sum(occ, axis=0, keepdims=True)
  return occ


def gamma_occupation(num_k, num_electrons, spin=0, num_bands=None,
                     spin_restricted=True):
  """jrystal/_src/occupation.py:193-237."""
  num_bands = num_electrons if num_bands is None else num_bands
  occ = np.zeros([2, num_k, num_bands])
  occ[0, 0, :(num_electrons + spin) // 2] = 1
  occ[1, 0, :(num_electrons - spin) // 2] = 1
  if spin_restricted:
    return np.sum(occ, axis=0, keepdims=True)
  return occ


def simplex_proj(x, total):
  """jrystal/_src/occupation.py:294-343 (push down / push up)."""
  x = np.asarray(x, dtype=np.float64)
  n = x.shape[0]
  ar = np.arange(n)
  xsum = x.sum()
  with np.errstate(divide="ignore", invalid="ignore"):
    if xsum <= total:
      xs = np.sort(x)[::-1]
      cs = np.cumsum(xs)
      rho = (xsum - total + (ar + 1 - cs)) / (n - ar - 1)
      k = int(np.argmax(xs - rho < 1.0))
      lam = (total - xsum) / n if k == 0 else (total - xsum - (k - cs[k - 1])) / (n - k)
      return np.minimum(x + lam, 1.0)
    xs = np.sort(x)
    cs = np.cumsum(xs)
    rho = (xsum - total - cs) / (n - ar - 1)
    k = int(np.argmax(xs > rho))
    lam = (xsum - total) / n if k == 0 else (xsum - total - cs[k - 1]) / (n - k)
    return np.maximum(x - lam, 0.0)


def simplex_projector(param_up, param_down, num_electrons, spin=0, spin_restricted=True):
  """jrystal/_src/occupation.py:346-375."""
  nk, nb = param_up.shape
  out = []
  for p, m in ((param_up, (num_electrons + spin) // 2), (param_down, (num_electrons - spin) // 2)):
    x = 1.0 / (1.0 + np.exp(-np.asarray(p, dtype=np.float64).ravel()))
    out.append((simplex_proj(x, m * nk) / nk).reshape(nk, nb))
  occ = np.stack(out)
  return occ.sum(0, keepdims=True) if spin_restricted else occ


def fermi_dirac_entropy(occ, eps=1e-8):
  """jrystal/_src/entropy.py:19-54."""
  num_spin, num_k, _ = occ.shape
  top = (3 - num_spin) / num_k
  return -np.sum(occ * np.log(eps + occ) + (top - occ) * np.log(eps + top - occ))


# --------------------------------------------------------------------------
# exchange-correlation: jax_xc 0.0.8 lda_x + lda_c_vwn (unpolarised)
# restated from Slater exchange and the VWN (1980) paramagnetic fit.
# --------------------------------------------------------------------------
DENS_THRESHOLD = 1e-15
VWN_A, VWN_B, VWN_C, VWN_X0 = 0.0310907, 3.72744, 12.9352, -0.10498


def lda_x(rho):
  """Slater exchange energy per particle and its potential d(rho e)/d rho."""
  rho = np.asarray(rho, dtype=np.float64)
  ok = rho > DENS_THRESHOLD
  r = np.where(ok, rho, 1.0)
  eps = -0.75 * (3.0 / np.pi)**(1.0 / 3.0) * np.cbrt(r)
  return np.where(ok, eps, 0.0), np.where(ok, 4.0 / 3.0 * eps, 0.0)


def lda_c_vwn(rho):
  """VWN5 paramagnetic correlation energy per particle and potential."""
  rho = np.asarray(rho, dtype=np.float64)
  ok = rho > DENS_THRESHOLD
  r = np.where(ok, rho, 1.0)
  a, b, c, x0 = VWN_A, VWN_B, VWN_C, VWN_X0
  q = math.sqrt(4 * c - b * b)
  xx0 = x0 * x0 + b * x0 + c
  rs = np.cbrt(3.0 / (4.0 * np.pi * r))
  x = np.sqrt(rs)
  xx = x * x + b * x + c
  at = np.arctan(q / (2 * x + b))
  eps = a * (np.log(x * x / xx) + 2 * b / q * at - b * x0 / xx0 *
             (np.log((x - x0)**2 / xx) + 2 * (b + 2 * x0) / q * at))
  den = (2 * x + b)**2 + q * q
  deps_dx = a * (2 / x - (2 * x + b) / xx - 4 * b / den - b * x0 / xx0 *
                 (2 / (x - x0) - (2 * x + b) / xx - 4 * (b + 2 * x0) / den))
  # v = eps + rho d eps/d rho, and rho d/d rho = -(rs/3) d/d rs = -(x/6) d/dx
  v = eps - x / 6.0 * deps_dx
  return np.where(ok, eps, 0.0), np.where(ok, v, 0.0)


# PBE generalised-gradient approximation (Perdew, Burke & Ernzerhof, Phys.
# Rev. Lett. 77, 3865 (1996)), unpolarised, with the libxc parameters that
# jax_xc's gga_x_pbe / gga_c_pbe use: kappa 0.804, mu 0.2195149727645171,
# beta 0.06672455060314922, gamma (1 - ln 2)/pi^2, and the Perdew-Wang 1992
# correlation (Phys. Rev. B 45, 13244) with A = 0.0310907 underneath.
# Written with operations that accept complex arguments, so that exact first
# derivatives come from the complex step f'(x) = Im f(x + i h) / h.
PBE_KAPPA, PBE_MU = 0.804, 0.2195149727645171
PBE_BETA = 0.06672455060314922
PBE_GAMMA = (1.0 - math.log(2.0)) / math.pi**2
PW92_A, PW92_A1 = 0.0310907, 0.21370
PW92_B = (7.5957, 3.5876, 1.6382, 0.49294)


def pw92_c(rho):
  """Perdew-Wang 1992 paramagnetic correlation energy per particle."""
  rs = (3.0 / (4.0 * np.pi * rho))**(1.0 / 3.0)
  srs = np.sqrt(rs)
  b1, b2, b3, b4 = PW92_B
  den = 2.0 * PW92_A * (b1 * srs + b2 * rs + b3 * rs * srs + b4 * rs * rs)
  return -2.0 * PW92_A * (1.0 + PW92_A1 * rs) * np.log(1.0 + 1.0 / den)


def pbe_x(rho, sigma):
  """PBE exchange energy per particle."""
  kf = (3.0 * np.pi**2 * rho)**(1.0 / 3.0)
  s2 = sigma / (4.0 * kf * kf * rho * rho)
  fx = 1.0 + PBE_KAPPA - PBE_KAPPA / (1.0 + PBE_MU * s2 / PBE_KAPPA)
  return -0.75 * (3.0 / np.pi)**(1.0 / 3.0) * rho**(1.0 / 3.0) * fx


def pbe_c(rho, sigma):
  """PBE correlation energy per particle: PW92 + H(r_s, t), phi = 1."""
  ec = pw92_c(rho)
  kf = (3.0 * np.pi**2 * rho)**(1.0 / 3.0)
  ks2 = 4.0 * kf / np.pi
  t2 = sigma / (4.0 * ks2 * rho * rho)
  a = (PBE_BETA / PBE_GAMMA) / (np.exp(-ec / PBE_GAMMA) - 1.0)
  at2 = a * t2
  h = PBE_GAMMA * np.log(1.0 + (PBE_BETA / PBE_GAMMA) * t2 * (1.0 + at2) / (1.0 + at2 + at2 * at2))
  return ec + h


_GGA = {"gga_x_pbe": pbe_x, "gga_c_pbe": pbe_c}


def is_gga(xc_type):
  parts = xc_type.split("+")
  g = [p in _GGA for p in parts]
  if any(g) and not all(g):
    raise NotImplementedError("mixed LDA/GGA functional strings are not supported")
  return all(g)


def gga_f(rho, sigma, xc_type):
  """f = rho * eps(rho, sigma) summed over the parts, 0 below the density
  threshold; with complex-step derivatives f_rho and f_sigma."""
  rho = np.asarray(rho, dtype=np.float64)
  sigma = np.maximum(np.asarray(sigma, dtype=np.float64), 0.0)
  ok = rho > DENS_THRESHOLD
  r = np.where(ok, rho, 1.0)
  sg = np.where(ok, sigma, 0.0)
  h = 1e-40

  def f(rr, ss):
    return rr * sum(_GGA[p](rr, ss) for p in xc_type.split("+"))

  val = f(r.astype(complex), sg.astype(complex)).real
  f_rho = f(r + 1j * h * r, sg.astype(complex)).imag / (h * r)
  f_sig = f(r.astype(complex), sg + 1j * h).imag / h
  return (np.where(ok, val, 0.0), np.where(ok, f_rho, 0.0), np.where(ok, f_sig, 0.0))


def grad_real(x, g_vector_grid):
  """Cartesian gradient of a real grid function by FFT, (3, x, y, z)."""
  xg = _fftn(x)
  return np.stack([np.real(_ifftn(1j * g_vector_grid[..., a] * xg)) for a in range(3)])


def gga_energy_potential(rho, g_vector_grid, vol, xc_type):
  """E_xc = sum f(rho, |grad rho|^2) vol/N and dE_xc/d rho(r) (vol/N units):
  v = f_rho - 2 div(f_sigma grad rho)  (jrystal/_src/xc.py:67-219: the local
  term minus 2 (grad t . grad rho + t lap rho), t = f_sigma)."""
  n = rho.size
  gr = grad_real(rho, g_vector_grid)
  sigma = np.sum(gr * gr, axis=0)
  fval, f_rho, f_sig = gga_f(rho, sigma, xc_type)
  t = np.where(sigma > 0, f_sig, 0.0)
  hg = [_fftn(t * gr[a]) for a in range(3)]
  div = np.real(_ifftn(sum(1j * g_vector_grid[..., a] * hg[a] for a in range(3))))
  return float(np.sum(fval) * vol / n), f_rho - 2.0 * div, fval


_XC = {"lda_x": lda_x, "lda_c_vwn": lda_c_vwn}

# --------------------------------------------------------------------------
# spin-polarised LDA (jrystal/_src/xc.py:40-64, polarised branches).
# Exchange: jrystal applies the unpolarised functional to 2 rho_s and takes
# eps_x = (e_x(2 rho_up) + e_x(2 rho_dn)) / 2 per particle of the TOTAL
# density (xc.py:57-60; xc_energy multiplies by rho_up + rho_dn,
# energy.py:205-211).  Correlation: jax_xc's lda_c_vwn "pol" form, the VWN
# (1980) interpolation between the paramagnetic (P) and ferromagnetic (F)
# fits with the spin-stiffness fit alpha:
#   eps_c = eps_P + alpha f(z) (1 - z^4) / f''(0) + (eps_F - eps_P) f(z) z^4,
#   f(z) = ((1 + z)^(4/3) + (1 - z)^(4/3) - 2) / (2^(4/3) - 2),
#   f''(0) = 4 / (9 (2^(1/3) - 1)),
# each fit A (ln(x^2/X) + 2b/Q atan(Q/(2x+b)) - b x0/X(x0) (ln((x-x0)^2/X)
# + 2(b+2x0)/Q atan(Q/(2x+b)))), x = sqrt(rs), with the published VWN5
# parameters (P above; F: 0.01554535, 7.06042, 18.0578, -0.32500; alpha:
# -1/(6 pi^2), 1.13107, 13.0045, -0.0047584).  Parity unpinned, as the
# unpolarised forms.  Each function returns eps and d eps / d rho_s.
# --------------------------------------------------------------------------
VWN_PARA = (VWN_A, VWN_B, VWN_C, VWN_X0)
VWN_FERRO = (0.01554535, 7.06042, 18.0578, -0.32500)
VWN_STIFF = (-1.0 / (6.0 * np.pi**2), 1.13107, 13.0045, -0.0047584)
VWN_FPP = 4.0 / (9.0 * (2.0**(1.0 / 3.0) - 1.0))


def _vwn_fit(x, a, b, c, x0):
  """One VWN fit F(x) and dF/dx, x = sqrt(rs)."""
  q = math.sqrt(4 * c - b * b)
  xx0 = x0 * x0 + b * x0 + c
  xx = x * x + b * x + c
  at = np.arctan(q / (2 * x + b))
  f = a * (np.log(x * x / xx) + 2 * b / q * at - b * x0 / xx0 *
           (np.log((x - x0)**2 / xx) + 2 * (b + 2 * x0) / q * at))
  den = (2 * x + b)**2 + q * q
  df = a * (2 / x - (2 * x + b) / xx - 4 * b / den - b * x0 / xx0 *
            (2 / (x - x0) - (2 * x + b) / xx - 4 * (b + 2 * x0) / den))
  return f, df


def lda_x_pol(rho_up, rho_dn):
  """Polarised Slater exchange by jrystal's scaling (xc.py:57-60)."""
  eps = np.zeros(np.shape(rho_up))
  ds = []
  for r in (np.asarray(rho_up, np.float64), np.asarray(rho_dn, np.float64)):
    e, _ = lda_x(2.0 * r)
    eps = eps + 0.5 * e
    ok = 2.0 * r > DENS_THRESHOLD
    # d/d rho_s of e_x(2 rho_s)/2 = e_x'(2 rho_s) = e_x(2 rho_s) / (3 * 2 rho_s)
    ds.append(np.where(ok, e / (6.0 * np.where(ok, r, 1.0)), 0.0))
  return eps, ds[0], ds[1]


def lda_c_vwn_pol(rho_up, rho_dn):
  """VWN5 correlation, spin-interpolated (jax_xc lda_c_vwn pol)."""
  up = np.asarray(rho_up, np.float64)
  dn = np.asarray(rho_dn, np.float64)
  rho = up + dn
  ok = rho > DENS_THRESHOLD
  r = np.where(ok, rho, 1.0)
  z = np.clip((up - dn) / r, -1.0, 1.0)
  x = np.sqrt(np.cbrt(3.0 / (4.0 * np.pi * r)))
  ep, dep = _vwn_fit(x, *VWN_PARA)
  ef, def_ = _vwn_fit(x, *VWN_FERRO)
  al, dal = _vwn_fit(x, *VWN_STIFF)
  norm = 2.0**(4.0 / 3.0) - 2.0
  cp, cm = np.cbrt(1.0 + z), np.cbrt(1.0 - z)
  fz = ((1.0 + z) * cp + (1.0 - z) * cm - 2.0) / norm
  dfz = 4.0 / 3.0 * (cp - cm) / norm
  z3 = z**3
  z4 = z3 * z
  eps = ep + al * fz * (1.0 - z4) / VWN_FPP + (ef - ep) * fz * z4
  deps_dx = dep + dal * fz * (1.0 - z4) / VWN_FPP + (def_ - dep) * fz * z4
  deps_dz = (al / VWN_FPP * (dfz * (1.0 - z4) - 4.0 * z3 * fz) +
             (ef - ep) * (dfz * z4 + 4.0 * z3 * fz))
  # rho d/d rho_s = -(x/6) d/dx + (+-1 - z) d/dz   (rs ~ rho^(-1/3), z = (up - dn)/rho)
  t = -x / 6.0 * deps_dx
  d_up = (t + (1.0 - z) * deps_dz) / r
  d_dn = (t - (1.0 + z) * deps_dz) / r
  return (np.where(ok, eps, 0.0), np.where(ok, d_up, 0.0), np.where(ok, d_dn, 0.0))


_XC_POL = {"lda_x": lda_x_pol, "lda_c_vwn": lda_c_vwn_pol}


def xc_eps_pol(rho, xc_type="lda_x"):
  """Polarised sum over the '+'-separated parts: eps (x,y,z) and
  d eps / d rho_s (2,x,y,z) of a (2,x,y,z) density."""
  eps = np.zeros(rho.shape[1:], dtype=np.float64)
  d = np.zeros(rho.shape, dtype=np.float64)
  for name in xc_type.split("+"):
    if name not in _XC_POL:
      raise NotImplementedError(f"polarised xc functional {name!r} is not restated")
    e, du, dd = _XC_POL[name](rho[0], rho[1])
    eps += e
    d[0] += du
    d[1] += dd
  return eps, d


def xc_eps_v(rho, xc_type="lda_x"):
  """Sum over the '+'-separated parts (jrystal/_src/xc.py:242-253)."""
  eps = np.zeros_like(rho, dtype=np.float64)
  v = np.zeros_like(rho, dtype=np.float64)
  for name in xc_type.split("+"):
    if name not in _XC:
      raise NotImplementedError(f"xc functional {name!r} is not restated")
    e, vv = _XC[name](rho)
    eps += e
    v += vv
  return eps, v


def xc_density(density_grid, kohn_sham=False, xc_type="lda_x"):
  """jrystal/_src/xc.py:222-253 (LDA branch).  Polarised, the Kohn-Sham
  form is vxc_lda's (xc.py:109-124): eps + rho_s d eps / d rho_s per spin."""
  if density_grid.shape[0] == 2:
    eps, d = xc_eps_pol(density_grid, xc_type)
    return eps[None] + d * density_grid if kohn_sham else eps
  if density_grid.shape[0] != 1:
    raise ValueError("density_grid must have 1 or 2 spin channels")
  eps, v = xc_eps_v(density_grid[0], xc_type)
  return v[None] if kohn_sham else eps


# --------------------------------------------------------------------------
# potentials and energies   (jrystal/_src/potential.py, energy.py, braket.py)
# --------------------------------------------------------------------------
def _g2_safe(g_vector_grid):
  g2 = np.sum(g_vector_grid**2, axis=-1)
  return g2


def hartree_reciprocal(density_grid_reciprocal, g_vector_grid,
                       kohn_sham=False):
  """jrystal/_src/potential.py:24-77."""
  rho_g = np.sum(density_grid_reciprocal, axis=0)
  g2 = _g2_safe(g_vector_grid).copy()
  g2[0, 0, 0] = 1.0
  out = rho_g / g2
  out[0, 0, 0] = 0.0
  out = out * 4 * np.pi
  if not kohn_sham:
    out = out / 2
  return out


def external_reciprocal(position, charge, g_vector_grid, vol):
  """jrystal/_src/potential.py:121-166."""
  g2 = _g2_safe(g_vector_grid)[..., None]
  si = np.exp(-1j * (g_vector_grid @ np.asarray(position).T))
  num = np.prod(g_vector_grid.shape[:-1])
  vi = np.asarray(charge, dtype=np.float64)[None, None, None] / (g2 + 1e-10)
  vi[0, 0, 0] = 0.0
  vi = vi * 4 * np.pi
  return -np.sum(vi * si, axis=-1) * num / vol


def reciprocal_braket(bra, ket, vol):
  """jrystal/_src/braket.py:27-72."""
  num = np.prod(bra.shape)
  return (np.sum(np.conj(bra) * ket) / num * vol / num).real


def real_braket(bra, ket, vol):
  """jrystal/_src/braket.py:75-114."""
  num = np.prod(bra.shape)
  return np.sum(bra * ket) * vol / num


def expectation(bra, hamiltonian, vol, diagonal=True, mode="real"):
  """jrystal/_src/braket.py:117-206 (diagonal=True/False, 3/4-dim operator)."""
  num = np.prod(bra.shape[-3:])
  factor = {"real": vol / num, "reciprocal": vol / num / num,
            "kinetic": 1.0}[mode]
  h = hamiltonian if hamiltonian.ndim == 4 else hamiltonian[None]
  hb = h[None, :, None] * bra                   # (s,k,b,x,y,z)
  if diagonal:
    out = np.einsum("skbxyz,skbxyz->skb", np.conj(bra), hb)
  else:
    out = np.einsum("skixyz,skjxyz->skij", np.conj(bra), hb)
  return out * factor


def hartree_energy(density_grid_reciprocal, g_vector_grid, vol,
                   kohn_sham=False):
  """jrystal/_src/energy.py:29-82."""
  v = hartree_reciprocal(density_grid_reciprocal, g_vector_grid, kohn_sham)
  return reciprocal_braket(v[None], density_grid_reciprocal, vol)


def external_energy(density_grid_reciprocal, position, charge, g_vector_grid,
                    vol):
  """jrystal/_src/energy.py:85-135."""
  v = external_reciprocal(position, charge, g_vector_grid, vol)
  return reciprocal_braket(v[None], density_grid_reciprocal, vol)


def kinetic_operator(g_vector_grid, kpts=None):
  """jrystal/_src/kinetic.py:21-44."""
  kpts = np.zeros([1, 3]) if kpts is None else np.asarray(kpts)
  return np.sum((g_vector_grid[None] + kpts[:, None, None, None])**2,
                axis=-1) / 2


def kinetic_energy(g_vector_grid, kpts, coeff_dense, occupation=None):
  """jrystal/_src/energy.py:138-182."""
  ek = 2 * kinetic_operator(g_vector_grid, kpts)           # (k,x,y,z)
  e = np.einsum("kxyz,skbxyz->skb", ek, np.abs(coeff_dense)**2)
  if occupation is not None:
    return np.sum(e * occupation) / 2
  return e / 2


def xc_energy(density_grid, vol, xc_type="lda_x", kohn_sham=False):
  """jrystal/_src/energy.py:185-211."""
  num = np.prod(density_grid.shape[-3:])
  e = xc_density(density_grid, kohn_sham, xc_type)
  return np.sum(e * density_grid) * vol / num


def effective(density_grid, position, charge, g_vector_grid, vol,
              split=False, xc_type="lda_x", kohn_sham=False):
  """jrystal/_src/potential.py:203-279."""
  if density_grid.ndim == 3:
    density_grid = density_grid[None]
  rho_g = _fftn(density_grid)
  v_h = _ifftn(hartree_reciprocal(rho_g, g_vector_grid, kohn_sham))
  v_e = _ifftn(external_reciprocal(position, charge, g_vector_grid, vol))
  v_xc = xc_density(density_grid, kohn_sham, xc_type)
  if split:
    return v_h, v_e, v_xc
  return v_h[None] + v_e[None] + v_xc


def total_energy(coeff_dense, position, charge, g_vector_grid, kpts, vol,
                 occupation=None, kohn_sham=False, xc="lda_x", split=False):
  """jrystal/_src/energy.py:246-307 (no Ewald term)."""
  wave = wave_grid(coeff_dense, vol)
  if occupation is None:
    occupation = np.ones(coeff_dense.shape[:3])
  rho = wave_to_density(wave, occupation)
  rho_g = _fftn(rho)
  e_kin = kinetic_energy(g_vector_grid, kpts, coeff_dense, occupation)
  e_ext = external_energy(rho_g, position, charge, g_vector_grid, vol)
  e_har = hartree_energy(rho_g, g_vector_grid, vol, kohn_sham)
  e_xc = xc_energy(rho, vol, xc, kohn_sham)
  if split:
    return e_kin, e_ext, e_har, e_xc
  return e_kin + e_ext + e_har + e_xc


def hamiltonian_matrix_trace(coeff_dense, position, charge, density_grid,
                             g_vector_grid, kpts, vol, xc="lda_x",
                             kohn_sham=True, keep_kpts_axis=False):
  """jrystal/_src/hamiltonian.py:105-168."""
  v_eff = effective(density_grid, position, charge, g_vector_grid, vol,
                    False, xc, kohn_sham)
  wave = wave_grid(coeff_dense, vol)
  f_eff = expectation(wave, v_eff, vol, diagonal=True, mode="real")
  t_kin = kinetic_operator(g_vector_grid, kpts)
  f_kin = expectation(coeff_dense, t_kin, vol, diagonal=True, mode="kinetic")
  tr = (f_eff + f_kin).real
  return np.sum(tr, axis=(1, 2)) if keep_kpts_axis else np.sum(tr)


def hamiltonian_matrix(coeff_dense, position, charge, density_grid,
                       g_vector_grid, kpts, vol, xc="lda_x", kohn_sham=True):
  """jrystal/_src/hamiltonian.py:171-240: H_ij = <psi_i|T + V_eff|psi_j> per
  (spin, kpt).  jrystal forms it as the complex Hessian of half the trace of
  a single combined band; for an operator independent of the coefficients
  that is the matrix of T + V_eff in the band basis, formed here directly."""
  v_eff = effective(density_grid, position, charge, g_vector_grid, vol,
                    False, xc, kohn_sham)
  wave = wave_grid(coeff_dense, vol)
  f_eff = expectation(wave, v_eff, vol, diagonal=False, mode="real")
  t_kin = kinetic_operator(g_vector_grid, kpts)
  f_kin = expectation(coeff_dense, t_kin, vol, diagonal=False, mode="kinetic")
  return f_eff + f_kin


def band_trace_terms(w_re, w_im, v_eff, sysm, weights=None, with_grad=True):
  """Band-structure objective for a fixed effective potential
  (calc/calc_band_structure_all_electrons.py:78-92 with
  hamiltonian_matrix_trace, kohn_sham=True): trace = sum w <psi|T+V|psi>,
  its kinetic part, the weighted band Hamiltonian A_ij = w_j <psi_i|H|psi_j>
  and d trace / d {w_re, w_im} through the same orthonormalisation adjoint as
  energy_terms (g_C = w (T c + sqrt(vol)/N FFT(V psi))|_sphere).  v_eff is
  one grid or one per spin channel (the bands of spin s see grid s)."""
  vol = sysm.vol
  gvec = sysm.g_vector_grid
  mask = sysm.mask
  n = np.prod(sysm.grid)
  c, r = cholesky_qr(w_re, w_im)                  # (s,k,g,b)
  if weights is None:
    weights = np.ones(c.shape[:2] + c.shape[-1:])
  dense = expand_coefficient(c, mask)
  wave = _ifftn(dense) * n / np.sqrt(vol)
  v = np.asarray(v_eff).reshape((-1,) + tuple(sysm.grid))      # (1 or S, x, y, z)
  hpsi = _fftn(v[:, None, None] * wave)[..., mask] * (np.sqrt(vol) / n)
  tk = kinetic_operator(gvec, sysm.kpts)[:, mask]  # (k,g)
  hc = tk[None, :, None, :] * np.swapaxes(c, -1, -2) + hpsi   # (s,k,b,g) = H c_b
  if sysm.proj is not None:      # + V_nl c_b (nloc.py:251-303)
    hc = hc + _nonlocal_grad_c(dense, sysm.proj, vol, np.ones(weights.shape), mask)
  g_c = np.swapaxes(weights[..., None] * hc, -1, -2)          # (s,k,g,b)
  a = np.einsum("...gi,...gj->...ij", c.conj(), g_c)
  kin = np.sum(weights * np.einsum("kg,skgb->skb", tk, np.abs(c)**2))
  out = dict(trace=float(np.sum(np.einsum("...ii->...i", a).real)), kinetic=float(kin), hmat=a)
  if not with_grad:
    return out
  up = np.triu(a, 1)
  kmat = up + np.swapaxes(up.conj(), -1, -2)
  kmat = kmat + np.einsum("...ii->...i", a).real[..., None] * np.eye(a.shape[-1])
  rinv_h = np.swapaxes(np.linalg.inv(r).conj(), -1, -2)
  g_w = (g_c - c @ kmat) @ rinv_h
  out["grad_re"], out["grad_im"] = 2 * g_w.real, 2 * g_w.imag
  return out


def plane_wave_hamiltonian(v_eff, sysm, k_index):
  """Full Hamiltonian of one k-point in the sphere basis:
  H[G, G'] = |G+k|^2/2 delta_GG' + V(G - G'), V(G) = (1/N) sum_r V(r) e^{-iG.r},
  in the normalisation of braket.expectation (real mode) and the kinetic
  mode; its lowest eigenvalues are what the band-structure minimisation
  converges to."""
  v = np.asarray(v_eff).reshape(sysm.grid)
  vg = np.fft.fftn(v) / np.prod(sysm.grid)
  idx = np.argwhere(sysm.mask)                    # (g, 3) FFT indices, row-major mask order
  d = (idx[:, None, :] - idx[None, :, :]) % np.asarray(sysm.grid)
  h = vg[d[..., 0], d[..., 1], d[..., 2]]
  tk = kinetic_operator(sysm.g_vector_grid, sysm.kpts[k_index:k_index + 1])[0][sysm.mask]
  h = h + np.diag(tk)
  if sysm.proj is not None:
    # V_nl[G, G'] = sum_j conj(P_j(G)) P_j(G') / vol (nloc.py:143-157)
    p = np.asarray(sysm.proj).reshape(sysm.proj.shape[0], -1, *sysm.grid)[k_index][:, sysm.mask]
    h = h + p.conj().T @ p / sysm.vol
  return h


def ewald_coulomb_repulsion(positions, charges, g_vector_grid, vol, ewald_eta,
                            ewald_grid):
  """jrystal/_src/ewald.py:21-86, evaluated pair by pair (same sums)."""
  from scipy.special import erfc
  positions = np.asarray(positions, dtype=np.float64)
  charges = np.asarray(charges, dtype=np.float64)
  na = positions.shape[0]
  g2 = np.sum(g_vector_grid**2, axis=-1)
  g2 = g2.copy()
  g2[0, 0, 0] = 1e16
  kernel = np.exp(-g2 / 4 / ewald_eta**2) / g2
  kernel[0, 0, 0] = 0.0
  ovlp = np.zeros((na, na))
  rec = np.zeros((na, na))
  for i in range(na):
    for j in range(na):
      tau = positions[j] - positions[i]
      d = tau[None] - ewald_grid
      nrm = np.sqrt(np.sum(d**2, axis=-1) + 1e-20)
      nrm = np.where(nrm <= 1e-9, 1e20, nrm)
      ovlp[i, j] = np.sum(erfc(ewald_eta * nrm) / nrm)
      rec[i, j] = np.sum(kernel * np.cos(g_vector_grid @ tau))
  rec = rec * 4 * np.pi / vol
  ew_aa = charges @ (ovlp + rec) @ charges / 2
  ew_a = -np.sum(charges**2) * 2 * ewald_eta / np.sqrt(np.pi) / 2
  ew_a -= np.sum(charges)**2 * np.pi / ewald_eta**2 / vol / 2
  return ew_aa + ew_a


def nuclear_repulsion(position, charge, cell_vectors, g_vector_grid, vol,
                      ewald_eta, ewald_cutoff):
  """jrystal/_src/energy.py:214-243."""
  tgrid = translation_vectors(cell_vectors, ewald_cutoff)
  return ewald_coulomb_repulsion(position, charge, g_vector_grid, vol,
                                 ewald_eta, tgrid)


# --------------------------------------------------------------------------
# energy + hand-derived gradient of the direct-minimisation loss
# (calc/calc_ground_state_energy_all_electrons.py:119-147, value_and_grad :178)
# --------------------------------------------------------------------------
@dataclass
class System:
  """Everything the energy path needs besides the parameters."""
  cell_vectors: np.ndarray
  positions: np.ndarray
  charges: np.ndarray
  grid: tuple
  mask: np.ndarray
  kpts: np.ndarray
  occupation: np.ndarray     # (spin, kpt, band)
  xc: str = "lda_x+lda_c_vwn"
  # norm-conserving pseudopotential: complex V_loc(G) grid replacing the
  # Coulomb external potential, and dense beta-projector rows (k, j, x, y, z)
  v_local: Optional[np.ndarray] = None
  proj: Optional[np.ndarray] = None

  @property
  def vol(self):
    return abs(np.linalg.det(self.cell_vectors))

  @property
  def g_vector_grid(self):
    return g_vectors(self.cell_vectors, self.grid)


def nonlocal_projections(coeff_dense, proj):
  """F[s,k,b,j] = sum_xyz c P (c not conjugated; nloc.py:143-151)."""
  p = np.asarray(proj).reshape(proj.shape[0], -1, *proj.shape[-3:])
  return np.einsum("skbxyz,kjxyz->skbj", coeff_dense, p)


def hamiltonian_nonlocal(coeff_dense, proj, vol):
  """H_nl = F^H F / vol per (s, k) (nloc.py:143-157)."""
  f = nonlocal_projections(coeff_dense, proj)
  return np.einsum("skbj,skcj->skbc", np.conj(f), f) / vol


def energy_nonlocal(coeff_dense, proj, vol, occupation):
  """sum_{s,k,b} f_skb H_nl[s,k,b,b] (nloc.py:238-248)."""
  h = hamiltonian_nonlocal(coeff_dense, proj, vol)
  return float(np.sum(np.einsum("skbb->skb", h) * occupation).real)


def _nonlocal_grad_c(coeff_dense, proj, vol, weights, mask):
  """d E_nl / d conj(c) on the sphere: w_b / vol sum_j F_bj conj(P_j) -> (s,k,b,g)."""
  p = np.asarray(proj).reshape(proj.shape[0], -1, *proj.shape[-3:])
  f = nonlocal_projections(coeff_dense, p)
  return weights[..., None] / vol * np.einsum("skbj,kjg->skbg", f, np.conj(p[..., mask]))


def energy_terms(w_re, w_im, sysm: System, with_grad=True):
  """Energy terms of the loss and d loss / d {w_re, w_im}.

  Forward follows total_energy in
  calc/calc_ground_state_energy_all_electrons.py:119-137.  The gradient is
  the analytic adjoint: per band g_C = f (T c + sqrt(vol)/N FFT(V psi))|_sphere
  and through the orthonormalisation g_W = (g_C - C K) R^{-H} with K the
  Hermitian completion of the upper triangle of C^H g_C; dE/dw_re = 2 Re g_W,
  dE/dw_im = 2 Im g_W.
  """
  vol = sysm.vol
  gvec = sysm.g_vector_grid
  mask = sysm.mask
  occ = sysm.occupation
  c, r = cholesky_qr(w_re, w_im)                 # (s,k,g,b)
  dense = expand_coefficient(c, mask)             # (s,k,b,x,y,z)
  n = np.prod(sysm.grid)
  wave = _ifftn(dense) * n / np.sqrt(vol)
  rho = wave_to_density(wave, occ)                # (s,x,y,z)
  rho_g = _fftn(rho)
  e_kin = kinetic_energy(gvec, sysm.kpts, dense, occ)
  if sysm.v_local is not None:     # normcons.energy_local (local.py:163-187)
    v_ext = np.asarray(sysm.v_local)
  else:
    v_ext = external_reciprocal(sysm.positions, sysm.charges, gvec, vol)
  e_ext = reciprocal_braket(v_ext[None], rho_g, vol)
  e_nl = energy_nonlocal(dense, sysm.proj, vol, occ) if sysm.proj is not None else 0.0
  e_har = hartree_energy(rho_g, gvec, vol, False)
  if is_gga(sysm.xc):
    if rho.shape[0] != 1:
      raise NotImplementedError("polarised GGA is not restated")
    e_xc, v_xc_gga, _ = gga_energy_potential(rho[0], gvec, vol, sysm.xc)
  else:
    e_xc = xc_energy(rho, vol, sysm.xc, False)
  terms = dict(kinetic=e_kin, external=e_ext + e_nl, hartree=e_har, xc=e_xc,
               external_local=e_ext, external_nonlocal=e_nl)
  terms["total"] = e_kin + e_ext + e_nl + e_har + e_xc
  if not with_grad:
    return terms
  # dE/d rho_s(r) = (vol/N) V_s(r)
  v_g = hartree_reciprocal(rho_g, gvec, kohn_sham=True) + v_ext
  if rho.shape[0] == 2:
    # d (eps rho_tot) / d rho_s = eps + rho_tot d eps / d rho_s
    eps, d = xc_eps_pol(rho, sysm.xc)
    v_xc = eps[None] + rho.sum(0)[None] * d
  else:
    v_xc = v_xc_gga if is_gga(sysm.xc) else xc_eps_v(rho[0], sysm.xc)[1]
  v_r = np.real(_ifftn(v_g)) + v_xc                # (x,y,z), or (2,x,y,z) polarised
  v_s = v_r if v_r.ndim == 4 else v_r[None]
  hpsi = _fftn(v_s[:, None, None] * wave)
  hpsi = hpsi[..., mask] * (np.sqrt(vol) / n)     # (s,k,b,g)
  tk = kinetic_operator(gvec, sysm.kpts)[:, mask]  # (k,g)
  g_c = occ[..., None] * (tk[None, :, None, :] * np.swapaxes(c, -1, -2) + hpsi)
  if sysm.proj is not None:
    g_c = g_c + _nonlocal_grad_c(dense, sysm.proj, vol, occ, mask)
  g_c = np.swapaxes(g_c, -1, -2)                   # (s,k,g,b)
  a = np.einsum("...gi,...gj->...ij", c.conj(), g_c)
  up = np.triu(a, 1)
  kmat = up + np.swapaxes(up.conj(), -1, -2)
  kmat = kmat + np.einsum("...ii->...i", a).real[..., None] * np.eye(a.shape[-1])
  rinv_h = np.swapaxes(np.linalg.inv(r).conj(), -1, -2)
  g_w = (g_c - c @ kmat) @ rinv_h
  return terms, 2 * g_w.real, 2 * g_w.imag, v_r


# --------------------------------------------------------------------------
# optimiser (optax.adam; calc/opt_utils.py:153-168) and convergence check
# --------------------------------------------------------------------------
def adam_update(param, grad, m, v, step, lr, b1=0.9, b2=0.99, eps=1e-8,
                scale=None):
  """One Adam step, optax placement of eps (outside the sqrt, after bias
  correction).  ``step`` is the 1-based count after this update.  ``scale``
  multiplies the update elementwise (the learned diagonal preconditioner)."""
  m = b1 * m + (1 - b1) * grad
  v = b2 * v + (1 - b2) * grad * grad
  mh = m / (1 - b1**step)
  vh = v / (1 - b2**step)
  upd = -lr * mh / (np.sqrt(vh) + eps)
  if scale is not None:
    upd = upd * scale
  return param + upd, m, v


class ConvergenceChecker:
  """calc/convergence.py:13-35."""

  def __init__(self, window_size=20, threshold=1e-5):
    self.window_size = window_size
    self.threshold = threshold
    self.history = []

  def check(self, value):
    self.history.append(value)
    if len(self.history) > self.window_size:
      self.history.pop(0)
    if len(self.history) < self.window_size:
      return False
    return bool(np.std(self.history) < self.threshold)


def geometry_path(name):
  return os.path.join(os.path.dirname(__file__), "..", "tests", "golden",
                      name)
