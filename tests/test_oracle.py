"""Pins the CPU oracle to the reference's own known answers and identities.

* crystal golden values: jrystal/_src/crystal_test.py:25-61 (diamond.xyz)
* FFT wave grid == direct O(G) sum: jrystal/_src/pw_test.py:36-49
* E_H, E_ext, E_xc == sum_b f <psi|V|psi>: jrystal/_src/energy_test.py:61-112
* KS Hamiltonian trace == total_energy(kohn_sham=True):
  jrystal/_src/hamiltonian_test.py:78-102
plus central finite differences of the hand-written gradient, and the
QR-variant (Householder vs Cholesky) invariance of the energy.
"""
import os

import numpy as np
import pytest

from oracle import restatement as R
from tests.systems import GOLDEN, make_system, random_params


@pytest.fixture(scope="module")
def diamond():
  return R.read_xyz(os.path.join(GOLDEN, "diamond.xyz"))


def test_crystal_golden_values(diamond):
  np.testing.assert_almost_equal(diamond.positions, [[-0.84251071] * 3, [0.84251071] * 3])
  np.testing.assert_almost_equal(diamond.charges, [6, 6])
  np.testing.assert_almost_equal(
    diamond.cell_vectors,
    [[0., 3.37004284, 3.37004284], [3.37004284, 0., 3.37004284], [3.37004284, 3.37004284, 0.]])
  # crystal_test asserts equality of the float; det rounding differs in the
  # last bit between LAPACK builds, so compare to 1 part in 1e14
  assert abs(diamond.vol - 76.5484253352856) <= 1e-14 * 76.5484253352856
  np.testing.assert_almost_equal(diamond.scaled_positions, [[-0.125] * 3, [0.125] * 3])
  np.testing.assert_almost_equal(
    diamond.reciprocal_vectors,
    [[-0.93221149, 0.93221149, 0.93221149], [0.93221149, -0.93221149, 0.93221149],
     [0.93221149, 0.93221149, -0.93221149]])


def _diamond_setup(diamond, kgrid=(1, 1, 1), seed=123):
  grid = (7, 8, 9)
  mask = R.cubic_mask(grid)
  kpts = R.k_vectors(diamond.cell_vectors, kgrid)
  nb = diamond.num_electron
  rng = np.random.default_rng(seed)
  shape = (1, kpts.shape[0], int(mask.sum()), nb)
  wr, wi = rng.uniform(size=shape), rng.uniform(size=shape)
  coeff = R.coeff(wr, wi, mask)
  gvec = R.g_vectors(diamond.cell_vectors, grid)
  return grid, mask, kpts, coeff, gvec


def test_wave_grid_equals_direct_sum(diamond):
  grid, mask, kpts, coeff, gvec = _diamond_setup(diamond)
  wave = R.wave_grid(coeff, diamond.vol)
  rvec = R.r_vectors(diamond.cell_vectors, grid)
  direct = np.empty_like(wave)
  for i in range(grid[0]):
    for j in range(grid[1]):
      for k in range(grid[2]):
        direct[..., i, j, k] = R.wave_r(rvec[i, j, k], coeff, diamond.cell_vectors, gvec)
  np.testing.assert_allclose(wave, direct, atol=1e-8)


@pytest.mark.parametrize("kohn_sham", [False])
def test_energy_potential_identities(diamond, kohn_sham):
  grid, mask, kpts, coeff, gvec = _diamond_setup(diamond)
  occ = R.gamma_occupation(kpts.shape[0], diamond.num_electron)
  wave = R.wave_grid(coeff, diamond.vol)
  rho = R.density_grid(coeff, diamond.vol, occ)
  rho_g = np.fft.fftn(rho, axes=(-3, -2, -1))
  xc = "lda_x+lda_c_vwn"
  vh, ve, vx = R.effective(rho, diamond.positions, diamond.charges, gvec, diamond.vol, split=True,
                           xc_type=xc, kohn_sham=kohn_sham)
  e = {}
  for name, v in (("h", vh), ("e", ve), ("x", vx)):
    e[name] = np.sum(R.expectation(wave, v, diamond.vol, diagonal=True, mode="real") * occ).real
  np.testing.assert_allclose(e["h"], R.hartree_energy(rho_g, gvec, diamond.vol, kohn_sham), atol=1e-7)
  np.testing.assert_allclose(e["e"], R.external_energy(rho_g, diamond.positions, diamond.charges,
                                                       gvec, diamond.vol), atol=1e-7)
  np.testing.assert_allclose(e["x"], R.xc_energy(rho, diamond.vol, xc, kohn_sham), atol=1e-7)


def test_hamiltonian_trace_equals_kohn_sham_energy(diamond):
  grid, mask, kpts, coeff, gvec = _diamond_setup(diamond, kgrid=(2, 2, 1))
  occ = np.ones((1, kpts.shape[0], diamond.num_electron))
  rho = R.density_grid(coeff, diamond.vol, occ)
  xc = "lda_x+lda_c_vwn"
  e1 = R.hamiltonian_matrix_trace(coeff, diamond.positions, diamond.charges, rho, gvec, kpts,
                                  diamond.vol, xc=xc, kohn_sham=True)
  e2 = R.total_energy(coeff, diamond.positions, diamond.charges, gvec, kpts, diamond.vol,
                      kohn_sham=True, xc=xc)
  np.testing.assert_allclose(e1, e2, atol=1e-7)


@pytest.mark.parametrize("case", [
  dict(kind="diamond", grid=(8, 9, 10), kgrid=(2, 1, 1), nb=4, nocc=2, mask="cubic"),
  dict(kind="si2", grid=(12, 12, 12), kgrid=(1, 1, 2), nb=5, nocc=3),
])
def test_gradient_central_differences(case):
  sysm = make_system(**case)
  wr, wi = random_params(sysm, seed=1)
  _, gr, gi, _ = R.energy_terms(wr, wi, sysm)
  rng = np.random.default_rng(2)
  h = 1e-5
  for _ in range(8):
    idx = tuple(int(rng.integers(0, s)) for s in wr.shape)
    for part, g in ((0, gr), (1, gi)):
      p = [wr.copy(), wi.copy()]
      p[part][idx] += h
      ep = R.energy_terms(p[0], p[1], sysm, with_grad=False)["total"]
      p[part][idx] -= 2 * h
      em = R.energy_terms(p[0], p[1], sysm, with_grad=False)["total"]
      fd = (ep - em) / (2 * h)
      assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(g[idx])), (idx, part, fd, g[idx])


def test_energy_invariant_to_qr_variant():
  sysm = make_system(kind="si2", grid=(12, 12, 12), kgrid=(2, 1, 1), nb=4, nocc=2)
  wr, wi = random_params(sysm, seed=4)
  t = R.energy_terms(wr, wi, sysm, with_grad=False)
  dense = R.coeff(wr, wi, sysm.mask)   # Householder QR, jnp.linalg.qr's convention
  ref = R.total_energy(dense, sysm.positions, sysm.charges, sysm.g_vector_grid, sysm.kpts,
                       sysm.vol, sysm.occupation, xc=sysm.xc)
  assert abs(t["total"] - ref) < 1e-10 * abs(ref)


def test_unoccupied_bands_have_zero_gradient():
  sysm = make_system(kind="si2", grid=(12, 12, 12), kgrid=(1, 1, 1), nb=5, nocc=2)
  wr, wi = random_params(sysm, seed=6)
  _, gr, gi, _ = R.energy_terms(wr, wi, sysm)
  assert np.abs(gr[..., 2:]).max() < 1e-12 and np.abs(gi[..., 2:]).max() < 1e-12


def test_lda_potential_is_derivative_of_energy_density():
  rho = np.geomspace(1e-6, 1e3, 60)
  for name in ("lda_x", "lda_c_vwn"):
    eps, v = R.xc_eps_v(rho, name)
    h = 1e-6 * rho
    ep, _ = R.xc_eps_v(rho + h, name)
    em, _ = R.xc_eps_v(rho - h, name)
    fd = ((rho + h) * ep - (rho - h) * em) / (2 * h)
    np.testing.assert_allclose(v, fd, rtol=1e-7)
  # Slater exchange closed form
  eps, _ = R.lda_x(np.array([1.0]))
  assert abs(eps[0] + 0.75 * (3 / np.pi)**(1 / 3)) < 1e-15
  # below the density threshold everything is zero
  assert R.xc_eps_v(np.array([1e-16]), "lda_x+lda_c_vwn")[0][0] == 0.0


def test_vwn_paramagnetic_fit_values():
  # closed-form spot values of the VWN5 paramagnetic fit at rs = 1 and rs = 4
  for rs in (1.0, 4.0):
    rho = 3.0 / (4.0 * np.pi * rs**3)
    eps, _ = R.lda_c_vwn(np.array([rho]))
    a, b, c, x0 = R.VWN_A, R.VWN_B, R.VWN_C, R.VWN_X0
    x = np.sqrt(rs)
    X = lambda t: t * t + b * t + c
    q = np.sqrt(4 * c - b * b)
    ref = a * (np.log(x * x / X(x)) + 2 * b / q * np.arctan(q / (2 * x + b)) -
               b * x0 / X(x0) * (np.log((x - x0)**2 / X(x)) +
                                 2 * (b + 2 * x0) / q * np.arctan(q / (2 * x + b))))
    assert abs(eps[0] - ref) < 1e-15
  # correlation energy per particle of the electron gas is about -0.06 Ha at rs = 1
  eps1, _ = R.lda_c_vwn(np.array([3.0 / (4.0 * np.pi)]))
  assert -0.065 < eps1[0] < -0.055


def test_adam_matches_hand_computation():
  p, g = np.array([1.0]), np.array([0.5])
  m, v = np.zeros(1), np.zeros(1)
  p1, m1, v1 = R.adam_update(p, g, m, v, 1, 0.1, b1=0.9, b2=0.99, eps=1e-8)
  # step 1: m_hat = g, v_hat = g^2 -> update = -lr * g / (|g| + eps)
  assert abs(p1[0] - (1.0 - 0.1 * 0.5 / (0.5 + 1e-8))) < 1e-15
  assert abs(m1[0] - 0.05) < 1e-15 and abs(v1[0] - 0.0025) < 1e-15


def test_convergence_checker():
  c = R.ConvergenceChecker(window_size=3, threshold=1e-3)
  assert not c.check(1.0) and not c.check(1.0001)
  assert c.check(1.0002)
  assert not c.check(2.0)


def test_ewald_structure_factor_form_equals_pair_form():
  sysm = make_system(kind="si2", grid=(12, 12, 12), kgrid=(1, 1, 1), nb=2, nocc=1)
  gvec = sysm.g_vector_grid
  tg = R.translation_vectors(sysm.cell_vectors, 500.0)
  e = R.ewald_coulomb_repulsion(sysm.positions, sysm.charges, gvec, sysm.vol, 0.1, tg)
  # reciprocal part through |S(G)|^2 instead of the pair cosine sum
  g2 = np.sum(gvec**2, -1)
  g2[0, 0, 0] = 1e16
  kern = np.exp(-g2 / 4 / 0.01) / g2
  kern[0, 0, 0] = 0
  s = np.sum(sysm.charges * np.exp(1j * gvec @ sysm.positions.T), -1)
  rec = 4 * np.pi / sysm.vol * np.sum(kern * np.abs(s)**2) / 2
  pos = sysm.positions
  real = 0.0
  from scipy.special import erfc
  for i in range(2):
    for j in range(2):
      d = np.linalg.norm(pos[j] - pos[i] - tg, axis=-1)
      d = d[d > 1e-9]
      real += sysm.charges[i] * sysm.charges[j] * np.sum(erfc(0.1 * d) / d) / 2
  z = sysm.charges
  self_e = -np.sum(z**2) * 0.1 / np.sqrt(np.pi) - np.sum(z)**2 * np.pi / 0.01 / sysm.vol / 2
  assert abs(e - (real + rec + self_e)) < 1e-9 * abs(e)
