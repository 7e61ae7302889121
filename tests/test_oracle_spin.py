"""Spin-polarised LDA of the oracle (jrystal/_src/xc.py:40-64 polarised
branches, energy.py:185-211): identities that pin the restatement without a
jax_xc value.

- at zeta = 0 the polarised energy density and the potential
  d(eps rho)/d rho_s reduce to the unpolarised ones;
- at zeta = +-1 the correlation is the VWN ferromagnetic fit;
- d eps / d rho_s agrees with central differences;
- an S = 2 system with the same parameters and half the occupation in both
  channels has the S = 1 energy and half its gradient per channel;
- the S = 2 gradient of energy_terms agrees with central differences.
"""
import dataclasses

import numpy as np
import pytest

from oracle import restatement as R
from systems import make_system, random_params

XC = "lda_x+lda_c_vwn"


def test_zero_polarisation_reduces_to_unpolarised():
  rho = np.geomspace(1e-6, 1e3, 50)
  for name in ("lda_x", "lda_c_vwn", XC):
    eps, d = R.xc_eps_pol(np.stack([rho / 2, rho / 2]), name)
    eps0, v0 = R.xc_eps_v(rho, name)
    np.testing.assert_allclose(eps, eps0, rtol=1e-13, atol=1e-300)
    for s in range(2):
      np.testing.assert_allclose(eps + rho * d[s], v0, rtol=1e-12)


def test_full_polarisation_is_ferromagnetic_fit():
  for rs in (0.5, 1.0, 4.0):
    rho = 3.0 / (4.0 * np.pi * rs**3)
    for up, dn in ((rho, 0.0), (0.0, rho)):
      eps, _, _ = R.lda_c_vwn_pol(np.array([up]), np.array([dn]))
      ref, _ = R._vwn_fit(np.sqrt(rs), *R.VWN_FERRO)
      assert abs(eps[0] - ref) < 1e-14
  # exchange of a fully polarised gas: 2^(1/3) times the unpolarised value
  e_pol, _, _ = R.lda_x_pol(np.array([1.0]), np.array([0.0]))
  e_unp, _ = R.lda_x(np.array([1.0]))
  assert abs(e_pol[0] / e_unp[0] - 0.5 * 2.0**(1.0 / 3.0)) < 1e-14


def test_polarised_derivatives_match_central_differences():
  rng = np.random.default_rng(3)
  up = np.geomspace(1e-4, 50, 40) * rng.uniform(0.2, 1.0, 40)
  dn = np.geomspace(1e-4, 50, 40)[::-1] * rng.uniform(0.2, 1.0, 40)
  for name in ("lda_x", "lda_c_vwn"):
    eps, d = R.xc_eps_pol(np.stack([up, dn]), name)
    for s in range(2):
      h = 1e-4 * (up if s == 0 else dn)
      hp = np.stack([up, dn]); hp[s] += h
      hm = np.stack([up, dn]); hm[s] -= h
      fd = (R.xc_eps_pol(hp, name)[0] - R.xc_eps_pol(hm, name)[0]) / (2 * h)
      np.testing.assert_allclose(d[s], fd, rtol=1e-6)


def test_kohn_sham_form_follows_vxc_lda():
  # vxc_lda (xc.py:109-124) polarised: eps + rho_s d eps / d rho_s per channel
  rng = np.random.default_rng(5)
  rho = rng.uniform(0.01, 1.0, size=(2, 3, 4, 5))
  eps, d = R.xc_eps_pol(rho, XC)
  v = R.xc_density(rho, kohn_sham=True, xc_type=XC)
  np.testing.assert_allclose(v, eps[None] + d * rho, rtol=1e-14)
  assert R.xc_density(rho, kohn_sham=False, xc_type=XC).shape == rho.shape[1:]


def _spin_system(sysm, occ_up, occ_dn):
  return dataclasses.replace(sysm, occupation=np.concatenate([occ_up, occ_dn]))


def test_unpolarised_state_as_two_channels():
  sysm = make_system(kind="si2", grid=(12, 12, 12), kgrid=(2, 1, 1), nb=5, nocc=3)
  wr, wi = random_params(sysm, seed=11)
  t1, gr1, gi1, v1 = R.energy_terms(wr, wi, sysm)
  half = sysm.occupation / 2
  s2 = _spin_system(sysm, half, half)
  t2, gr2, gi2, v2 = R.energy_terms(np.concatenate([wr, wr]), np.concatenate([wi, wi]), s2)
  for key in ("kinetic", "external", "hartree", "xc", "total"):
    assert abs(t2[key] - t1[key]) < 1e-11 * max(1.0, abs(t1[key])), key
  for s in range(2):
    np.testing.assert_allclose(gr2[s], gr1[0] / 2, atol=1e-12 * np.abs(gr1).max())
    np.testing.assert_allclose(gi2[s], gi1[0] / 2, atol=1e-12 * np.abs(gi1).max())
    np.testing.assert_allclose(v2[s], v1, atol=1e-11 * np.abs(v1).max())


@pytest.mark.parametrize("occ", [(3, 2), (4, 1)])
def test_polarised_gradient_central_differences(occ):
  sysm = make_system(kind="si2", grid=(12, 12, 12), kgrid=(1, 1, 2), nb=5, nocc=3)
  K = sysm.kpts.shape[0]
  up = np.zeros((1, K, 5)); up[0, :, :occ[0]] = 1.0 / K
  dn = np.zeros((1, K, 5)); dn[0, :, :occ[1]] = 1.0 / K
  s2 = _spin_system(sysm, up, dn)
  wr, wi = random_params(s2, seed=12, ns=2)
  _, gr, gi, v = R.energy_terms(wr, wi, s2)
  assert v.shape == (2,) + tuple(sysm.grid)
  rng = np.random.default_rng(13)
  h = 1e-5
  for _ in range(8):
    idx = tuple(int(rng.integers(0, s)) for s in wr.shape)
    for part, g in ((0, gr), (1, gi)):
      p = [wr.copy(), wi.copy()]
      p[part][idx] += h
      ep = R.energy_terms(p[0], p[1], s2, with_grad=False)["total"]
      p[part][idx] -= 2 * h
      em = R.energy_terms(p[0], p[1], s2, with_grad=False)["total"]
      fd = (ep - em) / (2 * h)
      assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(g[idx])), (idx, part, fd, g[idx])


def test_band_trace_per_spin_potential():
  """Two spin channels in their own potentials: the trace, band Hamiltonian
  and gradient are those of each channel alone in its potential."""
  sysm = make_system(kind="si2", grid=(12, 12, 12), kgrid=(1, 1, 2), nb=4, nocc=2)
  K = sysm.kpts.shape[0]
  s2 = _spin_system(sysm, np.ones((1, K, 4)), np.ones((1, K, 4)))
  rng = np.random.default_rng(21)
  v = rng.normal(size=(2,) + tuple(sysm.grid))
  wr, wi = random_params(s2, seed=22, ns=2)
  both = R.band_trace_terms(wr, wi, v, s2)
  one = dataclasses.replace(sysm, occupation=np.ones((1, K, 4)))
  parts = [R.band_trace_terms(wr[s:s + 1], wi[s:s + 1], v[s], one) for s in range(2)]
  assert abs(both["trace"] - sum(p["trace"] for p in parts)) < 1e-11 * abs(both["trace"])
  for s in range(2):
    np.testing.assert_allclose(both["hmat"][s], parts[s]["hmat"][0], atol=1e-12)
    np.testing.assert_allclose(both["grad_re"][s], parts[s]["grad_re"][0], atol=1e-12)
    np.testing.assert_allclose(both["grad_im"][s], parts[s]["grad_im"][0], atol=1e-12)
