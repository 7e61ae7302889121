"""Learnable occupations on the host (CPU torch) against the oracle's NumPy
restatement of jrystal/_src/occupation.py, the temperature schedule, and the
oracle relation dE/df = <psi|T + V_eff|psi> used by jrg_energy_grad_bands."""
import numpy as np
import pytest
import torch

from oracle import restatement as R
from tests.systems import make_system, random_params


@pytest.mark.parametrize("nelec,spin,nk,nb,shift", [(13, 1, 4, 8, 0.0), (8, 0, 2, 6, 3.0),
                                                    (8, 0, 2, 6, -3.0), (26, 0, 8, 16, 0.5)])
def test_simplex_projector_matches_oracle(nelec, spin, nk, nb, shift):
  from jrystal_gb300 import occupation as O
  rng = np.random.default_rng(nelec + nk)
  up = torch.tensor(rng.normal(size=(nk, nb)) + shift)
  down = torch.tensor(rng.normal(size=(nk, nb)) + shift)
  occ = O.simplex_projector({"param_up": up, "param_down": down}, nelec, spin)
  ref = R.simplex_projector(up.numpy(), down.numpy(), nelec, spin)
  np.testing.assert_allclose(occ.numpy(), ref, atol=1e-12)
  assert abs(float(occ.sum()) - nelec) < 1e-9
  assert float(occ.min()) >= -1e-12 and float(occ.max()) <= 2.0 / nk + 1e-12


def test_simplex_projector_gradient_flows_and_init():
  from jrystal_gb300 import occupation as O
  p = O.simplex_projector_init(6, 3, device="cpu")
  np.testing.assert_allclose(p["param_up"].numpy().ravel(), (np.arange(18) - 9) * 0.1)
  for t in p.values():
    t.requires_grad_(True)
  occ = O.simplex_projector(p, 8)
  w = torch.linspace(-1, 1, occ.numel(), dtype=torch.float64).reshape(occ.shape)
  g = torch.autograd.grad((occ * w).sum(), [p["param_up"]])[0]
  assert torch.isfinite(g).all() and float(g.abs().sum()) > 0


def test_idempotent_occupation_constraints():
  from jrystal_gb300 import occupation as O
  prm = O.idempotent_param_init(3, 6, 8, 2, device="cpu")
  occ = O.idempotent(prm, 2)
  assert occ.shape == (1, 2, 6)
  assert abs(float(occ.sum()) - 8) < 1e-10
  assert float(occ.min()) >= -1e-12 and float(occ.max()) <= 2.0 / 2 + 1e-12


def test_temperature_schedule():
  from jrystal_gb300.calc import temperature_schedule
  f = temperature_schedule({"smearing": 0.01, "epoch": 1000})
  assert f(0) == 100.0
  assert abs(f(250) - 100.0 * 1e-4 ** 0.5) < 1e-9
  assert f(500) == pytest.approx(0.01) and f(900) == 0.01
  assert temperature_schedule({"smearing": 0.0, "epoch": 10})(3) == 0.0


def test_band_energies_are_occupation_derivatives():
  sysm = make_system(kind="si2", grid=(8, 8, 8), kgrid=(2, 1, 1), nb=3, nocc=2)
  rng = np.random.default_rng(4)
  sysm.occupation = rng.uniform(0.1, 1.0, size=sysm.occupation.shape)
  wr, wi = random_params(sysm, seed=8)
  _, _, _, v = R.energy_terms(wr, wi, sysm)
  eps = np.einsum("...ii->...i", R.band_trace_terms(wr, wi, v, sysm, with_grad=False)["hmat"]).real
  h = 1e-5
  for idx in [(0, 0, 0), (0, 1, 2), (0, 0, 1)]:
    occ0 = sysm.occupation.copy()
    sysm.occupation = occ0.copy(); sysm.occupation[idx] += h
    ep = R.energy_terms(wr, wi, sysm, with_grad=False)["total"]
    sysm.occupation = occ0.copy(); sysm.occupation[idx] -= h
    em = R.energy_terms(wr, wi, sysm, with_grad=False)["total"]
    sysm.occupation = occ0
    assert abs((ep - em) / (2 * h) - eps[idx]) < 1e-6 * max(1.0, abs(eps[idx]))
