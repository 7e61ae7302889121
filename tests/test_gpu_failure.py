"""Numerical failure detection and recovery, with the failures made on the
host: parameters with two identical occupied columns (rank-deficient W) and
parameters holding a NaN.  Cholesky QR breaks down on both where the
reference's Householder QR (jrystal/_src/unitary_module.py:74-80) does not;
the call reports it in its status word and condition estimate (energies[6],
energies[5]), the fused step applies no update, and jrg_reorthonormalise
restores a valid parameter set from which the minimisation continues."""
import numpy as np
import pytest

from oracle import restatement as R
from tests.systems import make_system, random_params

pytestmark = pytest.mark.gpu


def _plan(sysm, prec):
  from jrystal_gb300.engine import PlaneWavePlan
  return PlaneWavePlan(sysm.cell_vectors, sysm.positions, sysm.charges, sysm.grid, sysm.mask,
                       sysm.kpts, sysm.occupation.shape[-1], 1, prec, sysm.xc)


def _system():
  return make_system(kind="si2", grid=(16, 16, 16), kgrid=(2, 1, 1), nb=8, nocc=4)


def _params(sysm, prec, seed=3):
  import torch
  wr, wi = random_params(sysm, seed=seed)
  dt = torch.float64 if prec == 64 else torch.float32
  return torch.tensor(np.stack([wr, wi]), dtype=dt, device="cuda").contiguous()


@pytest.mark.parametrize("prec", [64, 32])
def test_rank_deficient_parameters_are_flagged(prec):
  sysm = _system()
  plan = _plan(sysm, prec)
  p = _params(sysm, prec)
  e, _, _ = plan.energy_and_grad(p[0], p[1], sysm.occupation)
  assert not plan.needs_reorthonormalisation(e)
  assert 1.0 <= plan.status_of(e)["condition"] < 10.0
  p[:, :, :, :, 2] = p[:, :, :, :, 1]          # band 2 = band 1 (both occupied)
  e, _, _ = plan.energy_and_grad(p[0], p[1], sysm.occupation)
  st = plan.status_of(e)
  assert st["flags"] & 1, st
  assert plan.needs_reorthonormalisation(e)


@pytest.mark.parametrize("prec", [64, 32])
def test_nan_parameters_raise_numeric_error(prec):
  from jrystal_gb300 import _lib
  sysm = _system()
  plan = _plan(sysm, prec)
  p = _params(sysm, prec)
  p[0, 0, 1, 5, 2] = float("nan")
  e, _, _ = plan.energy_and_grad(p[0], p[1], sysm.occupation)
  st = plan.status_of(e)
  assert st["flags"] & 1
  assert not st["condition"] < np.inf
  with pytest.raises(_lib.NumericalError) as err:
    plan.check_numerics(e)
  assert err.value.code == _lib.JRG_ERR_NUMERIC


@pytest.mark.parametrize("prec", [64, 32])
def test_reorthonormalise_keeps_coefficients_and_energy(prec):
  """Full-rank W: W' = Q diag(|w_b|) with Q the oracle's Cholesky QR factor;
  the coefficients of W' equal those of W (no phase change), and so does
  the energy."""
  import torch
  sysm = _system()
  plan = _plan(sysm, prec)
  p = _params(sysm, prec)
  e0 = plan.energy_and_grad(p[0], p[1], sysm.occupation, with_grad=False)[0].cpu().numpy().copy()
  c0 = plan.coeff(p[0], p[1]).cpu().numpy()
  w = p.double().cpu().numpy()
  q, _ = R.cholesky_qr(w[0], w[1])
  norms = np.sqrt((w[0] ** 2 + w[1] ** 2).sum(axis=-2, keepdims=True))
  plan.reorthonormalise(p[0], p[1])
  torch.cuda.synchronize()
  wn = p.double().cpu().numpy()
  ref = q * norms
  tol = 1e-12 if prec == 64 else 2e-6
  assert np.abs(wn[0] + 1j * wn[1] - ref).max() <= tol * np.abs(ref).max()
  e1 = plan.energy_and_grad(p[0], p[1], sysm.occupation, with_grad=False)[0].cpu().numpy()
  etol = 1e-10 if prec == 64 else 2e-6
  assert np.abs(e1[:5] - e0[:5]).max() <= etol * np.abs(e0[:5]).max()
  c1 = plan.coeff(p[0], p[1]).cpu().numpy()
  assert np.abs(c1 - c0).max() <= (1e-11 if prec == 64 else 1e-5) * np.abs(c0).max()
  assert plan.status_of(e1)["condition"] < 1.0 + 1e-3


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("fault", ["duplicate", "nan"])
def test_reorthonormalise_recovers(prec, fault):
  import torch
  sysm = _system()
  plan = _plan(sysm, prec)
  p = _params(sysm, prec)
  if fault == "duplicate":
    p[:, :, :, :, 2] = p[:, :, :, :, 1]
  else:
    p[1, 0, 0, 7, 3] = float("nan")
  plan.reorthonormalise(p[0], p[1])
  assert torch.isfinite(p).all()
  e, _, _ = plan.energy_and_grad(p[0], p[1], sysm.occupation)
  st = plan.check_numerics(e)
  assert st["flags"] == 0 and st["condition"] < 1.0 + 1e-3
  c = plan.coeff(p[0], p[1]).cpu().numpy().astype(np.complex128)
  ovl = np.einsum("skgi,skgj->skij", c.conj(), c)
  assert np.abs(ovl - np.eye(c.shape[-1])).max() < (1e-12 if prec == 64 else 2e-6)


@pytest.mark.parametrize("prec", [64, 32])
def test_fused_step_applies_no_update_on_breakdown(prec):
  import torch
  sysm = _system()
  plan = _plan(sysm, prec)
  p = _params(sysm, prec)
  p[0, 0, 1, 5, 2] = float("nan")
  m = torch.zeros_like(p)
  v = torch.zeros_like(p)
  before = p.clone()
  e = plan.energy_grad_adam(p, m, v, sysm.occupation, 1, 1e-2)
  assert plan.status_of(e)["flags"] & 1
  assert torch.equal(torch.isnan(p), torch.isnan(before))
  fin = torch.isfinite(before)
  assert torch.equal(p[fin], before[fin])
  assert (m == 0).all() and (v == 0).all()


def test_minimizer_recovers_from_a_duplicated_band():
  """The driver's checked step: a duplicated occupied band injected between
  steps is detected, the parameters are re-orthonormalised, Adam restarts
  and the energy keeps decreasing."""
  import torch
  from jrystal_gb300.calc import Minimizer
  sysm = _system()
  plan = _plan(sysm, 64)
  mini = Minimizer(plan, sysm.occupation, _params(sysm, 64), lr=1e-2)
  for _ in range(20):
    mini.checked_step()
  assert mini.recoveries == 0
  mini.params[:, :, :, :, 2] = mini.params[:, :, :, :, 1]
  e = mini.checked_step()
  assert mini.recoveries == 1
  assert torch.isfinite(e[:5]).all()
  hist = [float(mini.checked_step()[4].item()) for _ in range(40)]
  assert mini.recoveries == 1
  assert np.isfinite(hist).all() and hist[-1] < hist[0]
