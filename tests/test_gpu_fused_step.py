"""The fused optimiser step (jrg_energy_grad_adam): energy + gradient + Adam
in one call, against the two-call path and the oracle's Adam."""
import numpy as np
import pytest

from oracle import restatement as R
from tests.systems import make_system, random_params

pytestmark = pytest.mark.gpu


def _plan(sysm, prec, nb):
  from jrystal_gb300.engine import PlaneWavePlan
  return PlaneWavePlan(sysm.cell_vectors, sysm.positions, sysm.charges, sysm.grid, sysm.mask,
                       sysm.kpts, nb, 1, prec, sysm.xc)


def _state(sysm, plan, seed):
  import torch
  dt = np.float64 if plan.precision == 64 else np.float32
  wr, wi = random_params(sysm, seed=seed, dtype=dt)
  p = torch.tensor(np.stack([wr, wi]), device="cuda").contiguous()
  return p, torch.zeros_like(p), torch.zeros_like(p)


@pytest.mark.parametrize("prec,nb,nocc,grid", [(64, 4, 2, (16, 16, 16)), (32, 12, 6, (24, 24, 24)),
                                               (32, 30, 16, (16, 16, 16)),
                                               # more than 32 bands: pipelined, 40-band tiles of 32 + 8
                                               (32, 40, 20, (16, 16, 16)), (64, 40, 20, (16, 16, 16))])
def test_fused_step_matches_two_call_path(prec, nb, nocc, grid):
  import torch
  from jrystal_gb300.engine import adam_update
  sysm = make_system(kind="si2", grid=grid, kgrid=(2, 1, 1), nb=nb, nocc=nocc)
  plan = _plan(sysm, prec, nb)
  occ = torch.tensor(sysm.occupation, device="cuda")
  p1, m1, v1 = _state(sysm, plan, 5)
  p2, m2, v2 = p1.clone(), m1.clone(), v1.clone()
  g1, g2 = torch.empty_like(p1), torch.empty_like(p1)
  scale = torch.rand(p1.shape, device="cuda", dtype=torch.float32, generator=torch.Generator(
      device="cuda").manual_seed(1)) + 0.5
  tol = dict(rtol=1e-12, atol=1e-14) if prec == 64 else dict(rtol=2e-5, atol=1e-6)
  for t in range(1, 5):
    sc = scale if t % 2 == 0 else None
    e1, _, _ = plan.energy_and_grad(p1[0], p1[1], occ, g1[0], g1[1])
    e1 = e1.clone()
    adam_update(p1, g1, m1, v1, t, 1e-2, scale=sc)
    e2 = plan.energy_grad_adam(p2, m2, v2, occ, t, 1e-2, scale=sc, grad=g2).clone()
    np.testing.assert_allclose(e2.cpu().numpy()[:5], e1.cpu().numpy()[:5],
                               rtol=1e-12 if prec == 64 else 1e-5)
    np.testing.assert_allclose(g2.cpu().numpy(), g1.cpu().numpy(), **tol)
    np.testing.assert_allclose(m2.cpu().numpy(), m1.cpu().numpy(), **tol)
    np.testing.assert_allclose(v2.cpu().numpy(), v1.cpu().numpy(), rtol=tol["rtol"] * 4,
                               atol=tol["atol"] ** 2)
    np.testing.assert_allclose(p2.cpu().numpy(), p1.cpu().numpy(), **tol)
  plan.close()


def test_fused_step_matches_oracle_adam():
  import torch
  sysm = make_system(kind="si2", grid=(16, 16, 16), kgrid=(2, 1, 1), nb=4, nocc=2)
  plan = _plan(sysm, 64, 4)
  occ = torch.tensor(sysm.occupation, device="cuda")
  p, m, v = _state(sysm, plan, 7)
  w = p.cpu().numpy()
  _, gr, gi, _ = R.energy_terms(w[0], w[1], sysm, with_grad=True)
  g = np.stack([gr, gi])
  mo, vo = np.zeros_like(w), np.zeros_like(w)
  wo, mo, vo = R.adam_update(w, g, mo, vo, 1, 1e-2, 0.9, 0.99, 1e-8)
  plan.energy_grad_adam(p, m, v, occ, 1, 1e-2)
  # the first Adam step is -lr * sign(g) up to eps: compare away from g ~ 0
  np.testing.assert_allclose(p.cpu().numpy(), wo, atol=1e-9)
  np.testing.assert_allclose(m.cpu().numpy(), mo, atol=1e-10)
  plan.close()


def test_fused_learned_step_matches_host_scaled_step():
  import torch
  from jrystal_gb300.calc import Minimizer
  from jrystal_gb300.precond import MLP, GuardedScale
  sysm = make_system(kind="si2", grid=(24, 24, 24), kgrid=(2, 1, 1), nb=8, nocc=4)
  plan = _plan(sysm, 32, 8)
  mlp = MLP(seed=11)
  p0, _, _ = _state(sysm, plan, 9)
  runs = {}
  for fused in (False, True):
    mini = Minimizer(plan, sysm.occupation, p0.clone(), lr=1e-2,
                     scale_fn=GuardedScale(mlp, total_steps=50), fused=fused, keep_grad=True)
    es = [float(mini.step()[4]) for _ in range(6)]
    runs[fused] = (mini.params.cpu().numpy(), es, mini.last_scale.cpu().numpy())
  np.testing.assert_allclose(runs[True][1], runs[False][1], rtol=1e-6)
  # the in-step form interpolates the network tabulated in x1 (4096 points
  # per band); BF16 inference: FP32-rounding differences of the inputs can
  # also move a hidden activation across a BF16 rounding boundary
  np.testing.assert_allclose(runs[True][2], runs[False][2], rtol=1e-3)
  np.testing.assert_allclose(runs[True][0], runs[False][0], rtol=1e-3, atol=1e-6)
  plan.close()


def test_fused_step_rejects_bad_arguments():
  import torch
  from jrystal_gb300 import _lib
  sysm = make_system(kind="si2", grid=(16, 16, 16), kgrid=(1, 1, 1), nb=40, nocc=4)
  plan = _plan(sysm, 32, 40)
  occ = torch.tensor(sysm.occupation, device="cuda")
  p, m, v = _state(sysm, plan, 1)
  lib = _lib.load()
  prev = lib.jrg_tensor_core_paths(3)   # register-blocked rotations: at most 32 bands
  try:
    with pytest.raises(NotImplementedError, match="num_band > 32"):
      plan.energy_grad_adam(p, m, v, occ, 1, 1e-2)
  finally:
    lib.jrg_tensor_core_paths(prev)
  with pytest.raises(ValueError):
    plan.energy_grad_adam(p, m.double(), v, occ, 1, 1e-2)
  with pytest.raises(ValueError, match="bad argument"):
    plan.energy_grad_adam(p, m, v, occ, 0, 1e-2)
  plan.close()
