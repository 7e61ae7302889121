"""The workspace bound (jrg_plan_set_memory_limit): with room for one
(s,k) block of plane transforms the energy entry points recompute the
planes per block instead of keeping them, and give the same energies and
gradients as the unbounded plan (and the same band trace)."""
import numpy as np
import pytest

from tests.systems import make_system, random_params

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", [64, 32])
def test_bounded_workspace_recomputes_planes_with_same_results(prec):
  import torch
  from jrystal_gb300.engine import PlaneWavePlan
  sysm = make_system(kind="si2", grid=(16, 16, 16), kgrid=(2, 2, 1), nb=6, nocc=3)
  mk = lambda: PlaneWavePlan(sysm.cell_vectors, sysm.positions, sysm.charges, sysm.grid, sysm.mask,
                             sysm.kpts, 6, 1, prec, sysm.xc)
  full, small = mk(), mk()
  nsk = sysm.kpts.shape[0]
  assert small.set_memory_limit(0) == nsk
  kc = small.set_memory_limit(small.workspace_bytes // 2)
  assert 1 <= kc < nsk
  assert small.set_memory_limit(1) == 1          # below the fixed part: one block at a time
  assert small.workspace_bytes < full.workspace_bytes
  wr, wi = random_params(sysm, seed=9)
  dt = torch.float64 if prec == 64 else torch.float32
  a = torch.tensor(wr, dtype=dt, device="cuda")
  b = torch.tensor(wi, dtype=dt, device="cuda")
  e1, g1r, g1i = full.energy_and_grad(a, b, sysm.occupation)
  e1 = e1.cpu().numpy().copy()
  g1 = torch.stack([g1r, g1i]).cpu().numpy()
  e2, g2r, g2i = small.energy_and_grad(a, b, sysm.occupation)
  e2 = e2.cpu().numpy()
  g2 = torch.stack([g2r, g2i]).cpu().numpy()
  tol = 1e-12 if prec == 64 else 1e-6
  assert np.abs(e1[:5] - e2[:5]).max() <= tol * np.abs(e1[:5]).max()
  assert np.abs(g1 - g2).max() <= tol * np.abs(g1).max()
  v = torch.tensor(np.random.default_rng(2).normal(size=sysm.grid), dtype=dt, device="cuda")
  t1 = full.band_trace_grad(a, b, v)[0].cpu().numpy()
  t2 = small.band_trace_grad(a, b, v)[0].cpu().numpy()
  assert np.abs(t1 - t2).max() <= tol * np.abs(t1).max()
  # the fused step takes the chunked single-stream path
  p = torch.stack([a, b]).contiguous()
  m, vv = torch.zeros_like(p), torch.zeros_like(p)
  e3 = small.energy_grad_adam(p, m, vv, sysm.occupation, 1, 1e-2).cpu().numpy()
  assert np.abs(e3[:5] - e1[:5]).max() <= tol * np.abs(e1[:5]).max()
