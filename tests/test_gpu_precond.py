"""Preconditioner kernels against the CPU oracle (oracle/mlp.py)."""
import numpy as np
import pytest

from oracle import mlp as M

pytestmark = pytest.mark.gpu


def _records(n, seed):
  rng = np.random.default_rng(seed)
  x = np.stack([rng.gamma(1.0, 2.0, n), rng.uniform(0, 1, n), rng.uniform(0, 1, n)], 1)
  a = rng.normal(size=n)
  c = np.abs(rng.normal(size=n)) + 0.1
  w = rng.uniform(0.5, 1.5, n)
  return x.astype(np.float32), a.astype(np.float32), c.astype(np.float32), w.astype(np.float32)


def test_mlp_forward_loss_and_gradient_match_oracle():
  import torch
  from jrystal_gb300.precond import MLP
  mlp = MLP(seed=5)
  # perturb the output bias so the loss gradient is not trivially small
  w = mlp.w32.cpu().numpy()
  x, a, c, wt = _records(3000, 1)
  t = lambda v: torch.tensor(v, device="cuda")
  s = mlp.forward(t(x)).cpu().numpy()
  s_ref, _ = M.forward(w, x)
  # tanh.approx.f32 in the device GELU: about 1e-3 relative on the output
  np.testing.assert_allclose(s, s_ref, rtol=5e-3, atol=1e-4)
  loss, grad = mlp.loss_and_grad(t(x), t(a), t(c), t(wt))
  l_ref, g_ref = M.loss_and_grad(w, x, a, c, wt)
  assert abs(float(loss) - l_ref) <= 5e-3 * abs(l_ref) + 1e-3
  g = grad.cpu().numpy()
  assert np.abs(g - g_ref).max() <= 2e-2 * np.abs(g_ref).max()
  cos = float(g @ g_ref / np.linalg.norm(g) / np.linalg.norm(g_ref))
  assert cos > 0.999


def test_tensor_core_inference_matches_training_forward():
  import torch
  from jrystal_gb300.precond import MLP
  from jrystal_gb300.engine import PlaneWavePlan
  from tests.systems import make_system, random_params
  sysm = make_system(kind="si2", grid=(16, 16, 16), kgrid=(2, 1, 1), nb=5, nocc=3)
  plan = PlaneWavePlan(sysm.cell_vectors, sysm.positions, sysm.charges, sysm.grid, sysm.mask,
                       sysm.kpts, 5, 1, 32, sysm.xc)
  wr, wi = random_params(sysm, seed=2, dtype=np.float32)
  occ = torch.tensor(sysm.occupation, device="cuda")
  plan.energy_and_grad(torch.tensor(wr, device="cuda"), torch.tensor(wi, device="cuda"), occ)
  mlp = MLP(seed=7)
  scale = mlp.scale(plan, 0.3, occ, smax=100.0).cpu().numpy()
  # features on the host from the plan's tables
  import ctypes as ct
  from jrystal_gb300 import _lib
  lib = _lib.load()
  S, K, G, B = plan.param_shape
  tk = torch.empty(K * G, dtype=torch.float64, device="cuda")
  ek = torch.empty(S * K * B, dtype=torch.float64, device="cuda")
  st = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
  assert lib.jrg_kinetic_table(plan._h, ct.c_void_p(tk.data_ptr()), st) == 0
  assert lib.jrg_band_kinetic(plan._h, ct.c_void_p(plan.workspace.data_ptr()),
                              ct.c_void_p(ek.data_ptr()), st) == 0
  tk, ek = tk.cpu().numpy().reshape(K, G), ek.cpu().numpy().reshape(S, K, B)
  x1 = tk[None, :, :, None] / ek[:, :, None, :]
  x2 = np.broadcast_to(np.arange(B) / B, (S, K, G, B))
  x = np.stack([x1.reshape(-1), x2.reshape(-1), np.full(x1.size, 0.3)], 1).astype(np.float32)
  ref = mlp.forward(torch.tensor(x, device="cuda")).cpu().numpy().reshape(S, K, G, B)
  occb = sysm.occupation[:, :, None, :] > 0
  got = scale[0]
  np.testing.assert_allclose(got[np.broadcast_to(occb, got.shape)],
                             ref[np.broadcast_to(occb, ref.shape)], rtol=2e-2, atol=2e-3)
  assert np.all(got[~np.broadcast_to(occb, got.shape)] == 1.0)
  np.testing.assert_array_equal(scale[0], scale[1])
  # the per-band kinetic energies agree with the oracle
  from oracle import restatement as R
  c, _ = R.cholesky_qr(wr.astype(np.float64), wi.astype(np.float64))
  tko = R.kinetic_operator(sysm.g_vector_grid, sysm.kpts)[:, sysm.mask]
  ek_ref = np.einsum("kg,skgb->skb", tko, np.abs(c)**2)
  np.testing.assert_allclose(ek, ek_ref, rtol=1e-5)
