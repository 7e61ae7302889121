"""Batched trajectory generation (jrg_batch_*) against the single-cell loop.

A mixed batch of strained Si / C / Al cells (different grids, band counts and
sphere sizes) takes plain Adam steps through one graph launch per step; each
cell must follow exactly (bit for bit: the kernels are deterministic) the
trajectory of the same cell stepped alone (jrg_energy_grad, then
jrg_adam_update), its first energy must match the FP64 oracle, and the records
drawn on the device must equal the one-step secant records recomputed on the
host from that single-cell trajectory at the drawn elements."""
import numpy as np
import pytest

from oracle import restatement as R

pytestmark = pytest.mark.gpu

STEPS, PER_STEP, LR = 6, 5, 1e-2


def _cells():
  from jrystal_gb300 import cells
  rng = np.random.default_rng(5)
  kinds = ["si", "c", "al", "si"]
  grids = [(24,), (27,), (24,), (32,)]
  bands = [(8, 8), (10, 10), (9, 9), (12, 12)]
  return [cells.strained_cell(rng, kind=k, grids=g, bands=b) for k, g, b in zip(kinds, grids, bands)]


def _single(wl):
  """Energies (steps, 8), parameters before each update (steps + 1), the
  gradient and band kinetic energies of each step, from the one-cell loop."""
  import ctypes as ct
  import torch
  from jrystal_gb300 import _lib
  from jrystal_gb300.batch import _plan
  from jrystal_gb300.engine import _ptr, _stream, adam_update
  plan = _plan(wl)
  wr, wi = wl.init_params()
  p = torch.tensor(np.stack([wr, wi]), dtype=plan.rdtype, device="cuda")
  m, v, g = torch.zeros_like(p), torch.zeros_like(p), torch.zeros_like(p)
  occ = torch.as_tensor(np.asarray(wl.occupation), dtype=torch.float64, device="cuda")
  ekin = torch.empty(plan.num_kpt * plan.num_band, dtype=torch.float64, device="cuda")
  es, ps, gs, ks = [], [p.clone()], [], []
  for t in range(STEPS):
    e, _, _ = plan.energy_and_grad(p[0], p[1], occ, g[0], g[1])
    _lib.check(plan.lib.jrg_band_kinetic(plan._h, _ptr(plan.workspace), _ptr(ekin), _stream()), "")
    es.append(e.clone()); gs.append(g.clone()); ks.append(ekin.clone())
    adam_update(p, g, m, v, t + 1, LR)
    ps.append(p.clone())
  tk = torch.empty(plan.num_kpt * plan.num_g, dtype=torch.float64, device="cuda")
  _lib.check(plan.lib.jrg_kinetic_table(plan._h, _ptr(tk), _stream()), "")
  out = dict(e=torch.stack(es).cpu().numpy(), p=torch.stack(ps).cpu().numpy().astype(np.float64),
             g=torch.stack(gs).cpu().numpy().astype(np.float64), ekin=torch.stack(ks).cpu().numpy(),
             tk=tk.cpu().numpy(), shape=plan.param_shape)
  plan.close()
  return out


def _expected_records(ref, idx, occ):
  """Host recomputation of the secant records of the drawn elements."""
  S, K, G, B = ref["shape"]
  n = S * K * G * B
  P = PER_STEP
  xs, As, Cs, Ws = [], [], [], []
  for t in range(STEPS - 1):
    ii = idx[t * P:(t + 1) * P]
    pt, pn = ref["p"][t].reshape(2, n), ref["p"][t + 1].reshape(2, n)
    gt, gn = ref["g"][t].reshape(2, n), ref["g"][t + 1].reshape(2, n)
    u = pn[:, ii] - pt[:, ii]
    a = (gt[:, ii] * u).sum(0)
    c = np.maximum(((gn[:, ii] - gt[:, ii]) * u).sum(0), 0.25 * np.abs(a))
    tot = np.abs(a).sum()
    Ws.append(np.full(P, (np.abs(a) > 0).sum() / tot if tot > 0 else 0.0))
    b = ii % B
    sk = ii // (G * B)
    gi = (ii // B) % G
    band = sk * B + b
    assert np.all(occ.reshape(-1)[band] > 0)
    xs.append(np.stack([ref["tk"][(sk % K) * G + gi] / ref["ekin"][t][band], b / B,
                        np.full(P, t / STEPS)], 1))
    As.append(a); Cs.append(c)
  return np.concatenate(xs), np.concatenate(As), np.concatenate(Cs), np.concatenate(Ws)


def test_batch_matches_single_cell_trajectories_and_records():
  import torch
  from jrystal_gb300.batch import TrajectoryBatch
  wls = _cells()
  batch = TrajectoryBatch(wls, STEPS, lr=LR, per_step=PER_STEP, seed=11)
  batch.step(graph=False)           # eager first step, graph replay after it
  batch.run()
  torch.cuda.synchronize()
  assert batch.steps_done == STEPS
  with pytest.raises(ValueError):
    batch.step()
  hist = batch.energies.cpu().numpy()
  rec = {k: v.cpu().numpy() for k, v in batch.records().items()}
  idx = batch.record_index().cpu().numpy()
  rows = (STEPS - 1) * PER_STEP
  for c, wl in enumerate(wls):
    ref = _single(wl)
    assert np.array_equal(hist[:, c, :], ref["e"]), wl.name
    assert np.array_equal(batch.params[c].cpu().numpy().astype(np.float64), ref["p"][-1]), wl.name
    assert np.all(hist[:, c, 6] == 0.0)
    x, a, cc, w = _expected_records(ref, idx[c], np.asarray(wl.occupation))
    sl = slice(c * rows, (c + 1) * rows)
    np.testing.assert_allclose(rec["x"][sl], x, rtol=1e-6, atol=0)
    np.testing.assert_allclose(rec["a"][sl], a, rtol=1e-5, atol=1e-6 * np.abs(a).max())
    np.testing.assert_allclose(rec["c"][sl], cc, rtol=1e-5, atol=1e-6 * np.abs(cc).max())
    np.testing.assert_allclose(rec["w"][sl], w, rtol=1e-5)
  batch.close()


def test_batch_first_energies_match_oracle():
  """FP64 and FP32 cells in one batch; FP64 to 1e-10 relative per term, FP32
  within the FP32 path's per-term tolerance of 2e-6 relative."""
  import dataclasses
  from jrystal_gb300.batch import TrajectoryBatch
  wls = [dataclasses.replace(wl, precision=p) for wl, p in zip(_cells()[:3], (64, 32, 64))]
  batch = TrajectoryBatch(wls, 1, lr=LR, per_step=0)
  batch.run()
  hist = batch.energies.cpu().numpy()
  for c, wl in enumerate(wls):
    sysm = R.System(wl.cell, wl.positions, wl.charges, wl.grid_sizes, wl.mask, wl.kpts,
                    np.asarray(wl.occupation), wl.xc)
    wr, wi = wl.init_params()
    terms, _, _, _ = R.energy_terms(wr.astype(np.float64), wi.astype(np.float64), sysm)
    tol = 1e-10 if wl.precision == 64 else 2e-6
    for i, name in enumerate(["kinetic", "external", "hartree", "xc", "total"]):
      ref = terms[name]
      assert abs(hist[0, c, i] - ref) <= tol * max(1.0, abs(ref)), (wl.name, name, hist[0, c, i], ref)
  batch.close()


def test_batch_graph_and_eager_agree():
  import torch
  from jrystal_gb300.batch import TrajectoryBatch
  wls = _cells()[:2]
  a = TrajectoryBatch(wls, 4, lr=LR, per_step=3, seed=1)
  a.run(graph=True)
  b = TrajectoryBatch(wls, 4, lr=LR, per_step=3, seed=1)
  b.run(graph=False)
  torch.cuda.synchronize()
  assert torch.equal(a.energies, b.energies)
  for k in ("x", "a", "c", "w"):
    assert torch.equal(a.records()[k], b.records()[k])
  for c in range(2):
    assert torch.equal(a.params[c], b.params[c])
  a.close()
  b.close()
