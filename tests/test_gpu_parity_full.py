"""Full-size parity of the benchmarked configurations, through the C ABI.

* Si8 cubic cell, 64^3 grid, 27 k-points, 24 bands (16 occupied), N(0, 1)
  parameters from seed 1: the FP32 path against the FP64 path of the same
  kernels, at the initial parameters and after 200 Adam steps of the FP32
  path; the FP64 path against the FP64 CPU oracle; the gradient against
  central differences (h = 1e-4) on 64 seeded coefficients.
* Si2 FCC cell, 48^3 grid, 8 k-points, 8 bands, FP64, seed 0: against the
  oracle.

Tolerances: energies within 1e-6 Ha per atom (each term and the total) and
gradients within 1e-5 relative (2-norm over all parameters) for FP32 against
FP64; 1e-10 Ha per atom and 1e-10 relative for FP64 against the oracle.
"""
import os

import numpy as np
import pytest

from oracle import restatement as R

pytestmark = pytest.mark.gpu

E_ATOM_FP32 = 1e-6
G_REL_FP32 = 1e-5
E_ATOM_FP64 = 1e-10
G_REL_FP64 = 1e-10
NAMES = ["kinetic", "external", "hartree", "xc", "total"]


def _setup(wl, prec):
  import torch
  from jrystal_gb300.engine import PlaneWavePlan
  plan = PlaneWavePlan(wl.cell, wl.positions, wl.charges, wl.grid_sizes, wl.mask, wl.kpts,
                       wl.num_band, 1, prec, wl.xc, device="cuda:0")
  occ = torch.tensor(wl.occupation, dtype=torch.float64, device="cuda:0")
  return plan, occ


def _eval(plan, params, occ):
  import torch
  p = params.to(plan.rdtype)
  e, gr, gi = plan.energy_and_grad(p[0].contiguous(), p[1].contiguous(), occ)
  torch.cuda.synchronize()
  return e.cpu().numpy().copy(), torch.stack([gr, gi]).double().cpu().numpy()


def _check(e32, g32, e64, g64, natom, etol, gtol):
  for i, n in enumerate(NAMES):
    assert abs(e32[i] - e64[i]) / natom <= etol, (n, e32[i], e64[i])
  rel = np.linalg.norm(g32 - g64) / np.linalg.norm(g64)
  assert rel <= gtol, rel
  assert np.abs(g32 - g64).max() <= gtol * np.abs(g64).max()
  assert e32[6] == 0.0 and e64[6] == 0.0


@pytest.fixture(scope="module")
def si8():
  import torch
  from jrystal_gb300 import workloads
  wl = workloads.si8_cubic(32)
  p32, occ = _setup(wl, 32)
  p64, _ = _setup(wl, 64)
  wr, wi = wl.init_params()
  params = torch.tensor(np.stack([wr, wi]), dtype=torch.float32, device="cuda:0").contiguous()
  return wl, p32, p64, occ, params


def test_si8_fp32_vs_fp64_initial(si8):
  wl, p32, p64, occ, params = si8
  e32, g32 = _eval(p32, params, occ)
  e64, g64 = _eval(p64, params.double(), occ)
  _check(e32, g32, e64, g64, len(wl.charges), E_ATOM_FP32, G_REL_FP32)


def test_si8_fp32_vs_fp64_after_200_steps(si8):
  import torch
  wl, p32, p64, occ, params = si8
  p = params.clone()
  m = torch.zeros_like(p)
  v = torch.zeros_like(p)
  for t in range(1, 201):
    p32.energy_grad_adam(p, m, v, occ, t, wl.lr)
  e32, g32 = _eval(p32, p, occ)
  e64, g64 = _eval(p64, p.double(), occ)
  # the parameters moved: the energy is no longer the initial one
  assert e64[4] < -400.0
  _check(e32, g32, e64, g64, len(wl.charges), E_ATOM_FP32, G_REL_FP32)


def test_si8_fp64_vs_oracle(si8):
  wl, p32, p64, occ, params = si8
  R.FFT_WORKERS = len(os.sched_getaffinity(0))
  w = params.double().cpu().numpy()
  sysm = R.System(wl.cell, wl.positions, wl.charges, wl.grid_sizes, wl.mask, wl.kpts, wl.occupation,
                  wl.xc)
  terms, gr, gi, _ = R.energy_terms(w[0], w[1], sysm)
  e64, g64 = _eval(p64, params.double(), occ)
  ref = np.array([terms[n] for n in NAMES])
  assert np.abs(e64[:5] - ref).max() / len(wl.charges) <= E_ATOM_FP64, (e64[:5], ref)
  g = np.stack([gr, gi])
  assert np.linalg.norm(g64 - g) / np.linalg.norm(g) <= G_REL_FP64


def test_si8_central_differences(si8):
  """Central differences (h = 1e-4) of the FP64 energy on 64 seeded
  coefficients of the occupied bands against the FP64 and FP32 gradients,
  and a zero gradient on the empty bands.  The difference quotient carries
  the rounding of E (~1e-12 Ha) over 2h, about 1e-5 of these entries, so the
  bound is 1e-4 relative (2-norm); an adjoint error would show at O(1)."""
  import torch
  wl, p32, p64, occ, params = si8
  rng = np.random.default_rng(1)
  _, K, G, B = params.shape[1:]
  idx = [(int(rng.integers(2)), int(rng.integers(K)), int(rng.integers(G)), int(rng.integers(wl.num_occ)))
         for _ in range(64)]
  h = 1e-4
  base = params.double()
  fd = []
  for (part, k, g, b) in idx:
    vals = []
    for s in (1.0, -1.0):
      w = base.clone()
      w[part, 0, k, g, b] += s * h
      e, _, _ = p64.energy_and_grad(w[0].contiguous(), w[1].contiguous(), occ, with_grad=False)
      vals.append(float(e[4].item()))
    fd.append((vals[0] - vals[1]) / (2 * h))
  fd = np.array(fd)
  _, g64 = _eval(p64, base, occ)
  _, g32 = _eval(p32, params, occ)
  for g in (g64, g32):
    an = np.array([g[p, 0, k, gg, b] for (p, k, gg, b) in idx])
    assert np.linalg.norm(an - fd) / np.linalg.norm(fd) <= 1e-4
  # empty bands do not enter the energy (Cholesky QR keeps the first columns)
  assert np.abs(g64[:, :, :, :, wl.num_occ:]).max() <= 1e-10 * np.abs(g64).max()
  torch.cuda.synchronize()


def test_si2_fp64_vs_oracle():
  import torch
  from jrystal_gb300 import workloads
  wl = workloads.si2_fcc(64)
  plan, occ = _setup(wl, 64)
  wr, wi = wl.init_params()
  params = torch.tensor(np.stack([wr, wi]), dtype=torch.float64, device="cuda:0")
  e, g = _eval(plan, params, occ)
  sysm = R.System(wl.cell, wl.positions, wl.charges, wl.grid_sizes, wl.mask, wl.kpts, wl.occupation,
                  wl.xc)
  terms, gr, gi, _ = R.energy_terms(wr, wi, sysm)
  ref = np.array([terms[n] for n in NAMES])
  assert np.abs(e[:5] - ref).max() / len(wl.charges) <= E_ATOM_FP64
  gref = np.stack([gr, gi])
  assert np.linalg.norm(g - gref) / np.linalg.norm(gref) <= G_REL_FP64
