"""Occupation gradient on the GPU (jrg_energy_grad_bands) against the oracle,
and the learnable-occupation driver path (simplex projector, smearing)."""
import numpy as np
import pytest

from oracle import restatement as R
from tests.systems import make_system, random_params

pytestmark = pytest.mark.gpu

TOL = {64: dict(e=1e-10, g=1e-9), 32: dict(e=2e-6, g=2e-4)}


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("case", [dict(kind="si2", grid=(16, 16, 16), kgrid=(2, 1, 1), nb=6, nocc=3),
                                  dict(kind="si8", grid=(24, 24, 24), kgrid=(1, 1, 2), nb=20, nocc=16)])
def test_energy_grad_bands_matches_oracle(prec, case):
  import torch
  from jrystal_gb300.engine import PlaneWavePlan
  sysm = make_system(**case)
  rng = np.random.default_rng(5)
  sysm.occupation = rng.uniform(0.0, 2.0 / sysm.kpts.shape[0], size=sysm.occupation.shape)
  sysm.occupation[0, 0, -1] = 0.0                  # an empty band in the middle of the set
  wr, wi = random_params(sysm, seed=6)
  terms, gr, gi, v = R.energy_terms(wr, wi, sysm)
  eps = np.einsum("...ii->...i", R.band_trace_terms(wr, wi, v, sysm, with_grad=False)["hmat"]).real
  plan = PlaneWavePlan(sysm.cell_vectors, sysm.positions, sysm.charges, sysm.grid, sysm.mask,
                       sysm.kpts, case["nb"], 1, prec, sysm.xc)
  dt = torch.float64 if prec == 64 else torch.float32
  twr = torch.tensor(wr, dtype=dt, device="cuda")
  twi = torch.tensor(wi, dtype=dt, device="cuda")
  e, g1, g2, be = plan.energy_grad_bands(twr, twi, sysm.occupation)
  e = e.cpu().numpy()
  tol = TOL[prec]
  for i, name in enumerate(["kinetic", "external", "hartree", "xc", "total"]):
    assert abs(e[i] - terms[name]) <= tol["e"] * max(1.0, abs(terms[name])), name
  scale = max(np.abs(gr).max(), np.abs(gi).max())
  assert max(np.abs(g1.cpu().numpy() - gr).max(), np.abs(g2.cpu().numpy() - gi).max()) <= tol["g"] * scale
  np.testing.assert_allclose(be.cpu().numpy(), eps, rtol=0, atol=tol["e"] * 10 * np.abs(eps).max())
  plan.close()


def test_learnable_occupation_driver_on_aluminium():
  import jrystal_gb300 as jr
  from jrystal_gb300 import grid as G
  a = 7.65
  cell = np.array([[0, a / 2, a / 2], [a / 2, 0, a / 2], [a / 2, a / 2, 0]])
  crystal = jr.Crystal(charges=np.array([13.0]), positions=np.zeros((1, 3)), cell_vectors=cell)
  grid = 16
  cfg = {"crystal": crystal, "grid_sizes": grid, "k_grid_sizes": [2, 2, 2],
         "cutoff_energy": float(G.alias_free_cutoff(cell, grid)), "epoch": 600,
         "occupation": "simplex-projector", "smearing": 0.01, "empty_bands": 4,
         "optimizer_args": {"learning_rate": 1e-2, "b1": 0.9, "b2": 0.99},
         "convergence_condition": 1e-12, "seed": 3, "jax_enable_x64": True}
  out = jr.calc.energy_all_electrons(cfg)
  occ = out.occupation.cpu().numpy()
  assert abs(occ.sum() - 13.0) < 1e-8
  assert occ.min() >= -1e-12 and occ.max() <= 2.0 / 8 + 1e-12
  h = np.array(out.total_energy_history)
  assert h[-1] < h[0] and h[-1] < h[len(h) // 2]
  # the reported energy terms equal the oracle's at the final parameters and occupations
  mask = G.spherical_mask(cell, (grid,) * 3, cfg["cutoff_energy"])
  sysm = R.System(cell, crystal.positions, crystal.charges, (grid,) * 3, mask,
                  G.k_vectors(cell, (2, 2, 2)), occ, "lda_x+lda_c_vwn")
  terms = R.energy_terms(out.params_pw["w_re"].cpu().numpy(), out.params_pw["w_im"].cpu().numpy(),
                         sysm, with_grad=False)
  assert abs(out.energy_terms["total"] - terms["total"]) < 1e-9 * abs(terms["total"])
  ent = R.fermi_dirac_entropy(occ)
  assert abs(out.energy_terms["entropy"] - ent) < 1e-9 * max(1.0, abs(ent))
