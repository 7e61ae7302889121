"""PBE (gga_x_pbe + gga_c_pbe) on the GPU against the oracle: energy terms
and gradient of the fused path, the Kohn-Sham potential and the energy
density of jrg_potential, and the ground-state driver with a PBE config."""
import numpy as np
import pytest

from oracle import restatement as R
from tests.systems import make_system, random_params

pytestmark = pytest.mark.gpu

XC = "gga_x_pbe+gga_c_pbe"
TOL = {64: dict(e=1e-9, g=1e-8), 32: dict(e=3e-6, g=3e-4)}


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("case", [dict(kind="si2", grid=(16, 16, 16), kgrid=(2, 1, 1), nb=4, nocc=2),
                                  dict(kind="diamond", grid=(24, 24, 24), kgrid=(1, 1, 2), nb=6, nocc=4),
                                  dict(kind="si2", grid=(15, 12, 10), kgrid=(1, 1, 1), nb=3, nocc=2)])
def test_pbe_energy_and_gradient(prec, case):
  import torch
  from jrystal_gb300.engine import PlaneWavePlan
  sysm = make_system(xc=XC, **case)
  wr, wi = random_params(sysm, seed=12)
  terms, gr, gi, _ = R.energy_terms(wr, wi, sysm)
  plan = PlaneWavePlan(sysm.cell_vectors, sysm.positions, sysm.charges, sysm.grid, sysm.mask,
                       sysm.kpts, case["nb"], 1, prec, XC)
  dt = torch.float64 if prec == 64 else torch.float32
  e, g1, g2 = plan.energy_and_grad(torch.tensor(wr, dtype=dt, device="cuda"),
                                   torch.tensor(wi, dtype=dt, device="cuda"), sysm.occupation)
  e = e.cpu().numpy()
  tol = TOL[prec]
  for i, name in enumerate(["kinetic", "external", "hartree", "xc", "total"]):
    assert abs(e[i] - terms[name]) <= tol["e"] * max(1.0, abs(terms[name])), (name, e[i], terms[name])
  scale = max(np.abs(gr).max(), np.abs(gi).max())
  err = max(np.abs(g1.cpu().numpy() - gr).max(), np.abs(g2.cpu().numpy() - gi).max())
  assert err <= tol["g"] * scale, (err, scale)
  plan.close()


def test_pbe_potential_and_energy_density():
  import torch
  from jrystal_gb300.engine import PlaneWavePlan
  sysm = make_system(kind="si2", grid=(16, 16, 16), kgrid=(2, 1, 1), nb=4, nocc=2, xc=XC)
  wr, wi = random_params(sysm, seed=13)
  c, _ = R.cholesky_qr(wr, wi)
  rho = R.density_grid(R.expand_coefficient(c, sysm.mask), sysm.vol, sysm.occupation)
  e_xc, v_xc, fval = R.gga_energy_potential(rho[0], sysm.g_vector_grid, sysm.vol, XC)
  plan = PlaneWavePlan(sysm.cell_vectors, sysm.positions, sysm.charges, sysm.grid, sysm.mask,
                       sysm.kpts, 4, 1, 64, XC)
  t = torch.tensor(rho, device="cuda")
  vks = plan.potential(t, kohn_sham=True).cpu().numpy()
  np.testing.assert_allclose(vks[2], v_xc, atol=1e-9 * np.abs(v_xc).max())
  eps = plan.potential(t, kohn_sham=False).cpu().numpy()[2]
  ok = rho[0] > 1e-15
  np.testing.assert_allclose(eps[ok], fval[ok] / rho[0][ok], rtol=1e-9)
  plan.close()


def test_pbe_driver():
  import jrystal_gb300 as jr
  from jrystal_gb300 import grid as G
  a = 6.74
  cell = np.array([[0, a / 2, a / 2], [a / 2, 0, a / 2], [a / 2, a / 2, 0]])
  pos = np.array([[0, 0, 0], [0.25, 0.25, 0.25]]) @ cell
  crystal = jr.Crystal(charges=np.array([6.0, 6.0]), positions=pos, cell_vectors=cell)
  cfg = {"crystal": crystal, "grid_sizes": 16, "k_grid_sizes": [1, 1, 1], "xc": XC,
         "cutoff_energy": float(G.alias_free_cutoff(cell, 16)), "epoch": 200,
         "optimizer_args": {"learning_rate": 1e-2, "b1": 0.9, "b2": 0.99},
         "convergence_condition": 1e-12, "jax_enable_x64": True}
  out = jr.calc.energy_all_electrons(cfg)
  h = out.total_energy_history
  assert h[-1] < h[0]
  mask = G.spherical_mask(cell, (16,) * 3, cfg["cutoff_energy"])
  occ = np.zeros((1, 1, 6))
  occ[..., :6] = 2.0
  sysm = R.System(cell, pos, np.array([6.0, 6.0]), (16,) * 3, mask, G.k_vectors(cell, (1, 1, 1)),
                  occ, XC)
  ref = R.energy_terms(out.params_pw["w_re"].cpu().numpy(), out.params_pw["w_im"].cpu().numpy(),
                       sysm, with_grad=False)
  assert abs(out.energy_terms["total"] - ref["total"]) < 1e-8 * abs(ref["total"])


def test_pbe_functional_api():
  import torch
  import jrystal_gb300 as jr
  jr.set_precision(64)
  sysm = make_system(kind="diamond", grid=(16, 16, 16), kgrid=(1, 1, 1), nb=4, nocc=3, xc=XC)
  wr, wi = random_params(sysm, seed=14)
  c, _ = R.cholesky_qr(wr, wi)
  rho = R.density_grid(R.expand_coefficient(c, sysm.mask), sysm.vol, sysm.occupation)
  g = sysm.g_vector_grid
  e_xc, v_xc, fval = R.gga_energy_potential(rho[0], g, sysm.vol, XC)
  t = torch.tensor(rho, device="cuda")
  v = jr.xc.xc_density(t, g, kohn_sham=True, xc_type=XC).cpu().numpy()
  np.testing.assert_allclose(v[0], v_xc, atol=1e-9 * np.abs(v_xc).max())
  e = float(jr.energy.xc_energy(t, g, sysm.vol, XC))
  assert abs(e - e_xc) < 1e-9 * abs(e_xc)
  vh, ve, vx = jr.potential.effective(t, sysm.positions, sysm.charges, g, sysm.vol, split=True,
                                      xc_type=XC, kohn_sham=True)
  np.testing.assert_allclose(vx.cpu().numpy()[0], v_xc, atol=1e-9 * np.abs(v_xc).max())
