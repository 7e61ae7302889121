"""torch.autograd through the jrystal-named functional modules.

jrystal differentiates pw.coeff -> energy.total_energy with jax.grad
(calc/calc_ground_state_energy_all_electrons.py:119-181); here the same
composition runs on the library's FFT, LDA/PBE and Cholesky-QR kernels with
their vector-Jacobian products, and its gradient is compared with the FP64
oracle's hand-derived gradient (oracle.restatement.energy_terms)."""
import numpy as np
import pytest

from oracle import restatement as R
from tests.systems import make_system, random_params

pytestmark = pytest.mark.gpu


def test_fft_vjp_gradcheck():
  import torch
  from jrystal_gb300._ops import fftn, ifftn
  rng = np.random.default_rng(0)
  x = rng.normal(size=(2, 4, 5, 6)) + 1j * rng.normal(size=(2, 4, 5, 6))
  t = torch.tensor(x, dtype=torch.complex128, device="cuda", requires_grad=True)
  assert torch.autograd.gradcheck(fftn, (t,), eps=1e-6, atol=1e-8)
  assert torch.autograd.gradcheck(ifftn, (t,), eps=1e-6, atol=1e-8)
  r = torch.tensor(rng.normal(size=(1, 4, 5, 6)), dtype=torch.float64, device="cuda", requires_grad=True)
  assert torch.autograd.gradcheck(lambda a: fftn(a).abs().sum(), (r,), eps=1e-6, atol=1e-8)


def test_lda_eps_vjp_gradcheck():
  import torch
  from jrystal_gb300._ops import lda_eps
  rng = np.random.default_rng(1)
  rho = torch.tensor(rng.uniform(0.01, 2.0, size=(3, 4, 5)), dtype=torch.float64, device="cuda",
                     requires_grad=True)
  assert torch.autograd.gradcheck(lambda r: lda_eps(r, "lda_x+lda_c_vwn"), (rho,), eps=1e-7, atol=1e-7,
                                  rtol=1e-5)


@pytest.mark.parametrize("prec", [64, 32])
def test_functional_total_energy_gradient_matches_oracle(prec):
  import torch
  from jrystal_gb300 import energy, pw
  from jrystal_gb300._ops import set_precision
  set_precision(prec)
  try:
    sysm = make_system(kind="si2", grid=(16, 16, 16), kgrid=(2, 1, 1), nb=6, nocc=3)
    wr, wi = random_params(sysm, seed=4)
    dt = torch.float64 if prec == 64 else torch.float32
    tr = torch.tensor(wr, dtype=dt, device="cuda", requires_grad=True)
    ti = torch.tensor(wi, dtype=dt, device="cuda", requires_grad=True)
    c = pw.coeff({"w_re": tr, "w_im": ti}, sysm.mask)
    e = energy.total_energy(c, sysm.positions, sysm.charges, sysm.g_vector_grid, sysm.kpts, sysm.vol,
                            occupation=sysm.occupation, kohn_sham=False, xc=sysm.xc)
    gr, gi = torch.autograd.grad(e, [tr, ti])
    terms, ogr, ogi, _ = R.energy_terms(wr, wi, sysm)
    etol, gtol = (1e-10, 1e-9) if prec == 64 else (1e-5, 1e-4)
    assert abs(float(e.detach()) - terms["total"]) <= etol * abs(terms["total"])
    g = np.stack([gr.double().cpu().numpy(), gi.double().cpu().numpy()])
    og = np.stack([ogr, ogi])
    assert np.linalg.norm(g - og) <= gtol * np.linalg.norm(og)
  finally:
    set_precision(64)


def test_functional_terms_gradients_by_central_differences():
  """Each differentiable term of energy.py on its own (hartree, external,
  xc_energy, kinetic) against central differences in two parameters."""
  import torch
  from jrystal_gb300 import energy, pw
  sysm = make_system(kind="diamond", grid=(12, 12, 12), kgrid=(1, 1, 1), nb=3, nocc=2)
  wr, wi = random_params(sysm, seed=5)
  g = sysm.g_vector_grid

  def terms(a, b):
    c = pw.coeff({"w_re": a, "w_im": b}, sysm.mask)
    rho = pw.density_grid(c, sysm.vol, sysm.occupation)
    rho_g = pw.density_grid_reciprocal(c, sysm.vol, sysm.occupation)
    return [energy.hartree(rho_g, g, sysm.vol), energy.external(rho_g, sysm.positions, sysm.charges, g, sysm.vol),
            energy.xc_energy(rho, g, sysm.vol, sysm.xc), energy.kinetic(g, sysm.kpts, c, sysm.occupation)]

  tr = torch.tensor(wr, device="cuda", requires_grad=True)
  ti = torch.tensor(wi, device="cuda", requires_grad=True)
  vals = terms(tr, ti)
  h = 1e-5
  for n, val in enumerate(vals):
    gr, gi = torch.autograd.grad(val, [tr, ti], retain_graph=True)
    for (part, idx) in ((0, (0, 0, 7, 1)), (1, (0, 0, 3, 0))):
      diffs = []
      for s in (1.0, -1.0):
        a, b = tr.detach().clone(), ti.detach().clone()
        (a if part == 0 else b)[idx] += s * h
        diffs.append(float(terms(a, b)[n]))
      fd = (diffs[0] - diffs[1]) / (2 * h)
      an = float((gr if part == 0 else gi)[idx])
      assert abs(an - fd) <= 1e-6 * max(1.0, abs(fd)), (n, part, an, fd)


def test_pbe_xc_energy_gradient_by_central_differences():
  import torch
  from jrystal_gb300 import energy
  sysm = make_system(kind="si2", grid=(16, 16, 16), kgrid=(1, 1, 1), nb=2, nocc=1)
  rng = np.random.default_rng(6)
  base = 0.05 + 0.02 * rng.random(size=(1, 16, 16, 16))
  rho = torch.tensor(base, device="cuda", requires_grad=True)
  xc = "gga_x_pbe+gga_c_pbe"
  e = energy.xc_energy(rho, sysm.g_vector_grid, sysm.vol, xc)
  (gr,) = torch.autograd.grad(e, [rho])
  h = 1e-6
  for idx in ((0, 1, 2, 3), (0, 9, 4, 15)):
    vals = []
    for s in (1.0, -1.0):
      r = rho.detach().clone()
      r[idx] += s * h
      vals.append(float(energy.xc_energy(r, sysm.g_vector_grid, sysm.vol, xc)))
    fd = (vals[0] - vals[1]) / (2 * h)
    assert abs(float(gr[idx]) - fd) <= 1e-5 * abs(fd), (idx, float(gr[idx]), fd)
