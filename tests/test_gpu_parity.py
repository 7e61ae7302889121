"""CUDA path vs the FP64 oracle, called through the C ABI (ctypes)."""
import numpy as np
import pytest

from oracle import restatement as R
from tests.systems import make_system, random_params

pytestmark = pytest.mark.gpu

# Tolerances: the FP64 path must agree with the FP64 oracle to rounding; the
# FP32 path (FFT/density/potential in FP32, Gram/Cholesky/energy sums in FP64)
# within 2e-6 relative on each energy term and 1e-4 of the gradient scale.
TOL = {64: dict(e_rel=1e-10, g_rel=1e-9), 32: dict(e_rel=2e-6, g_rel=1e-4)}


def _torch():
  import torch
  return torch


def _plan(sysm, prec):
  from jrystal_gb300.engine import PlaneWavePlan
  return PlaneWavePlan(sysm.cell_vectors, sysm.positions, sysm.charges, sysm.grid, sysm.mask,
                       sysm.kpts, sysm.occupation.shape[-1], 1, prec, sysm.xc)


CASES = [
  dict(kind="diamond", grid=(12, 12, 12), kgrid=(2, 1, 1), nb=4, nocc=2),
  dict(kind="si2", grid=(16, 16, 16), kgrid=(2, 2, 2), nb=8, nocc=4),
  dict(kind="diamond", grid=(14, 15, 16), kgrid=(1, 1, 1), nb=3, nocc=3),
  dict(kind="si2", grid=(10, 12, 9), kgrid=(1, 2, 1), nb=5, nocc=2, mask="cubic"),
  # cubic grids covered by the register-resident slab kernels
  dict(kind="diamond", grid=(24, 24, 24), kgrid=(1, 1, 2), nb=4, nocc=2),
  dict(kind="si2", grid=(27, 27, 27), kgrid=(1, 1, 1), nb=3, nocc=2),
  dict(kind="si2", grid=(32, 32, 32), kgrid=(2, 1, 1), nb=4, nocc=2, mask="cubic"),
  dict(kind="si8", grid=(36, 36, 36), kgrid=(1, 1, 1), nb=5, nocc=3),
  dict(kind="si2", grid=(48, 48, 48), kgrid=(1, 1, 1), nb=3, nocc=2),
  dict(kind="si8", grid=(64, 64, 64), kgrid=(1, 1, 1), nb=3, nocc=2),
  # register-blocked Gram with 2, 3 and 4 rows per thread (9-32 bands)
  dict(kind="si2", grid=(16, 16, 16), kgrid=(1, 1, 1), nb=12, nocc=6),
  dict(kind="si8", grid=(24, 24, 24), kgrid=(1, 1, 1), nb=20, nocc=16),
  dict(kind="si8", grid=(16, 16, 16), kgrid=(2, 1, 1), nb=30, nocc=16),
  # more than 32 bands: tiled Gram, 32-wide rotation tiles, global-memory Cholesky
  dict(kind="si2", grid=(16, 16, 16), kgrid=(1, 1, 2), nb=40, nocc=20),
  # 32^3 sphere: the pruned eight-values-per-thread transforms
  dict(kind="si8", grid=(32, 32, 32), kgrid=(2, 1, 1), nb=4, nocc=2),
  # the band count of the Si64 supercell workload (160 bands, 128 occupied)
  dict(kind="si8", grid=(32, 32, 32), kgrid=(1, 1, 1), nb=160, nocc=128),
  # more than 32 bands, not a multiple of 4 (scalar loads and stores, a
  # partial last tile), two k-points (pipelined step)
  dict(kind="si2", grid=(16, 16, 16), kgrid=(1, 1, 2), nb=37, nocc=18),
]


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_energy_and_grad(prec, case):
  torch = _torch()
  sysm = make_system(**CASES[case])
  wr, wi = random_params(sysm, seed=case)
  terms, gr, gi, _ = R.energy_terms(wr, wi, sysm)
  plan = _plan(sysm, prec)
  dt = torch.float64 if prec == 64 else torch.float32
  twr = torch.tensor(wr, dtype=dt, device="cuda")
  twi = torch.tensor(wi, dtype=dt, device="cuda")
  e, tgr, tgi = plan.energy_and_grad(twr, twi, sysm.occupation)
  e = e.cpu().numpy()
  tol = TOL[prec]
  for i, name in enumerate(["kinetic", "external", "hartree", "xc", "total"]):
    ref = terms[name]
    assert abs(e[i] - ref) <= tol["e_rel"] * max(1.0, abs(ref)), (name, e[i], ref)
  assert e[6] == 0.0
  scale = max(np.abs(gr).max(), np.abs(gi).max())
  err = max(np.abs(tgr.cpu().numpy() - gr).max(), np.abs(tgi.cpu().numpy() - gi).max())
  assert err <= tol["g_rel"] * scale, (err, scale)


@pytest.mark.parametrize("prec", [64, 32])
def test_coeff_orthonormal_and_density(prec):
  torch = _torch()
  sysm = make_system(**CASES[1])
  wr, wi = random_params(sysm, seed=7)
  plan = _plan(sysm, prec)
  dt = torch.float64 if prec == 64 else torch.float32
  c = plan.coeff(torch.tensor(wr, dtype=dt, device="cuda"), torch.tensor(wi, dtype=dt, device="cuda"))
  cn = c.cpu().numpy().astype(np.complex128)
  ovl = np.einsum("skgi,skgj->skij", cn.conj(), cn)
  eye = np.eye(cn.shape[-1])
  assert np.abs(ovl - eye).max() < (1e-12 if prec == 64 else 2e-6)
  # same column space and phase-equal columns as Householder QR
  q = R.unitary_householder(wr, wi)
  ph = np.einsum("skgb,skgb->skb", q.conj(), cn)
  assert np.abs(np.abs(ph) - 1).max() < (1e-10 if prec == 64 else 1e-5)
  rho = plan.density(c, sysm.occupation).cpu().numpy()
  dense = R.expand_coefficient(cn, sysm.mask)
  rref = R.density_grid(dense, sysm.vol, sysm.occupation)
  assert np.abs(rho - rref).max() <= (1e-12 if prec == 64 else 1e-6) * np.abs(rref).max()


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("grid", [(12, 12, 12), (7, 10, 12), (16, 9, 20), (24, 27, 32), (27, 27, 27), (64, 64, 64)])
def test_fft3d(prec, grid):
  torch = _torch()
  from jrystal_gb300.engine import fft3d
  rng = np.random.default_rng(3)
  x = rng.normal(size=(2,) + grid) + 1j * rng.normal(size=(2,) + grid)
  dt = torch.complex128 if prec == 64 else torch.complex64
  tx = torch.tensor(x, dtype=dt, device="cuda")
  f = fft3d(tx).cpu().numpy()
  fi = fft3d(tx, inverse=True).cpu().numpy()
  rf = np.fft.fftn(x, axes=(-3, -2, -1))
  ri = np.fft.ifftn(x, axes=(-3, -2, -1))
  tol = 1e-12 if prec == 64 else 2e-6
  assert np.abs(f - rf).max() <= tol * np.abs(rf).max()
  assert np.abs(fi - ri).max() <= tol * np.abs(ri).max()


@pytest.mark.parametrize("prec", [64, 32])
def test_potential_split(prec):
  torch = _torch()
  sysm = make_system(**CASES[0])
  wr, wi = random_params(sysm, seed=11)
  dense = R.coeff(wr, wi, sysm.mask)
  rho = R.density_grid(dense, sysm.vol, sysm.occupation)
  plan = _plan(sysm, prec)
  for ks in (False, True):
    vh, ve, vx = R.effective(rho, sysm.positions, sysm.charges, sysm.g_vector_grid, sysm.vol,
                             split=True, xc_type=sysm.xc, kohn_sham=ks)
    out = plan.potential(torch.tensor(rho, device="cuda"), kohn_sham=ks).cpu().numpy()
    tol = 1e-11 if prec == 64 else 2e-5
    for got, ref in ((out[0], vh.real), (out[1], ve.real), (out[2], np.reshape(vx, out[2].shape))):
      assert np.abs(got - ref).max() <= tol * max(1.0, np.abs(ref).max())


def test_ewald_matches_oracle():
  sysm = make_system(kind="si2", grid=(16, 16, 16), kgrid=(1, 1, 1), nb=2, nocc=1)
  plan = _plan(sysm, 64)
  got = plan.ewald(0.1, 2e3)
  tgrid = R.translation_vectors(sysm.cell_vectors, 2e3)
  ref = R.ewald_coulomb_repulsion(sysm.positions, sysm.charges, sysm.g_vector_grid, sysm.vol, 0.1,
                                  tgrid)
  assert abs(got - ref) <= 1e-10 * abs(ref)


@pytest.mark.parametrize("prec", [64, 32])
def test_adam_matches_oracle(prec):
  torch = _torch()
  from jrystal_gb300.engine import adam_update
  rng = np.random.default_rng(5)
  p, g = rng.normal(size=1000), rng.normal(size=1000)
  m, v = np.zeros(1000), np.zeros(1000)
  dt = torch.float64 if prec == 64 else torch.float32
  tp, tm, tv = (torch.tensor(a, dtype=dt, device="cuda") for a in (p, m, v))
  for step in (1, 2, 3):
    tg = torch.tensor(g * step, dtype=dt, device="cuda")
    adam_update(tp, tg, tm, tv, step, 1e-2)
    p, m, v = R.adam_update(p, g * step, m, v, step, 1e-2)
  tol = 1e-14 if prec == 64 else 1e-6
  assert np.abs(tp.cpu().numpy() - p).max() < tol * 10


@pytest.mark.parametrize("prec", [64, 32])
def test_fast_and_generic_slab_kernels_agree(prec):
  torch = _torch()
  from jrystal_gb300 import _lib
  lib = _lib.load()
  sysm = make_system(kind="si2", grid=(32, 32, 32), kgrid=(2, 1, 1), nb=4, nocc=2)
  wr, wi = random_params(sysm, seed=21)
  plan = _plan(sysm, prec)
  dt = torch.float64 if prec == 64 else torch.float32
  twr = torch.tensor(wr, dtype=dt, device="cuda")
  twi = torch.tensor(wi, dtype=dt, device="cuda")
  out = {}
  prev = lib.jrg_fast_paths(-1)
  try:
    for fast in (1, 0):
      lib.jrg_fast_paths(fast)
      e, gr, gi = plan.energy_and_grad(twr, twi, sysm.occupation)
      out[fast] = (e.cpu().numpy().copy(), gr.cpu().numpy(), gi.cpu().numpy())
  finally:
    lib.jrg_fast_paths(prev)
  tol = TOL[prec]
  assert np.abs(out[1][0][:5] - out[0][0][:5]).max() <= tol["e_rel"] * np.abs(out[0][0][:5]).max()
  scale = np.abs(out[0][1]).max()
  assert np.abs(out[1][1] - out[0][1]).max() <= tol["g_rel"] * scale
  assert np.abs(out[1][2] - out[0][2]).max() <= tol["g_rel"] * scale


@pytest.mark.parametrize("nb,nocc,grid,kgrid", [(24, 12, (36, 36, 36), (2, 1, 1)),
                                                (5, 3, (24, 24, 24), (1, 1, 2)),
                                                (12, 8, (16, 16, 16), (2, 1, 1)),
                                                (30, 16, (24, 24, 24), (1, 1, 1))])
def test_tensor_core_and_cuda_core_contractions_agree(nb, nocc, grid, kgrid):
  """mode 1: mma.sync TF32 x 3 Gram and rotation; mode 2: tcgen05 TF32 x 3
  Gram (tensor memory accumulator); mode 0: CUDA cores.  All against the
  oracle, and the flag word (energies[6]) stays clear."""
  torch = _torch()
  from jrystal_gb300 import _lib
  lib = _lib.load()
  sysm = make_system(kind="si8", grid=grid, kgrid=kgrid, nb=nb, nocc=nocc)
  wr, wi = random_params(sysm, seed=31)
  terms, gr, gi, _ = R.energy_terms(wr, wi, sysm)
  plan = _plan(sysm, 32)
  twr = torch.tensor(wr, dtype=torch.float32, device="cuda")
  twi = torch.tensor(wi, dtype=torch.float32, device="cuda")
  out = {}
  prev = lib.jrg_tensor_core_paths(-1)
  try:
    for tc in (3, 2, 1, 0):
      lib.jrg_tensor_core_paths(tc)
      e, g1, g2 = plan.energy_and_grad(twr, twi, sysm.occupation)
      out[tc] = (e.cpu().numpy().copy(), g1.cpu().numpy(), g2.cpu().numpy())
  finally:
    lib.jrg_tensor_core_paths(prev)
  tol = TOL[32]
  scale = max(np.abs(gr).max(), np.abs(gi).max())
  for tc in (3, 2, 1, 0):
    e, g1, g2 = out[tc]
    assert e[6] == 0.0, (tc, e[6])
    for i, name in enumerate(["kinetic", "external", "hartree", "xc", "total"]):
      assert abs(e[i] - terms[name]) <= tol["e_rel"] * max(1.0, abs(terms[name])), (tc, name)
    assert max(np.abs(g1 - gr).max(), np.abs(g2 - gi).max()) <= tol["g_rel"] * scale, tc


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("case", [dict(kind="si2", grid=(16, 16, 16), kgrid=(2, 2, 2), nb=8, nocc=4),
                                  dict(kind="si8", grid=(24, 24, 24), kgrid=(3, 1, 1), nb=12, nocc=8),
                                  dict(kind="si2", grid=(27, 27, 27), kgrid=(1, 1, 2), nb=5, nocc=3)])
def test_two_stream_pipeline_matches_serial_and_oracle(prec, case):
  """jrg_pipeline(1) splits the k-points over two streams; results equal the
  single-stream path to summation order and the oracle to the usual tolerance."""
  torch = _torch()
  from jrystal_gb300 import _lib
  lib = _lib.load()
  sysm = make_system(**case)
  wr, wi = random_params(sysm, seed=41)
  terms, gr, gi, _ = R.energy_terms(wr, wi, sysm)
  plan = _plan(sysm, prec)
  dt = torch.float64 if prec == 64 else torch.float32
  twr = torch.tensor(wr, dtype=dt, device="cuda")
  twi = torch.tensor(wi, dtype=dt, device="cuda")
  out = {}
  prev = lib.jrg_pipeline(-1)
  try:
    for pipe in (1, 0):
      lib.jrg_pipeline(pipe)
      e, g1, g2 = plan.energy_and_grad(twr, twi, sysm.occupation)
      out[pipe] = (e.cpu().numpy().copy(), g1.cpu().numpy(), g2.cpu().numpy())
  finally:
    lib.jrg_pipeline(prev)
  tol = TOL[prec]
  scale = max(np.abs(gr).max(), np.abs(gi).max())
  for pipe in (1, 0):
    e, g1, g2 = out[pipe]
    assert e[6] == 0.0
    for i, name in enumerate(["kinetic", "external", "hartree", "xc", "total"]):
      assert abs(e[i] - terms[name]) <= tol["e_rel"] * max(1.0, abs(terms[name])), (pipe, name)
    assert max(np.abs(g1 - gr).max(), np.abs(g2 - gi).max()) <= tol["g_rel"] * scale, pipe
  same = 1e-12 if prec == 64 else 1e-5
  np.testing.assert_allclose(out[1][0][:5], out[0][0][:5], rtol=same)
  assert np.abs(out[1][1] - out[0][1]).max() <= same * scale


MULTIBAND_CASES = [
  # 64^3, 4 k-points x 24 bands: single stream 96 bands x 31 planes selects the
  # multi-band inverse plane pass (4 bands per CTA) and the register-prefetch
  # forward plane pass, both with the pruned 64-point transforms
  dict(kind="si8", grid=(64, 64, 64), kgrid=(2, 2, 1), nb=24, nocc=16),
  # 48^3 (not pruned), 4 k-points x 30 bands
  dict(kind="si8", grid=(48, 48, 48), kgrid=(2, 2, 1), nb=30, nocc=16),
]


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("pipe", [0, 1])
@pytest.mark.parametrize("case", range(len(MULTIBAND_CASES)))
def test_multiband_plane_passes(prec, pipe, case):
  """Several bands per CTA in the plane passes (chosen only when the call
  fills the GPU) against the oracle, with and without the two-stream pipeline."""
  torch = _torch()
  from jrystal_gb300 import _lib
  lib = _lib.load()
  sysm = make_system(**MULTIBAND_CASES[case])
  wr, wi = random_params(sysm, seed=77 + case)
  terms, gr, gi, _ = R.energy_terms(wr, wi, sysm)
  plan = _plan(sysm, prec)
  dt = torch.float64 if prec == 64 else torch.float32
  prev = lib.jrg_pipeline(pipe)
  try:
    e, g1, g2 = plan.energy_and_grad(torch.tensor(wr, dtype=dt, device="cuda"),
                                     torch.tensor(wi, dtype=dt, device="cuda"), sysm.occupation)
  finally:
    lib.jrg_pipeline(prev)
  e = e.cpu().numpy()
  tol = TOL[prec]
  for i, name in enumerate(["kinetic", "external", "hartree", "xc", "total"]):
    assert abs(e[i] - terms[name]) <= tol["e_rel"] * max(1.0, abs(terms[name])), (name, e[i], terms[name])
  scale = max(np.abs(gr).max(), np.abs(gi).max())
  err = max(np.abs(g1.cpu().numpy() - gr).max(), np.abs(g2.cpu().numpy() - gi).max())
  assert err <= tol["g_rel"] * scale, (err, scale)
