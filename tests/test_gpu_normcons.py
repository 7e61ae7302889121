"""Norm-conserving pseudopotential path on the GPU (jrg_plan_set_pseudopotential)
against the FP64 oracle: local V_loc(G) in place of the Coulomb table and the
beta-projector term (jrystal/pseudopotential/local.py, nloc.py;
calc/calc_ground_state_energy_normcons.py:160-181), through the two-call,
pipelined and fused paths, the band trace and the functional API."""
import numpy as np
import pytest

from oracle import restatement as R
from tests.synthetic_upf import write_set
from tests.systems import make_system, nc_tables, random_params, with_pseudopotential

pytestmark = pytest.mark.gpu

TOL = {64: dict(e_rel=1e-10, g_rel=1e-9), 32: dict(e_rel=2e-6, g_rel=1e-4)}
SI = {"Si": dict(z_valence=4, dij=(0.8, 1.6))}
NAMES = ["kinetic", "external", "hartree", "xc", "total"]


def _plan(sysm, prec, vloc, table, nb=None):
  from jrystal_gb300.engine import PlaneWavePlan
  p = PlaneWavePlan(sysm.cell_vectors, sysm.positions, sysm.charges, sysm.grid, sysm.mask,
                    sysm.kpts, nb or sysm.occupation.shape[-1], 1, prec, sysm.xc)
  p.set_pseudopotential(vloc, table)
  return p


def _setup(tmp_path, specs=SI, symbols=("Si", "Si"), **case):
  write_set(str(tmp_path), specs)
  sysm = make_system(**case)
  pp, vloc, dense, table = nc_tables(sysm, list(symbols), str(tmp_path))
  return sysm, with_pseudopotential(sysm, vloc, dense), vloc, table


def _check(e, tgr, tgi, terms, gr, gi, prec):
  tol = TOL[prec]
  for i, name in enumerate(NAMES):
    assert abs(e[i] - terms[name]) <= tol["e_rel"] * max(1.0, abs(terms[name])), (name, e[i], terms[name])
  assert abs(e[7] - terms["external_nonlocal"]) <= tol["e_rel"] * max(1.0, abs(terms["external_nonlocal"]))
  assert e[6] == 0.0
  scale = max(np.abs(gr).max(), np.abs(gi).max())
  err = max(np.abs(tgr - gr).max(), np.abs(tgi - gi).max())
  assert err <= tol["g_rel"] * scale, (err, scale)


CASES = [
  dict(kind="si2", grid=(16, 16, 16), kgrid=(2, 1, 1), nb=4, nocc=2),
  dict(kind="si2", grid=(15, 16, 18), kgrid=(1, 1, 1), nb=6, nocc=4, mask="cubic"),
]


@pytest.mark.parametrize("prec", [64, 32])
@pytest.mark.parametrize("pipeline", [1, 0])
@pytest.mark.parametrize("case", range(len(CASES)))
def test_nc_energy_and_gradient(tmp_path, prec, pipeline, case):
  import torch
  from jrystal_gb300 import _lib
  sysm, nc, vloc, table = _setup(tmp_path, **CASES[case])
  wr, wi = random_params(nc, seed=11 + case)
  terms, gr, gi, _ = R.energy_terms(wr, wi, nc)
  plan = _plan(nc, prec, vloc, table)
  assert plan.num_proj == 8
  dt = torch.float64 if prec == 64 else torch.float32
  lib = _lib.load()
  prev = lib.jrg_pipeline(pipeline)
  try:
    e, g1, g2 = plan.energy_and_grad(torch.tensor(wr, dtype=dt, device="cuda"),
                                     torch.tensor(wi, dtype=dt, device="cuda"), nc.occupation)
  finally:
    lib.jrg_pipeline(prev)
  _check(e.cpu().numpy(), g1.cpu().numpy(), g2.cpu().numpy(), terms, gr, gi, prec)


@pytest.mark.parametrize("prec", [64, 32])
def test_nc_two_species_many_bands_and_projectors(tmp_path, prec):
  """Projector rows split over two 64-row tiles and several apply passes,
  bands over two 64-band tiles (si8 cell, l = 0, 1, 2 betas on Si: 9 rows per
  atom, 72 in all; a projector-free element would add none)."""
  import torch
  specs = {"Si": dict(z_valence=4, betas=((0, 0.9), (1, 0.8), (2, 0.7)), dij=(0.5, 1.0, 2.0))}
  sysm, nc, vloc, table = _setup(tmp_path, specs, ["Si"] * 8, kind="si8", grid=(16, 16, 16),
                                 kgrid=(1, 1, 1), nb=70, nocc=16)
  assert table.shape[1] == 72
  wr, wi = random_params(nc, seed=5)
  terms, gr, gi, _ = R.energy_terms(wr, wi, nc)
  plan = _plan(nc, prec, vloc, table)
  dt = torch.float64 if prec == 64 else torch.float32
  e, g1, g2 = plan.energy_and_grad(torch.tensor(wr, dtype=dt, device="cuda"),
                                   torch.tensor(wi, dtype=dt, device="cuda"), nc.occupation)
  _check(e.cpu().numpy(), g1.cpu().numpy(), g2.cpu().numpy(), terms, gr, gi, prec)


def test_nc_unsorted_negative_d_and_projector_free_species(tmp_path):
  """A D with a negative, unsorted diagonal (the reference's eigh pairing) and
  an element without projectors next to one with them."""
  import torch
  specs = {"Ge": dict(z_valence=4, dij=(3.0, -1.0)), "H": dict(z_valence=1, betas=(), dij=())}
  sysm, nc, vloc, table = _setup(tmp_path, specs, ["Ge", "H"], kind="si2", grid=(16, 16, 16),
                                 kgrid=(2, 1, 1), nb=4, nocc=2)
  assert table.shape[1] == 4
  wr, wi = random_params(nc, seed=21)
  terms, gr, gi, _ = R.energy_terms(wr, wi, nc)
  plan = _plan(nc, 64, vloc, table)
  e, g1, g2 = plan.energy_and_grad(torch.tensor(wr, device="cuda"), torch.tensor(wi, device="cuda"),
                                   nc.occupation)
  _check(e.cpu().numpy(), g1.cpu().numpy(), g2.cpu().numpy(), terms, gr, gi, 64)


@pytest.mark.parametrize("prec", [64, 32])
def test_nc_fused_adam_step_equals_two_call_step(tmp_path, prec):
  import torch
  from jrystal_gb300.engine import adam_update
  sysm, nc, vloc, table = _setup(tmp_path, kind="si2", grid=(16, 16, 16), kgrid=(2, 1, 1), nb=4,
                                 nocc=2)
  wr, wi = random_params(nc, seed=4)
  plan = _plan(nc, prec, vloc, table)
  dt = torch.float64 if prec == 64 else torch.float32
  p0 = torch.tensor(np.stack([wr, wi]), dtype=dt, device="cuda")
  pa, ma, va = p0.clone(), torch.zeros_like(p0), torch.zeros_like(p0)
  e1 = plan.energy_grad_adam(pa, ma, va, nc.occupation, 1, 1e-2, 0.9, 0.99, 1e-8).cpu().numpy()
  pb, mb, vb = p0.clone(), torch.zeros_like(p0), torch.zeros_like(p0)
  g = torch.empty_like(pb)
  e2, _, _ = plan.energy_and_grad(pb[0], pb[1], nc.occupation, g[0], g[1])
  adam_update(pb, g, mb, vb, 1, 1e-2, 0.9, 0.99, 1e-8)
  np.testing.assert_allclose(e1[:5], e2.cpu().numpy()[:5], rtol=1e-12 if prec == 64 else 1e-6)
  assert abs(e1[7] - float(e2[7])) <= 1e-12 * abs(e1[7]) + (0 if prec == 64 else 1e-6)
  tol = 1e-12 if prec == 64 else 2e-5
  assert (pa - pb).abs().max().item() <= tol


@pytest.mark.parametrize("prec", [64, 32])
def test_nc_band_trace_and_band_hamiltonian(tmp_path, prec):
  """hamiltonian_trace / hamiltonian_matrix of the normcons band driver
  (nloc.py:160-303): T + v_eff + V_nl with v_eff = V_H + v_loc + v_xc."""
  import torch
  sysm, nc, vloc, table = _setup(tmp_path, kind="si2", grid=(12, 12, 12), kgrid=(2, 1, 1), nb=4,
                                 nocc=2)
  wr0, wi0 = random_params(nc, seed=1)
  c, _ = R.cholesky_qr(wr0, wi0)
  rho = R.density_grid(R.expand_coefficient(c, nc.mask), nc.vol, nc.occupation)
  rho_g = R._fftn(rho)
  v = np.real(R._ifftn(R.hartree_reciprocal(rho_g, nc.g_vector_grid, True) + vloc)) + \
      R.xc_eps_v(rho[0], nc.xc)[1]
  wr, wi = random_params(nc, seed=2)
  ref = R.band_trace_terms(wr, wi, v, nc)
  plan = _plan(nc, prec, vloc, table)
  dt = torch.float64 if prec == 64 else torch.float32
  out, g1, g2, hmat = plan.band_trace_grad(torch.tensor(wr, dtype=dt, device="cuda"),
                                           torch.tensor(wi, dtype=dt, device="cuda"),
                                           torch.tensor(v, dtype=dt, device="cuda"), hmat=True)
  o = out.cpu().numpy()
  tol = TOL[prec]
  assert abs(o[0] - ref["trace"]) <= tol["e_rel"] * abs(ref["trace"])
  np.testing.assert_allclose(hmat.cpu().numpy(), ref["hmat"], atol=10 * tol["e_rel"] * np.abs(ref["hmat"]).max())
  scale = max(np.abs(ref["grad_re"]).max(), np.abs(ref["grad_im"]).max())
  assert np.abs(g1.cpu().numpy() - ref["grad_re"]).max() <= tol["g_rel"] * scale
  assert np.abs(g2.cpu().numpy() - ref["grad_im"]).max() <= tol["g_rel"] * scale


def test_nc_band_energies_include_the_nonlocal_term(tmp_path):
  """band_energies[s,k,b] = d total / d f[s,k,b] (central differences of the
  oracle total in the occupations)."""
  import torch
  sysm, nc, vloc, table = _setup(tmp_path, kind="si2", grid=(12, 12, 12), kgrid=(1, 1, 1), nb=4,
                                 nocc=2)
  wr, wi = random_params(nc, seed=8)
  plan = _plan(nc, 64, vloc, table)
  g1, g2 = torch.empty((2,) + plan.param_shape, dtype=torch.float64, device="cuda")
  _, _, _, be = plan.energy_grad_bands(torch.tensor(wr, device="cuda"), torch.tensor(wi, device="cuda"),
                                       nc.occupation, g1, g2)
  be = be.cpu().numpy().reshape(nc.occupation.shape)
  import dataclasses
  h = 1e-5
  for b in range(4):
    occ_p, occ_m = nc.occupation.copy(), nc.occupation.copy()
    occ_p[0, 0, b] += h
    occ_m[0, 0, b] -= h
    fp = R.energy_terms(wr, wi, dataclasses.replace(nc, occupation=occ_p), with_grad=False)["total"]
    fm = R.energy_terms(wr, wi, dataclasses.replace(nc, occupation=occ_m), with_grad=False)["total"]
    assert abs((fp - fm) / (2 * h) - be[0, 0, b]) < 1e-6 * max(1.0, abs(be[0, 0, b]))


def test_nc_functional_api(tmp_path):
  """normcons.energy_local / energy_nonlocal / hamiltonian_nonlocal on dense
  coefficients against the oracle's dense forms."""
  import jrystal_gb300 as jr
  from jrystal_gb300.pseudopotential import normcons
  jr.set_precision(64)
  sysm, nc, vloc, table = _setup(tmp_path, kind="si2", grid=(12, 12, 12), kgrid=(2, 1, 1), nb=4,
                                 nocc=2)
  wr, wi = random_params(nc, seed=9)
  c, _ = R.cholesky_qr(wr, wi)
  dense_c = R.expand_coefficient(c, nc.mask)
  dense_p = nc.proj
  e_nl = normcons.energy_nonlocal(dense_c, dense_p, nc.vol, nc.occupation)
  assert abs(float(e_nl) - R.energy_nonlocal(dense_c, dense_p, nc.vol, nc.occupation)) < 1e-10
  h = normcons.hamiltonian_nonlocal(dense_c, dense_p, nc.vol).cpu().numpy()
  np.testing.assert_allclose(h, R.hamiltonian_nonlocal(dense_c, dense_p, nc.vol), atol=1e-11)
  rho_g = R.density_grid_reciprocal(dense_c, nc.vol, nc.occupation)
  e_loc = normcons.energy_local(rho_g, vloc, nc.vol)
  assert abs(float(e_loc) - R.reciprocal_braket(vloc[None], rho_g, nc.vol)) < 1e-10


def test_nc_potential_external_part_is_ifft_of_v_local(tmp_path):
  import torch
  sysm, nc, vloc, table = _setup(tmp_path, kind="si2", grid=(12, 12, 12), kgrid=(1, 1, 1), nb=4,
                                 nocc=2)
  plan = _plan(nc, 64, vloc, table)
  rho = np.abs(np.random.default_rng(0).normal(size=nc.grid)) * 0.01
  out = plan.potential(torch.tensor(rho, device="cuda"), kohn_sham=True).cpu().numpy()
  np.testing.assert_allclose(out[1], np.real(R._ifftn(vloc)), atol=1e-10)


def test_set_pseudopotential_rejects_bad_shapes(tmp_path):
  sysm, nc, vloc, table = _setup(tmp_path, kind="si2", grid=(12, 12, 12), kgrid=(1, 1, 1), nb=4,
                                 nocc=2)
  plan = _plan(nc, 64, vloc, table)
  with pytest.raises(ValueError):
    plan.set_pseudopotential(vloc[:-1], table)
  with pytest.raises(ValueError):
    plan.set_pseudopotential(vloc, table[:, :, :-1])
  plan.set_pseudopotential(None, None)      # nonlocal term removed, local table kept
  assert plan.num_proj == 0


def _si_crystal():
  import jrystal_gb300 as jr
  a = 10.26
  cell = np.array([[0, a / 2, a / 2], [a / 2, 0, a / 2], [a / 2, a / 2, 0]])
  pos = np.array([[0, 0, 0], [0.25, 0.25, 0.25]]) @ cell
  return jr.Crystal(charges=np.array([14.0, 14.0]), positions=pos, cell_vectors=cell,
                    symbols=["Si", "Si"])


def test_energy_normcons_driver(tmp_path):
  """calc.energy_normcons (calc/calc_ground_state_energy_normcons.py:68-308):
  valence electrons only (8 -> 4 occupied bands), energy decreasing, the
  final terms equal the oracle's at the final parameters, Ewald with the
  nuclear charges."""
  import jrystal_gb300 as jr
  d = write_set(str(tmp_path / "pp"), SI)
  crystal = _si_crystal()
  grid = 16
  cfg = {"crystal": crystal, "grid_sizes": grid, "k_grid_sizes": [1, 1, 1], "cutoff_energy": 8.0,
         "epoch": 80, "convergence_condition": 1e-12, "empty_bands": 2, "use_pseudopotential": True,
         "pseudopotential_file_dir": d, "xc": "lda_x",
         "optimizer_args": {"learning_rate": 0.01, "b1": 0.9, "b2": 0.99}}
  out = jr.calc.energy_normcons(cfg)
  h = out.total_energy_history
  assert h[-1] < h[0]
  p = out.params_pw
  assert p["w_re"].shape[-1] == 6
  mask = R.spherical_mask(crystal.cell_vectors, (grid,) * 3, 8.0)
  kpts = R.k_vectors(crystal.cell_vectors, (1, 1, 1))
  occ = np.zeros((1, 1, 6))
  occ[..., :4] = 2.0
  sysm = R.System(crystal.cell_vectors, crystal.positions, crystal.charges, (grid,) * 3, mask, kpts,
                  occ, "lda_x")
  _, vloc, dense, _ = nc_tables(sysm, crystal.symbols, d)
  nc = with_pseudopotential(sysm, vloc, dense)
  ref = R.energy_terms(p["w_re"].cpu().numpy(), p["w_im"].cpu().numpy(), nc, with_grad=False)
  t = out.energy_terms
  for name in ("kinetic", "external", "hartree", "xc", "total", "external_nonlocal", "external_local"):
    assert abs(t[name] - ref[name]) < 1e-8 * max(1.0, abs(ref[name])), name
  ew = R.nuclear_repulsion(crystal.positions, crystal.charges, crystal.cell_vectors,
                           R.g_vectors(crystal.cell_vectors, (grid,) * 3), nc.vol, 0.1, 2e4)
  assert abs(out.ewald - ew) < 1e-8 * abs(ew)
  with pytest.raises(ValueError):
    jr.calc.energy_normcons(dict(cfg, pseudopotential_file_dir=None))


def test_band_normcons_driver_matches_full_diagonalisation(tmp_path):
  """calc.band_normcons (calc/calc_band_structure_normcons.py:68-299) against
  the lowest eigenvalues of the full plane-wave Hamiltonian T + v_eff + V_nl
  at every k-point of the path, with the beta transforms of the whole path."""
  import jrystal_gb300 as jr
  d = write_set(str(tmp_path / "pp"), SI)
  crystal = _si_crystal()
  grid, nk, nb = 16, 4, 6
  cfg = {"crystal": crystal, "grid_sizes": grid, "k_grid_sizes": [1, 1, 1], "cutoff_energy": 8.0,
         "epoch": 300, "use_pseudopotential": True, "pseudopotential_file_dir": d, "xc": "lda_x",
         "optimizer_args": {"learning_rate": 1e-2, "b1": 0.9, "b2": 0.99},
         "k_path_special_points": "LGX", "num_kpoints": nk, "band_structure_empty_bands": 2,
         "band_structure_epoch": 2500, "k_path_fine_tuning_epoch": 1500, "seed": 3,
         "jax_enable_x64": True}
  out = jr.calc.band_normcons(cfg)
  assert out.eigenvalues.shape == (1, nk, nb)
  v = out.effective_potential.cpu().numpy()
  mask = R.spherical_mask(crystal.cell_vectors, (grid,) * 3, 8.0)
  sysm = R.System(crystal.cell_vectors, crystal.positions, crystal.charges, (grid,) * 3, mask,
                  out.k_path, np.ones((1, nk, nb)), "lda_x")
  _, vloc, dense, _ = nc_tables(sysm, crystal.symbols, d, kpts=out.k_path)
  nc = with_pseudopotential(sysm, vloc, dense)
  exact = np.array([np.linalg.eigvalsh(R.plane_wave_hamiltonian(v, nc, k))[:nb] for k in range(nk)])
  err = np.abs(out.eigenvalues[0] - exact)
  print("band energies: max |error| per band", err.max(axis=0))
  assert np.all(out.eigenvalues[0] >= exact - 1e-8)
  assert err.max() < 1e-4


def test_nc_functional_hamiltonian_matrix_and_trace(tmp_path):
  """normcons.hamiltonian_matrix / hamiltonian_trace (nloc.py:160-303) on
  dense coefficients against the same sums of the oracle's dense pieces: the
  nonlocal F^H F / vol, the local and Hartree potentials as ifftn of their
  reciprocal tables (complex, as the reference keeps them), v_xc and T."""
  import jrystal_gb300 as jr
  from jrystal_gb300.pseudopotential import normcons
  jr.set_precision(64)
  sysm, nc, vloc, table = _setup(tmp_path, kind="si2", grid=(12, 12, 12), kgrid=(2, 1, 1), nb=4,
                                 nocc=2)
  g = nc.g_vector_grid
  wr0, wi0 = random_params(nc, seed=12)
  c0, _ = R.cholesky_qr(wr0, wi0)
  rho_h = R.density_grid(R.expand_coefficient(c0, nc.mask), nc.vol, nc.occupation)  # (1,x,y,z)
  wr, wi = random_params(nc, seed=13)
  c, _ = R.cholesky_qr(wr, wi)
  dense_c = R.expand_coefficient(c, nc.mask)
  wave = R.wave_grid(dense_c, nc.vol)
  v_h = R._ifftn(R.hartree_reciprocal(R._fftn(rho_h), g, kohn_sham=True))
  v_xc = R.xc_eps_v(rho_h[0], nc.xc)[1]
  h_ref = (R.hamiltonian_nonlocal(dense_c, nc.proj, nc.vol)
           + R.expectation(wave, R._ifftn(vloc), nc.vol, diagonal=False, mode="real")
           + R.expectation(wave, v_h + v_xc, nc.vol, diagonal=False, mode="real")
           + R.expectation(dense_c, R.kinetic_operator(g, nc.kpts), nc.vol, diagonal=False,
                           mode="kinetic"))
  h = normcons.hamiltonian_matrix(dense_c, rho_h, vloc, nc.proj, g, nc.kpts, nc.vol,
                                  xc=nc.xc, kohn_sham=True).cpu().numpy()
  np.testing.assert_allclose(h, h_ref, atol=1e-9 * np.abs(h_ref).max())
  tr = float(normcons.hamiltonian_trace(dense_c, rho_h, vloc, nc.proj, g, nc.kpts, nc.vol,
                                        xc=nc.xc, kohn_sham=True))
  assert abs(tr - np.einsum("skii->", h_ref).real) < 1e-9 * abs(tr)
