"""Norm-conserving pseudopotential path on the CPU: the UPF reader, the
numerical spherical Bessel transform, the real spherical harmonics, the
local and nonlocal tables (jrystal/pseudopotential/*.py) and the oracle's
energy/gradient with the pseudopotential, checked against known answers,
independent restatements and central finite differences."""
import os

import numpy as np
import pytest

from oracle import restatement as R
from tests.synthetic_upf import write_set, write_upf
from tests.systems import make_system, nc_tables, random_params, with_pseudopotential

REF_UPF = "/root/reference/pseudopotential/normconserving"


def test_synthetic_upf_round_trip(tmp_path):
  from jrystal_gb300.pseudopotential import load
  p = write_upf(str(tmp_path / "Si.synthetic.UPF"), "Si", 4, dij=(0.8, 1.6))
  d = load.parse_upf(p)
  assert float(d["PP_HEADER"]["z_valence"]) == 4.0
  assert int(d["PP_HEADER"]["number_of_proj"]) == 2
  assert len(d["PP_NONLOCAL"]["PP_BETA"]) == 2
  np.testing.assert_allclose(d["PP_NONLOCAL"]["PP_DIJ"], [1.6, 0, 0, 3.2])
  assert d["PP_MESH"]["PP_R"][0] == 0.0 and len(d["PP_MESH"]["PP_R"]) == 451
  assert d["PP_INFO"]["Valence configuration"][0]["l"] == 0
  assert load.find_upf(str(tmp_path), "si").endswith("Si.synthetic.UPF")
  with pytest.raises(ValueError):
    load.find_upf(str(tmp_path), "Ge")


def test_container_units(tmp_path):
  from types import SimpleNamespace
  from jrystal_gb300.pseudopotential import NormConservingPseudopotential
  write_set(str(tmp_path), {"Si": dict(z_valence=4, dij=(0.8, 1.6)),
                            "H": dict(z_valence=1, betas=(), dij=())})
  cr = SimpleNamespace(symbols=["Si", "H"], positions=np.zeros((2, 3)), charges=np.array([14, 1]))
  pp = NormConservingPseudopotential.create(cr, str(tmp_path))
  assert pp.valence_charges == [4, 1]
  assert pp.r_grid[0].size == 450 and np.all(pp.r_grid[0] > 0)
  np.testing.assert_allclose(np.diag(pp.nonlocal_d_matrix[0]), [0.8, 1.6])   # Ry -> Ha
  r = pp.r_grid[0]
  np.testing.assert_allclose(pp.nonlocal_beta_grid[0][1], r * np.exp(-(r / 0.9) ** 2), rtol=1e-12)
  # local potential tail -z/r in Hartree
  assert abs(pp.local_potential_grid[0][-1] * r[-1] + 4) < 1e-9
  # element without projectors: one zero l = 0 beta, zero D
  assert pp.num_beta[1] == 1 and np.all(pp.nonlocal_d_matrix[1] == 0)


@pytest.mark.skipif(not os.path.isdir(REF_UPF), reason="reference UPF files absent")
def test_reference_upf_files_parse():
  """Header facts of the reference's bundled files (pseudopotential/normconserving)."""
  from types import SimpleNamespace
  from jrystal_gb300.pseudopotential import NormConservingPseudopotential, load
  d = load.parse_upf(os.path.join(REF_UPF, "Si.pz-vbc.UPF"))
  assert int(d["PP_HEADER"]["mesh_size"]) == 431 and int(d["PP_HEADER"]["number_of_proj"]) == 2
  assert [b["angular_momentum"] for b in d["PP_NONLOCAL"]["PP_BETA"]] == ["0", "1"]
  np.testing.assert_allclose(d["PP_NONLOCAL"]["PP_DIJ"], [1.52388501179, 0, 0, 3.68330413052])
  cr = SimpleNamespace(symbols=["Si", "C", "Ge"], positions=np.zeros((3, 3)),
                       charges=np.array([14, 6, 32]))
  pp = NormConservingPseudopotential.create(cr, REF_UPF + "/")
  assert pp.valence_charges == [4, 4, 4]
  assert [len(l) for l in pp.nonlocal_angular_momentum] == [2, 1, 2]
  np.testing.assert_allclose(np.diag(pp.nonlocal_d_matrix[2]), [44.5849915611 / 2, -22.6924252259 / 2])


def test_real_spherical_harmonics():
  from jrystal_gb300.pseudopotential.spherical import (batch_sph_harm, batch_sph_harm_real,
                                                       cartesian_to_spherical)
  rng = np.random.default_rng(0)
  x = rng.normal(size=(50, 3))
  sph = cartesian_to_spherical(x)
  th, ph = sph[:, 1], sph[:, 2]
  u = x / np.linalg.norm(x, axis=1, keepdims=True)
  y1 = batch_sph_harm_real(1, th, ph)
  np.testing.assert_allclose(y1, np.sqrt(3 / (4 * np.pi)) * u[:, [1, 2, 0]], atol=1e-13)
  for l in range(5):   # addition theorem: sum_m Y_lm^2 = (2l+1)/(4 pi)
    yl = batch_sph_harm_real(l, th, ph)
    np.testing.assert_allclose(np.sum(yl ** 2, axis=-1), (2 * l + 1) / (4 * np.pi), rtol=1e-12)
  sp = pytest.importorskip("scipy.special")
  if hasattr(sp, "sph_harm_y"):
    for l in range(4):
      got = batch_sph_harm(l, th, ph)
      for i, m in enumerate(range(-l, l + 1)):
        np.testing.assert_allclose(got[:, i], sp.sph_harm_y(l, m, ph, th), atol=1e-12)
  # origin: r = eps, polar angle pi/2, azimuth 0
  np.testing.assert_allclose(cartesian_to_spherical(np.zeros(3)), [1e-10, 0.0, np.pi / 2])


def test_sbt_quadrature():
  from jrystal_gb300.pseudopotential.sbt import sbt
  from scipy.special import spherical_jn
  r = 1e-4 * np.exp(0.01 * np.arange(1400))
  f = np.stack([np.exp(-r ** 2), r * np.exp(-r ** 2)])
  g, out = sbt(r, f, l=[0, 1], kmax=8.0)
  assert g.size == 2 * r.size and g[0] == 1e-4 and g[-1] == 8.0
  dr = np.append(np.diff(r), 0.0)
  for row, l in ((0, 0), (1, 1)):   # the left Riemann sum it restates
    direct = np.array([np.sum(f[row] * spherical_jn(l, gi * r) * r * r * dr) for gi in g[::97]])
    np.testing.assert_allclose(out[row, ::97], direct, rtol=1e-12, atol=1e-15)
  # against the closed forms: int e^{-r^2} j0 r^2 = sqrt(pi)/4 e^{-g^2/4},
  # int r e^{-r^2} j1 r^2 = sqrt(pi)/8 g e^{-g^2/4}
  np.testing.assert_allclose(out[0], np.sqrt(np.pi) / 4 * np.exp(-g ** 2 / 4), atol=1e-2 * np.sqrt(np.pi) / 4)
  np.testing.assert_allclose(out[1], np.sqrt(np.pi) / 8 * g * np.exp(-g ** 2 / 4), atol=1e-2 * np.sqrt(np.pi) / 8)
  _, o1 = sbt(r, f[0], l=0, kmax=8.0)
  np.testing.assert_allclose(o1[0], out[0], rtol=1e-13)


def test_local_potential_of_a_pure_coulomb_tail_is_the_coulomb_table():
  """v(r) = -z/r: the short-range part vanishes and V_loc(G) equals the
  all-electron external table of charges z (potential.py:121-166)."""
  from jrystal_gb300.pseudopotential import local
  sysm = make_system(kind="si2", grid=(12, 12, 12), kgrid=(1, 1, 1))
  r = 1e-3 * np.exp(0.025 * np.arange(400))
  v = local.potential_local_reciprocal(sysm.positions, sysm.g_vector_grid, [r, r], [-4 / r, -4 / r],
                                       [4, 4], sysm.vol)
  ref = R.external_reciprocal(sysm.positions, np.array([4.0, 4.0]), sysm.g_vector_grid, sysm.vol)
  np.testing.assert_allclose(v, ref, rtol=1e-8, atol=1e-8 * np.abs(ref).max())


def test_projector_table_is_the_dense_rows_on_the_sphere(tmp_path):
  write_set(str(tmp_path), {"Si": dict(z_valence=4, betas=((0, 0.9), (1, 0.8), (2, 0.7)),
                                       dij=(0.5, 1.0, 2.0))})
  sysm = make_system(kind="si2", grid=(10, 10, 10), kgrid=(2, 1, 1))
  pp, vloc, dense, table = nc_tables(sysm, ["Si", "Si"], str(tmp_path))
  K = sysm.kpts.shape[0]
  rows = dense.reshape(K, -1, *sysm.grid)[..., sysm.mask]       # [k, beta*M, G]
  keep = np.any(rows != 0, axis=(0, 2))
  assert table.shape == (K, 2 * 9, int(sysm.mask.sum())) and keep.sum() == 18
  np.testing.assert_allclose(table, rows[:, keep], rtol=0, atol=0)
  # V_loc is Hermitian off the Nyquist planes and vanishes at G = 0
  assert vloc[0, 0, 0] == 0


def test_nonlocal_energy_reproduces_the_eigh_pairing(tmp_path):
  """E_nl = sum_b f/vol sum_{a,b2,m} |lambda_b2| |x_{a,b2,m}|^2 with lambda
  the ascending eigenvalues of D paired with the betas in file order
  (nloc.py:108-133 with nloc.py:143-157): exact for sorted D, and the
  reference's pairing for an unsorted, negative D."""
  from jrystal_gb300.pseudopotential import nloc
  sysm = make_system(kind="si2", grid=(10, 10, 10), kgrid=(1, 1, 1), nb=3, nocc=2)
  wr, wi = random_params(sysm, seed=2)
  c, _ = R.cholesky_qr(wr, wi)
  dense_c = R.expand_coefficient(c, sysm.mask)
  for dij in ((0.8, 1.6), (3.0, -1.0)):
    d = str(tmp_path / f"d{dij[1]}")
    write_set(d, {"Si": dict(z_valence=4, dij=dij)})
    pp, _, dense, _ = nc_tables(sysm, ["Si", "Si"], d)
    e = R.energy_nonlocal(dense_c, dense, sysm.vol, sysm.occupation)
    # unit-D rows: x_{a,b2,m} without the D factor
    unit = [np.eye(2), np.eye(2)]
    x = nloc.potential_nonlocal_psi_reciprocal(sysm.positions, sysm.g_vector_grid, sysm.kpts,
                                               pp.r_grid, pp.nonlocal_beta_grid,
                                               pp.nonlocal_angular_momentum, unit)
    xr = x.reshape(1, 2, 2, 3, *sysm.grid)                       # [k, atom, b2, m, ...]
    lam = np.sort(np.asarray(dij))
    f = np.einsum("skbxyz,kaqmxyz->skbaqm", dense_c, xr)
    expect = np.sum(sysm.occupation[..., None, None, None] * np.abs(lam)[None, None, None, None, :, None]
                    * np.abs(f) ** 2) / sysm.vol
    assert abs(e - expect) < 1e-12 * abs(expect)


def test_oracle_nc_gradient_central_differences(tmp_path):
  write_set(str(tmp_path), {"Si": dict(z_valence=4, dij=(0.8, 1.6))})
  sysm = make_system(kind="si2", grid=(8, 8, 8), kgrid=(2, 1, 1), nb=3, nocc=2)
  _, vloc, dense, _ = nc_tables(sysm, ["Si", "Si"], str(tmp_path))
  nc = with_pseudopotential(sysm, vloc, dense)
  wr, wi = random_params(nc, seed=7)
  terms, gr, gi, _ = R.energy_terms(wr, wi, nc)
  assert terms["external_nonlocal"] > 0
  assert abs(terms["external"] - terms["external_local"] - terms["external_nonlocal"]) < 1e-12
  rng = np.random.default_rng(1)
  h = 1e-5
  for _ in range(6):
    idx = tuple(rng.integers(0, s) for s in wr.shape)
    for part, g in ((0, gr), (1, gi)):
      p, m = [wr.copy(), wi.copy()], [wr.copy(), wi.copy()]
      p[part][idx] += h
      m[part][idx] -= h
      fd = (R.energy_terms(*p, nc, with_grad=False)["total"] -
            R.energy_terms(*m, nc, with_grad=False)["total"]) / (2 * h)
      assert abs(fd - g[idx]) < 1e-6 * max(1.0, abs(fd)), (part, idx, fd, g[idx])


def test_oracle_nc_rayleigh_ritz(tmp_path):
  """With the projector term the exact eigenvectors of the full plane-wave
  Hamiltonian (T + v + V_nl) make the band trace stationary, and their Ritz
  values equal the exact eigenvalues."""
  write_set(str(tmp_path), {"Si": dict(z_valence=4, dij=(0.8, 1.6))})
  sysm = make_system(kind="si2", grid=(8, 8, 8), kgrid=(1, 1, 1), nb=3, nocc=2)
  _, vloc, dense, _ = nc_tables(sysm, ["Si", "Si"], str(tmp_path))
  nc = with_pseudopotential(sysm, vloc, dense)
  v = np.real(R._ifftn(vloc))
  hk = R.plane_wave_hamiltonian(v, nc, 0)
  np.testing.assert_allclose(hk, hk.conj().T, atol=1e-12 * np.abs(hk).max())
  e, u = np.linalg.eigh(hk)
  x = u[:, :3][None, None]
  out = R.band_trace_terms(x.real, x.imag, v, nc)
  np.testing.assert_allclose(np.linalg.eigvalsh(out["hmat"][0, 0]), e[:3], atol=1e-10 * np.abs(e[:3]).max())
  assert np.abs(out["grad_re"]).max() < 1e-8 and np.abs(out["grad_im"]).max() < 1e-8


@pytest.mark.skipif(not os.path.isdir(REF_UPF), reason="reference UPF files absent")
def test_numerical_sbt_accuracy_on_reference_betas():
  """jrystal/sbt/sbt_test.py:42-71 holds its two transforms of the bundled Si
  betas (kmax 100, delta_r = PP_RAB, 2000 points up to 100) within 5e-3 of
  each other; the numerical transform restated here stays within that of an
  independent Simpson quadrature over the mesh (measured 8.9e-4)."""
  from types import SimpleNamespace
  from scipy.integrate import simpson
  from scipy.interpolate import CubicSpline
  from scipy.special import spherical_jn
  from jrystal_gb300.pseudopotential import NormConservingPseudopotential
  from jrystal_gb300.pseudopotential.sbt import sbt
  cr = SimpleNamespace(symbols=["Si"], positions=np.zeros((1, 3)), charges=np.array([14]))
  pp = NormConservingPseudopotential.create(cr, REF_UPF + "/")
  r, rab = pp.r_grid[0], pp.r_ab[0]
  beta, ls = pp.nonlocal_beta_grid[0], pp.nonlocal_angular_momentum[0]
  g, out = sbt(r, beta, l=list(ls), kmax=100, delta_r=rab)
  xx = np.linspace(0, 100, 2000)
  got = CubicSpline(g, out, axis=-1)(xx)
  ref = np.stack([[simpson(beta[b] * spherical_jn(int(ls[b]), k * r) * r * r * rab, dx=1.0)
                   for k in xx] for b in range(len(ls))])
  np.testing.assert_allclose(got, ref, rtol=0, atol=5e-3)
