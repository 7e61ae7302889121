"""Band-structure objective of the oracle (fixed effective potential): the
trace and band Hamiltonian against the dense forms of
jrystal/_src/hamiltonian.py, central finite differences of the gradient,
and the Rayleigh-Ritz relations with the full plane-wave Hamiltonian."""
import numpy as np

from oracle import restatement as R
from tests.systems import make_system, random_params


def _veff(sysm, seed=1):
  wr, wi = random_params(sysm, seed=seed)
  c, _ = R.cholesky_qr(wr, wi)
  dense = R.expand_coefficient(c, sysm.mask)
  rho = R.density_grid(dense, sysm.vol, sysm.occupation)
  v = R.effective(rho, sysm.positions, sysm.charges, sysm.g_vector_grid, sysm.vol, False,
                  sysm.xc, True)
  return rho, np.real(v[0])


def test_band_trace_and_matrix_equal_dense_forms():
  sysm = make_system(kind="si2", grid=(10, 10, 10), kgrid=(2, 1, 1), nb=3, nocc=2)
  rho, v = _veff(sysm)
  wr, wi = random_params(sysm, seed=4)
  out = R.band_trace_terms(wr, wi, v, sysm, with_grad=False)
  c, _ = R.cholesky_qr(wr, wi)
  dense = R.expand_coefficient(c, sysm.mask)
  tr = R.hamiltonian_matrix_trace(dense, sysm.positions, sysm.charges, rho, sysm.g_vector_grid,
                                  sysm.kpts, sysm.vol, sysm.xc, True)
  assert abs(out["trace"] - tr) < 1e-10 * abs(tr)
  h = R.hamiltonian_matrix(dense, sysm.positions, sysm.charges, rho, sysm.g_vector_grid,
                           sysm.kpts, sysm.vol, sysm.xc, True)
  np.testing.assert_allclose(out["hmat"], h, atol=1e-10 * np.abs(h).max())
  np.testing.assert_allclose(h, np.swapaxes(h.conj(), -1, -2), atol=1e-10 * np.abs(h).max())


def test_band_trace_gradient_central_differences():
  sysm = make_system(kind="si2", grid=(8, 8, 8), kgrid=(1, 1, 1), nb=3, nocc=2)
  _, v = _veff(sysm)
  wr, wi = random_params(sysm, seed=5)
  wts = np.array([[[1.0, 0.5, 2.0]]])
  out = R.band_trace_terms(wr, wi, v, sysm, weights=wts)
  rng = np.random.default_rng(0)
  h = 1e-5
  for _ in range(6):
    idx = tuple(rng.integers(0, s) for s in wr.shape)
    for part, g in ((0, out["grad_re"]), (1, out["grad_im"])):
      p, m = [wr.copy(), wi.copy()], [wr.copy(), wi.copy()]
      p[part][idx] += h
      m[part][idx] -= h
      fd = (R.band_trace_terms(*p, v, sysm, weights=wts, with_grad=False)["trace"] -
            R.band_trace_terms(*m, v, sysm, weights=wts, with_grad=False)["trace"]) / (2 * h)
      assert abs(fd - g[idx]) < 1e-6 * max(1.0, abs(fd)), (part, idx, fd, g[idx])


def test_rayleigh_ritz_against_full_plane_wave_hamiltonian():
  sysm = make_system(kind="si2", grid=(10, 10, 10), kgrid=(2, 1, 1), nb=4, nocc=2)
  _, v = _veff(sysm)
  nb = 4
  exact = []
  vecs = []
  for k in range(sysm.kpts.shape[0]):
    hk = R.plane_wave_hamiltonian(v, sysm, k)
    np.testing.assert_allclose(hk, hk.conj().T, atol=1e-12 * np.abs(hk).max())
    e, u = np.linalg.eigh(hk)
    exact.append(e[:nb])
    vecs.append(u[:, :nb])
  exact = np.array(exact)
  # any orthonormal basis: Ritz values lie above the exact ones (interlacing)
  wr, wi = random_params(sysm, seed=6)
  ritz = np.linalg.eigvalsh(R.band_trace_terms(wr, wi, v, sysm, with_grad=False)["hmat"][0])
  assert np.all(ritz >= exact - 1e-10)
  # the exact eigenvectors as parameters: Ritz values equal the exact ones
  u = np.stack(vecs)[None]                       # (1,k,g,b)
  out = R.band_trace_terms(u.real, u.imag, v, sysm)
  ritz = np.linalg.eigvalsh(out["hmat"][0])
  np.testing.assert_allclose(ritz, exact, atol=1e-10 * np.abs(exact).max())
  # and the trace is stationary there
  assert np.abs(out["grad_re"]).max() < 1e-8 and np.abs(out["grad_im"]).max() < 1e-8


def _wirtinger_hessian(f, n, h=1e-3):
  """2 d^2 f / (d conj(u_i) d u_j) at u = 1 by central differences, u = a + i b:
  d/d conj(u) = (d/da + i d/db) / 2, d/du = (d/da - i d/db) / 2."""
  u0 = np.ones(n, dtype=np.complex128)

  def d2(i, si, j, sj):   # second difference along the real directions si e_i, sj e_j
    ei = np.zeros(n, complex)
    ej = np.zeros(n, complex)
    ei[i] = si * h
    ej[j] = sj * h
    return (f(u0 + ei + ej) - f(u0 + ei - ej) - f(u0 - ei + ej) + f(u0 - ei - ej)) / (4 * h * h)

  out = np.zeros((n, n), dtype=np.complex128)
  for i in range(n):
    for j in range(n):
      faa, fab = d2(i, 1, j, 1), d2(i, 1, j, 1j)
      fba, fbb = d2(i, 1j, j, 1), d2(i, 1j, j, 1j)
      out[i, j] = 2 * 0.25 * (faa - 1j * fab + 1j * fba + fbb)
  return out


def test_complex_hessian_convention_and_band_hamiltonian():
  """jrystal builds H_ij as complex_hessian of efun(u) = 1/2 E(sum_i u_i psi_i)
  (jrystal/_src/hamiltonian.py:211-232) in the convention that
  _src/hessian_test.py:29-45 pins: the Hessian of 1/2 x^H H x is H, i.e.
  2 d^2 f / (d conj(x_i) d x_j).  The oracle's band Hamiltonian (the form the
  device returns) equals that construction."""
  rng = np.random.default_rng(3)
  a = rng.normal(size=(5, 5)) + 1j * rng.normal(size=(5, 5))
  hq = a + a.conj().T
  q = lambda x: float(np.real(0.5 * x.conj() @ hq @ x))
  np.testing.assert_allclose(_wirtinger_hessian(q, 5), hq, atol=1e-7)

  sysm = make_system(kind="si2", grid=(8, 8, 8), kgrid=(1, 1, 1), nb=3, nocc=2)
  rho, _ = _veff(sysm)
  wr, wi = random_params(sysm, seed=9)
  c, _ = R.cholesky_qr(wr, wi)
  dense = R.expand_coefficient(c, sysm.mask)                      # (1,1,b,x,y,z)

  def efun(u):
    psi = np.einsum("i,ixyz->xyz", u, dense[0, 0])[None, None, None]
    return 0.5 * float(R.hamiltonian_matrix_trace(psi, sysm.positions, sysm.charges, rho,
                                                  sysm.g_vector_grid, sysm.kpts, sysm.vol,
                                                  sysm.xc, True))

  h_fd = _wirtinger_hessian(efun, 3)
  h = R.hamiltonian_matrix(dense, sysm.positions, sysm.charges, rho, sysm.g_vector_grid,
                           sysm.kpts, sysm.vol, sysm.xc, True)[0, 0]
  np.testing.assert_allclose(h, h_fd, atol=1e-6 * np.abs(h).max())
  ref = R.band_trace_terms(wr, wi, np.real(R.effective(rho, sysm.positions, sysm.charges,
                                                       sysm.g_vector_grid, sysm.vol, False,
                                                       sysm.xc, True)[0]), sysm,
                           with_grad=False)["hmat"][0, 0]
  np.testing.assert_allclose(ref, h_fd, atol=1e-6 * np.abs(h).max())
