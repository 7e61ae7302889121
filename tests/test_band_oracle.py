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
