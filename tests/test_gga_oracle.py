"""PBE (gga_x_pbe + gga_c_pbe) in the oracle: published limits, complex-step
derivatives against central differences, and the GGA gradient of the total
energy (v_xc = f_rho - 2 div(f_sigma grad rho)) against central differences."""
import numpy as np

from oracle import restatement as R
from tests.systems import make_system, random_params

XC = "gga_x_pbe+gga_c_pbe"


def test_pbe_limits():
  rho = np.array([1e-3, 0.1, 1.0, 30.0])
  np.testing.assert_allclose(R.pbe_x(rho, 0 * rho), R.lda_x(rho)[0], rtol=1e-14)   # F_x(0) = 1
  np.testing.assert_allclose(R.pbe_x(rho, 1e16 * rho) / R.lda_x(rho)[0], 1.804, rtol=1e-6)
  np.testing.assert_allclose(R.pbe_c(rho, 0 * rho), R.pw92_c(rho), rtol=1e-14)    # H(t=0) = 0
  assert np.all(np.abs(R.pbe_c(rho, 1e20 * rho)) < 1e-6)        # correlation vanishes as t -> inf
  # PW92 and VWN fit the same electron-gas data
  for rs in (1.0, 2.0, 5.0, 10.0):
    r = 3 / (4 * np.pi * rs**3)
    assert abs(R.pw92_c(r) - R.lda_c_vwn(np.array([r]))[0][0]) < 5e-4


def test_complex_step_derivatives():
  rng = np.random.default_rng(1)
  rho = rng.uniform(1e-3, 5.0, 8)
  sig = rng.uniform(0.0, 3.0, 8) * rho**(8 / 3)
  f, fr, fs = R.gga_f(rho, sig, XC)
  for i in range(8):
    h = 1e-6 * rho[i]
    d = (R.gga_f(rho[i:i + 1] + h, sig[i:i + 1], XC)[0] - R.gga_f(rho[i:i + 1] - h, sig[i:i + 1], XC)[0]) / (2 * h)
    assert abs(d[0] - fr[i]) < 1e-6 * max(1.0, abs(fr[i]))
    hs = 1e-6 * max(sig[i], 1e-3)
    d = (R.gga_f(rho[i:i + 1], sig[i:i + 1] + hs, XC)[0] - R.gga_f(rho[i:i + 1], sig[i:i + 1] - hs, XC)[0]) / (2 * hs)
    assert abs(d[0] - fs[i]) < 1e-5 * max(1e-3, abs(fs[i]))


def test_gga_total_energy_gradient_central_differences():
  sysm = make_system(kind="si2", grid=(10, 10, 10), kgrid=(1, 1, 1), nb=3, nocc=2, xc=XC)
  wr, wi = random_params(sysm, seed=11)
  terms, gr, gi, _ = R.energy_terms(wr, wi, sysm)
  assert np.isfinite(terms["xc"]) and terms["xc"] < 0
  rng = np.random.default_rng(2)
  h = 1e-5
  for _ in range(5):
    idx = tuple(rng.integers(0, s) for s in wr.shape)
    for part, g in ((0, gr), (1, gi)):
      p, m = [wr.copy(), wi.copy()], [wr.copy(), wi.copy()]
      p[part][idx] += h
      m[part][idx] -= h
      fd = (R.energy_terms(*p, sysm, with_grad=False)["total"] -
            R.energy_terms(*m, sysm, with_grad=False)["total"]) / (2 * h)
      assert abs(fd - g[idx]) < 1e-6 * max(1.0, abs(fd)), (part, idx, fd, g[idx])
