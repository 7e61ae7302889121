"""CPU checks of the preconditioner oracle (oracle/mlp.py): its analytic
gradient against central differences, and the BF16 rounding it emulates."""
import numpy as np

from oracle import mlp as M


def test_bf16_round_to_nearest_even():
  x = np.array([1.0, 1.0 + 2**-8, 1.0 + 2**-9, 1.0 + 3 * 2**-9, -2.5, 3.14159], dtype=np.float32)
  r = M.bf16(x)
  assert r[0] == 1.0
  assert r[1] == 1.0                       # exactly halfway: ties to the even mantissa
  assert r[2] == 1.0                       # below halfway
  assert r[3] == 1.0 + 2**-7               # above halfway
  assert r[4] == -2.5
  assert abs(r[5] - 3.140625) < 1e-12


def test_mlp_oracle_gradient_central_differences(monkeypatch):
  rng = np.random.default_rng(0)
  w = rng.normal(size=8641) * 0.1
  n = 40
  x = np.stack([rng.gamma(1, 2, n), rng.uniform(0, 1, n), rng.uniform(0, 1, n)], 1)
  a = rng.normal(size=n)
  c = np.abs(rng.normal(size=n)) + 0.1
  wt = rng.uniform(0.5, 1.5, n)
  monkeypatch.setattr(M, "bf16", lambda v: np.asarray(v, dtype=np.float64))   # exact arithmetic
  _, g = M.loss_and_grad(w, x, a, c, wt)
  for i in (0, 5, 191, 200, 300, 4000, 8575, 8640):
    e = np.zeros_like(w)
    e[i] = 1e-6
    fd = (M.loss_and_grad(w + e, x, a, c, wt)[0] - M.loss_and_grad(w - e, x, a, c, wt)[0]) / 2e-6 / n
    assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_softplus_output_starts_at_one():
  # the initial output bias of jrystal_gb300.precond.MLP: softplus(b4) = 1
  assert abs(M.softplus(np.array([0.5413248546129181]))[0] - 1.0) < 1e-12
