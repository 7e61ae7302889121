"""Trains and evaluates the learned preconditioner on trajectories this
implementation generates.

  python -m jrystal_gb300.precond_train --out weights.npz [--eval-json eval.json]
  python -m jrystal_gb300.precond_train --weights weights.npz --eval-json eval.json

1. Trajectories (--recipe benchmark, the default): four plain Adam runs
   (lr 1e-2, 300 steps) of the Si8 64^3 benchmark cell from N(0,1)
   parameters of seeds 1, 5, 6, 7, stepped together as one TrajectoryBatch,
   80 sampled coefficient records per run and step (95 680 records).
   --recipe strained: 64 strained cells (Si, C, Al; seed 2; grids from
   {24, 27, 32, 36, 48}; 2x2x2 k-grid; 8-16 bands, the lower half doubly
   occupied), 300 plain Adam steps each, ~6 records per step (~1.2e5
   records), then ``passes - 1`` refinement passes whose records come from
   trajectories run under the current network (the one-step model is
   re-expressed for the absolute scale, see collect_records).
2. Training: Adam lr 1e-3, 2000 steps, seed 3, with the library's BF16/FP32
   training kernels.
3. Evaluation on 16 held-out strained cells: plain and learned (with the
   plain fallback) optimisers from the same start, both run for the same
   number of steps; E_ref is the converged energy of the plain run (its last
   energy; its own drift over the last 10 % of the run is reported beside
   it), and each method is charged the wall time until |E - E_ref| < 1e-5
   Ha/atom holds for the rest of its run.  A learned run that never settles
   within the tolerance of E_ref (also when it ends below it) counts as not
   reached.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import cells, precond
from .calc import Minimizer
from .engine import PlaneWavePlan


def _plan(wl):
  return PlaneWavePlan(wl.cell, wl.positions, wl.charges, wl.grid_sizes, wl.mask, wl.kpts,
                       wl.num_band, 1, wl.precision, wl.xc)


def _params(wl, plan):
  wr, wi = wl.init_params()
  return torch.tensor(np.stack([wr, wi]), dtype=plan.rdtype, device=plan.device)


def generate(ncells=64, steps=300, per_step=6, seed=2, grids=(24, 27, 32, 36, 48), mlp=None,
             smax=4.0, lr=1e-2, batched=True):
  """Training records from ``steps``-step trajectories of ``ncells`` strained
  cells: plain trajectories run as one batch (batch.TrajectoryBatch: one
  graph launch per step of every cell, records drawn on the device);
  trajectories under the network (``mlp``), or with ``batched=False``, one
  cell at a time (precond.collect_records)."""
  rng = np.random.default_rng(seed)
  if mlp is None and batched:
    from .batch import TrajectoryBatch
    wls = [cells.strained_cell(rng, grids=grids) for _ in range(ncells)]
    b = TrajectoryBatch(wls, steps, lr=lr, per_step=per_step, seed=seed)
    b.run()
    out = {k: v.clone() for k, v in b.records().items()}
    b.close()
    return out
  recs = []
  for i in range(ncells):
    wl = cells.strained_cell(rng, grids=grids)
    plan = _plan(wl)
    fn = precond.GuardedScale(mlp, steps, smax, rise_tol=1e9) if mlp is not None else None
    recs.append(precond.collect_records(plan, wl.occupation, _params(wl, plan), steps, lr,
                                        precond.RecordSpec(per_step=per_step), seed=seed * 1000 + i,
                                        scale_fn=fn))
    plan.close()
  return {k: torch.cat([r[k] for r in recs]) for k in recs[0]}


def fit(passes=3, ncells=64, steps=300, per_step=6, smax=4.0, grids=(24, 27, 32, 36, 48),
        refine_steps=1500, log=print):
  """Pass 1 on plain trajectories of ``steps`` steps; refinement passes on
  trajectories of ``refine_steps`` steps run under the current network (the
  horizon of the step feature x3 is refine_steps from pass 2 on)."""
  mlp = precond.MLP(seed=3)
  mlp.horizon = steps if passes == 1 else refine_steps
  t0 = time.time()
  R = generate(ncells, steps, per_step, 2, grids)
  log(f"pass 1: {R['x'].shape[0]} records from plain trajectories ({time.time() - t0:.1f} s)")
  precond.train(mlp, R, steps=2000, lr=1e-3, seed=3)
  for r in range(2, passes + 1):
    R2 = generate(ncells // 4, refine_steps, max(1, per_step * steps // refine_steps * 2),
                  2 + 10 * r, grids, mlp=mlp, smax=smax)
    R = {k: torch.cat([R[k], R2[k]]) for k in R}
    precond.train(mlp, R, steps=2000, lr=1e-3, seed=3 + r)
    log(f"pass {r}: {R['x'].shape[0]} records, loss {precond.evaluate_loss(mlp, R):.4f}")
  return mlp


def fit_benchmark_cell(name="si8_cubic_64", seeds=(1, 5, 6, 7), steps=300, per_step=80, train_steps=2000,
                       lr=1e-2, log=print):
  """The training recipe on the benchmark cell itself: plain Adam runs of the
  named workload (the Si8 64^3 cell, FP32) from N(0,1) parameters of each
  seed, ``steps`` steps each as one TrajectoryBatch, ``per_step`` records
  per run and step (4 x 299 x 80 = 95 680 records, ~1e5), then Adam (lr
  1e-3, ``train_steps`` steps, seed 3) with the library's training kernels."""
  import dataclasses
  from . import workloads
  from .batch import TrajectoryBatch
  base = workloads.WORKLOADS[name](32)
  wls = [dataclasses.replace(base, seed=s, name=f"{name}_s{s}") for s in seeds]
  t0 = time.time()
  b = TrajectoryBatch(wls, steps, lr=lr, per_step=per_step, seed=3)
  b.run()
  recs = {k: v.clone() for k, v in b.records().items()}
  b.close()
  log(f"{recs['x'].shape[0]} records from {len(wls)} runs of {name} ({time.time() - t0:.1f} s)")
  mlp = precond.MLP(seed=3)
  mlp.horizon = steps
  precond.train(mlp, recs, steps=train_steps, lr=1e-3, seed=3)
  log(f"loss {precond.evaluate_loss(mlp, recs):.4f}")
  return mlp


def run_pair(wl, mlp, nsteps, smax=4.0, total=None, lr=1e-2):
  """Plain and learned histories (energy per step) and ms per step of each."""
  plan = _plan(wl)
  out = {}
  for mode in ("plain", "learned"):
    g = precond.GuardedScale(mlp, total, smax) if mode == "learned" else None
    mini = Minimizer(plan, wl.occupation, _params(wl, plan), lr=lr, scale_fn=g, total_steps=total)
    hist = torch.empty(nsteps, dtype=torch.float64, device=plan.device)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for t in range(nsteps):
      e = mini.step()
      hist[t] = e[4]
      if g is not None and t % 20 == 0 and g.fallback_at is None:
        g.observe(float(e[4]), t)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / nsteps * 1e3
    out[mode] = (hist.cpu().numpy(), ms, None if g is None else g.fallback_at)
  plan.close()
  return out


def score_pair(res, natom, tol=1e-5):
  """Time to tolerance of a run_pair result against the converged plain
  energy E_ref (the plain run's last energy), two ways:
    * |E - E_ref| < tol Ha/atom holding for the rest of the run (steps,
      seconds, speedup_wall; a learned run that ends more than tol below
      E_ref never settles there and counts as not reached);
    * E - E_ref < tol Ha/atom holding for the rest of the run (the _below
      keys: at least as low as the converged plain energy, within tol).
  Also the plain run's drift over its last 10 % (per atom), which bounds how
  converged E_ref is, and each run's end energy relative to E_ref."""
  hp = res["plain"][0]
  n = len(hp)
  eref = float(hp[-1])
  row = {"E_ref": eref, "plain_drift_last10pct_ha_per_atom": float((hp[int(0.9 * n)] - hp[-1]) / natom)}
  for mode, (h, ms, fb) in res.items():
    t = precond.time_to_tolerance(h, eref, tol * natom)
    tb = precond.time_below(h, eref + tol * natom)
    row[mode] = {"steps": t, "ms_per_step": ms, "seconds": None if t is None else t * ms / 1e3,
                 "steps_below": tb, "seconds_below": None if tb is None else tb * ms / 1e3,
                 "fallback_at": fb, "E_end": float(h[-1]),
                 "end_minus_ref_ha_per_atom": float((h[-1] - eref) / natom)}
  for suffix in ("", "_below"):
    p, l = row["plain"]["seconds" + suffix], row["learned"]["seconds" + suffix]
    row["speedup_wall" + suffix] = None if (l is None or p is None or l <= 0) else p / l
  return row


def evaluate(mlp, ncells=16, nsteps=40000, seed=99, grids=(24, 27, 32), smax=4.0, tol=1e-5,
             total=None):
  """Learned vs plain on ``ncells`` held-out strained cells (score_pair)."""
  rng = np.random.default_rng(seed)
  rows = []
  for j in range(ncells):
    wl = cells.strained_cell(rng, grids=grids)
    res = run_pair(wl, mlp, nsteps, smax, total)
    row = {"cell": wl.name}
    row.update(score_pair(res, wl.positions.shape[0], tol))
    rows.append(row)
  return summarise(rows, nsteps, tol)


def summarise(rows, nsteps, tol):
  out = {"cells": rows, "nsteps": nsteps, "tol": tol, "reference_energy": "converged plain energy"}
  for suffix in ("", "_below"):
    sp = [r["speedup_wall" + suffix] for r in rows if r["speedup_wall" + suffix] is not None]
    # cells where the learned run never settled count as no gain (0)
    sp_all = [r["speedup_wall" + suffix] or 0.0 for r in rows]
    out["median_speedup_wall" + suffix] = float(np.median(sp)) if sp else None
    out["median_speedup_wall_all_cells" + suffix] = float(np.median(sp_all))
    out["learned_reached" + suffix] = sum(r["learned"]["steps" + suffix] is not None for r in rows)
    out["plain_reached" + suffix] = sum(r["plain"]["steps" + suffix] is not None for r in rows)
  return out


def transfer(mlp, nsteps=20000, smax=4.0, tol=1e-5, names=("si2_fcc_48", "si8_cubic_64")):
  """The same reference energy on the named benchmark cells (FP32)."""
  from . import workloads
  out = {}
  for name in names:
    wl = workloads.WORKLOADS[name](32)
    res = run_pair(wl, mlp, nsteps, smax)
    out[name] = score_pair(res, wl.positions.shape[0], tol)
  return out


def main():
  ap = argparse.ArgumentParser()
  ap.add_argument("--out", default=None)
  ap.add_argument("--weights", default=None, help="evaluate these weights instead of training")
  ap.add_argument("--eval-json", default=None)
  ap.add_argument("--passes", type=int, default=1)
  ap.add_argument("--recipe", default="benchmark", choices=["benchmark", "strained"],
                  help="records from runs of the Si8 64^3 benchmark cell, or from 64 strained "
                       "Si/C/Al cells with refinement passes")
  ap.add_argument("--eval-cells", type=int, default=16)
  ap.add_argument("--eval-steps", type=int, default=40000)
  ap.add_argument("--transfer-steps", type=int, default=0,
                  help="also score the benchmark cells (Si2 48^3, Si8 64^3) over this many steps")
  ap.add_argument("--refine-steps", type=int, default=1500)
  args = ap.parse_args()
  if args.weights:
    mlp = precond.MLP.load(args.weights)
  else:
    if not args.out:
      ap.error("--out is required when training")
    mlp = (fit_benchmark_cell() if args.recipe == "benchmark"
           else fit(passes=args.passes, refine_steps=args.refine_steps))
    mlp.save(args.out)
  if args.eval_json:
    res = evaluate(mlp, ncells=args.eval_cells, nsteps=args.eval_steps)
    if args.transfer_steps:
      res["transfer"] = transfer(mlp, nsteps=args.transfer_steps)
    with open(args.eval_json, "w") as f:
      json.dump(res, f, indent=1)
    print(json.dumps({k: v for k, v in res.items() if k != "cells"}))


if __name__ == "__main__":
  main()
