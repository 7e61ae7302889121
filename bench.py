#!/usr/bin/env python
"""Energy+gradient evaluations/s of the direct-minimisation step on one GB300.

A step is one optimiser iteration of jrystal's ground-state loop
(calc/calc_ground_state_energy_all_electrons.py:175-181): orthonormalise the
parameters, energy and hand-written gradient, and the Adam update of all
parameters.  The default workload is the all-electron Si 8-atom cubic cell
(a = 10.26 bohr, LDA, 64^3 grid, 17071 plane waves, 3x3x3 k-grid, 24 bands of
which 16 doubly occupied, complex64 parameters drawn N(0,1) from seed 1).

Prints one JSON line.  ``--impl reference`` times the CPU restatement of the
same path on the host cores instead (the reference arm).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
  sys.path.insert(0, ROOT)

METRIC = "energy+grad evals/s (direct-minimisation step incl. Adam)"
UNIT = "evals/s"


def _args():
  p = argparse.ArgumentParser()
  p.add_argument("--gpus", type=int, default=1)
  p.add_argument("--steps", type=int, default=300)
  p.add_argument("--warmup", type=int, default=3)
  p.add_argument("--impl", default="ours", choices=["ours", "reference"])
  p.add_argument("--workload", default="si8_cubic_64")
  p.add_argument("--no-cpu-baseline", action="store_true")
  p.add_argument("--pseudo", action="store_true",
                 help="attach the analytic norm-conserving model pseudopotential "
                      "(local table + beta projectors) to the workload")
  p.add_argument("--no-time-to-tol", action="store_true",
                 help="skip the learned-vs-plain time-to-tolerance runs")
  p.add_argument("--cpu-sample-kpts", type=int, default=27)
  p.add_argument("--step", default="fused", choices=["split", "fused"],
                 help="fused: one jrg_energy_grad_adam call per step (default); split: "
                      "jrg_energy_grad then jrg_adam_update")
  p.add_argument("--kgrid", type=int, nargs=3, default=None,
                 help="override the workload's k-grid (smaller cases for profiling)")
  return p.parse_args()


def _dist():
  ws = int(os.environ.get("WORLD_SIZE", "1"))
  rank = int(os.environ.get("RANK", "0"))
  local = int(os.environ.get("LOCAL_RANK", "0"))
  return ws, rank, local


def _max_over_ranks(x, device):
  """The maximum of x over the ranks of the process group (x itself without
  one): the job's time is its slowest rank's."""
  import torch
  import torch.distributed as dist
  if not dist.is_initialized() or dist.get_world_size() == 1:
    return float(x)
  t = torch.tensor([float(x)], dtype=torch.float64, device=device)
  dist.all_reduce(t, op=dist.ReduceOp.MAX)
  return float(t.item())


def _peaks():
  path = os.path.join(ROOT, "MEASURED_PEAKS.json")
  try:
    with open(path) as f:
      d = json.load(f)
    return float(d["hbm_gbs"]), "measured"
  except Exception:
    return 6800.0, "fallback"


class _Nvml:
  """The few NVML reads the clock record needs (libnvidia-ml from the
  driver, through ctypes): SM clock, its maximum and the active clock event
  reasons.  Reads only; nothing is set."""
  HW_SLOWDOWN, SW_THERMAL, HW_THERMAL, SW_POWER_CAP = 0x8, 0x20, 0x40, 0x4

  def __init__(self, index):
    import ctypes as ct
    self.ct = ct
    self.lib = ct.CDLL("libnvidia-ml.so.1")
    if self.lib.nvmlInit_v2() != 0:
      raise RuntimeError("nvmlInit failed")
    self.h = ct.c_void_p()
    if self.lib.nvmlDeviceGetHandleByIndex_v2(ct.c_uint(index), ct.byref(self.h)) != 0:
      raise RuntimeError("nvmlDeviceGetHandleByIndex failed")
    try:
      self._reasons = self.lib.nvmlDeviceGetCurrentClocksEventReasons
    except AttributeError:   # the name of older drivers
      self._reasons = self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
    mx = ct.c_uint()
    self.max_mhz = float(mx.value) if self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, ct.byref(mx)) == 0 \
        else None

  def sample(self):
    ct = self.ct
    mhz, reasons = ct.c_uint(), ct.c_ulonglong()
    if self.lib.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(mhz)) != 0:   # NVML_CLOCK_SM
      return None
    self._reasons(self.h, ct.byref(reasons))
    return float(mhz.value), int(reasons.value)


class ClockSampler:
  """SM clocks and throttle reasons sampled every 2 ms by a host thread
  through NVML while the region runs (a region of a few tens of ms still
  gets samples); nvidia-smi every 200 ms where NVML cannot be loaded."""
  Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
       "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
       "clocks_event_reasons.sw_power_cap")

  def __init__(self, index):
    self.index = index
    self.proc = None
    self.nvml = None
    self.lines = []
    self.samples = []
    self.stop = threading.Event()

  def __enter__(self):
    try:
      self.nvml = _Nvml(self.index)
    except Exception:
      self.nvml = None
    if self.nvml is not None:
      self.t = threading.Thread(target=self._poll, daemon=True)
      self.t.start()
      return self
    try:
      self.proc = subprocess.Popen(
        ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
         "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
      self.t = threading.Thread(target=self._read, daemon=True)
      self.t.start()
      # wait for nvidia-smi's first sample, then keep only samples taken
      # inside the region
      t0 = time.time()
      while not self.lines and time.time() - t0 < 5.0:
        time.sleep(0.01)
      self.lines = []
    except Exception:
      self.proc = None
    return self

  def _poll(self):
    while not self.stop.is_set():
      s = self.nvml.sample()
      if s is not None:
        self.samples.append(s)
      time.sleep(0.002)

  def _read(self):
    for ln in self.proc.stdout:
      self.lines.append(ln.strip())

  def __exit__(self, *a):
    self.stop.set()
    if self.nvml is not None:
      self.t.join(timeout=5)
    if self.proc:
      self.proc.terminate()
      try:
        self.proc.wait(timeout=5)
      except Exception:
        self.proc.kill()

  def summary(self):
    sm, mx, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    if self.nvml is not None:
      bits = [_Nvml.HW_SLOWDOWN, _Nvml.HW_THERMAL, _Nvml.SW_THERMAL, _Nvml.SW_POWER_CAP]
      for mhz, r in self.samples:
        sm.append(mhz)
        for n, b in zip(names, bits):
          if r & b:
            reasons.add(n)
      if self.nvml.max_mhz:
        mx.append(self.nvml.max_mhz)
      source = "nvml, 2 ms"
    else:
      for ln in self.lines:
        parts = [p.strip() for p in ln.split(",")]
        if len(parts) < 7:
          continue
        try:
          sm.append(float(parts[0]))
          mx.append(float(parts[1]))
        except ValueError:
          continue
        for n, v in zip(names, parts[3:7]):
          if v.lower() in ("active", "1", "yes"):
            reasons.add(n)
      source = "nvidia-smi, 200 ms"
    if not sm:
      return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx) if mx else None,
            "reasons": sorted(reasons), "samples": len(sm), "source": source}


def cpu_sample(wl, nk_sample, workers, min_seconds=10.0, max_repeats=50):
  """Seconds per full evaluation of the FP64 CPU restatement (energy,
  gradient and Adam of nk_sample k-points, all bands, full grid, scaled by
  K / nk_sample), the mean over evaluations repeated until min_seconds of CPU
  work; also returns the sample's total seconds and evaluation count."""
  from oracle import restatement as R
  R.FFT_WORKERS = workers
  occ = wl.occupation[:, :nk_sample]
  sysm = R.System(wl.cell, wl.positions, wl.charges, wl.grid_sizes, wl.mask,
                  wl.kpts[:nk_sample], occ, wl.xc)
  wr, wi = wl.init_params()
  wr = wr[:, :nk_sample].astype(np.float64)
  wi = wi[:, :nk_sample].astype(np.float64)
  m = np.zeros_like(wr)
  v = np.zeros_like(wr)
  times = []
  while not times or (sum(times) < min_seconds and len(times) < max_repeats):
    it = len(times)
    t0 = time.perf_counter()
    _, gr, gi, _ = R.energy_terms(wr, wi, sysm)
    R.adam_update(wr, gr, m, v, it + 1, wl.lr)
    R.adam_update(wi, gi, m, v, it + 1, wl.lr)
    times.append(time.perf_counter() - t0)
  t = sum(times) / len(times)
  return t * wl.num_kpt / nk_sample, sum(times), len(times)


def run_reference(args, wl):
  ws, rank, _ = _dist()
  if rank != 0:
    return
  workers = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
  nks = max(1, min(args.cpu_sample_kpts, wl.num_kpt))
  # one evaluation per step (min_seconds=0)
  for _ in range(args.warmup):
    cpu_sample(wl, nks, workers, min_seconds=0.0)
  per_eval = []
  t_start = time.time()
  for _ in range(args.steps):
    per_eval.append(cpu_sample(wl, nks, workers, min_seconds=0.0)[0])
    if time.time() - t_start > 150.0:   # bound the arm to a few minutes
      break
  t = statistics.median(per_eval)
  val = 1.0 / t
  sample = (f"FP64 NumPy/SciPy restatement of the path (not jrystal: jax is absent), "
            f"{nks} of {wl.num_kpt} k-points per step (all {wl.num_band} bands, full "
            f"{wl.grid_sizes[0]}^3 grid)"
            + (f", time scaled by {wl.num_kpt}/{nks}" if nks < wl.num_kpt else ""))
  out = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
         "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
         "steps_sampled": len(per_eval),
         "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
         "data": "synthetic", "config": _config(wl, args.gpus, precision=64),
         "cpu_baseline": {"value": val, "unit": UNIT, "cores": workers, "kind": "port",
                          "sample": sample},
         "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
  print(json.dumps(out))


def _config(wl, n, precision=None):
  return {"workload": wl.name, "cell": "all-electron Si", "grid": list(wl.grid_sizes),
          "num_g": int(wl.mask.sum()), "kpts": wl.num_kpt, "bands": wl.num_band,
          "occupied": wl.num_occ, "xc": wl.xc,
          "precision": f"fp{precision or wl.precision}",
          "parallelism": f"replicas{n}" if n > 1 else "single-gpu",
          "l2": "no explicit flush: each step streams >0.7 GB of plane buffers, >5x the 129 MB L2"}


# DRAM bytes (read + write) per band of one k_line_apply_v<float, 64> launch,
# from an ncu capture (dram__bytes_read.sum + dram__bytes_write.sum) of the
# 64^3 Si8 cell at 2x2x2 k-points (135 MB for the 96 bands of one pipeline
# half); a full launch is scaled by its band count
LINE_APPLY_V_DRAM_PER_BAND = (98.57996e6 + 36.56985e6) / 96


# algorithmic bytes per call of each phase of jrg_energy_grad (fused: the
# adjoint rotation also reads and writes the parameters and both moments)
def phase_bytes(plan, fused=False):
  c = 8 if plan.precision == 32 else 16
  r = c // 2
  nbt = plan.num_spin * plan.num_kpt * plan.num_band
  nsk = plan.num_spin * plan.num_kpt
  nx, ny, nz = plan.grid
  ngrid = nx * ny * nz
  nact = int(np.unique(np.flatnonzero(plan.mask.reshape(-1)) // (ny * nz)).size)
  planes = nact * ny * nz * c
  sph = plan.num_g * c
  return {
    "pack_params": 2 * nbt * sph,
    "gram": nbt * sph,
    "rotate": 2 * nbt * sph,
    # kinetic partials come out of the forward rotation; this phase sums them
    "kinetic": nbt * ((plan.num_g + 255) // 256) * r,
    "plane_inv_sphere": nbt * (sph + planes),
    "line_density": nbt * planes + nsk * ngrid * r,
    "reduce_density": nsk * ngrid * r + ngrid * r,
    "line_apply_v": nbt * 2 * planes + nsk * ngrid * r,
    "plane_fwd_sphere": nbt * (planes + 2 * sph) + plan.num_kpt * plan.num_g * 8,
    "adj_gram": 2 * nbt * sph,
    "adj_rotate": 2 * nbt * sph + (6 if fused else 1) * nbt * sph,
    # beta projectors: C and the table read once; the table again and g_C
    # read + written by the apply pass
    "nl_project": nbt * sph + plan.num_kpt * plan.num_proj * sph,
    "nl_apply": plan.num_kpt * plan.num_proj * sph + 2 * nbt * sph,
  }


def time_to_tolerance(nsteps=20000, ncells=16, cell_index=1):
  """Learned vs plain optimiser on the held-out strained cells of the
  preconditioner's evaluation sequence (seed 99), measured against the
  converged plain energy E_ref (the plain run's energy after nsteps): wall
  time until E stays within 1e-5 Ha/atom of E_ref (two-sided: |E - E_ref|)
  and until E stays below E_ref + 1e-5 Ha/atom (one-sided, the "_below"
  keys: at least as converged as the plain run; the learned runs end below
  E_ref, so the two-sided form charges them for going lower).  Medians over
  the cells, with cells where the learned run never settles counted as 0,
  the detail of one cell, and the same reference energy on the Si8 64^3 benchmark cell
  (8000 steps)."""
  from jrystal_gb300 import precond, precond_train
  mlp = precond.MLP.load(precond.DEFAULT_WEIGHTS)
  res = precond_train.evaluate(mlp, ncells=ncells, nsteps=nsteps, seed=99, grids=(24, 27, 32))
  row = res["cells"][cell_index]
  out = {"cell": row["cell"], "tol_ha_per_atom": 1e-5, "max_steps": nsteps,
         "reference_energy": "converged plain energy (the plain run's energy after max_steps)",
         "E_ref": row["E_ref"], "plain_drift_last10pct_ha_per_atom": row["plain_drift_last10pct_ha_per_atom"]}
  for mode in ("plain", "learned"):
    r = row[mode]
    out[mode] = {k: (round(r[k], 4) if isinstance(r[k], float) else r[k])
                 for k in ("steps", "steps_below", "ms_per_step", "seconds", "seconds_below",
                           "end_minus_ref_ha_per_atom")}
  out["speedup_wall"] = row["speedup_wall"]
  out["speedup_wall_below"] = row["speedup_wall_below"]
  out["heldout"] = {k: res[k] for k in res if k not in ("cells",)}
  out["heldout"]["cells"] = ncells
  out["heldout"]["speedups_below"] = [None if r["speedup_wall_below"] is None else round(r["speedup_wall_below"], 3)
                                      for r in res["cells"]]
  out["heldout"]["speedups"] = [None if r["speedup_wall"] is None else round(r["speedup_wall"], 3)
                                for r in res["cells"]]
  # the benchmark cell itself (Si8 64^3, FP32, N(0,1) seed 1), same reference energy
  b = precond_train.transfer(mlp, nsteps=8000, names=("si8_cubic_64",))["si8_cubic_64"]
  out["benchmark_cell"] = {"cell": "si8_cubic_64", "max_steps": 8000, "E_ref": b["E_ref"],
                           "plain_drift_last10pct_ha_per_atom": b["plain_drift_last10pct_ha_per_atom"],
                           "speedup_wall": b["speedup_wall"], "speedup_wall_below": b["speedup_wall_below"]}
  for mode in ("plain", "learned"):
    out["benchmark_cell"][mode] = {k: (round(b[mode][k], 4) if isinstance(b[mode][k], float) else b[mode][k])
                                   for k in ("steps", "steps_below", "ms_per_step", "seconds_below",
                                             "fallback_at", "end_minus_ref_ha_per_atom")}
  return out


def parity_at(plan, wl, params, occ, dev, pseudo=None):
  """Error of the timed (FP32) path against the FP64 path of the same
  kernels at the given parameters: energy per atom (each term and the total)
  and the gradient's 2-norm relative error and max-abs error over the max."""
  import torch
  from jrystal_gb300.engine import PlaneWavePlan
  if plan.precision == 64:
    return None
  try:
    p64 = PlaneWavePlan(wl.cell, wl.positions, wl.charges, wl.grid_sizes, wl.mask, wl.kpts,
                        wl.num_band, 1, 64, wl.xc, device=dev)
  except NotImplementedError as err:
    return {"against": "FP64 path of the same kernels", "unavailable": str(err)}
  if pseudo is not None:
    p64.set_pseudopotential(*pseudo)
  out = []
  for pl in (plan, p64):
    p = params.to(pl.rdtype)
    e, gr, gi = pl.energy_and_grad(p[0].contiguous(), p[1].contiguous(), occ)
    torch.cuda.synchronize()
    out.append((e.cpu().numpy().copy(), torch.stack([gr, gi]).double()))
  (e32, g32), (e64, g64) = out
  natom = len(wl.charges)
  names = ["kinetic", "external", "hartree", "xc", "total"]
  err = {n: float(abs(e32[i] - e64[i]) / natom) for i, n in enumerate(names)}
  d = g32 - g64
  res = {"against": "FP64 path of the same kernels at the parameters after the timed steps",
         "energy_err_ha_per_atom": err, "max_energy_err_ha_per_atom": max(err.values()),
         "grad_rel_err_2norm": float(torch.linalg.norm(d) / torch.linalg.norm(g64)),
         "grad_max_abs_err_over_max": float(d.abs().max() / g64.abs().max()),
         "tolerance": {"energy_ha_per_atom": 1e-6, "grad_rel": 1e-5},
         "energies_fp64": e64[:5].tolist()}
  res["within_tolerance"] = bool(res["max_energy_err_ha_per_atom"] <= 1e-6 and
                                 res["grad_rel_err_2norm"] <= 1e-5)
  del p64
  return res


def run_ours(args, wl):
  import torch
  import torch.distributed as dist
  from jrystal_gb300 import _lib
  from jrystal_gb300.engine import PlaneWavePlan, adam_update

  ws, rank, local = _dist()
  if ws > 1:
    dist.init_process_group("nccl")
  torch.cuda.set_device(local)
  dev = torch.device("cuda", local)
  lib = _lib.load()
  plan = PlaneWavePlan(wl.cell, wl.positions, wl.charges, wl.grid_sizes, wl.mask, wl.kpts,
                       wl.num_band, 1, wl.precision, wl.xc, device=dev)
  from jrystal_gb300.workloads import model_pseudopotential
  if args.pseudo:
    plan.set_pseudopotential(*model_pseudopotential(wl))
  wr, wi = wl.init_params()
  rdt = plan.rdtype
  params = torch.tensor(np.stack([wr, wi]), dtype=rdt, device=dev).contiguous()
  grads = torch.empty_like(params)
  m = torch.zeros_like(params)
  v = torch.zeros_like(params)
  occ = torch.tensor(wl.occupation, dtype=torch.float64, device=dev)
  state = {"t": 0}

  fused = args.step == "fused"

  def step_split(p):
    state["t"] += 1
    e, _, _ = plan.energy_and_grad(p[0], p[1], occ, grads[0], grads[1])
    adam_update(p, grads, m, v, state["t"], wl.lr)
    return e

  def step(p):
    if not fused:
      return step_split(p)
    # one call: energy, gradient and Adam (per k-point half in the pipeline)
    state["t"] += 1
    return plan.energy_grad_adam(p, m, v, occ, state["t"], wl.lr)

  def barrier():
    if ws > 1:
      dist.barrier()
    torch.cuda.synchronize()

  for _ in range(args.warmup):
    step(params)
  barrier()
  launches0 = lib.jrg_launch_count()
  stream = torch.cuda.current_stream()
  t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  with ClockSampler(local) as clk:
    barrier()
    t0.record(stream)
    for _ in range(args.steps):
      e = step(params)
    t1.record(stream)
    barrier()
  launches = lib.jrg_launch_count() - launches0
  ms = t0.elapsed_time(t1) / args.steps
  # per-phase CUDA-event times from a separate single-stream run of the
  # two-call step (phase events are kept out of the timed region above, and
  # the phases of the pipelined step overlap)
  nprof = min(args.steps, 50)
  lib.jrg_profile_enable(plan._h, nprof)
  for _ in range(nprof):
    step_split(params)
  barrier()
  nph = lib.jrg_profile_num_phases()
  import ctypes as ct
  arr = (ct.c_double * nph)()
  ncalls = ct.c_int()
  _lib.check(lib.jrg_profile_read(plan._h, arr, ct.byref(ncalls), nph), "jrg_profile_read")
  lib.jrg_profile_enable(plan._h, 0)
  phases = {lib.jrg_profile_phase_name(i).decode(): arr[i] / max(1, ncalls.value) for i in range(nph)}
  ms = _max_over_ranks(ms, dev)
  energies = e.cpu().numpy().tolist()

  # end to end through the public API with host buffers: H2D of the step's
  # parameters from pinned memory, energy+grad+Adam, D2H of the energies.
  # Two device parameter buffers: the copy engine fills one (side stream)
  # while the step runs on the other.
  host_params = params.cpu().pin_memory()
  host_e = torch.empty((2, 8), dtype=torch.float64).pin_memory()
  bufs = [params, torch.empty_like(params)]
  copy_stream = torch.cuda.Stream(device=dev)
  ready = [torch.cuda.Event(), torch.cuda.Event()]
  free = [torch.cuda.Event(), torch.cuda.Event()]

  def e2e_run(n):
    copy_stream.wait_stream(stream)
    with torch.cuda.stream(copy_stream):
      bufs[0].copy_(host_params, non_blocking=True)
      ready[0].record(copy_stream)
    for i in range(n):
      cur, nxt = i % 2, (i + 1) % 2
      if i + 1 < n:
        with torch.cuda.stream(copy_stream):
          if i >= 1:
            copy_stream.wait_event(free[nxt])
          bufs[nxt].copy_(host_params, non_blocking=True)
          ready[nxt].record(copy_stream)
      stream.wait_event(ready[cur])
      e = step(bufs[cur])
      free[cur].record(stream)
      host_e[cur].copy_(e, non_blocking=True)

  e2e_run(max(1, args.warmup))
  barrier()
  e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  e0.record(stream)
  e2e_run(args.steps)
  e1.record(stream)
  barrier()
  e2e_ms = e0.elapsed_time(e1) / args.steps
  e2e_ms = _max_over_ranks(e2e_ms, dev)

  if rank == 0:
    peak, peak_kind = _peaks()
    pb = phase_bytes(plan, False)
    top = max((k for k in phases if k in pb), key=lambda k: phases[k])
    achieved = pb[top] / (phases[top] * 1e-3) / 1e9
    traffic = None
    if top == "line_apply_v" and plan.grid == (64, 64, 64) and plan.precision == 32:
      traffic = LINE_APPLY_V_DRAM_PER_BAND * plan.num_spin * plan.num_kpt * plan.num_band
    # whole-evaluation models: the grid-streaming byte model 6 P G c + 10 P n_g c
    # (each band's grid crossing HBM once per FFT pass) and the compulsory
    # traffic (2 + 4) P n_g r 2 (parameters, gradient and Adam state), against
    # the measured step time; FFT flops 3 P 5 G log2 G
    c_b = 8 if wl.precision == 32 else 16
    P_b = plan.num_spin * plan.num_kpt * plan.num_band
    G_b = int(np.prod(plan.grid))
    model_bytes = 6 * P_b * G_b * c_b + 10 * P_b * plan.num_g * c_b
    compulsory = (2 + 4) * P_b * plan.num_g * (c_b // 2) * 2
    fft_flops = 3 * P_b * 5 * G_b * np.log2(G_b)
    step_model = {"model_bytes": int(model_bytes), "model_gbs": model_bytes / (ms * 1e-3) / 1e9,
                  "model_frac": model_bytes / (ms * 1e-3) / 1e9 / peak,
                  "compulsory_bytes": int(compulsory),
                  "compulsory_frac": compulsory / (ms * 1e-3) / 1e9 / peak,
                  "fft_tflops": fft_flops / (ms * 1e-3) / 1e12}
    roof = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
            "traffic_source": None if traffic is None else
            "ncu dram bytes per band (2x2x2 k-point capture) x bands of this launch",
            "algorithmic_bytes": pb[top], "ms_per_launch": phases[top],
            "phase_ms": {k: round(v, 4) for k, v in phases.items()}, "step_model": step_model}
    out = {"metric": METRIC, "value": 1000.0 / ms * ws, "unit": UNIT, "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32" if wl.precision == 32 else "f64", "data": "synthetic",
           "config": _config(wl, ws), "clocks": clk.summary(),
           "e2e": {"value": 1000.0 / e2e_ms * ws, "unit": UNIT,
                   "h2d_bytes_per_step": int(params.numel() * params.element_size()),
                   "d2h_bytes_per_step": 64},
           "gpu_launches": int(launches), "roofline": roof,
           "energies_last_step": energies[:5]}
    if args.pseudo:
      out["config"]["cell"] = "Si cell with the analytic norm-conserving model pseudopotential"
      out["config"]["projector_rows"] = int(plan.num_proj)
      out["energies_last_step"] = energies[:5] + [energies[7]]
      out["nonlocal"] = {k: {"ms_per_launch": round(phases[k], 5),
                             "algorithmic_bytes": pb[k],
                             "achieved_gbs": pb[k] / (phases[k] * 1e-3) / 1e9,
                             "frac": pb[k] / (phases[k] * 1e-3) / 1e9 / peak}
                         for k in ("nl_project", "nl_apply") if phases.get(k, 0) > 0}
    out["parity"] = parity_at(plan, wl, params, occ, dev,
                              model_pseudopotential(wl) if args.pseudo else None)
    if not args.no_time_to_tol:
      out["time_to_1e-5_Ha_per_atom"] = time_to_tolerance()
    if not args.no_cpu_baseline and not args.pseudo:
      workers = len(os.sched_getaffinity(0))
      nks = max(1, min(args.cpu_sample_kpts, wl.num_kpt))
      per_eval, t_sample, n_eval = cpu_sample(wl, nks, workers)
      out["cpu_baseline"] = {
        "value": 1.0 / per_eval, "unit": UNIT, "cores": workers, "kind": "port",
        "sample": f"FP64 CPU restatement (energy, gradient, Adam), {nks}/{wl.num_kpt} k-points, "
                  f"{n_eval} evaluations in {t_sample:.1f} s"
                  + (f", scaled by {wl.num_kpt}/{nks}" if nks < wl.num_kpt else "")}
    print(json.dumps(out))
  if ws > 1:
    dist.destroy_process_group()


BATCH_METRIC = "cell-steps/s (batched plain-Adam trajectory generation incl. records)"
BATCH_UNIT = "cell-steps/s"


def batch_cells(ncells=64, seed=2, grids=(24, 27, 32, 36, 48)):
  """The 64 strained Si / C / Al cells of the trajectory-generation workload
  (uniform +-3 % strain per lattice vector, grids 24^3-48^3, 2x2x2 k-points,
  8-16 bands, the lower half doubly occupied, FP32)."""
  from jrystal_gb300 import cells
  rng = np.random.default_rng(seed)
  return [cells.strained_cell(rng, grids=grids) for _ in range(ncells)]


def _batch_config(wls, n):
  return {"workload": "batch64_trajectories", "cells": len(wls),
          "kinds": {k: sum(w.name.startswith(k + "_") for w in wls) for k in ("si", "c", "al")},
          "grids": sorted({w.grid_sizes[0] for w in wls}), "kpts": 8,
          "bands": [min(w.num_band for w in wls), max(w.num_band for w in wls)],
          "records_per_step_per_cell": 6, "precision": "fp32", "xc": "lda_x+lda_c_vwn",
          "parallelism": f"replicas{n}" if n > 1 else "single-gpu",
          "l2": "no explicit flush: the 64 cells' plane buffers total > 1 GB, > 8x the 129 MB L2"}


def run_batch_reference(args, wls):
  """The FP64 CPU restatement stepping the cells one at a time (energy,
  gradient, Adam per cell-step), over a bounded sample of cells."""
  ws, rank, _ = _dist()
  if rank != 0:
    return
  workers = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()
  cpu_sample(wls[0], wls[0].num_kpt, workers, min_seconds=0.0)
  per, t_start, i = [], time.time(), 0
  while i < args.steps and time.time() - t_start < 60.0:
    wl = wls[i % len(wls)]
    per.append(cpu_sample(wl, wl.num_kpt, workers, min_seconds=0.0)[0])
    i += 1
  val = len(per) / sum(per)
  out = {"impl": "reference", "metric": BATCH_METRIC, "value": val, "unit": BATCH_UNIT,
         "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
         "ms_per_step": 1e3 / val, "steps_sampled": len(per), "higher_is_better": True,
         "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
         "config": _batch_config(wls, args.gpus),
         "cpu_baseline": {"value": val, "unit": BATCH_UNIT, "cores": workers, "kind": "port",
                          "sample": f"FP64 NumPy restatement, {len(per)} cell-steps of the first "
                                    f"{min(len(per), len(wls))} cells, one cell at a time"},
         "e2e": {"value": val, "unit": BATCH_UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
  print(json.dumps(out))


def run_batch(args, wls):
  """Batched trajectory generation: args.warmup + args.steps plain Adam
  steps of every cell (one CUDA graph launch per step of all cells, records
  drawn on the device), timed over the last args.steps; beside it the same
  cells stepped one at a time (the single-cell two-call loop, a bounded
  sample), and the whole job end to end (parameters copied in from pinned
  host memory, records and energies copied out)."""
  import torch
  import torch.distributed as dist
  from jrystal_gb300 import _lib
  from jrystal_gb300.batch import TrajectoryBatch, _plan
  from jrystal_gb300.engine import adam_update

  ws, rank, local = _dist()
  if ws > 1:
    dist.init_process_group("nccl")
  torch.cuda.set_device(local)
  dev = torch.device("cuda", local)
  lib = _lib.load()
  total = args.warmup + args.steps
  batch = TrajectoryBatch(wls, total, per_step=6, seed=2, device=dev)
  stream = torch.cuda.current_stream()

  def barrier():
    if ws > 1:
      dist.barrier()
    torch.cuda.synchronize()

  batch.run(args.warmup)
  barrier()
  launches0 = lib.jrg_launch_count()
  t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  with ClockSampler(local) as clk:
    barrier()
    t0.record(stream)
    batch.run(args.steps)
    t1.record(stream)
    barrier()
  kernels_per_step = (lib.jrg_launch_count() - launches0)
  ms = _max_over_ranks(t0.elapsed_time(t1) / args.steps, dev)
  last_e = batch.energies[-1].cpu().numpy()
  nrec = int(batch.rec_a.numel())
  # the graph's kernel launches are not counted by the library's host-side
  # launch counter; count one eager step instead
  probe = TrajectoryBatch(wls[:len(wls)], 1, per_step=6, seed=2, device=dev)
  c0 = lib.jrg_launch_count()
  probe.step(graph=False)
  barrier()
  launches_per_step = lib.jrg_launch_count() - c0
  probe.close()

  # the same cells one at a time (single-cell two-call loop), bounded sample
  seq_steps, seq_cells = 20, min(16, len(wls))
  seq_ms = 0.0
  for wl in wls[:seq_cells]:
    plan = _plan(wl, dev)
    wr, wi = wl.init_params()
    p = torch.tensor(np.stack([wr, wi]), dtype=plan.rdtype, device=dev)
    g, m, v = torch.zeros_like(p), torch.zeros_like(p), torch.zeros_like(p)
    occ = torch.as_tensor(np.asarray(wl.occupation), dtype=torch.float64, device=dev)
    for t in range(3):
      plan.energy_and_grad(p[0], p[1], occ, g[0], g[1])
      adam_update(p, g, m, v, t + 1, 1e-2)
    barrier()
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a0.record(stream)
    for t in range(seq_steps):
      plan.energy_and_grad(p[0], p[1], occ, g[0], g[1])
      adam_update(p, g, m, v, t + 4, 1e-2)
    a1.record(stream)
    barrier()
    seq_ms += a0.elapsed_time(a1)
    plan.close()
  seq_val = seq_cells * seq_steps / (seq_ms * 1e-3)

  # end to end: parameters from pinned host memory, all steps, records and
  # energies back to pinned host memory
  host_p = [torch.tensor(np.stack(wl.init_params())).pin_memory() for wl in wls]
  e2e = TrajectoryBatch(wls, args.steps, per_step=6, seed=3, device=dev)
  host_rec = {k: torch.empty(v.shape, dtype=v.dtype).pin_memory() for k, v in e2e.records().items()}
  host_hist = torch.empty(e2e.energies.shape, dtype=torch.float64).pin_memory()
  barrier()
  b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
  b0.record(stream)
  for dst, src in zip(e2e.params, host_p):
    dst.copy_(src, non_blocking=True)
  e2e.run()
  for k, v in e2e.records().items():
    host_rec[k].copy_(v, non_blocking=True)
  host_hist.copy_(e2e.energies, non_blocking=True)
  b1.record(stream)
  barrier()
  e2e_ms = _max_over_ranks(b0.elapsed_time(b1) / args.steps, dev)
  h2d = sum(p.numel() * p.element_size() for p in e2e.params)
  d2h = sum(v.numel() * v.element_size() for v in e2e.records().values()) + host_hist.numel() * 8
  e2e.close()

  if rank == 0:
    peak, peak_kind = _peaks()
    step_bytes = sum(sum(phase_bytes(p).values()) - phase_bytes(p)["pack_params"] for p in batch.plans)
    adam_bytes = sum(7 * p.numel() * p.element_size() for p in batch.params)
    achieved = (step_bytes + adam_bytes) / (ms * 1e-3) / 1e9
    ncell = len(wls)
    out = {"metric": BATCH_METRIC, "value": ncell * 1000.0 / ms * ws, "unit": BATCH_UNIT, "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic", "config": _batch_config(wls, ws), "clocks": clk.summary(),
           "e2e": {"value": ncell * 1000.0 / e2e_ms * ws, "unit": BATCH_UNIT,
                   "h2d_bytes_per_step": int(h2d / args.steps), "d2h_bytes_per_step": int(d2h / args.steps)},
           "gpu_launches": int(launches_per_step * args.steps),
           "graph_launches": args.steps,
           "roofline": {"bound": "hbm", "kernel": "whole batched step (every kernel of the 64 cells)",
                        "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                        "peak_source": peak_kind, "traffic": None,
                        "algorithmic_bytes": int(step_bytes + adam_bytes)},
           "sequential": {"value": seq_val, "unit": BATCH_UNIT,
                          "sample": f"{seq_cells} cells x {seq_steps} steps, one cell at a time "
                                    "(jrg_energy_grad + jrg_adam_update per step)",
                          "batched_over_sequential": ncell * 1000.0 / ms / seq_val},
           "records": {"rows": nrec, "records_per_s": nrec / ((args.warmup + args.steps) * ms * 1e-3)},
           "energies_last_step_cell0": last_e[0, :5].tolist()}
    if kernels_per_step:
      out["host_counted_launches_in_timed_region"] = int(kernels_per_step)
    print(json.dumps(out))
  batch.close()
  if ws > 1:
    dist.destroy_process_group()


def main():
  args = _args()
  from jrystal_gb300 import workloads
  if args.workload == "batch64_trajectories":
    wls = batch_cells()
    if args.impl == "reference":
      run_batch_reference(args, wls)
    else:
      run_batch(args, wls)
    return
  wl = workloads.WORKLOADS[args.workload]()
  if args.kgrid:
    wl.kgrid = tuple(args.kgrid)
    wl.name += "_k" + "x".join(map(str, args.kgrid))
  if args.impl == "reference":
    run_reference(args, wl)
  else:
    run_ours(args, wl)


if __name__ == "__main__":
  main()
