"""Batched trajectory generation: plain Adam on many independent cells at once.

jrystal runs one cell per driver loop
(calc/calc_ground_state_energy_all_electrons.py:205-220).  The learned
preconditioner's training set needs a few hundred plain Adam steps on dozens
of small strained cells (grids 24^3-48^3, 8-16 bands); one such cell leaves
most of the GPU idle.  :class:`TrajectoryBatch` hands all of them to the C ABI
batch (``jrg_batch_*``): each cell's step (energy and gradient, the record
kernel, Adam) runs on its own stream branch, one CUDA graph launch per step
of every cell, and the one-step secant records are drawn on the device.
Every cell's trajectory equals the single-cell loop of ``calc.Minimizer``
with ``fused=False`` (the kernels are deterministic).
"""
from __future__ import annotations

import ctypes as ct
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib
from .engine import PlaneWavePlan, _stream


def _plan(wl, device=None):
  return PlaneWavePlan(wl.cell, wl.positions, wl.charges, wl.grid_sizes, wl.mask, wl.kpts,
                       wl.num_band, 1, wl.precision, wl.xc, device=device)


class TrajectoryBatch:
  """``steps`` plain Adam steps on every workload in ``workloads``.

  params: optional list of (2, 1, K, G, B) starting parameters (default: each
  workload's ``init_params``).  per_step: records drawn per step and cell (0
  for none).  energies: (steps, cells, 8) float64 on the device after
  :meth:`run`; records(): {x[n][3], a[n], c[n], w[n]} in cell-major, step,
  draw order; record_index(): the flat [S][K][G][B] element of each draw."""

  def __init__(self, workloads: Sequence, steps: int, lr: float = 1e-2, b1: float = 0.9,
               b2: float = 0.99, eps: float = 1e-8, per_step: int = 6, seed: int = 2,
               c_floor: float = 0.25, params: Optional[list] = None, device=None):
    self.lib = _lib.load()
    self.workloads = list(workloads)
    self.steps = int(steps)
    self.per_step = int(per_step)
    self.plans = [_plan(wl, device) for wl in self.workloads]
    dev = self.plans[0].device
    self.device = dev
    self.params, self.m, self.v, self.grads, self.occ = [], [], [], [], []
    for i, (wl, plan) in enumerate(zip(self.workloads, self.plans)):
      if params is not None:
        p = params[i].to(device=dev, dtype=plan.rdtype).contiguous().clone()
      else:
        wr, wi = wl.init_params()
        p = torch.tensor(np.stack([wr, wi]), dtype=plan.rdtype, device=dev)
      if tuple(p.shape) != (2,) + plan.param_shape:
        raise ValueError(f"params[{i}] shape {tuple(p.shape)} != {(2,) + plan.param_shape}")
      self.params.append(p)
      self.m.append(torch.zeros_like(p))
      self.v.append(torch.zeros_like(p))
      self.grads.append(torch.zeros_like(p))
      self.occ.append(torch.as_tensor(np.asarray(wl.occupation).reshape(-1), dtype=torch.float64,
                                      device=dev).contiguous())
    n = len(self.plans)
    self.energies = torch.zeros(self.steps, n, 8, dtype=torch.float64, device=dev)
    rows = max(self.steps - 1, 0) * self.per_step
    self.rec_x = torch.zeros(n, rows, 3, dtype=torch.float32, device=dev)
    self.rec_a = torch.zeros(n, rows, dtype=torch.float32, device=dev)
    self.rec_c = torch.zeros(n, rows, dtype=torch.float32, device=dev)
    self.rec_w = torch.zeros(n, rows, dtype=torch.float32, device=dev)
    self.rec_idx = torch.zeros(n, rows, dtype=torch.int64, device=dev)
    arr = lambda xs: (ct.c_void_p * n)(*[ct.c_void_p(x) for x in xs])
    self._keep = dict(
      plans=arr([p._h.value for p in self.plans]),
      ws=arr([p.workspace.data_ptr() for p in self.plans]),
      params=arr([t.data_ptr() for t in self.params]),
      m=arr([t.data_ptr() for t in self.m]),
      v=arr([t.data_ptr() for t in self.v]),
      grads=arr([t.data_ptr() for t in self.grads]),
      occ=arr([t.data_ptr() for t in self.occ]))
    d = _lib.BatchDesc()
    d.num_cells = n
    d.plans = ct.cast(self._keep["plans"], ct.POINTER(ct.c_void_p))
    d.workspaces = ct.cast(self._keep["ws"], ct.POINTER(ct.c_void_p))
    d.params = ct.cast(self._keep["params"], ct.POINTER(ct.c_void_p))
    d.m = ct.cast(self._keep["m"], ct.POINTER(ct.c_void_p))
    d.v = ct.cast(self._keep["v"], ct.POINTER(ct.c_void_p))
    d.grads = ct.cast(self._keep["grads"], ct.POINTER(ct.c_void_p))
    d.occupations = ct.cast(self._keep["occ"], ct.POINTER(ct.c_void_p))
    d.steps = self.steps
    d.lr, d.b1, d.b2, d.eps = float(lr), float(b1), float(b2), float(eps)
    d.energies = self.energies.data_ptr()
    d.per_step = self.per_step
    d.seed = int(seed) & (2**64 - 1)
    d.c_floor = float(c_floor)
    if self.per_step > 0 and rows > 0:
      d.rec_x, d.rec_a = self.rec_x.data_ptr(), self.rec_a.data_ptr()
      d.rec_c, d.rec_w = self.rec_c.data_ptr(), self.rec_w.data_ptr()
      d.rec_idx = self.rec_idx.data_ptr()
    elif self.per_step > 0:
      d.per_step = 0
    torch.cuda.synchronize(dev)
    h = ct.c_void_p()
    _lib.check(self.lib.jrg_batch_create(ct.byref(d), ct.byref(h)), "jrg_batch_create")
    self._h = h

  @property
  def steps_done(self) -> int:
    n = ct.c_int()
    _lib.check(self.lib.jrg_batch_steps_done(self._h, ct.byref(n)), "jrg_batch_steps_done")
    return int(n.value)

  def step(self, graph: bool = True):
    """One Adam step of every cell on torch's current stream."""
    _lib.check(self.lib.jrg_batch_step(self._h, 1 if graph else 0, _stream()), "jrg_batch_step")

  def run(self, nsteps: Optional[int] = None, graph: bool = True):
    """The remaining steps (or ``nsteps`` of them)."""
    left = self.steps - self.steps_done
    for _ in range(left if nsteps is None else min(int(nsteps), left)):
      self.step(graph)

  def records(self) -> dict:
    return {"x": self.rec_x.reshape(-1, 3), "a": self.rec_a.reshape(-1),
            "c": self.rec_c.reshape(-1), "w": self.rec_w.reshape(-1)}

  def record_index(self) -> torch.Tensor:
    return self.rec_idx

  def close(self):
    if getattr(self, "_h", None) is not None and self._h.value:
      _lib.check(self.lib.jrg_batch_destroy(self._h), "jrg_batch_destroy")
      self._h = None
    for p in self.plans:
      p.close()
    self.plans = []

  def __del__(self):
    try:
      self.close()
    except Exception:
      pass
