"""Learned diagonal preconditioner of the direct-minimisation optimiser.

An MLP (3-64-64-64-1, GELU, softplus output; BF16 weights, FP32
accumulation) maps per-coefficient features
  x1 = |G+k|^2 / E_kin,band,   x2 = band / num_band,   x3 = step / total_steps
to a positive scale of each Adam update element (no counterpart in jrystal).

Training data are the optimiser's own trajectories: for sampled occupied
coefficients at step t the record holds the features, a = g_t . u_t (the
slope of the step u_t along the gradient) and c = (g_{t+1} - g_t) . u_t
(its secant curvature).  A scale s changes the energy by about
s a + s^2 c / 2 along that coefficient; the network is trained to minimise
the sum of these one-step model changes (each step's records normalised by
their total |a|), i.e. to predict the step-length correction the secant
model asks for.  Both training (forward/backward) and inference run on the
library's kernels; the plain optimiser is the fallback whenever the energy
rises under the learned scaling.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass
from typing import List, Optional

import numpy as np
import torch

from . import _lib
from .engine import PlaneWavePlan, adam_update

NUM_PARAMS = 64 * 3 + 64 + 2 * (64 * 64 + 64) + 64 + 1


def _p(t):
  return None if t is None else ct.c_void_p(t.data_ptr())


def _st():
  return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


class MLP:
  """Parameters of the preconditioner network (FP32 master + BF16 copy)."""

  def __init__(self, seed: int = 3, device=None):
    lib = _lib.load()
    assert lib.jrg_mlp_num_params() == NUM_PARAMS
    self.device = torch.device(device or "cuda")
    rng = np.random.default_rng(seed)
    w = np.zeros(NUM_PARAMS, dtype=np.float32)
    o = 0
    for din, dout in ((3, 64), (64, 64), (64, 64), (64, 1)):
      bound = np.sqrt(6.0 / (din + dout))
      w[o:o + din * dout] = rng.uniform(-bound, bound, din * dout)
      o += din * dout + dout
    w[-1] = 0.5413248546129181        # softplus(b4) = 1: start at the plain update
    self.w32 = torch.tensor(w, device=self.device)
    self.wb = torch.empty(NUM_PARAMS, dtype=torch.bfloat16, device=self.device)
    self.horizon = 300          # total_steps the step feature x3 was trained with
    self.sync()

  def sync(self):
    """Refresh the BF16 copy from the FP32 master."""
    _lib.check(_lib.load().jrg_mlp_to_bf16(_p(self.w32), _p(self.wb), _st()), "jrg_mlp_to_bf16")

  def state_dict(self):
    return {"w32": self.w32.detach().cpu().numpy(), "horizon": np.array(self.horizon)}

  def load_state_dict(self, d):
    self.w32.copy_(torch.as_tensor(d["w32"], device=self.device))
    if "horizon" in d:
      self.horizon = int(np.asarray(d["horizon"]))
    self.sync()

  def save(self, path):
    np.savez(path, **self.state_dict())

  @classmethod
  def load(cls, path, device=None):
    m = cls(device=device)
    m.load_state_dict(dict(np.load(path)))
    return m

  # -- training kernels ----------------------------------------------------
  def _ws(self, n):
    nbytes = ct.c_size_t()
    _lib.check(_lib.load().jrg_mlp_workspace_size(n, ct.byref(nbytes)), "jrg_mlp_workspace_size")
    return torch.empty(int(nbytes.value), dtype=torch.uint8, device=self.device)

  def forward(self, x: torch.Tensor) -> torch.Tensor:
    """Scales of records x[n][3] (training forward path)."""
    x = x.to(self.device, torch.float32).contiguous()
    n = x.shape[0]
    s = torch.empty(n, dtype=torch.float32, device=self.device)
    _lib.check(_lib.load().jrg_mlp_train_eval(n, _p(x), _p(self.w32), _p(self.wb), None, None,
                                              None, _p(s), None, None, _p(self._ws(n)), _st()),
               "jrg_mlp_train_eval")
    return s

  def loss_and_grad(self, x, a, c, w=None, ws=None):
    """Summed loss sum w (s a + s^2 c/2) and d(mean loss)/d params."""
    x = x.contiguous()
    n = x.shape[0]
    loss = torch.zeros(1, dtype=torch.float64, device=self.device)
    grad = torch.empty(NUM_PARAMS, dtype=torch.float32, device=self.device)
    _lib.check(_lib.load().jrg_mlp_train_eval(n, _p(x), _p(self.w32), _p(self.wb), _p(a), _p(c),
                                              _p(w), None, _p(loss), _p(grad),
                                              _p(ws if ws is not None else self._ws(n)), _st()),
               "jrg_mlp_train_eval")
    return loss, grad

  def scale(self, plan: PlaneWavePlan, t_frac: float, occupation: torch.Tensor,
            smax: float = 8.0, out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Tensor-core inference: one scale per parameter element (2,S,K,G,B)."""
    if out is None:
      out = torch.empty((2,) + plan.param_shape, dtype=torch.float32, device=plan.device)
    occ = occupation.to(torch.float64).contiguous()
    _lib.check(_lib.load().jrg_precond_scale(plan._h, _p(self.w32), _p(self.wb), float(t_frac),
                                             float(smax), _p(occ), _p(out), _p(plan.workspace),
                                             _st()), "jrg_precond_scale")
    return out


def train(mlp: MLP, records: dict, steps: int = 2000, lr: float = 1e-3, batch: int = 16384,
          seed: int = 3, log_every: int = 0) -> List[float]:
  """Adam (lr 1e-3) on the MLP parameters with the library's training
  kernels; minibatches drawn with the given seed."""
  x, a, c, w = (records[k] for k in ("x", "a", "c", "w"))
  n = x.shape[0]
  batch = min(batch, n)
  g = torch.Generator(device=mlp.device)
  g.manual_seed(seed)
  m = torch.zeros_like(mlp.w32)
  v = torch.zeros_like(mlp.w32)
  ws = mlp._ws(batch)
  hist = []
  for t in range(1, steps + 1):
    idx = torch.randint(0, n, (batch,), generator=g, device=mlp.device)
    loss, grad = mlp.loss_and_grad(x[idx].contiguous(), a[idx].contiguous(), c[idx].contiguous(),
                                   w[idx].contiguous(), ws)
    adam_update(mlp.w32, grad, m, v, t, lr, 0.9, 0.999, 1e-8)
    mlp.sync()
    if log_every and t % log_every == 0:
      hist.append(float(loss.item()) / batch)
  return hist


def evaluate_loss(mlp: MLP, records: dict) -> float:
  loss, _ = mlp.loss_and_grad(records["x"], records["a"], records["c"], records["w"])
  return float(loss.item()) / records["x"].shape[0]


# weights of the benchmark-cell recipe (precond_train.fit_benchmark_cell: ~1e5
# records of plain runs of the Si8 64^3 cell); precond_si_c_al.npz holds the
# strained-cell recipe's (precond_train.fit)
DEFAULT_WEIGHTS = __import__("os").path.join(__import__("os").path.dirname(__file__), "data",
                                             "precond_si8_cubic_64.npz")


class GuardedScale:
  """scale_fn for calc.Minimizer: learned scales, plain fallback after the
  energy rises above its best value by more than ``rise_tol``.  The step
  feature is step / total_steps (the network's training horizon by default)."""

  def __init__(self, mlp: MLP, total_steps: Optional[int] = None, smax: float = 4.0,
               rise_tol: float = 0.0):
    total_steps = total_steps or mlp.horizon
    self.mlp, self.total, self.smax, self.rise_tol = mlp, total_steps, smax, rise_tol
    self.best = None
    self.fallback_at = None
    self.buf = None

  def observe(self, energy: float, step: int):
    if self.best is None or energy < self.best:
      self.best = energy
    elif self.fallback_at is None and energy > self.best + self.rise_tol:
      self.fallback_at = step

  def _buf(self, mini):
    if self.buf is None:
      self.buf = torch.empty((2,) + mini.plan.param_shape, dtype=torch.float32,
                             device=mini.plan.device)
    return self.buf

  def __call__(self, mini):
    if self.fallback_at is not None:
      return None
    return self.mlp.scale(mini.plan, min(1.0, mini.t / self.total), mini.occ, self.smax,
                          self._buf(mini))

  def in_step(self, mini):
    """(mlp, step fraction, cap, scale buffer) for the fused device step, or
    None after the fallback to the plain update."""
    if self.fallback_at is not None:
      return None
    return self.mlp, min(1.0, mini.t / self.total), self.smax, self._buf(mini)


@dataclass
class RecordSpec:
  per_step: int = 400       # sampled occupied coefficients per step
  c_floor: float = 0.25     # secant curvature floor relative to |a| (target scale <= 4)


def collect_records(plan: PlaneWavePlan, occupation, params: torch.Tensor, steps: int, lr: float,
                    spec: RecordSpec = RecordSpec(), seed: int = 0, scale_fn=None,
                    b1: float = 0.9, b2: float = 0.99) -> dict:
  """Runs the optimiser for ``steps`` steps (plain, or with ``scale_fn``) and
  returns training records {x[n][3], a[n], c[n], w[n]} on the device."""
  from .calc import Minimizer
  mini = Minimizer(plan, occupation, params.clone(), lr=lr, b1=b1, b2=b2, scale_fn=scale_fn,
                   total_steps=steps)
  occ = mini.occ
  S, K, G, B = plan.param_shape
  occ_flat = occ.reshape(-1)
  occupied = torch.nonzero(occ_flat > 0, as_tuple=False).reshape(-1)     # (s k b) bands
  tk = torch.empty(K * G, dtype=torch.float64, device=plan.device)
  _lib.check(_lib.load().jrg_kinetic_table(plan._h, _p(tk), _st()), "jrg_kinetic_table")
  ekin = torch.empty(S * K * B, dtype=torch.float64, device=plan.device)
  gen = torch.Generator(device=plan.device)
  gen.manual_seed(seed)
  xs, As, Cs, Ws = [], [], [], []
  prev = None
  for t in range(steps):
    before = mini.params.clone()
    mini.energy_and_grad()
    _lib.check(_lib.load().jrg_band_kinetic(plan._h, _p(plan.workspace), _p(ekin), _st()),
               "jrg_band_kinetic")
    g_now = mini.grads
    if prev is not None:
      idx, x, u, g_prev, s_prev = prev
      gv = g_now.reshape(2, -1)[:, idx]
      # one-step model of the applied (already scaled) step u = s_prev u_adam,
      # rewritten for the absolute scale sigma of u_adam: a/s_prev, c/s_prev^2
      a = (g_prev * u).sum(0)
      c = ((gv - g_prev) * u).sum(0)
      c = torch.maximum(c, spec.c_floor * a.abs())
      a = a / s_prev
      c = c / (s_prev * s_prev)
      keep = a.abs() > 0
      wts = torch.zeros_like(a)
      tot = a.abs().sum()
      if tot > 0:
        wts = torch.full_like(a, 1.0) / tot * keep.sum()
      xs.append(x); As.append(a.float()); Cs.append(c.float()); Ws.append(wts.float())
    # sample occupied coefficients for this step's record
    band = occupied[torch.randint(0, occupied.numel(), (spec.per_step,), generator=gen,
                                  device=plan.device)]
    sk, b = band // B, band % B
    gi = torch.randint(0, G, (spec.per_step,), generator=gen, device=plan.device)
    k = sk % K
    idx = (sk * G + gi) * B + b
    x = torch.stack([(tk[k * G + gi] / ekin[band]).float(), (b.float() / B),
                     torch.full_like(b, t, dtype=torch.float32) / steps], dim=1)
    g_t = g_now.reshape(2, -1)[:, idx].clone()
    mini.t += 1
    scale = mini.scale_fn(mini) if mini.scale_fn is not None else None
    adam_update(mini.params, mini.grads, mini.m, mini.v, mini.t, mini.lr, mini.b1, mini.b2,
                mini.eps, scale=scale)
    u = (mini.params - before).reshape(2, -1)[:, idx]
    s_prev = scale.reshape(2, -1)[0, idx].double() if scale is not None else torch.ones_like(u[0])
    prev = (idx, x, u, g_t, s_prev)
  return {"x": torch.cat(xs), "a": torch.cat(As), "c": torch.cat(Cs), "w": torch.cat(Ws)}


def time_below(history: np.ndarray, e_max: float) -> Optional[int]:
  """First step after which E < e_max for the rest of the run (None if never)."""
  bad = np.nonzero(np.asarray(history) >= e_max)[0]
  if len(bad) == 0:
    return 0
  if bad[-1] == len(history) - 1:
    return None
  return int(bad[-1] + 1)


def time_to_tolerance(history: np.ndarray, e_ref: float, tol: float) -> Optional[int]:
  """First step after which |E - e_ref| stays below tol (None if never)."""
  bad = np.nonzero(np.abs(np.asarray(history) - e_ref) >= tol)[0]
  if len(bad) == 0:
    return 0
  if bad[-1] == len(history) - 1:
    return None
  return int(bad[-1] + 1)
