"""Direct-minimisation driver: jrystal's ground-state loop
(calc/calc_ground_state_energy_all_electrons.py:63-247) on the fused GPU path.

Each step runs the orthonormalisation, energy and hand-written gradient
(jrg_energy_grad) and the Adam update (jrg_adam_update) on the device; the
host reads back the energy for the windowed convergence check
(calc/convergence.py:13-35), as the reference does after every update.
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np
import torch

from . import grid as _grid
from .crystal import Crystal
from .engine import PlaneWavePlan, adam_update

DEFAULT_CONFIG = {
  "crystal": None,
  "crystal_file_path_path": None,
  "spin": 0,
  "xc": "lda_x+lda_c_vwn",
  "freq_mask_method": "spherical",
  "cutoff_energy": 40.0,
  "grid_sizes": 16,
  "k_grid_sizes": [1, 1, 1],
  "occupation": "uniform",
  "smearing": 0.0,
  "empty_bands": 0,
  "spin_restricted": True,
  "ewald_args": {"ewald_eta": 0.1, "ewald_cutoff": 2.0e4},
  "epoch": 1000,
  "optimizer": "adam",
  "optimizer_args": {"learning_rate": 0.01, "b1": 0.9, "b2": 0.99},
  "convergence_window_size": 20,
  "convergence_condition": 1e-6,
  "seed": 123,
  "jax_enable_x64": True,
  "verbose": False,
  "use_pseudopotential": False,
  "pseudopotential_type": "nc",
  "pseudopotential_file_dir": None,
}


class ConvergenceChecker:
  """Standard deviation of the last ``window_size`` energies below the
  threshold (calc/convergence.py:13-35)."""

  def __init__(self, window_size: int = 20, threshold: float = 1e-5):
    self.window_size = window_size
    self.threshold = threshold
    self.history: List[float] = []

  def check(self, value: float) -> bool:
    self.history.append(float(value))
    if len(self.history) > self.window_size:
      self.history.pop(0)
    if len(self.history) < self.window_size:
      return False
    return bool(np.std(self.history) < self.threshold)

  def reset(self):
    self.history = []


class Minimizer:
  """Adam on the raw plane-wave parameters with the fused device step.

  params: tensor (2, S, K, G, B) holding w_re and w_im.  ``scale_fn``, when
  given, is called as scale_fn(minimizer) before each update and returns a
  float32 tensor of one positive scale per parameter element (the learned
  diagonal preconditioner) or None for the plain update.  A scale_fn with an
  ``in_step(minimizer)`` method (precond.GuardedScale) instead hands the
  network to the device step, which evaluates it between the kinetic and the
  density phases.  With ``fused`` (the default where supported: more than
  32 bands with the default contraction kernels) each step is one
  jrg_energy_grad_adam call: with
  the two-stream k-point pipeline each half of the k-points takes its Adam
  step as soon as its gradient is done (1.951 vs 1.963 ms per step for the
  two-call path on the 64^3 Si8 cell); ``grads`` is only filled when
  ``keep_grad`` is set."""

  def __init__(self, plan: PlaneWavePlan, occupation, params: torch.Tensor, lr: float = 1e-2,
               b1: float = 0.9, b2: float = 0.99, eps: float = 1e-8, scale_fn=None,
               total_steps: Optional[int] = None, fused: bool = True,
               keep_grad: bool = False):
    self.plan = plan
    self.occ = torch.as_tensor(np.asarray(occupation), dtype=torch.float64, device=plan.device)
    if tuple(params.shape) != (2,) + plan.param_shape:
      raise ValueError(f"params shape {tuple(params.shape)} != {(2,) + plan.param_shape}")
    self.params = params.contiguous()
    self.grads = torch.empty_like(self.params)
    self.m = torch.zeros_like(self.params)
    self.v = torch.zeros_like(self.params)
    self.lr, self.b1, self.b2, self.eps = lr, b1, b2, eps
    self.t = 0
    self.total_steps = total_steps
    self.scale_fn = scale_fn
    self.last_scale = None
    supported = plan.num_band <= 32 or plan.lib.jrg_tensor_core_paths(-1) == 0
    self.fused = fused and supported
    self.keep_grad = keep_grad
    self.recoveries = 0

  def energy_and_grad(self):
    e, _, _ = self.plan.energy_and_grad(self.params[0], self.params[1], self.occ, self.grads[0],
                                        self.grads[1])
    return e

  def recover(self):
    """Re-orthonormalise the parameters (same subspace, same column norms)
    and restart Adam from them: the response to a Cholesky breakdown or a
    large Gram condition estimate (the step applies no update when it reports
    a breakdown, so the parameters are those before it)."""
    self.plan.reorthonormalise(self.params[0], self.params[1])
    self.m.zero_()
    self.v.zero_()
    self.t = 0
    self.recoveries += 1

  def checked_step(self) -> torch.Tensor:
    """step(), then the host check of its status (the energies are read back
    every step, as the reference does): on a breakdown, non-finite energies
    or a condition estimate above the plan's limit the parameters are
    re-orthonormalised and the step is taken again; a second failure raises
    NumericalError."""
    e = self.step()
    if not self.plan.needs_reorthonormalisation(e):
      return e
    self.recover()
    e = self.step()
    self.plan.check_numerics(e, "step after re-orthonormalisation")
    return e

  def step(self) -> torch.Tensor:
    """One update; returns the device energy vector of the parameters before it."""
    in_step = getattr(self.scale_fn, "in_step", None)
    if self.fused and (self.scale_fn is None or in_step is not None):
      self.t += 1
      spec = in_step(self) if in_step is not None else None
      kw = {} if spec is None else dict(mlp=spec[0], t_frac=spec[1], smax=spec[2], scale=spec[3])
      self.last_scale = None if spec is None else spec[3]
      return self.plan.energy_grad_adam(self.params, self.m, self.v, self.occ, self.t, self.lr,
                                        self.b1, self.b2, self.eps,
                                        grad=self.grads if self.keep_grad else None, **kw)
    e = self.energy_and_grad()
    if self.plan.status_of(e)["flags"] & 1:
      return e   # a Cholesky breakdown: no update from this gradient (as the fused step)
    self.t += 1
    scale = self.scale_fn(self) if self.scale_fn is not None else None
    self.last_scale = scale
    adam_update(self.params, self.grads, self.m, self.v, self.t, self.lr, self.b1, self.b2,
                self.eps, scale=scale)
    return e

  def energy(self) -> float:
    e, _, _ = self.plan.energy_and_grad(self.params[0], self.params[1], self.occ, with_grad=False)
    return float(e[4].item())


@dataclass
class GroundStateEnergyOutput:
  config: dict
  crystal: Crystal
  params_pw: dict
  total_energy: float
  total_energy_history: List[float]
  energy_terms: dict = field(default_factory=dict)
  ewald: float = 0.0
  steps: int = 0
  converged: bool = False
  train_time: float = 0.0
  density_grid: Optional[torch.Tensor] = None
  occupation: Optional[torch.Tensor] = None


def _merge(config):
  cfg = dict(DEFAULT_CONFIG)
  cfg.update(config or {})
  return cfg


def create_crystal(cfg) -> Crystal:
  if isinstance(cfg.get("crystal"), Crystal):
    return cfg["crystal"]
  path = cfg.get("crystal_file_path_path")
  if cfg.get("crystal") is not None and path is None:
    raise ValueError("pass the geometry as a Crystal object or through crystal_file_path_path")
  return Crystal.create_from_file(path, spin=cfg.get("spin"))


def create_pseudopotential(cfg, crystal):
  """NormConservingPseudopotential of the crystal's atoms from the UPF files
  in ``pseudopotential_file_dir`` (calc/opt_utils.py:117-140); jrystal's
  bundled files are not shipped, so the directory is required."""
  from .pseudopotential import NormConservingPseudopotential
  kind = cfg.get("pseudopotential_type", "nc")
  if kind not in ("normcons", "normconserving", "nc"):
    if kind in ("ultrasoft", "us"):
      raise NotImplementedError("ultrasoft pseudopotentials are not implemented")
    raise ValueError(f"Pseudopotential type {kind} is not supported.")
  d = cfg.get("pseudopotential_file_dir")
  if d is None:
    raise ValueError("pseudopotential_file_dir must name the directory of the UPF files")
  return NormConservingPseudopotential.create(crystal, d)


@dataclass
class _Setup:
  crystal: Crystal
  pseudo: object          # NormConservingPseudopotential or None (all-electron)
  precision: int
  grid_sizes: tuple
  kpts: np.ndarray
  mask: np.ndarray
  nelec: int              # valence electrons with a pseudopotential
  num_bands: int


def _setup(cfg, pseudo: bool) -> _Setup:
  crystal = create_crystal(cfg)
  precision = 64 if cfg["jax_enable_x64"] else 32
  grid_sizes = tuple(int(g) for g in _grid.proper_grid_size(cfg["grid_sizes"]))
  k_grid = tuple(int(k) for k in np.broadcast_to(cfg["k_grid_sizes"], 3))
  kpts = _grid.k_vectors(crystal.cell_vectors, k_grid)
  if cfg["freq_mask_method"] == "spherical":
    mask = _grid.spherical_mask(crystal.cell_vectors, grid_sizes, cfg["cutoff_energy"])
  elif cfg["freq_mask_method"] == "cubic":
    mask = _grid.cubic_mask(grid_sizes)
  else:
    raise ValueError("freq_mask_method must be either cubic or spherical.")
  pp = create_pseudopotential(cfg, crystal) if pseudo else None
  nelec = int(sum(pp.valence_charges)) if pp is not None else int(crystal.num_electron)
  num_bands = math.ceil(nelec / 2) + cfg["empty_bands"]
  return _Setup(crystal, pp, precision, grid_sizes, kpts, mask, nelec, num_bands)


def attach_pseudopotential(plan: PlaneWavePlan, pp, kmax: Optional[float] = None):
  """Local V_loc(G) and beta-projector tables of ``pp`` on ``plan``
  (calc/calc_ground_state_energy_normcons.py:115-153): built on the host as
  the reference builds them, consumed by the device kernels."""
  from .pseudopotential import local, nloc
  g = _grid.g_vectors(plan.cell, plan.grid)
  vloc = local.potential_local_reciprocal(plan.positions, g, pp.r_grid, pp.local_potential_grid,
                                          pp.local_potential_charge, plan.vol)
  table = nloc.projector_table(plan.positions, g, plan.kpts, plan.mask, pp.r_grid,
                               pp.nonlocal_beta_grid, pp.nonlocal_angular_momentum,
                               pp.nonlocal_d_matrix, kmax=kmax)
  plan.set_pseudopotential(vloc, table)
  return plan


def _num_spin(cfg) -> int:
  """1 spin channel (restricted) or 2; the polarised path is LDA only."""
  if cfg["spin_restricted"]:
    return 1
  if "gga" in cfg["xc"]:
    raise NotImplementedError("spin-polarised PBE is not implemented")
  return 2


def _make_plan(su: _Setup, cfg, kpts=None, num_bands=None, kmax=None, num_spin=1) -> PlaneWavePlan:
  c = su.crystal
  plan = PlaneWavePlan(c.cell_vectors, c.positions, c.charges, su.grid_sizes, su.mask,
                       su.kpts if kpts is None else kpts, num_bands or su.num_bands, num_spin,
                       su.precision, cfg["xc"])
  if su.pseudo is not None:
    attach_pseudopotential(plan, su.pseudo, kmax=kmax)
  return plan


def _energy_terms_dict(e, pseudo: bool):
  terms = dict(kinetic=e[0], external=e[1], hartree=e[2], xc=e[3], total=e[4])
  if pseudo:
    terms.update(external_local=e[1] - e[7], external_nonlocal=e[7])
  return terms


def energy_all_electrons(config: dict) -> GroundStateEnergyOutput:
  """All-electron ground state by direct minimisation with fixed occupations
  (calc/calc_ground_state_energy_all_electrons.py:63-247)."""
  return _ground_state(_merge(config), pseudo=False)


def energy_normcons(config: dict) -> GroundStateEnergyOutput:
  """Ground state with norm-conserving pseudopotentials
  (calc/calc_ground_state_energy_normcons.py:68-308): valence electrons only,
  the local table in place of the Coulomb external potential, the nonlocal
  beta-projector energy added to the loss (energy_terms carries
  external_local and external_nonlocal).  The Ewald constant uses the
  crystal's nuclear charges, as the reference's get_ewald_coulomb_repulsion
  does (calc/opt_utils.py:186-200)."""
  return _ground_state(_merge(config), pseudo=True)


def _ground_state(cfg, pseudo: bool) -> GroundStateEnergyOutput:
  if cfg["optimizer"] != "adam":
    raise NotImplementedError("only the adam optimiser is implemented on the device")
  if cfg["occupation"] in ("simplex-projector", "idempotent"):
    return _energy_learnable_occupation(cfg, pseudo)
  if cfg["occupation"] not in ("uniform", "gamma"):
    raise ValueError(f"Invalid method: {cfg['occupation']}")
  ns = _num_spin(cfg)
  su = _setup(cfg, pseudo)
  crystal, kpts, mask, nelec = su.crystal, su.kpts, su.mask, su.nelec
  num_bands = su.num_bands
  K = kpts.shape[0]
  if cfg["occupation"] == "uniform":
    occ = np.zeros((2, K, num_bands))
    occ[0, :, :(nelec + crystal.spin) // 2] = 1 / K
    occ[1, :, :(nelec - crystal.spin) // 2] = 1 / K
  else:
    occ = np.zeros((2, K, num_bands))
    occ[0, 0, :(nelec + crystal.spin) // 2] = 1
    occ[1, 0, :(nelec - crystal.spin) // 2] = 1
  if ns == 1:
    occ = occ.sum(0, keepdims=True)
  if "occupation_array" in cfg:
    occ = np.asarray(cfg["occupation_array"], dtype=np.float64)
    num_bands = occ.shape[-1]
  plan = _make_plan(su, cfg, num_bands=num_bands, num_spin=ns)
  ew = plan.ewald(cfg["ewald_args"]["ewald_eta"], cfg["ewald_args"]["ewald_cutoff"])
  ng = int(mask.sum())
  gen = torch.Generator(device=plan.device)
  gen.manual_seed(int(cfg["seed"]))
  if "init_params" in cfg:
    w_re, w_im = cfg["init_params"]
    params = torch.tensor(np.stack([w_re, w_im]), dtype=plan.rdtype, device=plan.device)
  else:
    params = torch.rand((2, ns, K, ng, num_bands), generator=gen, device=plan.device,
                        dtype=plan.rdtype)
  oa = cfg["optimizer_args"]
  mini = Minimizer(plan, occ, params, lr=oa.get("learning_rate", 1e-2), b1=oa.get("b1", 0.9),
                   b2=oa.get("b2", 0.999), eps=oa.get("eps", 1e-8),
                   scale_fn=cfg.get("scale_fn"), total_steps=cfg["epoch"])
  checker = ConvergenceChecker(cfg["convergence_window_size"], cfg["convergence_condition"])
  history, converged, train_time = [], False, 0.0
  i = 0
  for i in range(cfg["epoch"]):
    t0 = time.perf_counter()
    e = mini.checked_step()
    etot = float(e[4].item())          # the reference blocks on the energy every step
    train_time += time.perf_counter() - t0
    history.append(etot)
    if checker.check(etot):
      converged = True
      break
  e, _, _ = plan.energy_and_grad(mini.params[0], mini.params[1], mini.occ, with_grad=False)
  e = e.cpu().numpy()
  terms = _energy_terms_dict(e, pseudo)
  rho = plan.density(plan.coeff(mini.params[0], mini.params[1]), mini.occ)
  return GroundStateEnergyOutput(config=cfg, crystal=crystal,
                                 params_pw={"w_re": mini.params[0], "w_im": mini.params[1]},
                                 total_energy=float(e[4] + ew), total_energy_history=history,
                                 energy_terms=terms, ewald=ew, steps=i + 1, converged=converged,
                                 train_time=train_time, density_grid=rho)


def temperature_schedule(cfg):
  """Smearing temperature of step i (calc/…all_electrons.py:193-203):
  optax.exponential_decay(100, epoch // 2, smearing / 100, end_value=smearing),
  i.e. 100 (smearing/100)^(i / (epoch//2)) clipped below at smearing; 0
  without smearing."""
  sm = float(cfg.get("smearing", 0.0))
  if sm <= 0.0:
    return lambda i: 0.0
  steps = max(1, int(cfg["epoch"]) // 2)
  rate = sm / 100.0
  return lambda i: max(sm, 100.0 * rate ** (i / steps))


def _energy_learnable_occupation(cfg, pseudo: bool = False) -> GroundStateEnergyOutput:
  """Free-energy minimisation F = E - T S over the plane-wave parameters and
  learnable occupations (simplex projector or idempotent), the reference
  driver's path for metals (calc/calc_ground_state_energy_all_electrons.py:
  103-147 and 150-220; calc_ground_state_energy_normcons.py:155-257): the
  device returns E, dE/dW and the band energies dE/df
  (jrg_energy_grad_bands); dF/d(occupation parameters) follows by torch
  autograd through the occupation map and the Fermi-Dirac entropy; both
  parameter sets take Adam steps with the same hyper-parameters."""
  from . import entropy as _entropy
  from . import occupation as _occupation
  ns = _num_spin(cfg)
  restricted = ns == 1
  su = _setup(cfg, pseudo)
  crystal, kpts, mask, nelec, num_bands = su.crystal, su.kpts, su.mask, su.nelec, su.num_bands
  K = kpts.shape[0]
  plan = _make_plan(su, cfg, num_spin=ns)
  ew = plan.ewald(cfg["ewald_args"]["ewald_eta"], cfg["ewald_args"]["ewald_cutoff"])
  ng = int(mask.sum())
  gen = torch.Generator(device=plan.device)
  gen.manual_seed(int(cfg["seed"]))
  if "init_params" in cfg:
    w_re, w_im = cfg["init_params"]
    params = torch.tensor(np.stack([w_re, w_im]), dtype=plan.rdtype, device=plan.device)
  else:
    params = torch.rand((2, ns, K, ng, num_bands), generator=gen, device=plan.device,
                        dtype=plan.rdtype)
  method = cfg["occupation"]
  spin = int(crystal.spin)
  if method == "idempotent":
    occ_params = _occupation.idempotent_param_init(gen, num_bands, nelec, K, spin, restricted)
    leaves = [occ_params["param_up"]["w_re"]]
    if occ_params["param_down"] is not occ_params["param_up"]:
      leaves.append(occ_params["param_down"]["w_re"])
  else:
    occ_params = _occupation.simplex_projector_init(num_bands, K, device=plan.device)
    leaves = [occ_params["param_up"], occ_params["param_down"]]
  for t in leaves:
    t.requires_grad_(True)

  def occ_of():
    return _occupation.occupation(occ_params, K, nelec, spin, method, restricted)

  oa = cfg["optimizer_args"]
  lr, b1, b2, eps = (oa.get("learning_rate", 1e-2), oa.get("b1", 0.9), oa.get("b2", 0.999),
                     oa.get("eps", 1e-8))
  grads = torch.empty_like(params)
  m, v = torch.zeros_like(params), torch.zeros_like(params)
  om = [torch.zeros_like(t) for t in leaves]
  ov = [torch.zeros_like(t) for t in leaves]
  temp_of = temperature_schedule(cfg)
  checker = ConvergenceChecker(cfg["convergence_window_size"], cfg["convergence_condition"])
  history, converged, train_time = [], False, 0.0
  ent_eps = float(cfg.get("eps", 1e-8))
  i = 0
  for i in range(cfg["epoch"]):
    t0 = time.perf_counter()
    temp = temp_of(i)
    occ = occ_of()
    e, _, _, band_e = plan.energy_grad_bands(params[0], params[1], occ.detach(), grads[0], grads[1])
    ent = _entropy.fermi_dirac(occ, eps=ent_eps)
    # dF/dtheta = sum_b (dE/df_b) df_b/dtheta - T dS/dtheta
    surrogate = (occ * band_e).sum() - temp * ent
    og = torch.autograd.grad(surrogate, leaves)
    adam_update(params, grads, m, v, i + 1, lr, b1, b2, eps)
    with torch.no_grad():
      for t, g, mm, vv in zip(leaves, og, om, ov):
        adam_update(t.data, g.contiguous(), mm, vv, i + 1, lr, b1, b2, eps)
    etot = float(e[4].item())
    train_time += time.perf_counter() - t0
    history.append(etot)
    if checker.check(etot):
      converged = True
      break
  with torch.no_grad():
    occ = occ_of().detach()
  e, _, _ = plan.energy_and_grad(params[0], params[1], occ, with_grad=False)
  e = e.cpu().numpy()
  terms = _energy_terms_dict(e, pseudo)
  terms.update(entropy=float(_entropy.fermi_dirac(occ, eps=ent_eps)), temperature=temp_of(i))
  rho = plan.density(plan.coeff(params[0], params[1]), occ)
  return GroundStateEnergyOutput(config=cfg, crystal=crystal,
                                 params_pw={"w_re": params[0], "w_im": params[1]},
                                 total_energy=float(e[4] + ew), total_energy_history=history,
                                 energy_terms=terms, ewald=ew, steps=i + 1, converged=converged,
                                 train_time=train_time, density_grid=rho, occupation=occ)


@dataclass
class BandStructureOutput:
  config: dict
  crystal: Crystal
  k_path: np.ndarray                 # (num_kpoints, 3) Cartesian, 1/bohr
  eigenvalues: np.ndarray            # (spin, num_kpoints, bands), hartree
  ground_state: GroundStateEnergyOutput
  band_trace: float = 0.0
  train_time: float = 0.0
  effective_potential: Optional[torch.Tensor] = None   # V_H + V_ext + v_xc (nx, ny, nz), or (S, ...) for S = 2


BAND_DEFAULTS = {
  "k_path_special_points": None,
  "num_kpoints": 60,
  "band_structure_empty_bands": None,
  "band_structure_epoch": 1000,
  "k_path_fine_tuning": True,
  "k_path_fine_tuning_epoch": 400,
  "save_path": None,
}


def _band_minimise(plan, v_eff, params, m, v, steps, lr, b1, b2, eps, t0=0):
  """Adam on the band trace of a fixed potential; no host synchronisation."""
  grads = torch.empty_like(params)
  for t in range(t0 + 1, t0 + steps + 1):
    plan.band_trace_grad(params[0], params[1], v_eff, grad_re=grads[0], grad_im=grads[1])
    adam_update(params, grads, m, v, t, lr, b1, b2, eps)
  return t0 + steps


def band_structure_all_electrons(config: dict) -> BandStructureOutput:
  """Kohn-Sham band structure along a k path
  (calc/calc_band_structure_all_electrons.py:37-209): the ground state of the
  same config gives the density and V_eff = V_H + V_ext + v_xc; the band
  trace sum_b <psi_b|T + V_eff|psi_b> is minimised with Adam, first at the
  path's first k-point (``band_structure_epoch`` steps), then at all other
  k-points at once starting from those parameters and moments
  (``k_path_fine_tuning_epoch`` steps; jrystal walks the path one k-point
  at a time, each starting from the previous one); the eigenvalues of the
  band Hamiltonian H_ij = <psi_i|H|psi_j> at each k-point are returned as
  (spin, k, band)."""
  return _band_structure(config, pseudo=False)


def band_structure_normcons(config: dict) -> BandStructureOutput:
  """Band structure with norm-conserving pseudopotentials
  (calc/calc_band_structure_normcons.py:68-299): as the all-electron driver,
  with v_eff = V_H + v_loc + v_xc of the ground-state density and the
  nonlocal projector term in the band trace and band Hamiltonian
  (nloc.hamiltonian_trace / hamiltonian_matrix); the beta transforms use the
  largest |G+k| over the whole k path, as the reference's pre-computation
  over the path does."""
  return _band_structure(config, pseudo=True)


def _band_structure(config: dict, pseudo: bool) -> BandStructureOutput:
  from .band import get_k_path
  from .pseudopotential.beta import max_gk_radius
  cfg = dict(BAND_DEFAULTS)
  cfg.update(_merge(config))
  ns = _num_spin(cfg)
  gs = _ground_state(cfg, pseudo)
  su = _setup(cfg, pseudo)
  crystal, mask = su.crystal, su.mask
  k_path = get_k_path(crystal.cell_vectors, cfg["k_path_special_points"], int(cfg["num_kpoints"]))
  extra = cfg["band_structure_empty_bands"]
  num_bands = math.ceil(su.nelec / 2) + (int(extra) if extra is not None else 0)
  oa = cfg["optimizer_args"]
  lr, b1, b2, eps = (oa.get("learning_rate", 1e-2), oa.get("b1", 0.9), oa.get("b2", 0.999),
                     oa.get("eps", 1e-8))
  kmax = max_gk_radius(_grid.g_vectors(crystal.cell_vectors, su.grid_sizes), k_path) if pseudo else None

  def make_plan(kpts):
    return _make_plan(su, cfg, kpts=kpts, num_bands=num_bands, kmax=kmax, num_spin=ns)

  t_start = time.perf_counter()
  plan0 = make_plan(k_path[:1])
  parts = plan0.potential(gs.density_grid, kohn_sham=True)   # V_H, V_ext, v_xc per spin
  v_eff = (parts[0] + parts[1] + parts[2:]).contiguous()     # (S, x, y, z)
  if ns == 1:
    v_eff = v_eff[0]
  gen = torch.Generator(device=plan0.device)
  gen.manual_seed(int(cfg["seed"]))
  ng = int(mask.sum())
  p0 = torch.rand((2, ns, 1, ng, num_bands), generator=gen, device=plan0.device,
                  dtype=plan0.rdtype)
  m0, v0 = torch.zeros_like(p0), torch.zeros_like(p0)
  t = _band_minimise(plan0, v_eff, p0, m0, v0, int(cfg["band_structure_epoch"]), lr, b1, b2, eps)
  out0, _, _, h0 = plan0.band_trace_grad(p0[0], p0[1], v_eff, with_grad=False, hmat=True)
  hs, trace = [h0], float(out0[0])
  plan0.close()
  nk = k_path.shape[0]
  if nk > 1:
    plan1 = make_plan(k_path[1:])
    rep = lambda x: x.expand(2, ns, nk - 1, ng, num_bands).contiguous()
    if cfg["k_path_fine_tuning"]:
      p1, m1, v1 = rep(p0), rep(m0), rep(v0)
      steps = int(cfg["k_path_fine_tuning_epoch"])
    else:
      p1 = rep(p0.new_empty(p0.shape).uniform_(generator=gen))
      m1, v1, t, steps = torch.zeros_like(p1), torch.zeros_like(p1), 0, int(cfg["band_structure_epoch"])
    _band_minimise(plan1, v_eff, p1, m1, v1, steps, lr, b1, b2, eps, t0=t)
    out1, _, _, h1 = plan1.band_trace_grad(p1[0], p1[1], v_eff, with_grad=False, hmat=True)
    hs.append(h1)
    trace += float(out1[0])
    plan1.close()
  h = torch.cat(hs, dim=1)                               # (S, nk, B, B)
  eig = torch.linalg.eigvalsh(h).cpu().numpy()           # (S, nk, B), ascending
  torch.cuda.synchronize()
  out = BandStructureOutput(config=cfg, crystal=crystal, k_path=k_path, eigenvalues=eig,
                            ground_state=gs, band_trace=trace,
                            train_time=time.perf_counter() - t_start, effective_potential=v_eff)
  if cfg.get("save_path"):
    np.save(cfg["save_path"], eig)
  return out


# the reference's name for the all-electron band driver (jrystal/calc/__init__.py:18)
band_all_electrons = band_structure_all_electrons
band_normcons = band_structure_normcons
