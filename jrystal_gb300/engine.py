"""Device plans and the fused energy/gradient engine.

A :class:`PlaneWavePlan` owns the geometry tables of one (cell, grid,
sphere, k-points, bands) system on the current CUDA device and a workspace
tensor, and calls the C ABI with torch-allocated device buffers on torch's
current stream.  It is the engine under the jrystal-compatible modules
(``pw``, ``energy``, ``potential`` ...) and the optimiser loop.
"""
from __future__ import annotations

import ctypes as ct
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib

_DT = {32: (torch.float32, torch.complex64), 64: (torch.float64, torch.complex128)}


def _ptr(t: Optional[torch.Tensor]):
  return None if t is None else ct.c_void_p(t.data_ptr())


def _stream():
  return ct.c_void_p(torch.cuda.current_stream().cuda_stream)


def xc_flags(xc: str) -> int:
  flags = 0
  for name in xc.split("+"):
    if name not in _lib.XC_FLAGS:
      raise NotImplementedError(f"xc functional {name!r} is not implemented")
    flags |= _lib.XC_FLAGS[name]
  return flags


def precision_of(dtype) -> int:
  if dtype in (torch.float64, torch.complex128, np.float64, np.complex128):
    return 64
  return 32


class PlaneWavePlan:
  """Geometry tables + workspace of one system on one GPU.

  Args:
    cell_vectors: (3,3) lattice vectors as rows (bohr).
    positions: (atom,3) Cartesian positions (bohr); charges: (atom,).
    grid_sizes: FFT grid (nx, ny, nz).
    freq_mask: boolean (nx,ny,nz) plane-wave sphere (jrystal's mask order).
    kpts: (kpt,3) Cartesian k-points.
    num_band, num_spin: band and spin counts of the parameters.
    precision: 32 (complex64 path) or 64 (complex128 path).
    xc: '+'-separated LDA names ("lda_x", "lda_c_vwn").
  """

  def __init__(self, cell_vectors, positions, charges, grid_sizes, freq_mask, kpts,
               num_band: int, num_spin: int = 1, precision: int = 32,
               xc: str = "lda_x+lda_c_vwn", device=None):
    self.lib = _lib.load()
    dev = torch.device(device if device is not None else "cuda")
    if dev.type != "cuda":
      raise RuntimeError("jrystal_gb300 runs on CUDA devices only (no CPU fallback)")
    if dev.index is None:
      dev = torch.device("cuda", torch.cuda.current_device())
    self.device = dev
    torch.cuda.set_device(self.device)
    self.precision = int(precision)
    self.rdtype, self.cdtype = _DT[self.precision]
    self.cell = np.ascontiguousarray(np.asarray(cell_vectors, dtype=np.float64))
    self.positions = np.ascontiguousarray(np.asarray(positions, dtype=np.float64).reshape(-1, 3))
    self.charges = np.ascontiguousarray(np.asarray(charges, dtype=np.float64).reshape(-1))
    self.grid = tuple(int(g) for g in grid_sizes)
    mask = np.asarray(freq_mask, dtype=bool)
    if mask.shape != self.grid:
      raise ValueError(f"freq_mask shape {mask.shape} != grid {self.grid}")
    self.mask = mask
    self.kpts = np.ascontiguousarray(np.asarray(kpts, dtype=np.float64).reshape(-1, 3))
    self.num_spin, self.num_kpt, self.num_band = int(num_spin), self.kpts.shape[0], int(num_band)
    self.sphere_index = np.ascontiguousarray(np.flatnonzero(mask.reshape(-1)).astype(np.int32))
    self.num_g = int(self.sphere_index.size)
    self.xc = xc
    self.vol = float(abs(np.linalg.det(self.cell)))
    d = _lib.PlanDesc()
    d.precision = self.precision
    d.grid[:] = list(self.grid)
    d.cell[:] = list(self.cell.reshape(-1))
    d.num_atom = self.positions.shape[0]
    d.positions = self.positions.ctypes.data_as(ct.POINTER(ct.c_double))
    d.charges = self.charges.ctypes.data_as(ct.POINTER(ct.c_double))
    d.num_spin, d.num_kpt, d.num_band = self.num_spin, self.num_kpt, self.num_band
    d.kpts = self.kpts.ctypes.data_as(ct.POINTER(ct.c_double))
    d.num_g = self.num_g
    d.sphere_index = self.sphere_index.ctypes.data_as(ct.POINTER(ct.c_int32))
    d.xc = xc_flags(xc)
    h = ct.c_void_p()
    _lib.check(self.lib.jrg_plan_create(ct.byref(d), ct.byref(h)), "jrg_plan_create")
    self._h = h
    nbytes = ct.c_size_t()
    _lib.check(self.lib.jrg_workspace_size(h, ct.byref(nbytes)), "jrg_workspace_size")
    self.workspace_bytes = int(nbytes.value)
    self.workspace = torch.empty(self.workspace_bytes, dtype=torch.uint8, device=self.device)
    self.energies = torch.zeros(8, dtype=torch.float64, device=self.device)
    self.num_proj = 0

  def set_pseudopotential(self, v_local=None, projectors=None):
    """Norm-conserving pseudopotential tables (jrg_plan_set_pseudopotential).

    v_local: complex (nx, ny, nz) V_loc(G) of
    pseudopotential.local.potential_local_reciprocal, or None to keep the
    current external table; projectors: complex (K, J, G) beta-projector rows
    on the sphere (pseudopotential.nloc.projector_table), or None / J = 0 for
    no nonlocal term.  The workspace is reallocated to the new size."""
    vl = None
    if v_local is not None:
      v = np.asarray(v_local, dtype=np.complex128)
      if v.shape != self.grid:
        raise ValueError(f"v_local shape {v.shape} != grid {self.grid}")
      vl = np.ascontiguousarray(v.reshape(-1).view(np.float64))
    nproj, pj = 0, None
    if projectors is not None:
      p = np.asarray(projectors, dtype=np.complex128)
      if p.ndim != 3 or p.shape[0] != self.num_kpt or p.shape[2] != self.num_g:
        raise ValueError(f"projectors shape {p.shape} != (K={self.num_kpt}, J, G={self.num_g})")
      nproj = int(p.shape[1])
      pj = np.ascontiguousarray(p.reshape(-1).view(np.float64)) if nproj else None
    ptr = lambda a: None if a is None else a.ctypes.data_as(ct.c_void_p)
    torch.cuda.synchronize(self.device)
    _lib.check(self.lib.jrg_plan_set_pseudopotential(self._h, ptr(vl), nproj, ptr(pj)),
               "jrg_plan_set_pseudopotential")
    self.num_proj = nproj
    nbytes = ct.c_size_t()
    _lib.check(self.lib.jrg_workspace_size(self._h, ct.byref(nbytes)), "jrg_workspace_size")
    if int(nbytes.value) != self.workspace_bytes:
      self.workspace_bytes = int(nbytes.value)
      self.workspace = torch.empty(self.workspace_bytes, dtype=torch.uint8, device=self.device)

  def set_memory_limit(self, nbytes: int) -> int:
    """Bound the workspace (jrg_plan_set_memory_limit; 0 removes the bound):
    the plane transforms are recomputed per chunk of (s,k) blocks when all
    of them do not fit.  Reallocates the workspace; returns the (s,k) blocks
    per chunk."""
    torch.cuda.synchronize(self.device)
    _lib.check(self.lib.jrg_plan_set_memory_limit(self._h, int(nbytes)), "jrg_plan_set_memory_limit")
    nb = ct.c_size_t()
    _lib.check(self.lib.jrg_workspace_size(self._h, ct.byref(nb)), "jrg_workspace_size")
    self.workspace_bytes = int(nb.value)
    self.workspace = torch.empty(self.workspace_bytes, dtype=torch.uint8, device=self.device)
    kc = ct.c_int()
    _lib.check(self.lib.jrg_plan_memory_chunk(self._h, ct.byref(kc)), "jrg_plan_memory_chunk")
    return int(kc.value)

  # -- shapes -------------------------------------------------------------
  @property
  def param_shape(self):
    return (self.num_spin, self.num_kpt, self.num_g, self.num_band)

  def _check_param(self, t: torch.Tensor, name: str, dtype=None):
    dtype = dtype or self.rdtype
    if tuple(t.shape) != self.param_shape:
      raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {self.param_shape}")
    if t.dtype != dtype or t.device != self.device or not t.is_contiguous():
      raise ValueError(f"{name} must be a contiguous {dtype} tensor on {self.device}")

  def _occ(self, occupation) -> torch.Tensor:
    occ = torch.as_tensor(occupation, dtype=torch.float64, device=self.device).contiguous()
    if tuple(occ.shape) != (self.num_spin, self.num_kpt, self.num_band):
      raise ValueError(f"occupation shape {tuple(occ.shape)} != "
                       f"{(self.num_spin, self.num_kpt, self.num_band)}")
    return occ

  # -- entry points -------------------------------------------------------
  def energy_and_grad(self, w_re: torch.Tensor, w_im: torch.Tensor, occupation,
                      grad_re: Optional[torch.Tensor] = None,
                      grad_im: Optional[torch.Tensor] = None, with_grad: bool = True):
    """Energy terms (device float64[8]: kinetic, external, hartree, xc,
    total, -, cholesky-breakdown flag, nonlocal pseudopotential part of the
    external term) and d total/d{w_re, w_im}."""
    self._check_param(w_re, "w_re")
    self._check_param(w_im, "w_im")
    occ = self._occ(occupation)
    if with_grad:
      if grad_re is None:
        grad_re = torch.empty_like(w_re)
      if grad_im is None:
        grad_im = torch.empty_like(w_im)
    st = self.lib.jrg_energy_grad(self._h, _ptr(w_re), _ptr(w_im), _ptr(occ), _ptr(self.energies),
                                  _ptr(grad_re) if with_grad else None,
                                  _ptr(grad_im) if with_grad else None, _ptr(self.workspace),
                                  _stream())
    _lib.check(st, "jrg_energy_grad")
    return self.energies, grad_re, grad_im

  def energy_grad_bands(self, w_re: torch.Tensor, w_im: torch.Tensor, occupation,
                        grad_re: Optional[torch.Tensor] = None,
                        grad_im: Optional[torch.Tensor] = None):
    """energy_and_grad plus the band energies <psi|T + V_eff|psi> (S,K,B)
    float64 = d total / d occupation."""
    self._check_param(w_re, "w_re")
    self._check_param(w_im, "w_im")
    occ = self._occ(occupation)
    grad_re = torch.empty_like(w_re) if grad_re is None else grad_re
    grad_im = torch.empty_like(w_im) if grad_im is None else grad_im
    eps = torch.empty((self.num_spin, self.num_kpt, self.num_band), dtype=torch.float64,
                      device=self.device)
    st = self.lib.jrg_energy_grad_bands(self._h, _ptr(w_re), _ptr(w_im), _ptr(occ),
                                        _ptr(self.energies), _ptr(eps), _ptr(grad_re),
                                        _ptr(grad_im), _ptr(self.workspace), _stream())
    _lib.check(st, "jrg_energy_grad_bands")
    return self.energies, grad_re, grad_im, eps

  def band_trace_grad(self, w_re: torch.Tensor, w_im: torch.Tensor, v_eff, weights=None,
                      grad_re: Optional[torch.Tensor] = None,
                      grad_im: Optional[torch.Tensor] = None, with_grad: bool = True,
                      hmat: bool = False):
    """Band trace sum w <psi|T + V_eff|psi> for a fixed effective potential
    (device float64[2]: trace, kinetic part), its gradient with respect to
    {w_re, w_im}, and optionally the band Hamiltonian (S,K,B,B) complex128
    with entries w_j <psi_i|H|psi_j>.  ``v_eff`` is one grid or one per spin
    (S,x,y,z); ``weights`` (S,K,B) default to ones."""
    self._check_param(w_re, "w_re")
    self._check_param(w_im, "w_im")
    v = torch.as_tensor(v_eff, device=self.device).to(self.rdtype)
    if v.dim() == 3:
      v = v[None]
    if v.shape[0] == 1 and self.num_spin == 2:
      v = v.expand(2, *self.grid)
    if tuple(v.shape) != (self.num_spin,) + self.grid:
      raise ValueError(f"v_eff has shape {tuple(v.shape)}, expected {(self.num_spin,) + self.grid}")
    v = v.contiguous()
    wts = self._occ(torch.ones((self.num_spin, self.num_kpt, self.num_band), dtype=torch.float64)
                    if weights is None else weights)
    if with_grad:
      if grad_re is None:
        grad_re = torch.empty_like(w_re)
      if grad_im is None:
        grad_im = torch.empty_like(w_im)
    out = torch.empty(2, dtype=torch.float64, device=self.device)
    hm = None
    if hmat:
      hm = torch.empty((self.num_spin, self.num_kpt, self.num_band, self.num_band),
                       dtype=torch.complex128, device=self.device)
    st = self.lib.jrg_band_trace_grad(self._h, _ptr(w_re), _ptr(w_im), _ptr(v), _ptr(wts),
                                      _ptr(out), _ptr(hm), _ptr(grad_re) if with_grad else None,
                                      _ptr(grad_im) if with_grad else None, _ptr(self.workspace),
                                      _stream())
    _lib.check(st, "jrg_band_trace_grad")
    return out, grad_re if with_grad else None, grad_im if with_grad else None, hm

  def energy_grad_adam(self, params: torch.Tensor, m: torch.Tensor, v: torch.Tensor, occupation,
                       step: int, lr: float, b1: float = 0.9, b2: float = 0.99, eps: float = 1e-8,
                       scale: Optional[torch.Tensor] = None, mlp=None, t_frac: float = 0.0,
                       smax: float = 4.0, grad: Optional[torch.Tensor] = None) -> torch.Tensor:
    """One fused optimiser step in place on params (2,S,K,G,B) and the Adam
    moments m, v: the energies of the parameters before the update (device
    float64[8]) are returned.  ``mlp`` (a precond.MLP) makes the learned
    preconditioner's scales inside the step into ``scale`` (required then);
    otherwise ``scale`` is an optional input.  ``grad`` receives the gradient."""
    shape = (2,) + self.param_shape
    for name, t in (("params", params), ("m", m), ("v", v), ("grad", grad)):
      if t is None and name == "grad":
        continue
      if tuple(t.shape) != shape or t.dtype != self.rdtype or not t.is_contiguous() \
          or t.device != self.device:
        raise ValueError(f"{name}: expected contiguous {self.rdtype} {shape} on {self.device}")
    if scale is not None and (tuple(scale.shape) != shape or scale.dtype != torch.float32
                              or not scale.is_contiguous()):
      raise ValueError(f"scale: expected contiguous float32 {shape}")
    if mlp is not None and scale is None:
      raise ValueError("the learned scale needs a scale buffer")
    occ = self._occ(occupation)
    addr = lambda t: None if t is None else t.data_ptr()
    opt = _lib.AdamStep(int(step), float(lr), float(b1), float(b2), float(eps), addr(scale),
                        addr(None if mlp is None else mlp.w32), addr(None if mlp is None else mlp.wb),
                        float(t_frac), float(smax))
    st = self.lib.jrg_energy_grad_adam(self._h, _ptr(params), _ptr(m), _ptr(v), _ptr(occ),
                                       ct.byref(opt), _ptr(self.energies), _ptr(grad),
                                       _ptr(self.workspace), _stream())
    _lib.check(st, "jrg_energy_grad_adam")
    return self.energies

  # -- numerical status and recovery ------------------------------------
  # Gram condition estimates above which the parameters are re-orthonormalised
  # (the coefficients lose orthogonality as the Gram's rounding times this)
  CONDITION_LIMIT = {32: 1e3, 64: 1e8}

  @staticmethod
  def status_of(energies) -> dict:
    """The numerical status of an energy call from its energies vector (host
    or device): ``flags`` (bit 0: Cholesky breakdown, bit 1: a tensor-core
    wait ran out), ``condition`` (the Gram condition estimate) and ``finite``
    (every energy term finite)."""
    e = energies.detach().cpu().numpy() if isinstance(energies, torch.Tensor) else np.asarray(energies)
    return {"flags": int(e[6]), "condition": float(e[5]), "finite": bool(np.isfinite(e[:5]).all())}

  def check_numerics(self, energies, what: str = "energy call"):
    """Raise _lib.NumericalError (JRG_ERR_NUMERIC) when the call's status word
    is set or an energy is not finite; returns the status otherwise."""
    st = self.status_of(energies)
    if st["flags"] or not st["finite"]:
      raise _lib.NumericalError(
        f"{what}: status word {st['flags']}, condition estimate {st['condition']:.3g}, "
        f"finite energies {st['finite']} (JRG_ERR_NUMERIC)")
    return st

  def needs_reorthonormalisation(self, energies) -> bool:
    st = self.status_of(energies)
    return bool(st["flags"] & 1) or not st["finite"] or \
        not (st["condition"] <= self.CONDITION_LIMIT[self.precision])

  def reorthonormalise(self, w_re: torch.Tensor, w_im: torch.Tensor):
    """In place: W <- an orthonormal basis of W's columns times the original
    column norms (jrg_reorthonormalise); the energy of a full-rank W is
    unchanged, non-finite or dependent columns are replaced."""
    self._check_param(w_re, "w_re")
    self._check_param(w_im, "w_im")
    _lib.check(self.lib.jrg_reorthonormalise(self._h, _ptr(w_re), _ptr(w_im), _ptr(self.workspace),
                                             _stream()), "jrg_reorthonormalise")

  def coeff(self, w_re: torch.Tensor, w_im: torch.Tensor) -> torch.Tensor:
    self._check_param(w_re, "w_re")
    self._check_param(w_im, "w_im")
    out = torch.empty(self.param_shape, dtype=self.cdtype, device=self.device)
    st = self.lib.jrg_coeff(self._h, _ptr(w_re), _ptr(w_im), _ptr(out), _ptr(self.workspace),
                            _stream())
    _lib.check(st, "jrg_coeff")
    return out

  def coeff_adjoint(self, w_re: torch.Tensor, w_im: torch.Tensor, grad_coeff: torch.Tensor):
    """dL/dw_re, dL/dw_im from the cotangent of coeff(w_re, w_im) (torch's
    convention for complex tensors: dL/dRe + i dL/dIm)."""
    self._check_param(w_re, "w_re")
    self._check_param(w_im, "w_im")
    g = grad_coeff.to(self.cdtype).contiguous()
    self._check_param(g, "grad_coeff", self.cdtype)
    gr, gi = torch.empty_like(w_re), torch.empty_like(w_im)
    st = self.lib.jrg_coeff_adjoint(self._h, _ptr(w_re), _ptr(w_im), _ptr(g), _ptr(gr), _ptr(gi),
                                    _ptr(self.workspace), _stream())
    _lib.check(st, "jrg_coeff_adjoint")
    return gr, gi

  def density(self, coeff_sphere: torch.Tensor, occupation) -> torch.Tensor:
    self._check_param(coeff_sphere, "coeff", self.cdtype)
    occ = self._occ(occupation)
    out = torch.empty((self.num_spin,) + self.grid, dtype=self.rdtype, device=self.device)
    st = self.lib.jrg_density(self._h, _ptr(coeff_sphere), _ptr(occ), _ptr(out),
                              _ptr(self.workspace), _stream())
    _lib.check(st, "jrg_density")
    return out

  def potential(self, density: torch.Tensor, kohn_sham: bool = False) -> torch.Tensor:
    """(2 + S, nx, ny, nz): Hartree, external, then the xc part of each of
    the plan's S spin channels (real)."""
    rho = density.to(device=self.device, dtype=self.rdtype).contiguous()
    if rho.dim() == 3:
      rho = rho[None]
    if tuple(rho.shape) != (self.num_spin,) + self.grid:
      raise ValueError(f"density shape {tuple(rho.shape)} != {(self.num_spin,) + self.grid}")
    out = torch.empty((2 + self.num_spin,) + self.grid, dtype=self.rdtype, device=self.device)
    st = self.lib.jrg_potential(self._h, _ptr(rho), int(bool(kohn_sham)), _ptr(out),
                                _ptr(self.workspace), _stream())
    _lib.check(st, "jrg_potential")
    return out

  def ewald(self, eta: float, cutoff: float) -> float:
    out = torch.zeros(1, dtype=torch.float64, device=self.device)
    st = self.lib.jrg_ewald(self._h, float(eta), float(cutoff), _ptr(out), _ptr(self.workspace),
                            _stream())
    _lib.check(st, "jrg_ewald")
    return float(out.item())

  def close(self):
    if getattr(self, "_h", None):
      self.lib.jrg_plan_destroy(self._h)
      self._h = None

  def __del__(self):
    try:
      self.close()
    except Exception:
      pass


def fft3d(x: torch.Tensor, inverse: bool = False) -> torch.Tensor:
  """Complex FFT over the last three axes (jnp.fft.fftn / ifftn semantics)."""
  lib = _lib.load()
  if not x.is_cuda:
    raise RuntimeError("fft3d needs a CUDA tensor (no CPU fallback)")
  if not torch.is_complex(x):
    x = x.to(torch.complex128 if x.dtype == torch.float64 else torch.complex64)
  x = x.contiguous()
  prec = 64 if x.dtype == torch.complex128 else 32
  grid = (ct.c_int * 3)(*x.shape[-3:])
  batch = int(np.prod(x.shape[:-3])) if x.dim() > 3 else 1
  nbytes = ct.c_size_t()
  _lib.check(lib.jrg_fft3d_workspace_size(prec, grid, batch, ct.byref(nbytes)), "jrg_fft3d_workspace_size")
  ws = torch.empty(int(nbytes.value), dtype=torch.uint8, device=x.device)
  out = torch.empty_like(x)
  _lib.check(lib.jrg_fft3d(prec, grid, batch, 1 if inverse else -1, _ptr(x), _ptr(out), _ptr(ws),
                           _stream()), "jrg_fft3d")
  return out


def adam_update(param: torch.Tensor, grad: torch.Tensor, m: torch.Tensor, v: torch.Tensor,
                step: int, lr: float, b1: float = 0.9, b2: float = 0.99, eps: float = 1e-8,
                scale: Optional[torch.Tensor] = None):
  """In-place fused Adam step (optax.adam semantics); ``step`` is 1-based."""
  lib = _lib.load()
  prec = 64 if param.dtype == torch.float64 else 32
  for t in (param, grad, m, v):
    if t.dtype != param.dtype or not t.is_contiguous() or t.numel() != param.numel():
      raise ValueError("adam_update: param, grad, m, v must match and be contiguous")
  if scale is not None and (scale.dtype != torch.float32 or scale.numel() != param.numel()):
    raise ValueError("adam_update: scale must be float32 with one entry per element")
  _lib.check(lib.jrg_adam_update(prec, param.numel(), _ptr(param), _ptr(grad), _ptr(m), _ptr(v),
                                 _ptr(scale), int(step), float(lr), float(b1), float(b2),
                                 float(eps), _stream()), "jrg_adam_update")
