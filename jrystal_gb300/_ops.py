"""Device helpers shared by the jrystal-compatible modules: tensor
conversion, the library's 3-D FFT and elementwise LDA with their
vector-Jacobian products (torch.autograd), and plan caches.

Gradients follow torch's convention for complex tensors (the cotangent of z
is dL/dRe z + i dL/dIm z).  The FFTs carry the transpose rules of
jrystal/_src/spmd/fft.py:88-101 in that convention: the adjoint of the
unnormalised forward transform is N times the normalised inverse, and the
reverse."""
from __future__ import annotations

import ctypes as ct
from typing import Optional

import numpy as np
import torch

from . import _lib
from .engine import fft3d as _fft3d, xc_flags

_DEFAULT_PRECISION = [64]   # jrystal defaults to jax_enable_x64 = True


def set_precision(bits: int):
  """Default precision (32 or 64) of arrays the modules create."""
  if bits not in (32, 64):
    raise ValueError("precision must be 32 or 64")
  _DEFAULT_PRECISION[0] = bits


def get_precision() -> int:
  return _DEFAULT_PRECISION[0]


def real_dtype(bits: Optional[int] = None):
  return torch.float64 if (bits or get_precision()) == 64 else torch.float32


def complex_dtype(bits: Optional[int] = None):
  return torch.complex128 if (bits or get_precision()) == 64 else torch.complex64


def device():
  if not torch.cuda.is_available():
    raise RuntimeError("jrystal_gb300 needs a CUDA device (no CPU fallback)")
  return torch.device("cuda", torch.cuda.current_device())


def as_tensor(x, dtype=None) -> torch.Tensor:
  """Array-like -> CUDA tensor (numpy, lists, scalars or tensors)."""
  if isinstance(x, torch.Tensor):
    t = x if x.is_cuda else x.to(device())
    return t.to(dtype) if dtype is not None and t.dtype != dtype else t
  a = np.asarray(x)
  if dtype is None:
    if a.dtype == np.bool_:
      dtype = torch.bool
    elif np.iscomplexobj(a):
      dtype = complex_dtype()
    elif np.issubdtype(a.dtype, np.integer):
      dtype = torch.int64
    else:
      dtype = real_dtype()
  return torch.as_tensor(a, device=device()).to(dtype)


def to_numpy(x) -> np.ndarray:
  if isinstance(x, torch.Tensor):
    return x.detach().cpu().numpy()
  return np.asarray(x)


def precision_of(t: torch.Tensor) -> int:
  return 64 if t.dtype in (torch.float64, torch.complex128) else 32


class _Fft3(torch.autograd.Function):
  """The library's batched 3-D FFT with its adjoint as the backward."""

  @staticmethod
  def forward(ctx, x, inverse):
    ctx.inverse = bool(inverse)
    ctx.n = float(np.prod(x.shape[-3:]))
    return _fft3d(x.contiguous(), inverse=ctx.inverse)

  @staticmethod
  def backward(ctx, g):
    g = g.contiguous()
    if ctx.inverse:   # y = conj(F) x / N  ->  x_bar = F y_bar / N
      return _fft3d(g, inverse=False) / ctx.n, None
    return _fft3d(g, inverse=True) * ctx.n, None   # y = F x  ->  x_bar = conj(F) y_bar


def _complex(x: torch.Tensor) -> torch.Tensor:
  if torch.is_complex(x):
    return x
  return x.to(torch.complex128 if x.dtype == torch.float64 else torch.complex64)


def fftn(x: torch.Tensor) -> torch.Tensor:
  """Unnormalised forward FFT over the last three axes (jnp.fft.fftn)."""
  return _Fft3.apply(_complex(x), False)


def ifftn(x: torch.Tensor) -> torch.Tensor:
  """Inverse FFT over the last three axes with 1/N (jnp.fft.ifftn)."""
  return _Fft3.apply(_complex(x), True)


class _LdaEps(torch.autograd.Function):
  """LDA energy per particle eps(rho), elementwise; its derivative
  d eps / d rho = (v_xc - eps) / rho from the library's v_xc."""

  @staticmethod
  def forward(ctx, rho, xc):
    eps = _lda_raw(rho, xc, False)
    ctx.save_for_backward(rho, eps)
    ctx.xc = xc
    return eps

  @staticmethod
  def backward(ctx, g):
    rho, eps = ctx.saved_tensors
    v = _lda_raw(rho, ctx.xc, True)
    d = torch.where(rho > 1e-15, (v - eps) / torch.where(rho > 1e-15, rho, torch.ones_like(rho)),
                    torch.zeros_like(rho))
    return g * d, None


def lda_eps(rho: torch.Tensor, xc: str) -> torch.Tensor:
  """Differentiable LDA energy per particle (the non-Kohn-Sham xc_density)."""
  return _LdaEps.apply(rho, xc)


def lda(rho: torch.Tensor, xc: str, kohn_sham: bool) -> torch.Tensor:
  """Elementwise LDA energy per particle (or potential) on the device, no
  gradient (the Kohn-Sham potential is taken at a stopped density, as
  jrystal/_src/xc.py:246-250 does)."""
  return _lda_raw(rho.detach(), xc, kohn_sham)


def _lda_raw(rho: torch.Tensor, xc: str, kohn_sham: bool) -> torch.Tensor:
  """Elementwise LDA energy per particle (or potential) on the device."""
  lib = _lib.load()
  rho = rho.contiguous()
  if torch.is_complex(rho):
    raise TypeError("density must be real")
  out = torch.empty_like(rho)
  prec = precision_of(rho)
  st = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
  _lib.check(lib.jrg_lda(prec, rho.numel(), xc_flags(xc), int(bool(kohn_sham)),
                         ct.c_void_p(rho.data_ptr()), ct.c_void_p(out.data_ptr()), st), "jrg_lda")
  return out


def lda_pol_raw(rho: torch.Tensor, xc: str, mode: int) -> torch.Tensor:
  """Spin-polarised LDA of a (2, ...) density on the device (jrg_lda_polarized):
  mode 0 eps (...), 1 vxc_lda's eps + rho_s d eps/d rho_s (2, ...), 2 the
  derivative of eps (rho_up + rho_dn), eps + rho d eps/d rho_s (2, ...)."""
  lib = _lib.load()
  rho = rho.contiguous()
  if torch.is_complex(rho) or rho.shape[0] != 2:
    raise TypeError("a polarised density is real with 2 channels")
  out = torch.empty(rho.shape[1:] if mode == 0 else rho.shape, dtype=rho.dtype, device=rho.device)
  st = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
  _lib.check(lib.jrg_lda_polarized(precision_of(rho), rho[0].numel(), xc_flags(xc), int(mode),
                                   ct.c_void_p(rho.data_ptr()), ct.c_void_p(out.data_ptr()), st),
             "jrg_lda_polarized")
  return out


class _LdaEpsPol(torch.autograd.Function):
  """Polarised LDA energy per particle eps(rho_up, rho_dn); d eps / d rho_s =
  (v_s - eps) / rho with v_s the library's derivative of eps rho."""

  @staticmethod
  def forward(ctx, rho, xc):
    eps = lda_pol_raw(rho, xc, 0)
    ctx.save_for_backward(rho, eps)
    ctx.xc = xc
    return eps

  @staticmethod
  def backward(ctx, g):
    rho, eps = ctx.saved_tensors
    v = lda_pol_raw(rho, ctx.xc, 2)
    tot = rho.sum(0)
    ok = tot > 1e-15
    d = torch.where(ok, (v - eps) / torch.where(ok, tot, torch.ones_like(tot)), torch.zeros_like(v))
    return g * d, None


def lda_eps_pol(rho: torch.Tensor, xc: str) -> torch.Tensor:
  """Differentiable polarised LDA energy per particle of a (2, ...) density."""
  return _LdaEpsPol.apply(rho, xc)


def safe_real(x: torch.Tensor, tol: float = 1e-8) -> torch.Tensor:
  """jrystal/_src/utils.py:25-59."""
  if torch.is_complex(x):
    if bool(torch.all(torch.abs(x.imag) <= tol)):
      return x.real
    raise ValueError("Array has non-zero imaginary part")
  return x
