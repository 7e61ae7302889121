"""Device helpers shared by the jrystal-compatible modules: tensor
conversion, the library's 3-D FFT and elementwise LDA, and plan caches."""
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


def fftn(x: torch.Tensor) -> torch.Tensor:
  """Unnormalised forward FFT over the last three axes (jnp.fft.fftn)."""
  return _fft3d(x, inverse=False)


def ifftn(x: torch.Tensor) -> torch.Tensor:
  """Inverse FFT over the last three axes with 1/N (jnp.fft.ifftn)."""
  return _fft3d(x, inverse=True)


def lda(rho: torch.Tensor, xc: str, kohn_sham: bool) -> torch.Tensor:
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


def safe_real(x: torch.Tensor, tol: float = 1e-8) -> torch.Tensor:
  """jrystal/_src/utils.py:25-59."""
  if torch.is_complex(x):
    if bool(torch.all(torch.abs(x.imag) <= tol)):
      return x.real
    raise ValueError("Array has non-zero imaginary part")
  return x
