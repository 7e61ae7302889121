"""ctypes binding of the C ABI in ``include/jrystal_gb300.h``.

The library is the in-tree ``libjrystal_gb300.so``; loading fails loudly when
it is missing -- there is no CPU or PyTorch fallback for any entry point.
"""
from __future__ import annotations

import ctypes as ct
import os
import threading

from . import build as _build

_LOCK = threading.Lock()
_LIB = None

JRG_OK = 0
JRG_ERR_INVALID = 1
JRG_ERR_CUDA = 2
JRG_ERR_NUMERIC = 3
JRG_ERR_UNSUPPORTED = 4
XC_FLAGS = {"lda_x": 1, "lda_c_vwn": 2, "gga_x_pbe": 4, "gga_c_pbe": 8}

# exported entry points and their argument types
_vp = ct.c_void_p


class AdamStep(ct.Structure):
  """jrg_adam_step."""
  _fields_ = [
    ("step", ct.c_int),
    ("lr", ct.c_double),
    ("b1", ct.c_double),
    ("b2", ct.c_double),
    ("eps", ct.c_double),
    ("scale", ct.c_void_p),
    ("mlp_w32", ct.c_void_p),
    ("mlp_wb", ct.c_void_p),
    ("t_frac", ct.c_float),
    ("smax", ct.c_float),
  ]


class BatchDesc(ct.Structure):
  """jrg_batch_desc."""
  _fields_ = [
    ("num_cells", ct.c_int),
    ("plans", ct.POINTER(ct.c_void_p)),
    ("workspaces", ct.POINTER(ct.c_void_p)),
    ("params", ct.POINTER(ct.c_void_p)),
    ("m", ct.POINTER(ct.c_void_p)),
    ("v", ct.POINTER(ct.c_void_p)),
    ("grads", ct.POINTER(ct.c_void_p)),
    ("occupations", ct.POINTER(ct.c_void_p)),
    ("steps", ct.c_int),
    ("lr", ct.c_double),
    ("b1", ct.c_double),
    ("b2", ct.c_double),
    ("eps", ct.c_double),
    ("energies", ct.c_void_p),
    ("per_step", ct.c_int),
    ("seed", ct.c_ulonglong),
    ("c_floor", ct.c_double),
    ("rec_x", ct.c_void_p),
    ("rec_a", ct.c_void_p),
    ("rec_c", ct.c_void_p),
    ("rec_w", ct.c_void_p),
    ("rec_idx", ct.c_void_p),
  ]


_SIGS = {
  "jrg_version": ([], ct.c_int),
  "jrg_last_error": ([], ct.c_char_p),
  "jrg_launch_count": ([], ct.c_longlong),
  "jrg_plan_create": ([_vp, ct.POINTER(_vp)], ct.c_int),
  "jrg_plan_destroy": ([_vp], ct.c_int),
  "jrg_workspace_size": ([_vp, ct.POINTER(ct.c_size_t)], ct.c_int),
  "jrg_plan_set_memory_limit": ([_vp, ct.c_size_t], ct.c_int),
  "jrg_batch_create": ([ct.POINTER(BatchDesc), ct.POINTER(_vp)], ct.c_int),
  "jrg_batch_step": ([_vp, ct.c_int, _vp], ct.c_int),
  "jrg_batch_steps_done": ([_vp, ct.POINTER(ct.c_int)], ct.c_int),
  "jrg_batch_destroy": ([_vp], ct.c_int),
  "jrg_plan_memory_chunk": ([_vp, ct.POINTER(ct.c_int)], ct.c_int),
  "jrg_plan_set_pseudopotential": ([_vp, _vp, ct.c_int, _vp], ct.c_int),
  "jrg_coeff": ([_vp, _vp, _vp, _vp, _vp, _vp], ct.c_int),
  "jrg_density": ([_vp, _vp, _vp, _vp, _vp, _vp], ct.c_int),
  "jrg_coeff_adjoint": ([_vp] * 8, ct.c_int),
  "jrg_energy_grad": ([_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp], ct.c_int),
  "jrg_band_trace_grad": ([_vp] * 11, ct.c_int),
  "jrg_pipeline": ([ct.c_int], ct.c_int),
  "jrg_energy_grad_bands": ([_vp] * 10, ct.c_int),
  "jrg_energy_grad_adam": ([_vp, _vp, _vp, _vp, _vp, ct.POINTER(AdamStep), _vp, _vp, _vp, _vp],
                           ct.c_int),
  "jrg_potential": ([_vp, _vp, ct.c_int, _vp, _vp, _vp], ct.c_int),
  "jrg_reorthonormalise": ([_vp, _vp, _vp, _vp, _vp], ct.c_int),
  "jrg_fft3d_workspace_size": ([ct.c_int, ct.POINTER(ct.c_int), ct.c_int,
                                ct.POINTER(ct.c_size_t)], ct.c_int),
  "jrg_fft3d": ([ct.c_int, ct.POINTER(ct.c_int), ct.c_int, ct.c_int, _vp, _vp, _vp,
                 _vp], ct.c_int),
  "jrg_fft3d_noalloc": ([ct.c_int, ct.POINTER(ct.c_int), ct.c_int, ct.c_int, _vp, _vp, _vp],
                        ct.c_int),
  "jrg_lda": ([ct.c_int, ct.c_int64, ct.c_int, ct.c_int, _vp, _vp, _vp], ct.c_int),
  "jrg_lda_polarized": ([ct.c_int, ct.c_int64, ct.c_int, ct.c_int, _vp, _vp, _vp], ct.c_int),
  "jrg_adam_update": ([ct.c_int, ct.c_int64, _vp, _vp, _vp, _vp, _vp, ct.c_int,
                       ct.c_double, ct.c_double, ct.c_double, ct.c_double, _vp], ct.c_int),
  "jrg_ewald": ([_vp, ct.c_double, ct.c_double, _vp, _vp, _vp], ct.c_int),
  "jrg_fast_paths": ([ct.c_int], ct.c_int),
  "jrg_tensor_core_paths": ([ct.c_int], ct.c_int),
  "jrg_mlp_num_params": ([], ct.c_int),
  "jrg_mlp_to_bf16": ([_vp, _vp, _vp], ct.c_int),
  "jrg_mlp_workspace_size": ([ct.c_int, ct.POINTER(ct.c_size_t)], ct.c_int),
  "jrg_mlp_train_eval": ([ct.c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
                         ct.c_int),
  "jrg_precond_scale": ([_vp, _vp, _vp, ct.c_float, ct.c_float, _vp, _vp, _vp, _vp], ct.c_int),
  "jrg_band_kinetic": ([_vp, _vp, _vp, _vp], ct.c_int),
  "jrg_kinetic_table": ([_vp, _vp, _vp], ct.c_int),
  "jrg_profile_enable": ([_vp, ct.c_int], ct.c_int),
  "jrg_profile_read": ([_vp, ct.POINTER(ct.c_double), ct.POINTER(ct.c_int), ct.c_int], ct.c_int),
  "jrg_profile_phase_name": ([ct.c_int], ct.c_char_p),
  "jrg_profile_num_phases": ([], ct.c_int),
}


class PlanDesc(ct.Structure):
  _fields_ = [
    ("precision", ct.c_int),
    ("grid", ct.c_int * 3),
    ("cell", ct.c_double * 9),
    ("num_atom", ct.c_int),
    ("positions", ct.POINTER(ct.c_double)),
    ("charges", ct.POINTER(ct.c_double)),
    ("num_spin", ct.c_int),
    ("num_kpt", ct.c_int),
    ("num_band", ct.c_int),
    ("kpts", ct.POINTER(ct.c_double)),
    ("num_g", ct.c_int),
    ("sphere_index", ct.POINTER(ct.c_int32)),
    ("xc", ct.c_int),
  ]


def library_path() -> str:
  return _build.LIB


def exported_symbols():
  return list(_SIGS)


def load(build_if_missing: bool = True):
  """Load (building first if allowed and needed) the CUDA library."""
  global _LIB
  with _LOCK:
    if _LIB is not None:
      return _LIB
    path = _build.LIB
    if build_if_missing and _build.needs_build():
      _build.build()
    if not os.path.exists(path):
      raise RuntimeError(
        f"jrystal_gb300 CUDA library not found at {path}; run "
        "jrystal_gb300.build.build() (nvcc required). There is no CPU fallback.")
    lib = ct.CDLL(path)
    for name, (args, res) in _SIGS.items():
      fn = getattr(lib, name)
      fn.argtypes = args
      fn.restype = res
    _LIB = lib
    return lib


class NumericalError(FloatingPointError):
  """JRG_ERR_NUMERIC: a Cholesky breakdown or non-finite values (the status
  word of an energy call, or a status the library returned)."""
  code = JRG_ERR_NUMERIC


def check(status: int, what: str = ""):
  if status != JRG_OK:
    msg = load().jrg_last_error().decode(errors="replace")
    kind = {JRG_ERR_INVALID: ValueError, JRG_ERR_UNSUPPORTED: NotImplementedError,
            JRG_ERR_NUMERIC: NumericalError}.get(status, RuntimeError)
    raise kind(f"{what} failed (status {status}): {msg}")
