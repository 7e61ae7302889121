"""The C-ABI library loads without a GPU and exports every entry point that
include/jrystal_gb300.h declares (no compute calls here)."""
import ctypes as ct
import os
import re

import pytest

from jrystal_gb300 import _lib, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "jrystal_gb300.h")


def declared_symbols():
  src = open(HEADER).read()
  src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
  return sorted(set(re.findall(r"\b(jrg_[a-z0-9_]+)\s*\(", src)))


def test_header_declares_entry_points():
  names = declared_symbols()
  for must in ("jrg_plan_create", "jrg_energy_grad", "jrg_coeff", "jrg_density", "jrg_fft3d",
               "jrg_adam_update", "jrg_ewald", "jrg_potential"):
    assert must in names


def test_library_exports_every_declared_symbol():
  lib = _lib.load()
  missing = [n for n in declared_symbols() if not hasattr(lib, n)]
  assert not missing, missing
  # and the Python binding covers them
  assert set(declared_symbols()) <= set(_lib.exported_symbols())


def test_version_and_error_string_without_gpu():
  lib = _lib.load()
  assert lib.jrg_version() >= 1
  assert isinstance(lib.jrg_last_error(), bytes)
  assert lib.jrg_profile_num_phases() > 5


def test_invalid_arguments_are_rejected_on_the_host():
  lib = _lib.load()
  out = ct.c_void_p()
  assert lib.jrg_plan_create(None, ct.byref(out)) == _lib.JRG_ERR_INVALID
  assert b"null" in lib.jrg_last_error()
  assert lib.jrg_adam_update(16, 10, None, None, None, None, None, 1, 1e-2, 0.9, 0.99, 1e-8,
                             None) == _lib.JRG_ERR_INVALID


def test_build_recipe_targets_sm_103a():
  assert "arch=compute_103a,code=sm_103a" in " ".join(build.ARCH)
  assert os.path.exists(build.LIB)


def test_plan_refuses_a_cpu_device():
  """There is no CPU fallback: a plan on the CPU is refused before any work."""
  import numpy as np
  from jrystal_gb300.engine import PlaneWavePlan
  mask = np.zeros((8, 8, 8), dtype=bool)
  mask[0, 0, 0] = mask[0, 0, 1] = True
  with pytest.raises(RuntimeError, match="CUDA"):
    PlaneWavePlan(np.eye(3) * 5.0, np.zeros((1, 3)), np.array([1.0]), (8, 8, 8), mask,
                  np.zeros((1, 3)), 1, 1, 64, "lda_x", device="cpu")


def test_pseudopotential_setter_rejects_bad_arguments_on_the_host():
  lib = _lib.load()
  assert lib.jrg_plan_set_pseudopotential(None, None, 0, None) == _lib.JRG_ERR_INVALID
  assert lib.jrg_plan_set_pseudopotential(None, None, 4, None) == _lib.JRG_ERR_INVALID


def test_pseudopotential_types():
  from types import SimpleNamespace
  from jrystal_gb300 import calc
  cr = SimpleNamespace(symbols=["Si"], positions=[[0, 0, 0]], charges=[14])
  with pytest.raises(NotImplementedError):
    calc.create_pseudopotential({"pseudopotential_type": "us", "pseudopotential_file_dir": "."}, cr)
  with pytest.raises(ValueError):
    calc.create_pseudopotential({"pseudopotential_type": "paw", "pseudopotential_file_dir": "."}, cr)
  with pytest.raises(ValueError):
    calc.create_pseudopotential({"pseudopotential_type": "nc", "pseudopotential_file_dir": None}, cr)


def test_batch_create_rejects_bad_descriptions_without_gpu():
  """jrg_batch_create checks its description before touching the device."""
  lib = _lib.load()
  h = ct.c_void_p()
  assert lib.jrg_batch_create(None, ct.byref(h)) == _lib.JRG_ERR_INVALID
  d = _lib.BatchDesc()
  d.num_cells = 0
  assert lib.jrg_batch_create(ct.byref(d), ct.byref(h)) == _lib.JRG_ERR_INVALID
  assert b"num_cells" in lib.jrg_last_error()
  one = (ct.c_void_p * 1)(ct.c_void_p(8))
  p = ct.cast(one, ct.POINTER(ct.c_void_p))
  d.num_cells = 1
  d.plans = d.workspaces = d.params = d.m = d.v = d.grads = d.occupations = p
  d.steps, d.lr, d.b1, d.b2, d.eps = 0, 1e-2, 0.9, 0.99, 1e-8
  assert lib.jrg_batch_create(ct.byref(d), ct.byref(h)) == _lib.JRG_ERR_INVALID
  d.steps, d.per_step = 10, 4      # records without record buffers
  assert lib.jrg_batch_create(ct.byref(d), ct.byref(h)) == _lib.JRG_ERR_INVALID
  assert b"record" in lib.jrg_last_error()
  assert lib.jrg_batch_step(None, 1, None) == _lib.JRG_ERR_INVALID
  assert lib.jrg_batch_destroy(None) == _lib.JRG_OK
