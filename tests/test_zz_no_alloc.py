"""jrg_fft3d_noalloc against jrg_fft3d, both called through the C ABI.

jrg_fft3d_noalloc exists for callers that may not allocate device memory
when they transform (a runtime that owns the GPU's memory, a fixed memory
budget, a path that must avoid cudaMalloc's implicit synchronisation): it
keeps its scratch in a fixed 16 MiB array inside the library instead of a
caller workspace.  This file is collected last so that a stop-at-first-
failure run has already run every other test before it.
"""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# same tolerances as the jrg_fft3d parity tests
TOL = {64: 1e-12, 32: 2e-6}


def _call_workspace(lib, prec, grid, batch, direction, x, torch):
  g = (ct.c_int * 3)(*grid)
  nbytes = ct.c_size_t()
  assert lib.jrg_fft3d_workspace_size(prec, g, batch, ct.byref(nbytes)) == 0
  ws = torch.empty(int(nbytes.value), dtype=torch.uint8, device="cuda")
  out = torch.empty_like(x)
  st = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
  assert lib.jrg_fft3d(prec, g, batch, direction, ct.c_void_p(x.data_ptr()),
                       ct.c_void_p(out.data_ptr()), ct.c_void_p(ws.data_ptr()), st) == 0
  return out


def _call_noalloc(lib, prec, grid, batch, direction, x, out, torch):
  g = (ct.c_int * 3)(*grid)
  st = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
  return lib.jrg_fft3d_noalloc(prec, g, batch, direction, ct.c_void_p(x.data_ptr()),
                               ct.c_void_p(out.data_ptr()), st)


@pytest.mark.parametrize("prec", [32, 64])
@pytest.mark.parametrize("grid,batch", [((16, 18, 20), 3), ((64, 64, 64), 2)])
def test_noalloc_matches_workspace_fft(prec, grid, batch):
  import torch
  from jrystal_gb300 import _lib
  lib = _lib.load()
  rng = np.random.default_rng(11)
  cdt = torch.complex128 if prec == 64 else torch.complex64
  # two calls in a row with different inputs and directions: the second call
  # must not see anything the first one left in the shared scratch array
  for call, direction in enumerate((-1, +1)):
    xn = rng.normal(size=(batch,) + grid) + 1j * rng.normal(size=(batch,) + grid)
    x = torch.tensor(xn, dtype=cdt, device="cuda")
    ref = _call_workspace(lib, prec, grid, batch, direction, x, torch)
    out = torch.full_like(x, complex(np.nan, np.nan))
    rc = _call_noalloc(lib, prec, grid, batch, direction, x, out, torch)
    assert rc == 0, lib.jrg_last_error().decode()
    torch.cuda.synchronize()
    a, b = out.cpu().numpy(), ref.cpu().numpy()
    assert np.isfinite(a).all(), f"call {call}"
    assert np.abs(a - b).max() <= TOL[prec] * np.abs(b).max(), f"call {call}"
    # and both agree with numpy's transform
    npref = (np.fft.fftn(xn, axes=(-3, -2, -1)) if direction < 0 else
             np.fft.ifftn(xn, axes=(-3, -2, -1)))
    assert np.abs(a - npref).max() <= TOL[prec] * np.abs(npref).max(), f"call {call}"


@pytest.mark.parametrize("prec", [32, 64])
def test_noalloc_in_place(prec):
  """out = in: the result equals the workspace transform of the same input."""
  import torch
  from jrystal_gb300 import _lib
  lib = _lib.load()
  rng = np.random.default_rng(12)
  grid, batch = (24, 24, 24), 2
  cdt = torch.complex128 if prec == 64 else torch.complex64
  for direction in (-1, +1):
    xn = rng.normal(size=(batch,) + grid) + 1j * rng.normal(size=(batch,) + grid)
    x = torch.tensor(xn, dtype=cdt, device="cuda")
    ref = _call_workspace(lib, prec, grid, batch, direction, x, torch)
    rc = _call_noalloc(lib, prec, grid, batch, direction, x, x, torch)
    assert rc == 0, lib.jrg_last_error().decode()
    torch.cuda.synchronize()
    a, b = x.cpu().numpy(), ref.cpu().numpy()
    assert np.abs(a - b).max() <= TOL[prec] * np.abs(b).max()


def test_noalloc_rejects_oversize_request():
  import torch
  from jrystal_gb300 import _lib
  lib = _lib.load()
  x = torch.zeros(1, dtype=torch.complex64, device="cuda")
  # 8 x 64^3 complex64 = 16 MiB of planes plus the twiddle tables: too large
  g = (ct.c_int * 3)(64, 64, 64)
  st = ct.c_void_p(torch.cuda.current_stream().cuda_stream)
  rc = lib.jrg_fft3d_noalloc(32, g, 8, -1, ct.c_void_p(x.data_ptr()), ct.c_void_p(x.data_ptr()), st)
  assert rc == _lib.JRG_ERR_INVALID
  assert b"16 MiB" in lib.jrg_last_error()
