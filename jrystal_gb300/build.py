"""Build recipe of the in-tree CUDA library ``libjrystal_gb300.so`` (sm_103a).

The translation units are compiled in parallel with ``nvcc -gencode
arch=compute_103a,code=sm_103a`` and linked into a shared library next to
this file.  Rebuilds happen only when a source or header is newer than the
library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libjrystal_gb300.so")
SOURCES = ["k_fft.cu", "k_fft_fast.cu", "k_orth.cu", "k_orth_tc.cu", "k_gram_tc5.cu", "k_grid.cu", "capi.cu", "noalloc.cu", "k_precond.cu", "k_nonlocal.cu", "batch.cu", "k_rotate_g.cu", "k_gram_big.cu", "k_chol_df.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", CSRC, "-I", INCLUDE]


def nvcc() -> str:
  exe = shutil.which("nvcc")
  if exe:
    return exe
  cand = "/usr/local/cuda/bin/nvcc"
  if os.path.exists(cand):
    return cand
  raise RuntimeError("nvcc not found: the CUDA toolkit is required to build jrystal_gb300")


def _deps():
  files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
  files.append(os.path.join(INCLUDE, "jrystal_gb300.h"))
  return files


def needs_build() -> bool:
  if not os.path.exists(LIB):
    return True
  t = os.path.getmtime(LIB)
  return any(os.path.getmtime(f) > t for f in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
  """Compile the library if needed and return its path."""
  if not force and not needs_build():
    return LIB
  os.makedirs(BUILD, exist_ok=True)
  exe = nvcc()

  def compile_one(src):
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    cmd = [exe, *ARCH, *FLAGS, "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
      raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr}")
    if verbose and r.stderr:
      print(r.stderr)
    return obj

  with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
    objs = list(pool.map(compile_one, SOURCES))
  tmp = LIB + ".tmp"
  cmd = [exe, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"]
  r = subprocess.run(cmd, capture_output=True, text=True)
  if r.returncode != 0:
    raise RuntimeError(f"nvcc link failed:\n{r.stderr}")
  os.replace(tmp, LIB)
  return LIB


if __name__ == "__main__":
  print(build(force=True, verbose=True))
