"""The benchmark's multi-rank plumbing on the CPU (world size 2): the job
time is the maximum over ranks (gloo), and under torchrun the reference arm
prints exactly one line, from rank 0, with every rank exiting 0.  The path
itself runs as independent replicas (one plan per GPU, no collective in the
data path), so these are the only cross-rank steps."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
  with socket.socket() as s:
    s.bind(("127.0.0.1", 0))
    return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
  import torch.distributed as dist
  sys.path.insert(0, ROOT)
  import bench
  dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                          world_size=world)
  try:
    m = bench._max_over_ranks(1.5 + 2.0 * rank, "cpu")
    with open(os.path.join(out_dir, f"r{rank}.txt"), "w") as f:
      f.write(repr(m))
  finally:
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
  import torch.multiprocessing as mp
  mp.start_processes(_rank_main, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True,
                     start_method="spawn")
  for r in range(2):
    assert float((tmp_path / f"r{r}.txt").read_text()) == 3.5


def test_max_over_ranks_single_process():
  sys.path.insert(0, ROOT)
  import bench
  assert bench._max_over_ranks(2.25, "cpu") == 2.25


def test_reference_arm_under_torchrun():
  cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
         "--master-addr", "127.0.0.1", "--master-port", str(_free_port()),
         os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
         "--workload", "si2_fcc_48", "--steps", "1", "--warmup", "0", "--cpu-sample-kpts", "1"]
  r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
  assert r.returncode == 0, r.stderr[-2000:]
  lines = [l for l in r.stdout.splitlines() if l.strip().startswith("{")]
  assert len(lines) == 1, r.stdout
  d = json.loads(lines[0])
  assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
