"""The N>1 path of bench.py on CPU: world_size-2 gloo ranks agree on the
slowest rank's time, and the whole-job value counts every replica."""
import os
import socket

import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
  with socket.socket() as s:
    s.bind(("127.0.0.1", 0))
    return s.getsockname()[1]


def _rank(rank, world, port, times, out):
  os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
  dist.init_process_group("gloo", rank=rank, world_size=world)
  try:
    dist.barrier()
    out[rank] = bench.max_over_ranks(times[rank], world, torch.device("cpu"))
  finally:
    dist.destroy_process_group()


def test_max_over_ranks_with_two_gloo_ranks():
  world, port = 2, _free_port()
  times = [3.5, 7.25]
  with mp.get_context("spawn").Manager() as manager:
    out = manager.dict()
    mp.start_processes(_rank, args=(world, port, times, out), nprocs=world,
                       start_method="spawn")
    assert dict(out) == {0: 7.25, 1: 7.25}


def test_single_rank_and_whole_job_value():
  assert bench.max_over_ranks(4.0, 1, None) == 4.0
  # 2 replicas x 28.4 Mpix in 7 ms each.
  assert abs(bench.whole_job_mpix(2, 28_377_088, 7.0) - 2 * 28_377_088 / 7.0 / 1e3) < 1e-9
