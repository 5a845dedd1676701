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


def test_cpu_baseline_loss_equals_autograd_of_the_l2_loss():
  """The CPU baseline's l2_loss (one pass each way over the images): loss
  and gradients of sum((out - t)^2)."""
  import bench
  gen = torch.Generator().manual_seed(0)
  v = torch.randn(40, 3, generator=gen, requires_grad=True)
  c = torch.randn(40, 4, generator=gen, requires_grad=True)
  w = torch.randn(3, 4, generator=gen)
  t = torch.randn(40, 4, generator=gen)

  def render(v, c):
    return torch.tanh(v @ w) * c + torch.sin(c)

  ref = ((render(v, c) - t) ** 2).sum()
  rv, rc = torch.autograd.grad(ref, (v, c))
  l2 = bench.l2_loss(render(v, c), t)
  # the loss sums in another order (a dot product): last bits may differ
  torch.testing.assert_close(l2.detach(), ref.detach(), rtol=1e-6, atol=0)
  gv, gc = torch.autograd.grad(l2, (v, c))
  assert torch.equal(gv, rv) and torch.equal(gc, rc)


def test_kernel_bytes_formulas():
  """The algorithmic bytes behind `roofline.achieved` and `kernels_gbs`:
  every input read and every output written once, per kernel."""
  import types
  wl = types.SimpleNamespace(num_layers=3, pixels=1000, triangles=50, vertices=30)
  S = 3000
  b = bench.kernel_bytes(wl, fg=400, near=600, C=4, K=4)
  assert b["raster"] == 50 * 12 + 30 * 32 + S * 4 + 400 * 44 + 16 * S
  assert b["splat_fwd"] == 4 * S + 32 * 400 + 16 * 1000 + 64 * 600
  assert b["splat_bwd"] == 600 * 80 + 4 * S + 32 * 400 + 16 * S + 16 * 400
  # pass-through colors: background attributes and color gradients unwritten
  p = bench.kernel_bytes(wl, fg=400, near=600, C=4, K=4, fg_attributes=True,
                         fg_color_grads=True, vids=False)
  assert p["raster"] == 50 * 12 + 30 * 32 + S * 4 + 400 * 32 + 16 * 400
  assert p["splat_bwd"] == 600 * 80 + 4 * S + 32 * 400 + 16 * 400 + 16 * 400
  assert b["samples_bwd"] == 4 * S + 400 * 64 + 30 * 32 * 3
  assert b["squared_error"] == 48 * 1000
  # near defaults to every pixel
  assert bench.kernel_bytes(wl, fg=400)["splat_fwd"] == 4 * S + 32 * 400 + 16 * 1000 + 64 * 1000
