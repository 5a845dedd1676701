"""The fused squared-error kernel (losses.py, csrc/loss.cu) through the C
ABI: loss against a float64 sum, the seed bit-exact against 2 (image -
target), gradients through a renderer equal to autograd of the loss."""
import pytest
import torch

import bench
from diffren_gb300 import losses

pytestmark = pytest.mark.gpu

DEV = "cuda"


def _pair(n, seed=0, offset=0):
  g = torch.Generator(device=DEV).manual_seed(seed)
  a = torch.rand(n + offset, generator=g, device=DEV)[offset:]
  b = torch.rand(n + offset, generator=g, device=DEV)[offset:]
  return a, b


@pytest.mark.parametrize("n,offset", [(1 << 20, 0), (4 * 1000003, 0), (999, 0),
                                      (1 << 16, 1), (1, 0), (0, 0)])
def test_loss_and_seed(n, offset):
  a, b = _pair(n, offset=offset)  # offset 1: unaligned rows, the scalar path
  loss, seed = losses.squared_error_seed(a, b)
  d = a - b
  want = float(((a.double() - b.double()) ** 2).sum())
  assert abs(float(loss) - want) <= 1e-6 * max(want, 1e-30)
  assert torch.equal(seed, d * 2.0)
  # deterministic: a second call gives the same bits
  loss2, _ = losses.squared_error_seed(a, b)
  assert torch.equal(loss, loss2)


def test_mean_weight_and_shapes():
  a, b = _pair(3 * 64 * 48 * 4, seed=1)
  a, b = a.view(3, 64, 48, 4), b.view(3, 64, 48, 4)
  w = 1.0 / a.numel()
  loss, seed = losses.squared_error_seed(a, b, w)
  want = float(((a.double() - b.double()) ** 2).mean())
  assert abs(float(loss) - want) <= 1e-6 * want
  assert seed.shape == a.shape
  torch.testing.assert_close(seed, (a - b) * (2.0 * w), rtol=1e-6, atol=0)
  with pytest.raises(ValueError, match="shapes differ"):
    losses.squared_error_seed(a, b[:1])


def test_autograd_function_matches_torch():
  a, b = _pair(4096, seed=2)
  x = a.clone().requires_grad_(True)
  t = b.clone().requires_grad_(True)
  loss = losses.squared_error(x, t)
  gx, gt = torch.autograd.grad(loss, (x, t))
  y = a.clone().requires_grad_(True)
  u = b.clone().requires_grad_(True)
  ref = ((y - u) ** 2).sum()
  ry, ru = torch.autograd.grad(ref, (y, u))
  assert torch.equal(gx, ry) and torch.equal(gt, ru)
  torch.testing.assert_close(loss, ref, rtol=1e-6, atol=0)


def test_bench_loss_gradients_equal_autograd_of_the_l2_loss():
  """The benchmark seeds the renderer's VJP with the fused kernel's
  2 (out - target): gradients bit-identical to autograd of
  sum((out - t)^2)."""
  gen = torch.Generator(device=DEV).manual_seed(0)
  v = torch.randn(40, 3, generator=gen, device=DEV, requires_grad=True)
  c = torch.randn(40, 4, generator=gen, device=DEV, requires_grad=True)
  w = torch.randn(3, 4, generator=gen, device=DEV)
  t = torch.randn(40, 4, generator=gen, device=DEV)

  def render(v, c):
    return torch.tanh(v @ w) * c + torch.sin(c)

  loss, (gv, gc) = bench.l2_loss_grads(render(v, c), t, (v, c))
  ref = ((render(v, c) - t) ** 2).sum()
  rv, rc = torch.autograd.grad(ref, (v, c))
  torch.testing.assert_close(loss, ref.detach(), rtol=1e-6, atol=0)
  assert torch.equal(gv, rv) and torch.equal(gc, rc)


def test_captured_in_a_cuda_graph():
  a, b = _pair(1 << 18, seed=3)
  s = torch.cuda.Stream()
  s.wait_stream(torch.cuda.current_stream())
  with torch.cuda.stream(s):
    losses.squared_error_seed(a, b)
  torch.cuda.current_stream().wait_stream(s)
  g = torch.cuda.CUDAGraph()
  with torch.cuda.graph(g):
    loss, seed = losses.squared_error_seed(a, b)
  a.mul_(0.5)
  g.replay()
  torch.cuda.synchronize()
  want = float(((a.double() - b.double()) ** 2).sum())
  assert abs(float(loss) - want) <= 1e-6 * want
  assert torch.equal(seed, (a - b) * 2.0)
