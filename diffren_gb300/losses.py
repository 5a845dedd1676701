"""Squared-error objective with a fused CUDA kernel.

The reference fits renders to target images with the mean squared error
(jnp.mean((image - target)**2), diffren/jax/internal/splat_test.py:137-167).
``squared_error_seed`` computes weight * sum((image - target)^2) and its
gradient (2 * weight) * (image - target) in one pass over the two images;
the gradient is the seed for the renderer's VJP
(``torch.autograd.grad(image, params, grad_outputs=seed)``), so no second
pass over the images forms it. ``squared_error`` is the same loss as an
autograd function. The sum order is fixed (deterministic).
"""
import torch

from . import _lib
from . import kernels


def squared_error_seed(image, target, weight=1.0):
  """(loss, seed): loss = weight * sum((image - target)^2) as a 0-dim CUDA
  tensor, seed = (2 * weight) * (image - target) shaped like image. Neither
  is tracked by autograd. With weight 1 the seed is exactly 2 (image -
  target)."""
  kernels._require_cuda(image, target)
  if image.shape != target.shape:
    raise ValueError("image and target shapes differ: %s vs %s"
                     % (tuple(image.shape), tuple(target.shape)))
  image = kernels._f32(image.detach())
  target = kernels._f32(target.detach(), image.device)
  seed = torch.empty_like(image)
  partials = torch.empty(_lib.DR_SQUARED_ERROR_PARTIALS, dtype=torch.float64,
                         device=image.device)
  loss = torch.empty((), dtype=torch.float32, device=image.device)
  lib = _lib.load()
  with torch.cuda.device(image.device), kernels._op("squared_error", 2):
    rc = lib.dr_squared_error(kernels._p(image), kernels._p(target), image.numel(),
                              float(weight), kernels._p(seed), kernels._p(partials),
                              kernels._p(loss), kernels._stream(image.device))
  _lib.check(rc, "dr_squared_error")
  return loss, seed


class _SquaredError(torch.autograd.Function):

  @staticmethod
  def forward(ctx, image, target, weight):
    loss, seed = squared_error_seed(image, target, weight)
    ctx.save_for_backward(seed)
    return loss

  @staticmethod
  def backward(ctx, g):
    (seed,) = ctx.saved_tensors
    d_image = seed * g if ctx.needs_input_grad[0] else None
    d_target = -(seed * g) if ctx.needs_input_grad[1] else None
    return d_image, d_target, None


def squared_error(image, target, weight=1.0):
  """weight * sum((image - target)^2), differentiable w.r.t. image and
  target; weight = 1 / image.numel() gives the reference's mean."""
  return _SquaredError.apply(image, target, float(weight))
