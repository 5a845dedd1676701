"""Shader building blocks with CUDA kernels (diffren/jax/utils/shaders.py,
diffren/jax/utils/image.py).

``texture_map`` is the reference's bilinear texture lookup with edge
clamping (shaders.py:40-65) and ``bilinear_resample`` the resampler under it
(image.py:21-118), as one CUDA kernel with a hand-written VJP to the
coordinates and the image. Any torch function remains usable as a shader.
"""
import torch

from . import _lib
from . import kernels


class _Resample(torch.autograd.Function):

  @staticmethod
  def forward(ctx, points, image, flags):
    lib = _lib.load()
    n = points.shape[0]
    H, W, C = image.shape
    out = torch.empty(n, C, dtype=torch.float32, device=points.device)
    with kernels._op("texture_fwd", 1):
      rc = lib.dr_texture_map_fwd(kernels._p(points), n, kernels._p(image), H, W, C, flags,
                                  kernels._p(out), kernels._stream(points.device))
    _lib.check(rc, "dr_texture_map_fwd")
    ctx.save_for_backward(points, image)
    ctx.flags = flags
    return out

  @staticmethod
  def backward(ctx, d_out):
    points, image = ctx.saved_tensors
    lib = _lib.load()
    H, W, C = image.shape
    d_pts = torch.empty_like(points) if ctx.needs_input_grad[0] else None
    d_img = torch.zeros_like(image) if ctx.needs_input_grad[1] else None
    if d_pts is None and d_img is None:
      return None, None, None
    with kernels._op("texture_bwd", 1):
      rc = lib.dr_texture_map_bwd(kernels._p(d_out.contiguous()), kernels._p(points),
                                  points.shape[0], kernels._p(image), H, W, C, ctx.flags,
                                  kernels._p(d_pts), kernels._p(d_img),
                                  kernels._stream(points.device))
    _lib.check(rc, "dr_texture_map_bwd")
    return d_pts, d_img, None


def _resample(points, image, flags):
  kernels._require_cuda(points, image)
  if image.dim() != 3:
    raise ValueError("image must be [H, W, C]")
  if points.shape[-1] != 2:
    raise ValueError("points must be [..., 2]")
  pts = points.reshape(-1, 2)
  pts = pts.float().contiguous() if pts.dtype != torch.float32 else pts.contiguous()
  out = _Resample.apply(pts, image.float().contiguous(), flags)
  return out.view(*points.shape[:-1], image.shape[-1])


def texture_map(uv_image, texture_image):
  """Bilinear texture lookup with edge clamping (shaders.py:40-65).

  uv_image [..., 2] with u along the texture's width and v along its height
  (range [0, 1]); texture_image [H, W, C]. Returns [..., C]. Differentiable
  w.r.t. both.
  """
  return _resample(uv_image, texture_image, 0)


def bilinear_resample(image, locations, pad_mode="constant"):
  """image.bilinear_resample (image.py:21-118) for 'HWC' order: samples
  image [H, W, C] at locations [..., 2] in texel units, 'xy' order, samples
  at half-integer coordinates; pad_mode 'constant' (zeros) or 'edge'."""
  if pad_mode not in ("constant", "edge"):
    raise ValueError("Unsupported padding mode: %s" % pad_mode)
  flags = _lib.DR_TEXTURE_TEXEL_UNITS | (_lib.DR_TEXTURE_PAD_ZERO if pad_mode == "constant"
                                         else 0)
  return _resample(locations, image, flags)
