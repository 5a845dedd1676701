"""Shader building blocks with CUDA kernels (diffren/jax/utils/shaders.py,
diffren/jax/utils/image.py).

``texture_map`` is the reference's bilinear texture lookup with edge
clamping (shaders.py:40-65) and ``bilinear_resample`` the resampler under it
(image.py:21-118), as one CUDA kernel with a hand-written VJP to the
coordinates and the image. ``diffuse_light``
(shaders.py:68-97) is the reference's formula as elementwise torch
expressions; ``point_light`` (shaders.py:100-173) runs as one CUDA kernel
each way with a hand-written VJP (torch expressions for tensor-valued
coefficients). Any torch function remains usable as a shader.
"""
import ctypes

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
    flags, scratch, launches = ctx.flags, None, 1
    if flags & _lib.DR_TEXTURE_DETERMINISTIC:
      if d_img is None:
        flags &= ~_lib.DR_TEXTURE_DETERMINISTIC  # d_uv is per point: nothing to sum
      else:
        scratch = torch.empty(lib.dr_texture_map_bwd_scratch_bytes(H, W, C),
                              dtype=torch.uint8, device=points.device)
        launches = 3
    with kernels._op("texture_bwd", launches):
      rc = lib.dr_texture_map_bwd_ex(kernels._p(d_out.contiguous()), kernels._p(points),
                                     points.shape[0], kernels._p(image), H, W, C, flags,
                                     kernels._p(d_pts), kernels._p(d_img), kernels._p(scratch),
                                     0 if scratch is None else scratch.numel(),
                                     kernels._stream(points.device))
    _lib.check(rc, "dr_texture_map_bwd_ex")
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


def _det(deterministic):
  return _lib.DR_TEXTURE_DETERMINISTIC if deterministic else 0


def texture_map(uv_image, texture_image, deterministic=False):
  """Bilinear texture lookup with edge clamping (shaders.py:40-65).

  uv_image [..., 2] with u along the texture's width and v along its height
  (range [0, 1]); texture_image [H, W, C]. Returns [..., C]. Differentiable
  w.r.t. both. ``deterministic`` (beyond the reference's arguments): the
  texture gradient is summed in fixed point, the same bits on every run.
  """
  return _resample(uv_image, texture_image, _det(deterministic))


def bilinear_resample(image, locations, pad_mode="constant", deterministic=False):
  """image.bilinear_resample (image.py:21-118) for 'HWC' order: samples
  image [H, W, C] at locations [..., 2] in texel units, 'xy' order, samples
  at half-integer coordinates; pad_mode 'constant' (zeros) or 'edge'."""
  if pad_mode not in ("constant", "edge"):
    raise ValueError("Unsupported padding mode: %s" % pad_mode)
  flags = _lib.DR_TEXTURE_TEXEL_UNITS | (_lib.DR_TEXTURE_PAD_ZERO if pad_mode == "constant"
                                         else 0) | _det(deterministic)
  return _resample(locations, image, flags)


def _vec3(v, like):
  """v (a tensor or three numbers) as a tensor like `like`; numbers are
  written with device-side fills, so that this works under CUDA graph
  capture."""
  if torch.is_tensor(v):
    return v.to(dtype=like.dtype, device=like.device)
  out = like.new_empty(3)
  for i, x in enumerate(v):
    out.narrow(0, i, 1).fill_(float(x))
  return out


def l2_normalize(x, dim=-1, eps=1e-12):
  """transforms.l2_normalize (transforms.py:26-37): x * rsqrt(|x|^2 + eps)."""
  return x * torch.rsqrt((x * x).sum(dim=dim, keepdim=True) + eps)


def diffuse_light(diffuse_image, normals_image, light_direction=(0.5, 0.5, 1.0), ka=0.5,
                  kd=0.5):
  """shaders.diffuse_light (shaders.py:68-97): ambient plus directional
  diffuse, diffuse * (ka + kd * clip(n . l, 0, 1)) with l normalized."""
  d = _vec3(light_direction, normals_image)
  d = l2_normalize(d.reshape(*([1] * (normals_image.dim() - 1)), 3))
  n_dot_l = (normals_image * d).sum(-1, keepdim=True).clamp(0.0, 1.0)
  return diffuse_image * ka + diffuse_image * kd * n_dot_l


def _row_stride(t):
  """Row stride (floats) of a [..., 3] float32 tensor whose rows lie evenly
  spaced in memory (columns of a packed buffer included), else None."""
  if t.dtype != torch.float32 or t.dim() < 1 or t.shape[-1] != 3 or t.stride(-1) != 1:
    return None
  try:
    rows = t.view(-1, 3)
  except RuntimeError:
    return None
  return 3 if rows.shape[0] <= 1 else rows.stride(0)


class _PointLight(torch.autograd.Function):
  """dr_point_light_fwd / _bwd: the whole shader in one kernel each way."""

  @staticmethod
  def forward(ctx, diffuse, normals, positions, params, out_channels):
    lib = _lib.load()
    ins = []
    for t in (diffuse, normals, positions):
      st = _row_stride(t)
      if st is None or st < 3:
        t, st = t.float().contiguous(), 3
      ins.append((t, st))
    (dif, sd), (nrm, sn), (pos, sp) = ins
    n = dif.numel() // 3 if dif.dim() > 0 else 0
    out = torch.empty(n, out_channels, dtype=torch.float32, device=dif.device)
    with kernels._op("point_light", 1):
      rc = lib.dr_point_light_fwd(kernels._p(dif), kernels._p(nrm), kernels._p(pos), n, sd, sn,
                                  sp, ctypes.byref(params), kernels._p(out), out_channels,
                                  kernels._stream(dif.device))
    _lib.check(rc, "dr_point_light_fwd")
    ctx.save_for_backward(dif, nrm, pos)
    ctx.strides, ctx.params, ctx.oc, ctx.n = (sd, sn, sp), params, out_channels, n
    ctx.shapes = (diffuse.shape, normals.shape, positions.shape)
    return out.view(*diffuse.shape[:-1], out_channels)

  @staticmethod
  def backward(ctx, d_out):
    dif, nrm, pos = ctx.saved_tensors
    lib = _lib.load()
    need = ctx.needs_input_grad[:3]
    if not any(need):
      return None, None, None, None, None
    d_out = d_out.float().contiguous()
    grads = [torch.empty(ctx.n, 3, dtype=torch.float32, device=dif.device) if w else None
             for w in need]
    sd, sn, sp = ctx.strides
    with kernels._op("point_light_bwd", 1):
      rc = lib.dr_point_light_bwd(kernels._p(d_out), ctx.oc, kernels._p(dif), kernels._p(nrm),
                                  kernels._p(pos), ctx.n, sd, sn, sp, ctypes.byref(ctx.params),
                                  *[kernels._p(g) for g in grads], 3,
                                  kernels._stream(dif.device))
    _lib.check(rc, "dr_point_light_bwd")
    return tuple(None if g is None else g.view(sh) for g, sh in zip(grads, ctx.shapes)) + (
        None, None)


def _three_numbers(v):
  """v as three Python floats when it is a length-3 sequence of numbers (or
  a CPU tensor), else None (tensors on the GPU stay on the torch path)."""
  if torch.is_tensor(v):
    if v.is_cuda or v.requires_grad or v.numel() != 3:
      return None
    return [float(x) for x in v.reshape(-1).tolist()]
  try:
    vals = [float(x) for x in v]
  except (TypeError, ValueError):
    return None
  return vals if len(vals) == 3 else None


def point_light(diffuse_image, normals_image, pixel_positions, point_locations,
                eye_position=(0.0, 0.0, 0.0), ka=0.3, kd=1.4, ks=0.0, ns=0.0,
                attenuation_constant=1.0, attenuation_linear=0.7,
                attenuation_quadratic=1.8, alpha=False):
  """shaders.point_light (shaders.py:100-173): a point light with ambient,
  diffuse and Blinn-Phong specular terms and quadratic distance attenuation
  1 / (c + l d + q d^2); images are [..., 3]. ``alpha`` (beyond the
  reference's arguments) appends an alpha channel of 1 (no gradient).

  CUDA images with scalar coefficients and a fixed light and eye run as one
  kernel each way (dr_point_light_fwd / _bwd); anything else as torch
  expressions."""
  light3, eye3 = _three_numbers(point_locations), _three_numbers(eye_position)
  coefs = (ka, kd, ks, ns, attenuation_constant, attenuation_linear, attenuation_quadratic)
  tensors = (diffuse_image, normals_image, pixel_positions)
  if (light3 is not None and eye3 is not None and
      all(isinstance(c, (int, float)) for c in coefs) and
      all(torch.is_tensor(t) and t.is_cuda and t.dtype == torch.float32 and t.shape[-1] == 3
          for t in tensors) and
      diffuse_image.shape == normals_image.shape == pixel_positions.shape):
    params = _lib.PointLight((ctypes.c_float * 3)(*light3), (ctypes.c_float * 3)(*eye3),
                             *[float(c) for c in coefs])
    return _PointLight.apply(diffuse_image, normals_image, pixel_positions, params,
                             4 if alpha else 3)
  light = _vec3(point_locations, pixel_positions)
  eye = _vec3(eye_position, pixel_positions)
  to_light = light - pixel_positions
  light_dir = l2_normalize(to_light)
  view_dir = l2_normalize(eye - pixel_positions)
  half = l2_normalize(light_dir + view_dir)
  nol = (normals_image * light_dir).sum(-1, keepdim=True).clamp(0.0, 1.0)
  noh = (normals_image * half).sum(-1, keepdim=True).clamp(0.0, 1.0)
  dist = torch.linalg.vector_norm(to_light, dim=-1, keepdim=True)
  decay = 1.0 / (attenuation_constant + attenuation_linear * dist +
                 attenuation_quadratic * dist * dist)
  luma = ka + kd * nol + ks * noh ** ns
  rgb = diffuse_image * luma * decay
  if alpha:
    rgb = torch.cat([rgb, torch.ones_like(rgb[..., :1])], -1)
  return rgb
