"""Test infrastructure only: CPU restatement of diffren's texture-map shader
(diffren/jax/utils/shaders.py:40-65) and its bilinear resampling with edge
padding (diffren/jax/utils/image.py:21-118), for checking the CUDA kernel.

texture_map(uv, texture): query = uv * (W, H) - 0.5 in texel units ('xy'
order, flipped to (row, col)), sampled from the texture padded by one texel
with its edge values: location += 1, floor clipped to [0, size], weights
ceil = clip(location - floor, 0, 1), floor = 1 - ceil, result
((ll + ul) + ur) + lr with each corner term (texel * w_row) * w_col.
`texture_map` follows the float32 operation order exactly; `texture_map_t`
is the same formula in torch (any dtype) for autograd, with jnp.clip's
gradient (1 strictly inside the bounds, 0 at or outside them, as lax.clamp).
"""
import numpy as np
import torch

F = np.float32


def _corners(loc, size):
  """floor index (padded), ceil weight, floor weight per axis; float32."""
  floor = np.floor(loc)
  floor = np.clip(floor, 0, size).astype(np.int64)  # padded shape - 2 = size
  cw = np.clip(loc - floor.astype(F), F(0), F(1)).astype(F)
  fw = (F(1) - cw).astype(F)
  return floor, cw, fw


def texture_map(uv, texture):
  """uv [..., 2] float32, texture [H, W, C] float32 -> [..., C] float32."""
  tex = np.asarray(texture, F)
  H, W, _ = tex.shape
  q = np.asarray(uv, F) * np.array([W, H], F)  # xy texel coordinates
  return bilinear_resample(tex, q, "edge")


def bilinear_resample(image, locations, pad_mode="constant"):
  """image.py:21-118 for HWC order: locations [..., 2] in texel units."""
  tex = np.asarray(image, F)
  H, W, C = tex.shape
  q = (np.asarray(locations, F) - F(0.5)).astype(F)
  loc_r = (q[..., 1] + F(1)).astype(F)
  loc_c = (q[..., 0] + F(1)).astype(F)
  fr, cwr, fwr = _corners(loc_r, H)
  fc, cwc, fwc = _corners(loc_c, W)
  pad = np.pad(tex, ((1, 1), (1, 1), (0, 0)), mode=pad_mode)
  d00 = pad[fr, fc]
  d10 = pad[fr + 1, fc]
  d11 = pad[fr + 1, fc + 1]
  d01 = pad[fr, fc + 1]
  ll = (d00 * fwr[..., None]).astype(F) * fwc[..., None]
  ul = (d10 * cwr[..., None]).astype(F) * fwc[..., None]
  ur = (d11 * cwr[..., None]).astype(F) * cwc[..., None]
  lr = (d01 * fwr[..., None]).astype(F) * cwc[..., None]
  return (((ll + ul).astype(F) + ur).astype(F) + lr).astype(F)


class _Clip01(torch.autograd.Function):
  """clip(x, 0, 1) with gradient 1 strictly inside (0, 1), else 0."""

  @staticmethod
  def forward(ctx, x):
    ctx.save_for_backward(x)
    return x.clamp(0.0, 1.0)

  @staticmethod
  def backward(ctx, g):
    (x,) = ctx.saved_tensors
    return g * ((x > 0) & (x < 1)).to(g.dtype)


def texture_map_t(uv, texture):
  """texture_map in torch: differentiable w.r.t. uv and texture."""
  H, W, _ = texture.shape
  q = uv * torch.tensor([W, H], dtype=uv.dtype, device=uv.device)
  return bilinear_resample_t(texture, q, "edge")


def bilinear_resample_t(image, locations, pad_mode="constant"):
  """bilinear_resample in torch: differentiable w.r.t. locations and image."""
  H, W, _ = image.shape
  q = locations - 0.5
  loc_r = q[..., 1] + 1.0
  loc_c = q[..., 0] + 1.0
  chw = image.permute(2, 0, 1)[None]
  if pad_mode == "edge":
    pad = torch.nn.functional.pad(chw, (1, 1, 1, 1), mode="replicate")
  else:
    pad = torch.nn.functional.pad(chw, (1, 1, 1, 1), mode="constant", value=0.0)
  pad = pad[0].permute(1, 2, 0)

  def axis(loc, size):
    floor = torch.floor(loc.detach()).clamp(0, size)
    cw = _Clip01.apply(loc - floor)
    return floor.long(), cw, 1.0 - cw

  fr, cwr, fwr = axis(loc_r, H)
  fc, cwc, fwc = axis(loc_c, W)
  ll = pad[fr, fc] * fwr[..., None] * fwc[..., None]
  ul = pad[fr + 1, fc] * cwr[..., None] * fwc[..., None]
  ur = pad[fr + 1, fc + 1] * cwr[..., None] * cwc[..., None]
  lr = pad[fr, fc + 1] * fwr[..., None] * cwc[..., None]
  return ((ll + ul) + ur) + lr
