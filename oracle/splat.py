"""Test infrastructure only: numpy float32 restatement of diffren's
interpolation, splatting, normalization and compositing.

Follows, operation by operation and in the same float32 order,
  diffren/jax/internal/interpolate.py:24-63, 118-145 (interpolate_layer),
  diffren/jax/internal/splat.py:26-175 (splat_at_pixel_centers),
  diffren/jax/internal/splat.py:207-221 (clip -> viewport),
  diffren/jax/composite.py:20-37 (over).
Where XLA's reduction order is unspecified (the 3-corner sum), the order is
left to right. Discrete decisions (floor, argmin, surface masks) depend only
on values computed here exactly as in the CUDA kernels.
"""
import math

import numpy as np

F = np.float32


def interpolate(attr, ids, z, bary, triangles, background=None):
  """[L, H, W, K] = fg * sum_i b_i attr[tri[id][i]] + (1 - fg) * bg."""
  attr = np.asarray(attr, F)
  K = attr.shape[1]
  fg = (z != F(1.0))[..., None]
  vids = np.asarray(triangles)[ids]  # [L, H, W, 3]; -1 wraps like jnp
  corners = attr[vids]  # [L, H, W, 3, K]
  b = np.asarray(bary, F)[..., None]
  s = (corners[..., 0, :] * b[..., 0, :] + corners[..., 1, :] * b[..., 1, :]) + \
      corners[..., 2, :] * b[..., 2, :]
  bg = np.zeros(K, F) if background is None else np.asarray(background, F)
  return np.where(fg, s, bg[None, None, None, :]).astype(F)


def viewport_xyz(clip_vertices, ids, z, bary, triangles, width, height):
  """splat.py:207-221: clip interpolation with background (0,0,1,1)."""
  c = interpolate(clip_vertices, ids, z, bary, triangles,
                  background=np.array([0, 0, 1, 1], F))
  ndc = c[..., :3] / c[..., 3:4]
  dims = np.array([width, height, 1], F)
  return ((ndc + F(1.0)) * dims) * F(0.5)


def gaussian_coef():
  s = 0.0
  for u in (-1, 0, 1):
    for v in (-1, 0, 1):
      s += math.exp(-2.0 * (u * u + v * v))
  return F((1.0 + 0.05) / s)


def splat_at_pixel_centers(xyz, color, fg):
  """xyz [L,H,W,3], color [L,H,W,C], fg [L,H,W,1] float32.

  Returns (out [H,W,C], accum [3,H,W,C], normalized [3,H,W,C]).
  """
  xyz = np.asarray(xyz, F)
  color = np.asarray(color, F)
  fg = np.asarray(fg, F)
  L, H, W, C = color.shape
  coef = gaussian_coef()
  acc = np.zeros((3, H + 2, W + 2, C), F)
  wacc = np.zeros((3, H + 2, W + 2, 1), F)
  zpad = np.pad(xyz[..., 2:3], ((0, 0), (1, 1), (1, 1), (0, 0)),
                constant_values=1.0)
  for l in range(L):
    col = color[l]
    p = xyz[l]
    center = (np.floor(p[..., :2]) + np.array([0.5, 0.5], F)) - p[..., :2]
    for u in (-1, 0, 1):
      for v in (-1, 0, 1):
        d = center + np.array([u, v], F)
        dist2 = (d[..., 0:1] * d[..., 0:1] + d[..., 1:2] * d[..., 1:2])
        w = (fg[l] * coef) * np.exp(F(-2.0) * dist2).astype(F)
        tc = w * col
        pad = ((max(v + 1, 0), abs(min(v - 1, 0))),
               (max(u + 1, 0), abs(min(u - 1, 0))), (0, 0))
        tc = np.pad(tc, pad)
        w = np.pad(w, pad)
        tapz = np.pad(xyz[..., 2:3], ((0, 0),) + pad, constant_values=1.0)
        dc = np.abs(tapz - zpad[0])
        c_idx = np.argmin(dc, axis=0)
        c_min = np.min(dc, axis=0)
        dt = np.abs(zpad - tapz[0])
        t_idx = np.argmin(dt, axis=0)
        t_min = np.min(dt, axis=0)
        surf = np.where(t_min < c_min, -t_idx, c_idx)
        masks = np.stack([(surf > l), (surf == l), (surf < l)]).astype(F)
        acc = acc + tc[None] * masks
        wacc = wacc + w[None] * masks
  acc = acc[:, 1:-1, 1:-1, :]
  wacc = wacc[:, 1:-1, 1:-1, :]
  scale = F(1.0) / (np.maximum(wacc - F(1.0), F(0.0)) + F(1.0))
  norm = acc * scale
  return over(norm), acc, norm


def over(layers):
  out = layers[-1]
  for i in range(2, layers.shape[0] + 1):
    alpha = layers[-i, ..., -1:]
    out = layers[-i] + (F(1.0) - alpha) * out
  return out


def splat_shaded_pixels(clip_vertices, ids, z, bary, triangles, shaded, width, height):
  xyz = viewport_xyz(clip_vertices, ids, z, bary, triangles, width, height)
  fg = (z != F(1.0)).astype(F)[..., None]
  return splat_at_pixel_centers(xyz, shaded, fg)
