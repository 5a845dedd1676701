"""Test infrastructure only: torch restatement of the continuous part of
diffren's rasterize-then-splat path, for gradients (torch autograd stands in
for jax.grad through the reference, which cannot run without JAX).

Same formulas as oracle/splat.py (interpolate.py:24-63, splat.py:26-229,
composite.py:20-37, rasterize.py:127-255) in any float dtype. The discrete
decisions of the float32 forward (floor of the splat positions, the per-tap
surface masks) are computed once in float32 by ``discrete_state`` and held
fixed, so that a float64 evaluation differentiates exactly the function the
float32 kernels compute. jnp.maximum's gradient splits 0.5/0.5 at equality
(lax.max) and that rule is kept.
"""
import numpy as np
import torch
import torch.nn.functional as Fn

from . import splat as np_splat


def interpolate(attr, ids, z, bary, triangles, background=None):
  fg = (z != 1.0)[..., None]
  vids = triangles[ids.long()]
  c = attr[vids]  # [L, H, W, 3, K]
  b = bary[..., None]
  s = (c[..., 0, :] * b[..., 0, :] + c[..., 1, :] * b[..., 1, :]) + c[..., 2, :] * b[..., 2, :]
  if background is None:
    background = torch.zeros(attr.shape[1], dtype=attr.dtype, device=attr.device)
  return torch.where(fg, s, background.to(attr.dtype))


def viewport_xyz(clip, ids, z, bary, triangles, width, height):
  c = interpolate(clip, ids, z, bary, triangles,
                  torch.tensor([0.0, 0.0, 1.0, 1.0], dtype=clip.dtype, device=clip.device))
  ndc = c[..., :3] / c[..., 3:4]
  dims = torch.tensor([width, height, 1.0], dtype=clip.dtype, device=clip.device)
  return ((ndc + 1.0) * dims) * 0.5


def discrete_state(clip32, ids, z, bary32, triangles, width, height):
  """float32 floor(xy) [L,H,W,2] and surface masks [L, 9, 3, H+2, W+2]."""
  xyz = np_splat.viewport_xyz(clip32, ids, z, bary32, triangles, width, height)
  return np.floor(xyz[..., :2]), discrete_state_xyz(xyz, None)


def discrete_state_xyz(xyz, fg):
  """Surface masks [L, 9, 3, H+2, W+2] of float32 viewport positions: for
  each layer and tap (u, v), one-hot over (in front, at, behind) the
  surface (splat.py:124-154)."""
  xyz = np.asarray(xyz, np.float32)
  L, H, W = xyz.shape[:3]
  zpad = np.pad(xyz[..., 2:3], ((0, 0), (1, 1), (1, 1), (0, 0)), constant_values=1.0)
  masks = np.zeros((L, 9, 3, H + 2, W + 2), np.float32)
  for l in range(L):
    for j, (u, v) in enumerate([(u, v) for u in (-1, 0, 1) for v in (-1, 0, 1)]):
      pad = ((max(v + 1, 0), abs(min(v - 1, 0))), (max(u + 1, 0), abs(min(u - 1, 0))),
             (0, 0))
      tapz = np.pad(xyz[..., 2:3], ((0, 0),) + pad, constant_values=1.0)
      dc = np.abs(tapz - zpad[0])
      dt = np.abs(zpad - tapz[0])
      surf = np.where(np.min(dt, 0) < np.min(dc, 0), -np.argmin(dt, 0), np.argmin(dc, 0))
      masks[l, j] = np.stack([(surf > l), (surf == l), (surf < l)])[..., 0]
  return masks


def _max0(x):
  """max(x, 0) with lax.max's gradient (0.5 at x == 0)."""
  pos = torch.where(x > 0, x, torch.zeros_like(x))
  return pos + torch.where(x == 0, 0.5 * (x - x.detach()), torch.zeros_like(x))


def splat_at_pixel_centers(xyz, color, fg, floors, masks):
  L, H, W, C = color.shape
  dt = color.dtype
  coef = float(np_splat.gaussian_coef())
  acc = torch.zeros(3, H + 2, W + 2, C, dtype=dt, device=color.device)
  wacc = torch.zeros(3, H + 2, W + 2, 1, dtype=dt, device=color.device)
  fl = torch.as_tensor(floors, dtype=dt, device=color.device)
  mk = torch.as_tensor(masks, dtype=dt, device=color.device)
  for l in range(L):
    center = (fl[l] + 0.5) - xyz[l, ..., :2]
    for j, (u, v) in enumerate([(u, v) for u in (-1, 0, 1) for v in (-1, 0, 1)]):
      d = center + torch.tensor([u, v], dtype=dt, device=color.device)
      dist2 = d[..., 0:1] * d[..., 0:1] + d[..., 1:2] * d[..., 1:2]
      w = (fg[l] * coef) * torch.exp(-2.0 * dist2)
      tc = w * color[l]
      pad = (0, 0, max(u + 1, 0), abs(min(u - 1, 0)), max(v + 1, 0), abs(min(v - 1, 0)))
      tc = Fn.pad(tc, pad)
      w = Fn.pad(w, pad)
      m = mk[l, j][..., None]  # [3, H+2, W+2, 1]
      acc = acc + tc[None] * m
      wacc = wacc + w[None] * m
  acc = acc[:, 1:-1, 1:-1, :]
  wacc = wacc[:, 1:-1, 1:-1, :]
  norm = acc * (1.0 / (_max0(wacc - 1.0) + 1.0))
  out = norm[2]
  for i in (1, 0):
    out = norm[i] + (1.0 - norm[i, ..., -1:]) * out
  return out, acc, norm


def splat_shaded_pixels(clip, ids, z, bary, triangles, shaded, width, height, state):
  xyz = viewport_xyz(clip, ids, z, bary, triangles, width, height)
  fg = (z != 1.0).to(clip.dtype)[..., None]
  return splat_at_pixel_centers(xyz, shaded, fg, *state)


def diff_barycentrics(clip, ids, z, triangles, width, height):
  """rasterize.py:127-255 in torch: per-triangle signed cofactors."""
  dt = clip.dtype
  x = (2 * torch.arange(width, device=clip.device) + 1).to(torch.float32) / width - 1
  y = (2 * torch.arange(height, device=clip.device) + 1).to(torch.float32) / height - 1
  py, px = torch.meshgrid(y.to(dt), x.to(dt), indexing="ij")
  v = clip[triangles.long()]  # [T, 3, 4]
  xs, ys, ws = v[..., 0], v[..., 1], v[..., 3]
  x0, x1, x2 = xs.unbind(-1)
  y0, y1, y2 = ys.unbind(-1)
  w0, w1, w2 = ws.unbind(-1)
  d = torch.stack([
      torch.stack([y1 * w2 - y2 * w1, w1 * x2 - w2 * x1, x1 * y2 - x2 * y1], -1),
      torch.stack([y2 * w0 - y0 * w2, w2 * x0 - w0 * x2, x2 * y0 - x0 * y2], -1),
      torch.stack([y0 * w1 - y1 * w0, w0 * x1 - w1 * x0, x0 * y1 - x1 * y0], -1)], -2)
  det = x0 * d[:, 0, 0] + y0 * d[:, 0, 1] + w0 * d[:, 0, 2]
  sign = torch.sign(det) + (det == 0).to(dt)
  m = sign[:, None, None] * d  # [T, 3, 3]
  mp = m[ids.long()]  # [L, H, W, 3, 3]
  u = mp[..., 0] * px[None, ..., None] + mp[..., 1] * py[None, ..., None] + mp[..., 2]
  b = u / u.sum(-1, keepdim=True)
  b = torch.where(torch.isfinite(b), b, torch.nan_to_num(b.detach()))
  return b * (z != 1.0).to(dt)[..., None]
