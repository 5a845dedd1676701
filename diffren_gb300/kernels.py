"""Torch-facing ops over the C ABI: rasterize, transform, interpolate,
differentiable barycentrics and splat, each with its VJP as an
``autograd.Function``.

This is the counterpart of diffren/jax/internal/kernels/
rasterize_triangles_xla.py (the FFI-call layer) extended to every kernel of
the rasterize-then-splat path. Tensors are device tensors; sizes and the
current CUDA stream go to the library through ctypes. The ops work on packed
ragged batches described by an ``ImageBatch``; a single image is a batch of
one.
"""
import contextlib
import ctypes
import threading

import numpy as np
import torch

from . import _lib
from ._lib import ImageDesc, RasterConfig


class _LaunchCounter:
  """Number of this library's kernels enqueued (per op call)."""

  def __init__(self):
    self.count = 0

  def reset(self):
    self.count = 0


LAUNCHES = _LaunchCounter()
_PROFILE = None  # list of (op, start event, end event) while profiling


@contextlib.contextmanager
def _op(name, kernels_launched):
  LAUNCHES.count += kernels_launched
  if _PROFILE is None:
    yield
    return
  e0 = torch.cuda.Event(enable_timing=True)
  e1 = torch.cuda.Event(enable_timing=True)
  e0.record()
  yield
  e1.record()
  _PROFILE.append((name, e0, e1))


def profile_step(step, steps, device):
  """Mean CUDA-event duration (ms) of each op over `steps` eager calls of
  `step`; events are recorded on the launching (current) stream."""
  global _PROFILE
  totals = {}
  for _ in range(steps):
    _PROFILE = []
    try:
      step()
      torch.cuda.synchronize(device)
      for name, e0, e1 in _PROFILE:
        totals[name] = totals.get(name, 0.0) + e0.elapsed_time(e1)
    finally:
      _PROFILE = None
  return {k: v / steps for k, v in totals.items()}


def _groups(batch):
  return (batch.n + _lib.DR_MAX_BATCH_INLINE - 1) // _lib.DR_MAX_BATCH_INLINE


def _p(t):
  return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream(device=None):
  return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _f32(t, device=None):
  t = torch.as_tensor(t, dtype=torch.float32, device=device)
  return t.contiguous()


def _i32(t, device=None):
  t = torch.as_tensor(t, device=device)
  return t.to(torch.int32).contiguous()


def _require_cuda(*ts):
  for t in ts:
    if t is not None and not t.is_cuda:
      raise ValueError("diffren_gb300 ops take CUDA tensors; got a %s tensor"
                       % t.device)


class ImageBatch:
  """Host-side table of a batch of images, each with its own mesh.

  Meshes are packed: vertices of image i are rows
  [vertex_offset[i], vertex_offset[i] + num_vertices[i]) of the packed
  vertex array, triangles likewise (indices local to the mesh). Layered
  per-pixel buffers are packed per image as [L, H_i, W_i] blocks, composited
  images as [H_i, W_i] blocks, in image order.
  """

  def __init__(self, widths, heights, num_vertices, num_triangles):
    n = len(widths)
    if not (len(heights) == len(num_vertices) == len(num_triangles) == n):
      raise ValueError("per-image lists must have the same length")
    self.n = n
    self.widths = [int(w) for w in widths]
    self.heights = [int(h) for h in heights]
    self.num_vertices = [int(v) for v in num_vertices]
    self.num_triangles = [int(t) for t in num_triangles]
    for w, h in zip(self.widths, self.heights):
      if w <= 0 or h <= 0:
        raise ValueError("image width and height must be > 0")
    self.pixel_offsets = np.concatenate(
        [[0], np.cumsum([w * h for w, h in zip(self.widths, self.heights)])])
    self.vertex_offsets = np.concatenate([[0], np.cumsum(self.num_vertices)])
    self.triangle_offsets = np.concatenate([[0], np.cumsum(self.num_triangles)])
    self.total_pixels = int(self.pixel_offsets[-1])
    self.total_vertices = int(self.vertex_offsets[-1])
    self.total_triangles = int(self.triangle_offsets[-1])
    self.descs = (ImageDesc * max(n, 1))()
    for i in range(n):
      d = self.descs[i]
      d.width, d.height = self.widths[i], self.heights[i]
      d.num_vertices, d.num_triangles = self.num_vertices[i], self.num_triangles[i]
      d.vertex_offset = int(self.vertex_offsets[i])
      d.triangle_offset = int(self.triangle_offsets[i])
      d.pixel_offset = int(self.pixel_offsets[i])

  def vertex_image_index(self, device):
    """[sum V] int64 image index of every packed vertex (cached per device)."""
    cache = self.__dict__.setdefault("_vidx", {})
    key = str(device)
    if key not in cache:
      idx = np.repeat(np.arange(self.n), self.num_vertices)
      cache[key] = torch.as_tensor(idx, device=device)
    return cache[key]

  @classmethod
  def single(cls, width, height, num_vertices, num_triangles):
    return cls([width], [height], [num_vertices], [num_triangles])

  @property
  def ptr(self):
    return ctypes.cast(self.descs, ctypes.c_void_p)

  def layered_view(self, flat, i, num_layers):
    """[L, H_i, W_i, ...] view of image i of a packed layered buffer."""
    h, w = self.heights[i], self.widths[i]
    a = int(self.pixel_offsets[i]) * num_layers
    return flat[a:a + num_layers * h * w].view(num_layers, h, w, *flat.shape[1:])

  def image_view(self, flat, i):
    """[H_i, W_i, ...] view of image i of a packed composited buffer."""
    h, w = self.heights[i], self.widths[i]
    a = int(self.pixel_offsets[i])
    return flat[a:a + h * w].view(h, w, *flat.shape[1:])


def raster_config(num_layers, face_culling_mode, depth_mode, tile=(0, 0),
                  large_tiles=0, flags=0):
  c = RasterConfig()
  c.num_layers = int(num_layers)
  c.face_culling_mode = int(face_culling_mode)
  c.depth_mode = int(depth_mode)
  c.tile_width, c.tile_height = int(tile[0]), int(tile[1])
  c.large_tiles = int(large_tiles)
  c.flags = int(flags)
  return c


def foreground_only(config, attributes=False):
  """A copy of `config` with DR_RASTER_FOREGROUND_ONLY set (and, with
  ``attributes``, DR_RASTER_FOREGROUND_ATTRIBUTES)."""
  return raster_config(config.num_layers, config.face_culling_mode, config.depth_mode,
                       (config.tile_width, config.tile_height), config.large_tiles,
                       config.flags | _lib.DR_RASTER_FOREGROUND_ONLY |
                       (_lib.DR_RASTER_FOREGROUND_ATTRIBUTES if attributes else 0))


class Workspace:
  """A growable device scratch buffer for one stream."""

  def __init__(self, device):
    self.device = device
    self.buf = None

  def get(self, nbytes):
    nbytes = max(int(nbytes), 256)
    if self.buf is None or self.buf.numel() < nbytes:
      self.buf = torch.empty(nbytes + (nbytes >> 3), dtype=torch.uint8,
                             device=self.device)
    return self.buf


_ws_lock = threading.Lock()
_workspaces = {}


def default_workspace(device):
  key = (device.index, torch.cuda.current_stream(device).cuda_stream)
  with _ws_lock:
    ws = _workspaces.get(key)
    if ws is None:
      ws = _workspaces[key] = Workspace(device)
  return ws


def raster_workspace_bytes(batch, config):
  lib = _lib.load()
  n = lib.dr_rasterize_batch_workspace_bytes(batch.ptr, batch.n,
                                             ctypes.byref(config))
  if n == 0:
    raise _lib.DiffrenError(lib.dr_last_error().decode())
  return n


def rasterize_packed(clip, triangles, batch, config, workspace=None, out=None):
  """Rasterizes a packed batch. Returns flat (ids [L*P], z [L*P], bary [L*P,3]).

  ``clip`` [sum V, 4] float32 and ``triangles`` [sum T, 3] int32 are CUDA
  tensors; P is the batch's total pixel count.
  """
  _require_cuda(clip, triangles)
  lib = _lib.load()
  dev = clip.device
  L = config.num_layers
  n = L * batch.total_pixels
  if out is None:
    ids = torch.empty(n, dtype=torch.int32, device=dev)
    z = torch.empty(n, dtype=torch.float32, device=dev)
    bary = torch.empty(n, 3, dtype=torch.float32, device=dev)
  else:
    ids, z, bary = out
  need = raster_workspace_bytes(batch, config)
  ws = (workspace or default_workspace(dev)).get(need)
  with torch.cuda.device(dev), _op("raster", 6 * _groups(batch)):
    rc = lib.dr_rasterize_batch(_p(clip), _p(triangles), batch.ptr, batch.n,
                                ctypes.byref(config), _p(ids), _p(z), _p(bary),
                                _p(ws), ws.numel(), _stream(dev))
  _lib.check(rc, "dr_rasterize_batch")
  return ids, z, bary


def read_error_flags(workspace, device):
  lib = _lib.load()
  flags = ctypes.c_uint32(0)
  ws = workspace.buf if isinstance(workspace, Workspace) else workspace
  rc = lib.dr_read_error_flags(_p(ws), ctypes.byref(flags), _stream(device))
  _lib.check(rc, "dr_read_error_flags")
  return flags.value


# ------------------------------------------------------------- transform
class _Transform(torch.autograd.Function):
  """clip = M @ [v, 1] per image (transforms.transform_homogeneous)."""

  @staticmethod
  def forward(ctx, vertices, matrices, batch):
    lib = _lib.load()
    clip = torch.empty(vertices.shape[0], 4, dtype=torch.float32,
                       device=vertices.device)
    if vertices.shape[0] > 0:
      with _op("transform", _groups(batch)):
        rc = lib.dr_transform_vertices(_p(matrices), _p(vertices),
                                       int(vertices.shape[1]), batch.ptr, batch.n,
                                       _p(clip), _stream(vertices.device))
      _lib.check(rc, "dr_transform_vertices")
    ctx.save_for_backward(vertices, matrices)
    ctx.save_for_forward(vertices, matrices)
    ctx.batch = batch
    return clip

  @staticmethod
  def jvp(ctx, d_vertices, d_matrices, _):
    vertices, matrices = ctx.saved_tensors
    batch = ctx.batch
    d_clip = torch.zeros(vertices.shape[0], 4, dtype=torch.float32, device=vertices.device)
    if d_vertices is not None:
      dv = d_vertices.float()
      if dv.shape[1] == 3:  # the tangent of the homogeneous 1 is 0
        dv = torch.cat([dv, torch.zeros_like(dv[:, :1])], 1)
      d_clip = _Transform.apply(dv.contiguous(), matrices, batch)
    if d_matrices is not None:
      idx = batch.vertex_image_index(vertices.device)
      vh = vertices if vertices.shape[1] == 4 else torch.cat(
          [vertices, torch.ones_like(vertices[:, :1])], dim=1)
      d_clip = d_clip + torch.einsum("vj,vij->vi", vh, d_matrices.float()[idx])
    return d_clip

  @staticmethod
  def backward(ctx, d_clip):
    vertices, matrices = ctx.saved_tensors
    batch = ctx.batch
    dim = vertices.shape[1]
    d_clip = d_clip.contiguous()
    d_v = d_m = None
    # Per image: clip_i = v_h @ M_i^T -> d v_h = d_clip @ M_i, d M_i = d^T v_h.
    if ctx.needs_input_grad[0]:
      d_v = torch.empty_like(vertices)
      with _op("transform_bwd", _groups(batch)):
        rc = _lib.load().dr_transform_vertices_bwd(_p(matrices), _p(d_clip), dim,
                                                 batch.ptr, batch.n, _p(d_v),
                                                 _stream(vertices.device))
      _lib.check(rc, "dr_transform_vertices_bwd")
    if ctx.needs_input_grad[1]:
      idx = batch.vertex_image_index(vertices.device)
      vh = vertices if dim == 4 else torch.cat(
          [vertices, torch.ones_like(vertices[:, :1])], dim=1)
      outer = d_clip[:, :, None] * vh[:, None, :]
      d_m = torch.zeros_like(matrices).index_add_(0, idx, outer)
    return d_v, d_m, None


def transform(vertices, matrices, batch):
  """Clip-space vertices [sum V, 4] of a packed batch (one matrix per image)."""
  vertices = _f32(vertices)
  matrices = _f32(matrices).reshape(batch.n, 4, 4)
  _require_cuda(vertices, matrices)
  if vertices.shape[1] not in (3, 4):
    raise ValueError("vertices must be [n, 3] or [n, 4]")
  return _Transform.apply(vertices, matrices, batch)


# ---------------------------------------------------------- interpolation
class _Interpolate(torch.autograd.Function):

  @staticmethod
  def forward(ctx, attributes, bary, background, triangles, ids, z, batch, L):
    lib = _lib.load()
    K = attributes.shape[1]
    out = torch.empty(ids.shape[0], K, dtype=torch.float32, device=ids.device)
    with _op("interp_fwd", _groups(batch)):
      rc = lib.dr_interpolate_fwd(_p(attributes), K, _p(triangles), _p(ids), _p(z),
                                _p(bary), _p(background), batch.ptr, batch.n, L,
                                _p(out), _stream(ids.device))
    _lib.check(rc, "dr_interpolate_fwd")
    ctx.save_for_backward(attributes, bary, triangles, ids, z)
    ctx.save_for_forward(attributes, bary, triangles, ids, z)
    ctx.batch, ctx.L, ctx.has_bg = batch, L, background is not None
    return out

  @staticmethod
  def jvp(ctx, d_attr, d_bary, d_bg, *unused):
    """fg (sum_i b_i a_i) + (1 - fg) bg is linear in the attributes, the
    barycentrics and the background separately."""
    attributes, bary, triangles, ids, z = ctx.saved_tensors
    batch, L = ctx.batch, ctx.L
    out = torch.zeros(ids.shape[0], attributes.shape[1], dtype=torch.float32,
                      device=ids.device)
    if d_attr is not None:
      out = out + _Interpolate.apply(d_attr.detach().float().contiguous(), bary, None,
                                     triangles, ids, z, batch, L)
    if d_bary is not None:
      out = out + _Interpolate.apply(attributes, d_bary.detach().float().contiguous(), None,
                                     triangles, ids, z, batch, L)
    if d_bg is not None:
      out = out + (z == 1.0).float()[:, None] * d_bg.detach().float()
    return out

  @staticmethod
  def backward(ctx, d_out):
    attributes, bary, triangles, ids, z = ctx.saved_tensors
    lib = _lib.load()
    d_out = d_out.contiguous()
    d_attr = torch.zeros_like(attributes)
    d_bary = torch.empty_like(bary) if ctx.needs_input_grad[1] else None
    d_bg = (torch.zeros(attributes.shape[1], device=attributes.device)
            if ctx.has_bg and ctx.needs_input_grad[2] else None)
    with _op("interp_bwd", _groups(ctx.batch)):
      rc = lib.dr_interpolate_bwd(_p(d_out), _p(attributes), attributes.shape[1],
                                _p(triangles), _p(ids), _p(z), _p(bary),
                                ctx.batch.ptr, ctx.batch.n, ctx.L, _p(d_attr),
                                _p(d_bary), _p(d_bg), _stream(d_out.device))
    _lib.check(rc, "dr_interpolate_bwd")
    return d_attr, d_bary, d_bg, None, None, None, None, None


def interpolate_packed(attributes, bary, triangles, ids, z, batch, num_layers,
                       background=None):
  """Interpolated attributes [L*P, K] of a packed batch."""
  attributes = _f32(attributes)
  if attributes.shape[1] > _lib.DR_MAX_CHANNELS:
    parts = torch.split(attributes, _lib.DR_MAX_CHANNELS, dim=1)
    bgs = (torch.split(_f32(background, attributes.device), _lib.DR_MAX_CHANNELS)
           if background is not None else [None] * len(parts))
    return torch.cat([
        interpolate_packed(a, bary, triangles, ids, z, batch, num_layers, b)
        for a, b in zip(parts, bgs)], dim=1)
  if background is not None:
    background = _f32(background, attributes.device).reshape(-1)
  return _Interpolate.apply(attributes, bary, background, triangles, ids, z,
                            batch, num_layers)


# ------------------------------------------- differentiable barycentrics
class _DiffBary(torch.autograd.Function):

  @staticmethod
  def forward(ctx, clip, triangles, ids, z, batch, L):
    lib = _lib.load()
    bary = torch.empty(ids.shape[0], 3, dtype=torch.float32, device=ids.device)
    with _op("diffbary_fwd", _groups(batch)):
      rc = lib.dr_diff_barycentrics_fwd(_p(clip), _p(triangles), _p(ids), _p(z),
                                      batch.ptr, batch.n, L, _p(bary),
                                      _stream(ids.device))
    _lib.check(rc, "dr_diff_barycentrics_fwd")
    ctx.save_for_backward(clip, triangles, ids, z)
    ctx.save_for_forward(clip, triangles, ids, z)
    ctx.batch, ctx.L = batch, L
    return bary

  @staticmethod
  def jvp(ctx, d_clip, *unused):
    """Tangent of the barycentrics (rasterize.py:127-255) for clip-vertex
    tangents, image by image in torch ops: the adjugate's cofactors by the
    product rule, u = M p, b = u / sum(u) by the quotient rule (0 where the
    barycentrics are not finite). Forward mode only; the VJP kernel serves
    reverse mode."""
    clip, triangles, ids, z = ctx.saved_tensors
    batch, L = ctx.batch, ctx.L
    out = torch.zeros(ids.shape[0], 3, dtype=torch.float32, device=ids.device)
    if d_clip is None:
      return out
    for i in range(batch.n):
      W, H = batch.widths[i], batch.heights[i]
      desc = batch.descs[i]
      v0, nv = int(desc.vertex_offset), int(desc.num_vertices)
      t0, nt = int(desc.triangle_offset), int(desc.num_triangles)
      if nt == 0 or nv == 0:
        continue
      ids_i = batch.layered_view(ids, i, L).reshape(-1).long().clamp(0, nt - 1)
      fg = (batch.layered_view(z, i, L).reshape(-1) != 1.0)[:, None].float()
      pix = torch.arange(L * H * W, device=ids.device) % (H * W)
      px = ((2 * (pix % W) + 1).float() / W - 1.0)[:, None]
      py = ((2 * (pix // W) + 1).float() / H - 1.0)[:, None]
      tri = triangles[t0:t0 + nt].long()

      v = clip[v0:v0 + nv][tri]  # [T, 3, 4]
      dv = d_clip[v0:v0 + nv].float()[tri]

      def cof(a, b, c, e, da, db_, dc, de):
        """a b - c e and its tangent."""
        return a * b - c * e, da * b + a * db_ - dc * e - c * de

      x, y, w = v[..., 0].unbind(-1), v[..., 1].unbind(-1), v[..., 3].unbind(-1)
      dx, dy, dw = dv[..., 0].unbind(-1), dv[..., 1].unbind(-1), dv[..., 3].unbind(-1)
      rows, drows = [], []
      for i0, i1, i2 in ((0, 1, 2), (1, 2, 0), (2, 0, 1)):
        # row i0 of the adjugate of [x; y; w] (cofactors of the other two)
        e0 = cof(y[i1], w[i2], y[i2], w[i1], dy[i1], dw[i2], dy[i2], dw[i1])
        e1 = cof(w[i1], x[i2], w[i2], x[i1], dw[i1], dx[i2], dw[i2], dx[i1])
        e2 = cof(x[i1], y[i2], x[i2], y[i1], dx[i1], dy[i2], dx[i2], dy[i1])
        rows.append(torch.stack([e0[0], e1[0], e2[0]], -1))
        drows.append(torch.stack([e0[1], e1[1], e2[1]], -1))
      d = torch.stack(rows, -2)
      dd = torch.stack(drows, -2)
      det = x[0] * d[:, 0, 0] + y[0] * d[:, 0, 1] + w[0] * d[:, 0, 2]
      sign = torch.sign(det) + (det == 0).float()  # locally constant
      m = (sign[:, None, None] * d)[ids_i]
      dm = (sign[:, None, None] * dd)[ids_i]
      u = m[..., 0] * px + m[..., 1] * py + m[..., 2]
      du = dm[..., 0] * px + dm[..., 1] * py + dm[..., 2]
      total = u.sum(-1, keepdim=True)
      bary = u / total
      db = (du - bary * du.sum(-1, keepdim=True)) / total
      db = torch.where(torch.isfinite(bary) & torch.isfinite(db), db, torch.zeros_like(db))
      db = db * fg
      dst = batch.layered_view(out, i, L)
      dst.copy_(db.view_as(dst))
    return out

  @staticmethod
  def backward(ctx, d_bary):
    clip, triangles, ids, z = ctx.saved_tensors
    lib = _lib.load()
    d_clip = torch.zeros_like(clip)
    with _op("diffbary_bwd", _groups(ctx.batch)):
      rc = lib.dr_diff_barycentrics_bwd(_p(d_bary.contiguous()), _p(clip),
                                      _p(triangles), _p(ids), _p(z), ctx.batch.ptr,
                                      ctx.batch.n, ctx.L, _p(d_clip),
                                      _stream(clip.device))
    _lib.check(rc, "dr_diff_barycentrics_bwd")
    return d_clip, None, None, None, None, None


def diff_barycentrics_packed(clip, triangles, ids, z, batch, num_layers):
  return _DiffBary.apply(clip, triangles, ids, z, batch, num_layers)


# --------------------------------------- fused attributes + splat positions
class _Samples(torch.autograd.Function):
  """interpolate (background 0) and splat positions in one pass per sample."""

  @staticmethod
  def forward(ctx, attributes, clip, bary, triangles, ids, z, batch, L):
    lib = _lib.load()
    K = attributes.shape[1]
    out = torch.empty(ids.shape[0], K, dtype=torch.float32, device=ids.device)
    vp = torch.empty(ids.shape[0], 4, dtype=torch.float32, device=ids.device)
    with _op("samples_fwd", _groups(batch)):
      rc = lib.dr_interpolate_with_positions_fwd(
          _p(attributes), K, _p(clip), _p(triangles), _p(ids), _p(z), _p(bary),
          batch.ptr, batch.n, L, _p(out), _p(vp), _stream(ids.device))
    _lib.check(rc, "dr_interpolate_with_positions_fwd")
    ctx.save_for_backward(attributes, clip, bary, triangles, ids, z)
    ctx.batch, ctx.L = batch, L
    ctx.set_materialize_grads(False)
    return out, vp

  @staticmethod
  def backward(ctx, d_out, d_vp):
    attributes, clip, bary, triangles, ids, z = ctx.saved_tensors
    d_attr, d_clip, d_bary = _samples_vjp(ctx, d_out, d_vp, attributes, clip, bary,
                                          triangles, ids, z, ctx.needs_input_grad[2],
                                          None, None)
    return (d_attr if ctx.needs_input_grad[0] else None,
            d_clip if ctx.needs_input_grad[1] else None,
            d_bary, None, None, None, None, None)


def _samples_vjp(ctx, d_out, d_vp, attributes, clip, bary, triangles, ids, z, want_bary,
                 positions, vertex_ids):
  """(d attributes, d clip, d barycentrics or None) of the fused pass;
  `positions` (w = clip w) and `vertex_ids` from the fused rasterizer, or
  None."""
  lib = _lib.load()
  if d_out is None and d_vp is None:
    return None, None, None
  if d_out is not None:
    d_out = d_out.contiguous()
  if d_vp is not None:
    d_vp = d_vp.contiguous()
    if d_vp.data_ptr() % 16:
      d_vp = d_vp.clone()
  # Both gradients accumulate (atomics) into one zeroed buffer: one fill.
  na, nc = attributes.numel(), clip.numel()
  na_pad = (na + 3) & ~3  # keeps d_clip 16-byte aligned
  zeros = torch.zeros(na_pad + nc, dtype=torch.float32, device=clip.device)
  d_attr = zeros[:na].view_as(attributes)
  d_clip = zeros[na_pad:].view_as(clip)
  d_bary = torch.empty_like(bary) if want_bary else None
  deterministic = getattr(ctx, "deterministic", False)
  flags, scratch, launches = 0, None, _groups(ctx.batch)
  if deterministic:
    flags = _lib.DR_SAMPLES_DETERMINISTIC
    nbytes = lib.dr_interpolate_with_positions_bwd_scratch_bytes(
        ctx.batch.ptr, ctx.batch.n, attributes.shape[1])
    scratch = torch.empty(nbytes, dtype=torch.uint8, device=clip.device)
    launches = 2 * _groups(ctx.batch) + 1
  with _op("samples_bwd", launches):
    rc = lib.dr_interpolate_with_positions_bwd_ex(
        _p(d_out), _p(d_vp), _p(attributes), attributes.shape[1], _p(clip),
        _p(triangles), _p(ids), _p(z), _p(bary), _p(positions), _p(vertex_ids),
        ctx.batch.ptr, ctx.batch.n, ctx.L, flags, _p(d_attr), _p(d_clip), _p(d_bary),
        _p(scratch), 0 if scratch is None else scratch.numel(), _stream(clip.device))
  _lib.check(rc, "dr_interpolate_with_positions_bwd_ex")
  return d_attr, d_clip, d_bary


def _viewport_tangent(q, dc, z, batch, L, w_from_vp):
  """Tangent of the splat positions vp = ((c.xyz / c.w) + 1) (W, H, 1) / 2
  (splat.py:207-221) for a tangent dc of the interpolated clip position c:
  d vp.xyz = (dc.xyz - ndc dc.w) / c.w (W, H, 1) / 2; background samples get
  0. With w_from_vp, q is the fused rasterizer's positions (viewport xyz,
  clip w); otherwise q is the interpolated clip position c itself. The
  tangent's w is dc.w (the clip w) with w_from_vp, else 0 (the foreground
  flag)."""
  d_vp = torch.zeros(q.shape[0], 4, dtype=torch.float32, device=q.device)
  for i in range(batch.n):
    half = torch.tensor([batch.widths[i] * 0.5, batch.heights[i] * 0.5, 0.5],
                        dtype=torch.float32, device=q.device)
    qi = batch.layered_view(q, i, L).reshape(-1, 4)
    d = batch.layered_view(dc, i, L).reshape(-1, 4)
    fg = (batch.layered_view(z, i, L).reshape(-1) != 1.0)[:, None]
    w = torch.where(fg, qi[:, 3:4], torch.ones_like(qi[:, 3:4]))
    ndc = qi[:, :3] / half - 1.0 if w_from_vp else qi[:, :3] / w
    t = (d[:, :3] - ndc * d[:, 3:4]) / w * half
    t = torch.cat([t, d[:, 3:4] if w_from_vp else torch.zeros_like(t[:, :1])], 1)
    t = torch.where(fg, t, torch.zeros_like(t))
    dst = batch.layered_view(d_vp, i, L)
    dst.copy_(t.view_as(dst))
  return d_vp


class _RasterSamples(torch.autograd.Function):
  """Rasterization fused with attribute interpolation and splat positions;
  the VJP is that of the fused pass (the rasterizer's own outputs carry no
  gradient, as in the reference).

  With ``recompute`` the forward keeps for the VJP only what the splat
  keeps anyway (depth and positions) plus the inputs: the triangle ids,
  barycentrics and vertex ids (28 bytes per layer sample) are not stored
  but recomputed in the backward by running the rasterizer again, which
  gives the same bits. This trades one rasterizer pass for memory."""

  @staticmethod
  def forward(ctx, attributes, clip, triangles, batch, config, workspace, recompute=False,
              deterministic=False):
    lib = _lib.load()
    dev = clip.device
    L = config.num_layers
    n = L * batch.total_pixels
    K = attributes.shape[1]
    ids = torch.empty(n, dtype=torch.int32, device=dev)
    z = torch.empty(n, dtype=torch.float32, device=dev)
    bary = torch.empty(n, 3, dtype=torch.float32, device=dev)
    out = torch.empty(n, K, dtype=torch.float32, device=dev)
    vp = torch.empty(n, 4, dtype=torch.float32, device=dev)
    vids = None if recompute else torch.empty(n, 3, dtype=torch.int32, device=dev)
    ws = workspace.get(raster_workspace_bytes(batch, config))
    with torch.cuda.device(dev), _op("raster", 6 * _groups(batch)):
      rc = lib.dr_rasterize_batch_interpolate(
          _p(clip), _p(triangles), batch.ptr, batch.n, ctypes.byref(config), _p(ids), _p(z),
          _p(bary), _p(attributes), K, _p(out), _p(vp), _p(vids), _p(ws), ws.numel(),
          _stream(dev))
    _lib.check(rc, "dr_rasterize_batch_interpolate")
    ctx.recompute = bool(recompute)
    ctx.deterministic = bool(deterministic)
    if recompute:
      ctx.save_for_backward(attributes, clip, triangles, z, vp)
      ctx.config, ctx.workspace = config, workspace
    else:
      ctx.save_for_backward(attributes, clip, bary, triangles, ids, z, vp, vids)
    ctx.save_for_forward(bary, triangles, ids, z, vp)
    ctx.batch, ctx.L, ctx.num_channels = batch, L, K
    ctx.set_materialize_grads(False)
    ctx.mark_non_differentiable(ids, z, bary)
    return out, vp, ids, z, bary

  @staticmethod
  def jvp(ctx, d_attributes, d_clip, *unused):
    """Tangents of the interpolated attributes and the splat positions at
    fixed barycentrics (the rasterizer's outputs carry no derivative)."""
    bary, triangles, ids, z, vp = ctx.saved_tensors
    batch, L = ctx.batch, ctx.L
    n = ids.shape[0]
    K = ctx.num_channels
    if d_attributes is not None:
      d_out = interpolate_packed(d_attributes.detach(), bary, triangles, ids, z, batch, L)
    else:
      d_out = torch.zeros(n, K, dtype=torch.float32, device=ids.device)
    if d_clip is not None:
      dc = interpolate_packed(d_clip.detach(), bary, triangles, ids, z, batch, L)
      # vp.w holds the clip w here, and xyz/w = 2 vp.xyz / (W, H, 1) - 1.
      d_vp = _viewport_tangent(vp, dc, z, batch, L, w_from_vp=True)
    else:
      d_vp = torch.zeros(n, 4, dtype=torch.float32, device=ids.device)
    return d_out, d_vp, None, None, None

  @staticmethod
  def backward(ctx, d_out, d_vp, *unused):
    if ctx.recompute:
      attributes, clip, triangles, z, vp = ctx.saved_tensors
      ids, bary, vids = _rerasterize(ctx, clip, triangles)
    else:
      attributes, clip, bary, triangles, ids, z, vp, vids = ctx.saved_tensors
    d_attr, d_clip, _ = _samples_vjp(ctx, d_out, d_vp, attributes, clip, bary, triangles,
                                     ids, z, False, vp, vids)
    return (d_attr if ctx.needs_input_grad[0] else None,
            d_clip if ctx.needs_input_grad[1] else None, None, None, None, None, None, None)


def _rerasterize(ctx, clip, triangles):
  """The forward's triangle ids, barycentrics and vertex ids, recomputed
  (the rasterizer is deterministic: same inputs, same bits)."""
  lib = _lib.load()
  dev = clip.device
  n = ctx.L * ctx.batch.total_pixels
  ids = torch.empty(n, dtype=torch.int32, device=dev)
  z = torch.empty(n, dtype=torch.float32, device=dev)
  bary = torch.empty(n, 3, dtype=torch.float32, device=dev)
  vp = torch.empty(n, 4, dtype=torch.float32, device=dev)
  vids = torch.empty(n, 3, dtype=torch.int32, device=dev)
  ws = ctx.workspace.get(raster_workspace_bytes(ctx.batch, ctx.config))
  with torch.cuda.device(dev), _op("raster_recompute", 6 * _groups(ctx.batch)):
    rc = lib.dr_rasterize_batch_interpolate(
        _p(clip), _p(triangles), ctx.batch.ptr, ctx.batch.n, ctypes.byref(ctx.config),
        _p(ids), _p(z), _p(bary), None, 0, None, _p(vp), _p(vids), _p(ws), ws.numel(),
        _stream(dev))
  _lib.check(rc, "dr_rasterize_batch_interpolate")
  return ids, bary, vids


def rasterize_interpolate_packed(attributes, clip, triangles, batch, config, workspace,
                                 recompute=False, deterministic=False):
  """Rasterizes a packed batch and, in the same pass, interpolates
  ``attributes`` [sum V, K <= 16] (background 0) and computes the splat
  positions. Returns (attributes [L*P, K], positions [L*P, 4], ids, z, bary);
  the first two are differentiable w.r.t. ``attributes`` and ``clip``.
  Positions are written for foreground samples only, as (viewport xyz,
  clip w): splat them with ``z`` so that the depth buffer marks the
  background. With ``recompute`` the VJP reruns the rasterizer instead of
  keeping ids, barycentrics and vertex ids from the forward. With
  ``deterministic`` the VJP sums the vertex gradients in fixed point, so
  they are the same bits on every run."""
  _require_cuda(clip, triangles)
  attributes = _f32(attributes)
  if attributes.shape[1] > _lib.DR_MAX_CHANNELS:
    raise ValueError("at most %d attribute channels" % _lib.DR_MAX_CHANNELS)
  return _RasterSamples.apply(attributes, clip, triangles, batch, config, workspace,
                              bool(recompute), bool(deterministic))


def interpolate_with_positions_packed(attributes, clip, bary, triangles, ids, z, batch,
                                      num_layers):
  """(interpolated attributes [L*P, K] with background 0, splat positions
  [L*P, 4]) of a packed batch, in one pass when K <= 16."""
  attributes = _f32(attributes)
  if attributes.shape[1] > _lib.DR_MAX_CHANNELS:
    return (interpolate_packed(attributes, bary, triangles, ids, z, batch, num_layers),
            splat_positions_packed(clip, bary, triangles, ids, z, batch, num_layers))
  return _Samples.apply(attributes, clip, bary, triangles, ids, z, batch, num_layers)


# ------------------------------------------------------------------ splat
class _Positions(torch.autograd.Function):
  """Viewport xyz + foreground flag of every layer sample (splat.py:207-221)."""

  @staticmethod
  def forward(ctx, clip, bary, triangles, ids, z, batch, L):
    lib = _lib.load()
    vp = torch.empty(ids.shape[0], 4, dtype=torch.float32, device=ids.device)
    with _op("splat_positions", _groups(batch)):
      rc = lib.dr_splat_positions_fwd(_p(clip), _p(triangles), _p(ids), _p(z), _p(bary),
                                      batch.ptr, batch.n, L, _p(vp), _stream(ids.device))
    _lib.check(rc, "dr_splat_positions_fwd")
    ctx.save_for_backward(clip, bary, triangles, ids, z)
    ctx.save_for_forward(clip, bary, triangles, ids, z)
    ctx.batch, ctx.L = batch, L
    return vp

  @staticmethod
  def jvp(ctx, d_clip, d_bary, *unused):
    clip, bary, triangles, ids, z = ctx.saved_tensors
    batch, L = ctx.batch, ctx.L
    c = interpolate_packed(clip, bary, triangles, ids, z, batch, L)
    dc = torch.zeros_like(c)
    if d_clip is not None:
      dc = dc + interpolate_packed(d_clip.detach(), bary, triangles, ids, z, batch, L)
    if d_bary is not None:
      dc = dc + interpolate_packed(clip, d_bary.detach().contiguous(), triangles, ids, z,
                                   batch, L)
    return _viewport_tangent(c, dc, z, batch, L, w_from_vp=False)

  @staticmethod
  def backward(ctx, d_vp):
    clip, bary, triangles, ids, z = ctx.saved_tensors
    lib = _lib.load()
    d_vp = d_vp.contiguous()
    if d_vp.data_ptr() % 16:
      d_vp = d_vp.clone()
    d_clip = torch.zeros_like(clip) if ctx.needs_input_grad[0] else None
    d_bary = torch.empty_like(bary) if ctx.needs_input_grad[1] else None
    if d_clip is None and d_bary is None:
      return None, None, None, None, None, None, None
    scratch = d_clip if d_clip is not None else torch.zeros_like(clip)
    with _op("splat_positions_bwd", _groups(ctx.batch)):
      rc = lib.dr_splat_positions_bwd(_p(d_vp), _p(clip), _p(triangles), _p(ids), _p(z),
                                      _p(bary), ctx.batch.ptr, ctx.batch.n, ctx.L,
                                      _p(scratch), _p(d_bary), _stream(d_vp.device))
    _lib.check(rc, "dr_splat_positions_bwd")
    return d_clip, d_bary, None, None, None, None, None


def splat_positions_packed(clip, bary, triangles, ids, z, batch, num_layers):
  """[L*P, 4] viewport positions (x, y, z, fg) of a packed batch."""
  return _Positions.apply(clip, bary, triangles, ids, z, batch, num_layers)


class _Splat(torch.autograd.Function):

  @staticmethod
  def forward(ctx, positions, colors, z, batch, L, want_accum, fg_grads=False):
    lib = _lib.load()
    C = colors.shape[1]
    dev = colors.device
    P = batch.total_pixels
    out = torch.empty(P, C, dtype=torch.float32, device=dev)
    needs_grad = positions.requires_grad or colors.requires_grad
    saved = (torch.empty(3 * (C + 1) + 2, P, dtype=torch.float32, device=dev)
             if needs_grad else None)
    accum = norm = None
    if want_accum:
      accum = torch.empty(3 * P, C, dtype=torch.float32, device=dev)
      norm = torch.empty_like(accum)
    with _op("splat_fwd", _splat_launches(batch, saved is not None and z is not None and
                                          not want_accum)):
      rc = lib.dr_splat_fwd(_p(positions), _p(z), _p(colors), C, batch.ptr, batch.n, L,
                            _p(out), _p(saved), _p(accum), _p(norm), _stream(dev))
    _lib.check(rc, "dr_splat_fwd")
    ctx.save_for_backward(positions, colors, saved, z)
    ctx.save_for_forward(positions, colors, z)
    ctx.batch, ctx.L = batch, L
    ctx.want_accum = want_accum
    ctx.fg_grads = bool(fg_grads) and z is not None
    if want_accum:
      ctx.mark_non_differentiable(accum, norm)
      return out, accum, norm
    return out

  @staticmethod
  def jvp(ctx, d_positions, d_colors, *unused):
    """Tangent of the image (discrete state held fixed), by dr_splat_jvp."""
    positions, colors, z = ctx.saved_tensors
    lib = _lib.load()
    C = colors.shape[1]
    d_image = torch.empty(ctx.batch.total_pixels, C, dtype=torch.float32, device=colors.device)
    dp = d_positions.float().contiguous() if d_positions is not None else None
    dc = d_colors.float().contiguous() if d_colors is not None else None
    with _op("splat_jvp", _groups(ctx.batch)):
      rc = lib.dr_splat_jvp(_p(positions), _p(z), _p(colors), _p(dp), _p(dc), C, ctx.batch.ptr,
                            ctx.batch.n, ctx.L, _p(d_image), _stream(colors.device))
    _lib.check(rc, "dr_splat_jvp")
    if ctx.want_accum:
      return d_image, None, None
    return d_image

  @staticmethod
  def backward(ctx, d_out, *unused):
    positions, colors, saved, z = ctx.saved_tensors
    lib = _lib.load()
    d_out = d_out.contiguous()
    if d_out.data_ptr() % 16:
      d_out = d_out.clone()
    d_colors = torch.empty_like(colors)
    d_pos = torch.empty_like(positions)
    flags = _lib.DR_SPLAT_FOREGROUND_GRADIENTS if ctx.fg_grads else 0
    with _op("splat_bwd", _splat_launches(ctx.batch, z is not None)):
      rc = lib.dr_splat_bwd_ex(_p(d_out), _p(positions), _p(z), _p(colors), _p(saved),
                               colors.shape[1], ctx.batch.ptr, ctx.batch.n, ctx.L, flags,
                               _p(d_colors), _p(d_pos), _stream(d_out.device))
    _lib.check(rc, "dr_splat_bwd_ex")
    return (d_pos if ctx.needs_input_grad[0] else None,
            d_colors if ctx.needs_input_grad[1] else None, None, None, None, None, None)


def split_channels(t, widths, dim=-1):
  """The per-attribute views of a packed [.., sum(widths)] tensor. One
  attribute is the tensor itself: torch.split's backward would copy the
  whole gradient to concatenate a single piece."""
  if len(widths) == 1:
    return (t,)
  return torch.split(t, list(widths), dim=dim)


def _splat_launches(batch, listed):
  """Kernels one splat call launches: with saved accumulators and a depth
  buffer (and a batch of at most DR_MAX_BATCH_INLINE images whose tile list
  fits its plane) a classifying (or zeroing) kernel plus the kernel over the
  listed tiles, else one kernel per group of images."""
  if listed and batch.n <= _lib.DR_MAX_BATCH_INLINE:
    tiles = sum(((w + 31) // 32) * ((h + 7) // 8) for w, h in zip(batch.widths, batch.heights))
    if 16 + ((4 * tiles + 15) & ~15) + tiles <= 4 * batch.total_pixels:
      return 2
  return _groups(batch)


def splat_packed(positions, colors, batch, num_layers, return_accum_buffers=False, z=None,
                 foreground_gradients=False):
  """Splatted, normalized, composited images [P, C] of a packed batch.

  positions [L*P, 4] (viewport xyz, fg) and colors [L*P, C]. ``z`` [L*P],
  the rasterizer's depth, marks background samples (z == 1), whose
  positions are then not read (nor their position gradients written). With
  ``return_accum_buffers`` also returns the accumulated and normalized
  fg/surface/bg layers, packed [3, H_i, W_i, C] per image (not
  differentiable). ``foreground_gradients`` (with ``z``): the color
  gradient of background samples is left unwritten, for colors whose VJP
  reads foreground samples only (the rasterizer's fused interpolation).
  """
  colors = colors.contiguous()
  if colors.dtype != torch.float32:
    colors = colors.float()
  if colors.data_ptr() % 16:
    colors = colors.clone()
  if colors.shape[1] > _lib.DR_MAX_SPLAT_CHANNELS:
    raise ValueError("splatting supports at most %d channels" %
                     _lib.DR_MAX_SPLAT_CHANNELS)
  positions = positions.contiguous()
  if z is not None:
    z = z.detach().contiguous()
  return _Splat.apply(positions, colors, z, batch, num_layers, bool(return_accum_buffers),
                      bool(foreground_gradients))


class _Over(torch.autograd.Function):

  @staticmethod
  def forward(ctx, shaded, z, batch, num_layers):
    lib = _lib.load()
    C = shaded.shape[1]
    out = torch.empty(batch.total_pixels, C, dtype=torch.float32, device=shaded.device)
    with _op("composite_over", _groups(batch)):
      rc = lib.dr_composite_over_fwd(_p(shaded), _p(z), C, batch.ptr, batch.n, num_layers,
                                     _p(out), _stream(shaded.device))
    _lib.check(rc, "dr_composite_over_fwd")
    ctx.save_for_backward(shaded, z)
    ctx.batch, ctx.L = batch, num_layers
    return out

  @staticmethod
  def backward(ctx, d_out):
    shaded, z = ctx.saved_tensors
    if not ctx.needs_input_grad[0]:
      return None, None, None, None
    lib = _lib.load()
    d_shaded = torch.empty_like(shaded)
    with _op("composite_over_bwd", _groups(ctx.batch)):
      rc = lib.dr_composite_over_bwd(_p(d_out.contiguous()), _p(shaded), _p(z),
                                     shaded.shape[1], ctx.batch.ptr, ctx.batch.n, ctx.L,
                                     _p(d_shaded), _stream(d_out.device))
    _lib.check(rc, "dr_composite_over_bwd")
    return d_shaded, None, None, None


def over_packed(shaded, z, batch, num_layers):
  """CompositingMode.OVER of a packed batch (render.py:134-140): shaded
  [L*P, C] (alpha last) times the foreground mask z != 1, composited front
  to back per pixel (composite.py:20-37). Returns [P, C]; differentiable
  w.r.t. shaded."""
  _require_cuda(shaded, z)
  shaded = shaded.contiguous()
  if shaded.dtype != torch.float32:
    shaded = shaded.float()
  return _Over.apply(shaded, z.detach().contiguous(), batch, int(num_layers))
