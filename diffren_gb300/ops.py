"""torch.library custom ops over the C ABI: the torch adapter of the
rasterize-then-splat path, for callers that want PyTorch operators
(`torch.ops.diffren_gb300.*`, visible to torch.compile and FakeTensor
tracing) rather than the Python API.

* ``rasterize_triangles`` mirrors rasterize_triangles_xla.rasterize_triangles
  (diffren/jax/internal/rasterize_triangles_xla.py:32-78): clip vertices
  [V, 4], triangles [T, 3] -> ids [L, H, W] int32, z [L, H, W], barycentrics
  [L, H, W, 3]; no gradient (as the reference's FFI op).
* ``splat`` is splat_at_pixel_centers + composite.over (splat.py:26-175,
  composite.py:20-37) on rasterized samples: positions [L, H, W, 4]
  (viewport xyz), colors [L, H, W, C], z_buffer [L, H, W] (1 = background)
  -> [H, W, C]; differentiable w.r.t. positions (x, y) and colors, with the
  gather-form VJP kernel.
"""
from typing import Tuple

import torch

from . import _lib
from . import kernels

_NS = "diffren_gb300"


def _single(width, height, num_vertices=0, num_triangles=0):
  return kernels.ImageBatch.single(width, height, num_vertices, num_triangles)


@torch.library.custom_op(_NS + "::rasterize_triangles", mutates_args=())
def rasterize_triangles(clip_vertices: torch.Tensor, triangles: torch.Tensor, width: int,
                        height: int, num_layers: int, face_culling_mode: int,
                        depth_mode: int) -> Tuple[torch.Tensor, torch.Tensor, torch.Tensor]:
  clip = kernels._f32(clip_vertices)
  tris = kernels._i32(triangles)
  batch = _single(width, height, clip.shape[0], tris.shape[0])
  cfg = kernels.raster_config(num_layers, face_culling_mode, depth_mode)
  ids, z, bary = kernels.rasterize_packed(clip, tris, batch, cfg)
  return (ids.view(num_layers, height, width), z.view(num_layers, height, width),
          bary.view(num_layers, height, width, 3))


@rasterize_triangles.register_fake
def _(clip_vertices, triangles, width, height, num_layers, face_culling_mode, depth_mode):
  shape = (num_layers, height, width)
  return (clip_vertices.new_empty(shape, dtype=torch.int32), clip_vertices.new_empty(shape),
          clip_vertices.new_empty(shape + (3,)))


@torch.library.custom_op(_NS + "::splat_fwd", mutates_args=())
def splat_fwd(positions: torch.Tensor, colors: torch.Tensor,
              z_buffer: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
  """(image [H, W, C], saved accumulators, surface codes and tile list [3 (C + 1) + 2, H * W])."""
  L, H, W, C = colors.shape
  lib = _lib.load()
  batch = _single(W, H)
  pos = positions.reshape(-1, 4).contiguous()
  col = colors.reshape(-1, C).contiguous()
  z = z_buffer.reshape(-1).contiguous()
  out = torch.empty(H, W, C, dtype=torch.float32, device=colors.device)
  saved = torch.empty(3 * (C + 1) + 2, H * W, dtype=torch.float32, device=colors.device)
  rc = lib.dr_splat_fwd(kernels._p(pos), kernels._p(z), kernels._p(col), C, batch.ptr, 1, L,
                        kernels._p(out), kernels._p(saved), None, None,
                        kernels._stream(colors.device))
  _lib.check(rc, "dr_splat_fwd")
  return out, saved


@splat_fwd.register_fake
def _(positions, colors, z_buffer):
  L, H, W, C = colors.shape
  return colors.new_empty((H, W, C)), colors.new_empty((3 * (C + 1) + 2, H * W))


@torch.library.custom_op(_NS + "::splat_bwd", mutates_args=())
def splat_bwd(d_out: torch.Tensor, positions: torch.Tensor, colors: torch.Tensor,
              z_buffer: torch.Tensor, saved: torch.Tensor) -> Tuple[torch.Tensor, torch.Tensor]:
  """(d positions [L, H, W, 4] as (d x, d y, 0, 0), d colors [L, H, W, C])."""
  L, H, W, C = colors.shape
  lib = _lib.load()
  batch = _single(W, H)
  pos = positions.reshape(-1, 4).contiguous()
  col = colors.reshape(-1, C).contiguous()
  z = z_buffer.reshape(-1).contiguous()
  d_pos = torch.zeros_like(pos)  # background samples get no gradient
  d_col = torch.empty_like(col)
  rc = lib.dr_splat_bwd(kernels._p(d_out.contiguous()), kernels._p(pos), kernels._p(z),
                        kernels._p(col), kernels._p(saved.contiguous()), C, batch.ptr, 1, L,
                        kernels._p(d_col), kernels._p(d_pos), kernels._stream(colors.device))
  _lib.check(rc, "dr_splat_bwd")
  return d_pos.view(L, H, W, 4), d_col.view(L, H, W, C)


@splat_bwd.register_fake
def _(d_out, positions, colors, z_buffer, saved):
  return torch.empty_like(positions), torch.empty_like(colors)


def _splat_setup(ctx, inputs, output):
  positions, colors, z_buffer = inputs
  ctx.save_for_backward(positions, colors, z_buffer, output[1])


def _splat_backward(ctx, d_out, d_saved):
  positions, colors, z_buffer, saved = ctx.saved_tensors
  d_pos, d_col = splat_bwd(d_out, positions, colors, z_buffer, saved)
  return d_pos, d_col, None


splat_fwd.register_autograd(_splat_backward, setup_context=_splat_setup)


def splat(positions, colors, z_buffer):
  """Splatted, normalized, composited image [H, W, C] of rasterized samples
  (see the module docstring); differentiable."""
  kernels._require_cuda(positions, colors, z_buffer)
  if colors.shape[-1] > _lib.DR_MAX_SPLAT_CHANNELS:
    raise ValueError("splatting supports at most %d channels" % _lib.DR_MAX_SPLAT_CHANNELS)
  return splat_fwd(positions.float(), colors.float(), z_buffer.float())[0]
