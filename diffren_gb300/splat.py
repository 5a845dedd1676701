"""Rasterize-then-splat (diffren/jax/internal/splat.py).

``splat_shaded_pixels`` re-derives the splat positions from the vertices by
interpolating clip coordinates with the rasterized barycentrics (so the
gradient reaches the vertices, splat.py:207-221), then
``splat_at_pixel_centers`` splats every shaded layer sample to its 3x3
neighbourhood with the per-tap surface test, normalizes and composites
(splat.py:26-175). Each step is a CUDA kernel with a hand-written VJP (see
csrc/splat.cu).
"""
import torch

from . import framebuffer as fb
from . import kernels
from . import rasterize as rasterize_lib


def _shaded_flat(shaded):
  C = shaded.shape[-1]
  s = shaded.reshape(-1, C)
  if s.dtype != torch.float32:
    s = s.float()
  return s.contiguous()


def _shape_outputs(res, lead, H, W, C, return_accum_buffers):
  if return_accum_buffers:
    out, accum, norm = res
    return (out.view(*lead, H, W, C), accum.view(*lead, 3, H, W, C),
            norm.view(*lead, 3, H, W, C))
  return res.view(*lead, H, W, C)


def splat_at_pixel_centers(xyz_layers, color_layers, foreground_mask):
  """Splats layered samples onto the pixel grid (splat.py:26-175).

  xyz_layers [L, H, W, 3] viewport positions, color_layers [L, H, W, C]
  (last channel alpha), foreground_mask [L, H, W, 1]. Returns the
  composited [H, W, C] image and the accumulated and normalized
  [3, H, W, C] fg/surface/bg buffers, like the reference. Differentiable
  w.r.t. the xy positions and the colors (the mask and the z used by the
  surface test carry no gradient, as in the reference).
  """
  L, H, W, C = color_layers.shape
  fg = torch.as_tensor(foreground_mask, device=color_layers.device).float()
  vp = torch.cat([xyz_layers.float(), fg.reshape(L, H, W, 1).detach()], -1)
  batch = kernels.ImageBatch.single(W, H, 0, 0)
  res = kernels.splat_packed(vp.reshape(-1, 4), _shaded_flat(color_layers), batch, L,
                             return_accum_buffers=True)
  return _shape_outputs(res, (), H, W, C, True)


def splat_clip(clip, frame: fb.Framebuffer, shaded_pixels, return_accum_buffers=False):
  """Splat with precomputed clip-space vertices (packed like the framebuffer)."""
  batch, tris, ids, z, bary = frame.kernel_inputs()
  vp = kernels.splat_positions_packed(clip, bary, tris, ids, z, batch, frame.num_layers)
  return splat_positions(vp, frame, shaded_pixels, return_accum_buffers)


def splat_positions(positions, frame: fb.Framebuffer, shaded_pixels,
                    return_accum_buffers=False, foreground_gradients=False):
  """Splat at packed splat positions [L*P, 4] of the framebuffer's samples
  (background samples are taken from its depth buffer).
  ``foreground_gradients``: see kernels.splat_packed."""
  batch, _, _, z, _ = frame.kernel_inputs()
  colors = _shaded_flat(shaded_pixels)
  res = kernels.splat_packed(positions, colors, batch, frame.num_layers,
                             return_accum_buffers, z=z,
                             foreground_gradients=foreground_gradients)
  lead = (frame.batch_size,) if frame.is_batched else ()
  return _shape_outputs(res, lead, frame.height, frame.width, colors.shape[1],
                        return_accum_buffers)


def splat_shaded_pixels(vertices, camera_matrices, rasterized_fb: fb.Framebuffer,
                        shaded_pixels, return_accum_buffers: bool = False):
  """Splats shaded layers back onto the pixel grid (splat.py:178-229).

  vertices [V, d] (or [B, V, d]); camera_matrices [4, 4] ([B, 4, 4]) or None
  for clip-space vertices; shaded_pixels [L, H, W, C] ([B, L, H, W, C]).
  Returns [H, W, C], plus the accumulated and normalized [3, H, W, C]
  fg/surface/bg buffers when ``return_accum_buffers``.
  """
  if rasterized_fb.packed is None:
    raise ValueError("splatting needs a framebuffer from rasterize_triangles")
  batch = rasterized_fb.packed[0]
  geom = rasterize_lib.Geometry(vertices, rasterized_fb.triangles, camera_matrices,
                                rasterized_fb.width, rasterized_fb.height)
  if geom.batch.total_vertices != batch.total_vertices:
    raise ValueError("vertices do not match the rasterized framebuffer")
  return splat_clip(geom.clip, rasterized_fb, shaded_pixels, return_accum_buffers)
