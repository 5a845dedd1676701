"""Rasterize-then-splat (diffren/jax/internal/splat.py:178-229).

``splat_shaded_pixels`` re-derives the splat positions from the vertices by
interpolating clip coordinates with the rasterized barycentrics (so the
gradient reaches the vertices), splats every shaded layer sample to its 3x3
neighbourhood with the per-tap surface test, normalizes and composites, all
in one CUDA kernel; the VJP is the gather-form kernel (see csrc/splat.cu).
"""
import torch

from . import framebuffer as fb
from . import kernels
from . import rasterize as rasterize_lib


def _shaded_flat(shaded, frame):
  C = shaded.shape[-1]
  s = shaded.reshape(-1, C)
  if s.dtype != torch.float32:
    s = s.float()
  return s.contiguous()


def splat_clip(clip, frame: fb.Framebuffer, shaded_pixels, return_accum_buffers=False):
  """Splat with precomputed clip-space vertices (packed like the framebuffer)."""
  batch, tris, ids, z, bary = frame.kernel_inputs()
  colors = _shaded_flat(shaded_pixels, frame)
  res = kernels.splat_packed(clip, colors, bary, tris, ids, z, batch, frame.num_layers,
                             return_accum_buffers)
  H, W = frame.height, frame.width
  C = colors.shape[1]
  lead = (frame.batch_size,) if frame.is_batched else ()
  if return_accum_buffers:
    out, accum, norm = res
    return (out.view(*lead, H, W, C), accum.view(*lead, 3, H, W, C),
            norm.view(*lead, 3, H, W, C))
  return res.view(*lead, H, W, C)


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
