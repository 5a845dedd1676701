"""Main entry point (diffren/jax/render.py:28-140).

``render_triangles`` keeps the reference's signature and behaviour:
rasterize, interpolate the attribute dict, run the user's deferred shader
(any differentiable torch function of a dict of [H, W, K] buffers) on each
layer, then splat+composite (SPLAT_OVER), composite (OVER) or return the
layers (NONE). Gradients reach vertices, attributes and camera through the
CUDA VJP kernels; the shader's own VJP is torch autograd.

A leading batch dimension on vertices / camera (/ attributes / triangles)
renders all images in one launch per kernel, the batched counterpart of
jax.vmap(render_triangles).
"""
from typing import Callable, Dict

import torch

from . import constants
from . import interpolate
from . import kernels
from . import rasterize
from . import splat


def _shade_layers(shading_function, interpolated, num_layers, batched):
  """vmap(shading_function) over layers (and images), as render.py:128."""
  outs = []
  if batched:
    B = next(iter(interpolated.values())).shape[0]
    for b in range(B):
      outs.append(torch.stack([
          shading_function({k: v[b, l] for k, v in interpolated.items()})
          for l in range(num_layers)]))
    return torch.stack(outs)
  return torch.stack([
      shading_function({k: v[l] for k, v in interpolated.items()})
      for l in range(num_layers)])


def _render_fused(geom, attributes, shading_function, num_layers, face_culling_mode,
                  depth_semantics, return_accum_buffers, recompute_raster=False,
                  deterministic_gradients=False):
  """SPLAT_OVER through the rasterizer that interpolates the attributes and
  the splat positions in its epilogue; None when the attributes exceed its
  channel limit."""
  keys = list(attributes.keys())
  parts = []
  for k in keys:
    a = torch.as_tensor(attributes[k], device=geom.clip.device)
    a = a.float() if not a.is_floating_point() or a.dtype != torch.float32 else a
    if geom.batched:
      a = (a.expand(geom.B, *a.shape) if a.dim() == 2 else a).reshape(-1, a.shape[-1])
    parts.append(a)
  widths = [p.shape[1] for p in parts]
  if sum(widths) > kernels._lib.DR_MAX_CHANNELS:
    return None
  cat = torch.cat(parts, dim=1) if len(parts) > 1 else parts[0].contiguous()
  # Background samples are told by the depth buffer downstream, so their
  # ids and barycentrics need not be written; with a pass-through shader
  # (None) the splat is the only reader of the attributes, so neither are
  # their attributes nor their color gradients.
  passthrough = shading_function is None
  cfg = kernels.raster_config(num_layers, face_culling_mode, int(depth_semantics),
                              flags=kernels._lib.DR_RASTER_FOREGROUND_ONLY |
                              (kernels._lib.DR_RASTER_FOREGROUND_ATTRIBUTES if passthrough
                               else 0))
  interp, vp, ids, z, bary = kernels.rasterize_interpolate_packed(
      cat, geom.clip, geom.triangles_packed, geom.batch, cfg,
      kernels.default_workspace(geom.clip.device), recompute_raster, deterministic_gradients)
  frame = rasterize.framebuffer_of(geom, num_layers, ids, z, bary)
  lead = (geom.B,) if geom.batched else ()
  interp = interp.view(*lead, num_layers, frame.height, frame.width, -1)
  if passthrough:
    shaded = interp
  else:
    interpolated = dict(zip(keys, kernels.split_channels(interp, widths)))
    shaded = _shade_layers(shading_function, interpolated, num_layers, geom.batched)
  return splat.splat_positions(vp, frame, shaded, return_accum_buffers,
                               foreground_gradients=passthrough)


def render_triangles(vertices, attributes: Dict[str, torch.Tensor], triangles,
                     camera_matrices, image_width: int, image_height: int,
                     shading_function: Callable[[Dict[str, torch.Tensor]],
                                                torch.Tensor],
                     num_layers: int = 1,
                     face_culling_mode=constants.FaceCullingMode.BACK,
                     compositing_mode=constants.CompositingMode.SPLAT_OVER,
                     return_accum_buffers=False, compute_diff_barys=False,
                     depth_semantics=constants.DepthSemantics.CUDA,
                     recompute_raster=False, deterministic_gradients=False):
  """Rendering with differentiable occlusion using rasterize-then-splat.

  Returns [H, W, C] ([num_layers, H, W, C] for CompositingMode.NONE), with a
  leading batch dimension when the inputs are batched. ``recompute_raster``
  (SPLAT_OVER, beyond the reference's arguments): the backward reruns the
  rasterizer instead of keeping its per-sample triangle ids, barycentrics
  and vertex ids, for memory-tight renders. ``shading_function`` None (also
  beyond the reference's arguments): the single attribute is the color, as
  ``lambda a: a[key]`` gives, and background samples' attributes and color
  gradients, which nothing then reads, are not written.
  ``deterministic_gradients`` (SPLAT_OVER; also beyond the reference): the
  vertex and attribute gradients of the fused pass are summed in fixed
  point, the same bits on every run.

  Raises:
    ValueError: if face_culling_mode is not BACK and compositing_mode is
      SPLAT_OVER (back faces would count as occluding layers).
  """
  if (compositing_mode == constants.CompositingMode.SPLAT_OVER and
      face_culling_mode != constants.FaceCullingMode.BACK):
    raise ValueError("Backface culling must be enabled when using splatting.")
  if shading_function is None and len(attributes) != 1:
    raise ValueError("shading_function=None needs exactly one attribute")
  vertices = torch.as_tensor(vertices)
  triangles = torch.as_tensor(triangles)
  camera = None if camera_matrices is None else torch.as_tensor(camera_matrices)
  rasterize._validate(vertices, triangles, camera, image_width, image_height,
                      num_layers)
  geom = rasterize.Geometry(vertices, triangles, camera, image_width, image_height)
  if (compositing_mode == constants.CompositingMode.SPLAT_OVER and not compute_diff_barys
      and attributes):
    fused = _render_fused(geom, attributes, shading_function, num_layers,
                          face_culling_mode, depth_semantics, return_accum_buffers,
                          recompute_raster, deterministic_gradients)
    if fused is not None:
      return fused
  frame, _ = rasterize.rasterize_geometry(geom, num_layers, face_culling_mode,
                                          depth_semantics, compute_diff_barys)
  interpolated = interpolate.interpolate_vertex_attributes(attributes, frame)
  if shading_function is None:
    shaded = next(iter(interpolated.values()))
  else:
    shaded = _shade_layers(shading_function, interpolated, num_layers, geom.batched)

  if compositing_mode == constants.CompositingMode.SPLAT_OVER:
    return splat.splat_clip(geom.clip, frame, shaded, return_accum_buffers)

  if compositing_mode == constants.CompositingMode.OVER:
    # Foreground mask and composite.over in one kernel.
    C = shaded.shape[-1]
    out = kernels.over_packed(shaded.reshape(-1, C), frame.z_buffer.reshape(-1), geom.batch,
                              num_layers)
    lead = (geom.B,) if geom.batched else ()
    return out.view(*lead, image_height, image_width, C)
  return shaded * frame.foreground_mask
