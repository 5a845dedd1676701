"""Ragged batches: many meshes, cameras and resolutions in one launch per
kernel.

The reference batches with jax.vmap, which lowers the rasterizer to one FFI
call per image (rasterize_triangles_xla.py:68-75, 'sequential_unrolled') and
needs equal shapes. ``BatchRenderer`` instead packs a fixed ragged batch
(per-mesh triangle lists and per-image resolutions) once, keeps its own
rasterizer workspace, and renders all images with one launch sequence:
transform, setup + tile binning + the persistent fine rasterizer over the
batch's (image, tile) queue whose epilogue also interpolates the attributes
and the splat positions, the user's shader on the packed buffers,
splat/normalize/composite, and the VJP kernels. Because no call
allocates outside torch's allocator or synchronizes, a whole forward+backward
step can be captured in a CUDA graph (``torch.cuda.graph``) and replayed.

The shader is called once on the packed buffers, each attribute viewed as
[1, N, K] with N = num_layers * total pixels, so it must be a per-pixel
function (the reference's shaders in diffren/jax/utils/shaders.py are).
"""
from typing import Callable, Dict, Sequence

import numpy as np
import torch

from . import constants
from . import kernels


class BatchRenderer:

  def __init__(self, triangles: Sequence, vertex_counts: Sequence[int],
               resolutions: Sequence, num_layers: int = 1,
               face_culling_mode=constants.FaceCullingMode.BACK,
               depth_semantics=constants.DepthSemantics.CUDA, device=None,
               tile=(0, 0), large_tiles=0, recompute_raster=False,
               deterministic_gradients=False):
    """``tile`` = (width, height) of the rasterizer's tiles, (0, 0) for the
    default, or "auto" to let the autotuner pick the tile and the
    large-triangle threshold on the first render (see autotune.py).
    ``recompute_raster``: for memory-tight batches, the backward reruns the
    rasterizer instead of keeping the triangle ids, barycentrics and vertex
    ids of every layer sample from the forward (28 bytes per sample).
    ``deterministic_gradients``: the vertex and attribute gradients of the
    fused pass are summed in fixed point instead of with float atomics, so
    they are the same bits on every run (one more pass over the samples)."""
    if len(triangles) != len(vertex_counts) or len(triangles) != len(resolutions):
      raise ValueError("triangles, vertex_counts and resolutions differ in length")
    self.device = torch.device(device or "cuda")
    tris = [torch.as_tensor(t).reshape(-1, 3).to(torch.int32) for t in triangles]
    self.batch = kernels.ImageBatch([r[0] for r in resolutions],
                                    [r[1] for r in resolutions],
                                    [int(v) for v in vertex_counts],
                                    [t.shape[0] for t in tris])
    self.triangles = torch.cat(tris).to(self.device).contiguous() if tris else \
        torch.zeros(0, 3, dtype=torch.int32, device=self.device)
    self.num_layers = int(num_layers)
    self.face_culling_mode = int(face_culling_mode)
    self._autotune = isinstance(tile, str)
    if self._autotune and tile != "auto":
      raise ValueError("tile must be (width, height) or 'auto'")
    self.config = kernels.raster_config(num_layers, face_culling_mode, int(depth_semantics),
                                        (0, 0) if self._autotune else tile, large_tiles)
    self.workspace = kernels.Workspace(self.device)
    self.workspace.get(kernels.raster_workspace_bytes(self.batch, self.config))
    self.recompute_raster = bool(recompute_raster)
    self.deterministic_gradients = bool(deterministic_gradients)

  def autotune(self, clip, attributes=None, **kw):
    """Picks the fastest tile / large-triangle configuration for this batch
    on these inputs (times the rasterizer; synchronizes, so call it before
    capturing a CUDA graph). Returns (tile_width, tile_height, large_tiles)."""
    from . import autotune as autotune_lib
    with torch.no_grad():
      choice = autotune_lib.tune(clip.detach(), self.triangles, self.batch, self.config,
                                 None if attributes is None else attributes.detach(),
                                 self.workspace, **kw)
    self.config = kernels.raster_config(self.config.num_layers, self.config.face_culling_mode,
                                        self.config.depth_mode, choice[:2], choice[2])
    self.workspace.get(kernels.raster_workspace_bytes(self.batch, self.config))
    self._autotune = False
    return choice

  def vertex_normals(self, vertices):
    """Area-weighted unit normals (mesh.py:22-52) of every mesh of the batch
    from packed world vertices [sum V, 3]; differentiable."""
    from . import mesh
    if getattr(self, "_adjacency", None) is None:
      self._adjacency = mesh.vertex_adjacency(self.triangles, self.batch)
    return mesh.vertex_normals_packed(vertices, self.triangles, self.batch, self._adjacency)

  @property
  def num_images(self):
    return self.batch.n

  @property
  def total_pixels(self):
    return self.batch.total_pixels

  def rasterize(self, clip):
    """(ids, z, bary) packed over the batch, from packed clip vertices."""
    return kernels.rasterize_packed(clip.detach(), self.triangles, self.batch,
                                    self.config, workspace=self.workspace)

  def render(self, vertices, attributes: Dict[str, torch.Tensor], cameras,
             shading_function: Callable, compositing_mode=constants.CompositingMode.SPLAT_OVER,
             return_accum_buffers=False):
    """Renders every image; returns packed [total_pixels, C] (see images()).

    vertices [sum V, 3|4] packed per mesh; attributes: dict of [sum V, K];
    cameras [N, 4, 4] (one per image) or None for clip-space vertices.
    ``shading_function`` None (beyond the reference's arguments): the single
    attribute is the color, as ``lambda a: a[key]`` gives; with splatting
    the background samples' attributes and color gradients, which nothing
    then reads, are not written.
    """
    if (compositing_mode == constants.CompositingMode.SPLAT_OVER and
        self.face_culling_mode != constants.FaceCullingMode.BACK):
      raise ValueError("Backface culling must be enabled when using splatting.")
    b = self.batch
    vertices = torch.as_tensor(vertices, device=self.device)
    if vertices.shape[0] != b.total_vertices:
      raise ValueError("expected %d packed vertices, got %d" % (b.total_vertices,
                                                                 vertices.shape[0]))
    if cameras is None:
      clip = vertices.float().contiguous()
    else:
      clip = kernels.transform(vertices.float().contiguous(),
                               torch.as_tensor(cameras, device=self.device), b)
    L = self.num_layers
    keys = list(attributes.keys())
    passthrough = shading_function is None
    if passthrough and len(keys) != 1:
      raise ValueError("shading_function=None needs exactly one attribute")
    parts = [kernels._f32(attributes[k], self.device) for k in keys]
    widths = [p.shape[1] for p in parts]
    cat = torch.cat(parts, dim=1) if len(parts) > 1 else parts[0]
    splatting = compositing_mode == constants.CompositingMode.SPLAT_OVER
    fused = splatting and cat.shape[1] <= kernels._lib.DR_MAX_CHANNELS
    if self._autotune:
      self.autotune(clip, cat if fused else None)
    if fused:
      # One pass: the rasterizer's epilogue interpolates the attributes and
      # the splat positions of every layer sample.
      # The splat path tells background samples by the depth buffer, so
      # their ids and barycentrics need not be written.
      # A pass-through shader leaves the splat the only reader of the
      # attributes: background rows need not be written either.
      interp, vp, ids, z, bary = kernels.rasterize_interpolate_packed(
          cat, clip, self.triangles, b,
          kernels.foreground_only(self.config, attributes=passthrough), self.workspace,
          self.recompute_raster, self.deterministic_gradients)
    else:
      ids, z, bary = self.rasterize(clip)
      if splatting:
        interp, vp = kernels.interpolate_with_positions_packed(cat, clip, bary,
                                                               self.triangles, ids, z, b, L)
      else:
        interp = kernels.interpolate_packed(cat, bary, self.triangles, ids, z, b, L)
    if passthrough:
      shaded = interp
    else:
      split = kernels.split_channels(interp, widths, dim=1)
      shaded = shading_function({k: s.view(1, -1, s.shape[1]) for k, s in zip(keys, split)})
      shaded = shaded.reshape(-1, shaded.shape[-1])
    if splatting:
      # Colors that are the fused pass's attribute buffer itself (a
      # pass-through shader such as lambda a: a[key]) send their gradient
      # only to that pass's VJP, which reads foreground samples: background
      # color gradients need not be written.
      colors_are_attributes = fused and (passthrough or (
          shaded.data_ptr() == interp.data_ptr() and shaded.shape == interp.shape and
          shaded.stride() == interp.stride()))
      return kernels.splat_packed(vp, shaded, b, L, return_accum_buffers, z=z,
                                  foreground_gradients=colors_are_attributes)
    if compositing_mode == constants.CompositingMode.NONE:
      return shaded * (z != 1.0).float()[:, None]
    return kernels.over_packed(shaded, z, b, L)

  def images(self, packed):
    """List of [H_i, W_i, C] views of a packed composited result."""
    return [self.batch.image_view(packed, i) for i in range(self.batch.n)]

  def layers(self, packed):
    """List of [L, H_i, W_i, C] views of a packed layered result."""
    return [self.batch.layered_view(packed, i, self.num_layers)
            for i in range(self.batch.n)]


def pack_meshes(vertices: Sequence, attributes: Sequence[Dict]):
  """Concatenates per-mesh vertex arrays and attribute dicts."""
  v = torch.cat([torch.as_tensor(x) for x in vertices])
  keys = attributes[0].keys() if attributes else []
  a = {k: torch.cat([torch.as_tensor(d[k]) for d in attributes]) for k in keys}
  return v, a


def render_triangles_batch(vertices: Sequence, attributes: Sequence[Dict],
                           triangles: Sequence, cameras, resolutions: Sequence,
                           shading_function: Callable, num_layers: int = 1,
                           face_culling_mode=constants.FaceCullingMode.BACK,
                           compositing_mode=constants.CompositingMode.SPLAT_OVER,
                           device=None):
  """render_triangles for a ragged list of meshes; returns a list of images."""
  r = BatchRenderer(triangles, [len(v) for v in vertices], resolutions, num_layers,
                    face_culling_mode, device=device)
  v, a = pack_meshes(vertices, attributes)
  cams = None if cameras is None else torch.as_tensor(np.asarray(cameras), dtype=torch.float32)
  out = r.render(v.to(r.device), {k: x.to(r.device) for k, x in a.items()},
                 None if cams is None else cams.to(r.device), shading_function,
                 compositing_mode)
  if compositing_mode == constants.CompositingMode.NONE:
    return r.layers(out)
  return r.images(out)
