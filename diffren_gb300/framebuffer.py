"""Framebuffer container (diffren/jax/internal/framebuffer.py:24-129).

Holds the rasterized buffers with the reference's layout: barycentrics
[L, H, W, 3], triangle_id [L, H, W, 1], vertex_ids [L, H, W, 3] and
foreground_mask [L, H, W, 1] (a leading batch dimension when batched). Unlike
the reference it also keeps what the CUDA kernels consume directly (the
triangle list and the depth buffer, from which the foreground mask is
derived exactly as z != 1), so vertex_ids and foreground_mask are computed on
first access instead of being materialized by every rasterization.
"""
from typing import Dict, Optional

import torch


class Framebuffer:

  def __init__(self, barycentrics: torch.Tensor, triangle_id: torch.Tensor,
               vertex_ids: Optional[torch.Tensor] = None,
               foreground_mask: Optional[torch.Tensor] = None,
               attributes: Optional[Dict[str, torch.Tensor]] = None,
               z_buffer: Optional[torch.Tensor] = None,
               triangles: Optional[torch.Tensor] = None):
    self.barycentrics = barycentrics
    self.triangle_id = triangle_id
    self._vertex_ids = vertex_ids
    self._foreground_mask = foreground_mask
    self.attributes = dict(attributes or {})
    self.z_buffer = z_buffer
    self.triangles = triangles
    # Set by the rasterizer: (ImageBatch, packed int32 triangles, flat ids,
    # flat z) exactly as the kernels consume them.
    self.packed = None
    if vertex_ids is None and triangles is None:
      raise ValueError("Framebuffer needs vertex_ids or triangles")
    if foreground_mask is None and z_buffer is None:
      raise ValueError("Framebuffer needs foreground_mask or z_buffer")
    shapes = [barycentrics.shape, triangle_id.shape]
    if vertex_ids is not None:
      shapes.append(vertex_ids.shape)
    if foreground_mask is not None:
      shapes.append(foreground_mask.shape)
    shapes += [v.shape for v in self.attributes.values()]
    for s in shapes[1:]:
      if tuple(s[:-1]) != tuple(shapes[0][:-1]):
        raise ValueError("Expected all input shapes to match (up to channels), "
                         "but found %s" % (shapes,))

  @property
  def vertex_ids(self):
    if self._vertex_ids is None:
      ids = self.triangle_id[..., 0].long()
      if self.is_batched:
        b = torch.arange(ids.shape[0], device=ids.device).view(-1, 1, 1, 1)
        tri = self.triangles if self.triangles.dim() == 3 else None
        self._vertex_ids = (tri[b, ids] if tri is not None else
                            self.triangles[ids])
      else:
        self._vertex_ids = self.triangles[ids]
    return self._vertex_ids

  @property
  def foreground_mask(self):
    if self._foreground_mask is None:
      self._foreground_mask = (self.z_buffer != 1.0).float()[..., None]
    return self._foreground_mask

  @property
  def is_batched(self):
    return self.barycentrics.dim() == 5

  @property
  def is_multi_layer(self):
    return self.barycentrics.dim() in (4, 5)

  @property
  def batch_size(self):
    return self.barycentrics.shape[0] if self.is_batched else 1

  @property
  def num_layers(self):
    if self.is_batched:
      return self.barycentrics.shape[1]
    if self.is_multi_layer:
      return self.barycentrics.shape[0]
    return 1

  @property
  def height(self):
    return self.barycentrics.shape[-3]

  @property
  def width(self):
    return self.barycentrics.shape[-2]

  @property
  def pixel_count(self):
    return self.num_layers * self.height * self.width

  @property
  def background_mask(self):
    return 1 - self.foreground_mask

  def layer(self, index):
    """Single-layer Framebuffer at `index` (framebuffer.py:116-129)."""
    if not self.is_multi_layer:
      if index > 0:
        raise ValueError("Invalid layer index %d for single-layer Framebuffer."
                         % index)
      return self
    sl = (slice(None), index) if self.is_batched else (index,)
    return Framebuffer(
        barycentrics=self.barycentrics[sl],
        triangle_id=self.triangle_id[sl],
        vertex_ids=self.vertex_ids[sl],
        foreground_mask=self.foreground_mask[sl],
        attributes={k: v[sl] for k, v in self.attributes.items()},
        z_buffer=None if self.z_buffer is None else self.z_buffer[sl])

  def replace(self, **kwargs):
    fields = dict(barycentrics=self.barycentrics, triangle_id=self.triangle_id,
                  vertex_ids=self._vertex_ids,
                  foreground_mask=self._foreground_mask,
                  attributes=self.attributes, z_buffer=self.z_buffer,
                  triangles=self.triangles)
    fields.update(kwargs)
    out = Framebuffer(**fields)
    out.packed = self.packed
    return out

  # Kernel-facing packed views -------------------------------------------
  def kernel_inputs(self):
    """(ImageBatch, triangles [T', 3] i32, ids [N] i32, z [N], bary [N, 3]).

    For a framebuffer built by this package these are the rasterizer's own
    packed buffers. For one built by hand (unbatched) from vertex_ids and a
    foreground mask, each pixel gets its own one-triangle entry so the same
    kernels apply.
    """
    from . import kernels  # local: kernels imports nothing from here
    bary = self.barycentrics.reshape(-1, 3)
    if bary.dtype != torch.float32:
      bary = bary.float()
    if self.packed is not None:
      batch, tris, ids, z = self.packed
      return batch, tris, ids, z, bary
    if self.is_batched:
      raise ValueError("hand-built framebuffers must be unbatched")
    vids = self.vertex_ids.reshape(-1, 3).to(torch.int32).contiguous()
    ids = torch.arange(vids.shape[0], dtype=torch.int32, device=vids.device)
    if self.z_buffer is not None:
      z = self.z_buffer.reshape(-1)
    else:
      z = torch.where(self.foreground_mask.reshape(-1) > 0, 0.0, 1.0).float()
    batch = kernels.ImageBatch.single(self.width, self.height, 0, vids.shape[0])
    return batch, vids, ids, z.float().contiguous(), bary.contiguous()
