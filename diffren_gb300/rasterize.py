"""Rasterization into framebuffers (diffren/jax/internal/rasterize.py).

``rasterize_triangles`` mirrors rasterize.py:26-124: validate, transform
vertices by the camera, rasterize, build the Framebuffer, and optionally
replace the barycentrics by differentiable ones (rasterize.py:127-165). The
raster outputs themselves carry no gradient, as in the reference
(rasterize_triangles_xla.py:49-52).

Besides the reference's [V, d] vertices with a [4, 4] camera, a leading batch
dimension ([B, V, d] vertices, [B, 4, 4] cameras, shared or [B, T, 3]
triangles) is accepted and rasterized in one launch sequence.
"""
from typing import Optional

import torch

from . import constants
from . import framebuffer as fb
from . import kernels


def normalized_pixel_coordinates(image_width, image_height, device=None):
  """Pixel-center NDC grids (rasterize.py:168-189), float32 [H, W] each."""
  x = (2 * torch.arange(image_width, device=device) + 1).float() / image_width - 1
  y = (2 * torch.arange(image_height, device=device) + 1).float() / image_height - 1
  yy, xx = torch.meshgrid(y, x, indexing="ij")
  return xx, yy


def _validate(vertices, triangles, camera, image_width, image_height, num_layers):
  if vertices.dim() not in (2, 3) or vertices.shape[-1] not in (3, 4):
    raise ValueError("vertices must have shape [n, 3] or [n, 4], but found %s"
                     % (tuple(vertices.shape),))
  if triangles.dim() not in (2, 3) or triangles.shape[-1] != 3:
    raise ValueError("triangles must have shape [n, 3], but found %s."
                     % (tuple(triangles.shape),))
  if camera is not None and tuple(camera.shape[-2:]) != (4, 4):
    raise ValueError("camera must be a (4, 4) matrix but found %s"
                     % (tuple(camera.shape),))
  if not image_width > 0:
    raise ValueError("image_width must be > 0 but is %s." % image_width)
  if not image_height > 0:
    raise ValueError("image_height must be > 0 but is %s." % image_height)
  if not num_layers > 0:
    raise ValueError("num_layers must be > 0 but is %s." % num_layers)
  if num_layers > 16:
    raise ValueError("num_layers must be <= 16 but is %s." % num_layers)
  if camera is None and vertices.shape[-1] != 4:
    raise ValueError("vertices must be [n, 4] clip coordinates when camera is None")


def _device(*ts):
  for t in ts:
    if isinstance(t, torch.Tensor) and t.is_cuda:
      return t.device
  return torch.device("cuda", torch.cuda.current_device())


class Geometry:
  """Packed clip-space geometry of a (possibly batched) rasterization."""

  def __init__(self, vertices, triangles, camera, image_width, image_height):
    dev = _device(vertices, triangles, camera)
    vertices = torch.as_tensor(vertices, device=dev)
    if not vertices.is_floating_point():
      vertices = vertices.float()
    triangles = torch.as_tensor(triangles, device=dev)
    camera = None if camera is None else torch.as_tensor(camera, device=dev)
    self.batched = vertices.dim() == 3 or (camera is not None and camera.dim() == 3) \
        or triangles.dim() == 3
    B = 1
    for t, d in ((vertices, 3), (triangles, 3), (camera, 3)):
      if t is not None and t.dim() == d:
        B = t.shape[0]
    self.B = B
    V = vertices.shape[-2]
    T = triangles.shape[-2]
    self.batch = kernels.ImageBatch([image_width] * B, [image_height] * B, [V] * B,
                                    [T] * B)
    v = vertices.expand(B, *vertices.shape[-2:]) if vertices.dim() == 2 else vertices
    self.world = v.reshape(B * V, vertices.shape[-1]).float()
    t = triangles.expand(B, T, 3) if triangles.dim() == 2 else triangles
    self.triangles_packed = t.reshape(B * T, 3).to(torch.int32).contiguous()
    self.triangles = triangles
    if camera is None:
      self.clip = self.world.contiguous()
    else:
      cam = camera.expand(B, 4, 4) if camera.dim() == 2 else camera
      self.clip = kernels.transform(self.world.contiguous(), cam.float(), self.batch)


def rasterize_geometry(geom: Geometry, num_layers, face_culling_mode,
                       depth_semantics=constants.DepthSemantics.CUDA,
                       compute_diff_barys=False, tile=(0, 0)):
  """Rasterizes packed geometry; returns (Framebuffer, flat kernel buffers)."""
  cfg = kernels.raster_config(num_layers, face_culling_mode, int(depth_semantics),
                              tile)
  ids, z, bary = kernels.rasterize_packed(geom.clip.detach(), geom.triangles_packed,
                                          geom.batch, cfg)
  if compute_diff_barys:
    bary = kernels.diff_barycentrics_packed(geom.clip, geom.triangles_packed, ids, z,
                                            geom.batch, num_layers)
  return framebuffer_of(geom, num_layers, ids, z, bary), (ids, z, bary)


def framebuffer_of(geom: Geometry, num_layers, ids, z, bary):
  """Framebuffer views of flat rasterizer outputs."""
  H, W = geom.batch.heights[0], geom.batch.widths[0]
  shape = (geom.B, num_layers, H, W) if geom.batched else (num_layers, H, W)
  frame = fb.Framebuffer(barycentrics=bary.view(*shape, 3),
                         triangle_id=ids.view(*shape, 1), z_buffer=z.view(*shape),
                         triangles=geom.triangles)
  frame.packed = (geom.batch, geom.triangles_packed, ids, z)
  return frame


def rasterize_triangles(vertices, triangles, camera: Optional[torch.Tensor],
                        image_width: int, image_height: int, num_layers=1,
                        face_culling_mode=constants.FaceCullingMode.NONE,
                        compute_diff_barys=False,
                        depth_semantics=constants.DepthSemantics.CUDA
                        ) -> fb.Framebuffer:
  """Rasterizes triangles and computes per-pixel ids and barycentrics.

  Layers are front to back. Nothing is differentiable unless
  ``compute_diff_barys`` (then the barycentrics are, w.r.t. vertices and
  camera). See rasterize.py:26-124 for the reference contract.
  """
  vertices = torch.as_tensor(vertices)
  triangles = torch.as_tensor(triangles)
  camera = None if camera is None else torch.as_tensor(camera)
  _validate(vertices, triangles, camera, image_width, image_height, num_layers)
  geom = Geometry(vertices, triangles, camera, image_width, image_height)
  frame, _ = rasterize_geometry(geom, num_layers, face_culling_mode,
                                depth_semantics, compute_diff_barys)
  return frame


def differentiable_barycentrics(framebuffer: fb.Framebuffer,
                                clip_space_vertices: torch.Tensor,
                                triangles: torch.Tensor) -> fb.Framebuffer:
  """Replaces the barycentrics by ones differentiable w.r.t. the clip-space
  vertices (rasterize.py:127-165), computed by the CUDA kernel."""
  if framebuffer.is_batched:
    raise ValueError("differentiable_barycentrics takes an unbatched framebuffer; "
                     "use rasterize_triangles(..., compute_diff_barys=True)")
  clip = clip_space_vertices.float().contiguous()
  tris = torch.as_tensor(triangles, device=clip.device).to(torch.int32).contiguous()
  L, H, W = framebuffer.num_layers, framebuffer.height, framebuffer.width
  batch = kernels.ImageBatch.single(W, H, clip.shape[0], tris.shape[0])
  z = framebuffer.z_buffer
  if z is None:
    z = torch.where(framebuffer.foreground_mask[..., 0] > 0, 0.0, 1.0)
  ids = framebuffer.triangle_id.reshape(-1).to(torch.int32).contiguous()
  bary = kernels.diff_barycentrics_packed(clip, tris, ids, z.reshape(-1).contiguous(),
                                          batch, L)
  return framebuffer.replace(barycentrics=bary.view(L, H, W, 3))
