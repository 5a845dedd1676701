"""Attribute interpolation (diffren/jax/internal/interpolate.py:118-170).

``interpolate_vertex_attribute`` computes, per layer and pixel,
fg * sum_i b_i attr[vertex_ids_i] + (1 - fg) * background with the CUDA
kernel; its VJP scatters to the vertex attributes (and to the barycentrics
when those are differentiable). ``interpolate_vertex_attributes`` packs all
attributes of the dict into one launch.
"""
from typing import Dict, Optional

import torch

from . import framebuffer as fb
from . import kernels


def _packed_attributes(attribute, frame: fb.Framebuffer):
  """[sum V, K] packed rows matching the framebuffer's image batch."""
  a = torch.as_tensor(attribute, device=frame.barycentrics.device)
  if not a.is_floating_point():
    a = a.float()
  if frame.is_batched:
    B = frame.batch_size
    if a.dim() == 2:
      a = a.expand(B, *a.shape)
    return a.reshape(-1, a.shape[-1]).float().contiguous()
  return a.float().contiguous()


def _reshape_like(frame, flat):
  K = flat.shape[-1]
  shape = (frame.batch_size,) if frame.is_batched else ()
  return flat.view(*shape, frame.num_layers, frame.height, frame.width, K)


def interpolate_vertex_attribute(attribute, framebuffer: fb.Framebuffer,
                                 background_value=None) -> torch.Tensor:
  """[L, H, W, K] (or [B, L, H, W, K]) interpolated attribute buffer."""
  batch, tris, ids, z, bary = framebuffer.kernel_inputs()
  attr = _packed_attributes(attribute, framebuffer)
  if framebuffer.packed is None:  # hand-built: per-pixel corner rows
    raise ValueError("interpolation needs a framebuffer from rasterize_triangles")
  bg = None
  if background_value is not None:
    bg = torch.as_tensor(background_value, dtype=torch.float32,
                         device=attr.device).reshape(-1)
  out = kernels.interpolate_packed(attr, bary, tris, ids, z, batch,
                                   framebuffer.num_layers, bg)
  return _reshape_like(framebuffer, out)


def interpolate_vertex_attributes(attributes: Dict[str, torch.Tensor],
                                  framebuffer: fb.Framebuffer,
                                  background_value: Optional[torch.Tensor] = None
                                  ) -> Dict[str, torch.Tensor]:
  """Interpolates every attribute of the dict in one kernel launch.

  ``background_value`` is None (zeros) or a tensor broadcastable to each
  attribute's channels (the reference passes a [L]-shaped zero vector from
  render_triangles, which broadcasts the same way).
  """
  if not attributes:
    return {}
  keys = list(attributes.keys())
  parts = [_packed_attributes(attributes[k], framebuffer) for k in keys]
  widths = [p.shape[1] for p in parts]
  cat = torch.cat(parts, dim=1) if len(parts) > 1 else parts[0]
  bg = None
  if background_value is not None:
    bgv = torch.as_tensor(background_value, dtype=torch.float32, device=cat.device)
    if bgv.numel() == 1 or bool((bgv == 0).all()):
      bg = bgv.reshape(-1)[:1].expand(cat.shape[1]).contiguous() if bgv.numel() else None
    else:
      bg = torch.cat([bgv.reshape(-1).expand(w) if bgv.numel() == 1 else
                      bgv.reshape(-1)[:w] for w in widths])
  batch, tris, ids, z, bary = framebuffer.kernel_inputs()
  out = kernels.interpolate_packed(cat, bary, tris, ids, z, batch,
                                   framebuffer.num_layers, bg)
  out = _reshape_like(framebuffer, out)
  return dict(zip(keys, kernels.split_channels(out, widths)))
