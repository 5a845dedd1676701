"""Mesh utilities with CUDA kernels (diffren/jax/utils/mesh.py).

``compute_vertex_normals`` is the reference's area-weighted vertex normal
(mesh.py:22-52): each face normal cross(v1 - v0, v2 - v0), whose length is
twice the face's area, is summed into its three vertices and the sums are
normalized with transforms.l2_normalize (x * rsqrt(|x|^2 + 1e-12)). Forward
and VJP are CUDA kernels over a ragged batch of meshes, summed without
atomics through a vertex -> corner adjacency built once per topology, so
that they are the same bits on every run.
"""
import weakref

import torch

from . import _lib
from . import kernels


def vertex_adjacency(triangles, batch):
  """The vertex -> corner adjacency of a ragged batch of meshes laid out as
  ``kernels.ImageBatch`` describes, for the deterministic normals: corner
  3 g + s is slot s of global triangle g (triangles numbered in mesh
  order); returns (offsets [V + 1] int64, corners int32) with vertex i's
  corners at corners[offsets[i]:offsets[i + 1]], slot 0 ones first, then
  slot 1, then slot 2, each in triangle order (a stable sort by vertex of
  the slot-major corner list). Triangles with an out-of-range index are
  left out, as the kernels skip them. Built once per topology."""
  dev = triangles.device
  descs = [batch.descs[i] for i in range(batch.n)]
  V = max([d.vertex_offset + d.num_vertices for d in descs] + [0])
  parts, vos, nvs = [], [], []
  for d in descs:
    nt = int(d.num_triangles)
    parts.append(triangles[int(d.triangle_offset):int(d.triangle_offset) + nt].long())
    vos.append(torch.full((nt,), int(d.vertex_offset), dtype=torch.int64, device=dev))
    nvs.append(torch.full((nt,), int(d.num_vertices), dtype=torch.int64, device=dev))
  if not parts or sum(p.shape[0] for p in parts) == 0:
    return (torch.zeros(V + 1, dtype=torch.int64, device=dev),
            torch.zeros(0, dtype=torch.int32, device=dev))
  tri = torch.cat(parts)
  vo, nv = torch.cat(vos), torch.cat(nvs)
  T = tri.shape[0]
  valid = ((tri >= 0) & (tri < nv[:, None])).all(1)
  keys = (tri + vo[:, None]).t()  # [3, T], slot-major
  g = torch.arange(T, dtype=torch.int64, device=dev)
  corners = torch.stack([3 * g, 3 * g + 1, 3 * g + 2])
  mask = valid[None, :].expand(3, T)
  keys, corners = keys[mask], corners[mask]
  order = torch.sort(keys, stable=True).indices
  offsets = torch.zeros(V + 1, dtype=torch.int64, device=dev)
  offsets[1:] = torch.cumsum(torch.bincount(keys, minlength=V), 0)
  return offsets, corners[order].to(torch.int32).contiguous()


class _VertexNormals(torch.autograd.Function):

  @staticmethod
  def forward(ctx, vertices, triangles, batch, adjacency):
    lib = _lib.load()
    off, corners = adjacency
    if corners.numel() == 0:  # no corner to list: a stand-in the kernels never read
      corners = torch.zeros(1, dtype=torch.int32, device=vertices.device)
    V = vertices.shape[0]
    T = int(batch.total_triangles)
    dev = vertices.device
    face = torch.empty(max(T, 1), 4, dtype=torch.float32, device=dev)
    accum = torch.empty(V, 4, dtype=torch.float32, device=dev)
    out = torch.empty(V, 3, dtype=torch.float32, device=dev)
    with kernels._op("normals_fwd", 2):
      rc = lib.dr_vertex_normals_csr_fwd(kernels._p(vertices), kernels._p(triangles), batch.ptr,
                                         batch.n, kernels._p(off), kernels._p(corners),
                                         kernels._p(face), kernels._p(accum), kernels._p(out),
                                         kernels._stream(dev))
    _lib.check(rc, "dr_vertex_normals_csr_fwd")
    ctx.save_for_backward(vertices, triangles, accum, off, corners)
    ctx.batch = batch
    return out

  @staticmethod
  def backward(ctx, d_out):
    vertices, triangles, accum, off, corners = ctx.saved_tensors
    if not ctx.needs_input_grad[0]:
      return None, None, None, None
    lib = _lib.load()
    T = int(ctx.batch.total_triangles)
    d_accum = torch.empty_like(accum)
    corner_grad = torch.empty(max(3 * T, 1), 4, dtype=torch.float32, device=vertices.device)
    d_v = torch.zeros_like(vertices)
    with kernels._op("normals_bwd", 3):
      rc = lib.dr_vertex_normals_csr_bwd(kernels._p(d_out.contiguous()), kernels._p(vertices),
                                         kernels._p(triangles), ctx.batch.ptr, ctx.batch.n,
                                         kernels._p(off), kernels._p(corners),
                                         kernels._p(accum), kernels._p(d_accum),
                                         kernels._p(corner_grad), kernels._p(d_v),
                                         kernels._stream(vertices.device))
    _lib.check(rc, "dr_vertex_normals_csr_bwd")
    return d_v, None, None, None


def vertex_normals_packed(vertices, triangles, batch, adjacency=None):
  """Normals of a ragged batch of meshes laid out as ``kernels.ImageBatch``
  describes (vertices [sum V, 3], triangles [sum T, 3] with mesh-local
  indices). Returns [sum V, 3]; differentiable w.r.t. vertices. Summed
  without atomics over ``adjacency`` (``vertex_adjacency``, built here when
  not given), so the normals and their gradients are the same bits on
  every run."""
  kernels._require_cuda(vertices, triangles)
  if vertices.dim() != 2 or vertices.shape[1] != 3:
    raise ValueError("vertices must be [V, 3]")
  if triangles.dim() != 2 or triangles.shape[1] != 3:
    raise ValueError("triangles must be [T, 3]")
  triangles = kernels._i32(triangles)
  if adjacency is None:
    adjacency = vertex_adjacency(triangles, batch)
  return _VertexNormals.apply(kernels._f32(vertices), triangles, batch, adjacency)


# Adjacency of each triangle tensor compute_vertex_normals has seen (the
# topology rarely changes between calls): id -> (weak reference, key of its
# contents' version and layout, adjacency), dropped with the tensor.
_ADJACENCY = {}


def _shared_batch(num_meshes, num_vertices, num_triangles):
  """num_meshes meshes of num_vertices rows each over one triangle list."""
  batch = kernels.ImageBatch([1] * num_meshes, [1] * num_meshes,
                             [num_vertices] * num_meshes, [num_triangles] * num_meshes)
  for i in range(num_meshes):
    batch.descs[i].triangle_offset = 0
  return batch


def compute_vertex_normals(vertices, triangles):
  """mesh.compute_vertex_normals (mesh.py:22-52).

  vertices [V, 3] (or [B, V, 3], the reference's vmap over a batch of
  meshes sharing one triangle list); triangles [T, 3] integer. Returns the
  normalized vertex normals with the vertices' shape.
  """
  kernels._require_cuda(vertices, triangles)
  if vertices.shape[-1] != 3 or vertices.dim() not in (2, 3):
    raise ValueError("vertices must be [V, 3] or [B, V, 3]")
  if triangles.dim() != 2 or triangles.shape[1] != 3:
    raise ValueError("triangles must be [T, 3]")
  shape = vertices.shape
  B = shape[0] if vertices.dim() == 3 else 1
  V, T = shape[-2], triangles.shape[0]
  if B * V == 0:
    return torch.zeros(shape, dtype=torch.float32, device=vertices.device)
  flat = vertices.reshape(B * V, 3)
  batch = _shared_batch(B, V, T)
  tris = kernels._i32(triangles)
  key = (B, V, T, tris.data_ptr(), triangles._version)
  entry = _ADJACENCY.get(id(triangles))
  if entry is None or entry[0]() is not triangles or entry[1] != key:
    adjacency = vertex_adjacency(tris, batch)
    _ADJACENCY[id(triangles)] = (weakref.ref(triangles), key, adjacency)
    weakref.finalize(triangles, _ADJACENCY.pop, id(triangles), None)
  else:
    adjacency = entry[2]
  out = vertex_normals_packed(flat, tris, batch, adjacency)
  return out.view(shape)
