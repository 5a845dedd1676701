"""The vertex -> corner adjacency behind the deterministic vertex normals
(mesh.vertex_adjacency), built with torch ops on the CPU here: every valid
corner listed once under its vertex, slot 0 corners first, then slot 1,
then slot 2, each in triangle order; triangles with an out-of-range index
left out; ragged meshes with their own vertex and triangle offsets."""
import numpy as np
import torch

from diffren_gb300 import kernels, mesh


def brute(tris_per_mesh, vcounts):
  out = {}
  g = 0
  vo = 0
  for tris, nv in zip(tris_per_mesh, vcounts):
    for t_local, tri in enumerate(tris):
      ok = all(0 <= int(i) < nv for i in tri)
      for s in range(3):
        if ok:
          out.setdefault(vo + int(tri[s]), []).append((s, g + t_local, 3 * (g + t_local) + s))
    g += len(tris)
    vo += nv
  return {v: [c for _, _, c in sorted(lst)] for v, lst in out.items()}


def test_vertex_adjacency_order_and_validity():
  rng = np.random.default_rng(0)
  vcounts = [7, 1, 12, 5]
  tris = [rng.integers(0, nv, (n, 3)) for nv, n in zip(vcounts, [9, 0, 20, 6])]
  tris[2][3] = [0, 12, 1]   # out of range: left out
  tris[3][1] = [-1, 0, 2]
  batch = kernels.ImageBatch([4] * 4, [4] * 4, vcounts, [len(t) for t in tris])
  packed = torch.tensor(np.concatenate([t for t in tris if len(t)]), dtype=torch.int32)
  off, corners = mesh.vertex_adjacency(packed, batch)
  assert off.dtype == torch.int64 and corners.dtype == torch.int32
  V = sum(vcounts)
  assert off.shape == (V + 1,) and int(off[0]) == 0
  want = brute(tris, vcounts)
  for v in range(V):
    got = corners[int(off[v]):int(off[v + 1])].tolist()
    assert got == want.get(v, []), v


def test_vertex_adjacency_shared_triangle_list():
  """B meshes over one triangle list (compute_vertex_normals of batched
  vertices): each mesh's triangles are numbered after the previous mesh's."""
  tris = torch.tensor([[0, 1, 2], [2, 1, 3]], dtype=torch.int32)
  batch = mesh._shared_batch(2, 4, 2)
  off, corners = mesh.vertex_adjacency(tris, batch)
  # vertex 4 + 1 (mesh 1's vertex 1): slot 1 of triangles 2 and 3
  assert corners[int(off[5]):int(off[6])].tolist() == [3 * 2 + 1, 3 * 3 + 1]
  # vertex 2: slot 2 of triangle 0, then slot 0 of triangle 1 -> slot order
  assert corners[int(off[2]):int(off[3])].tolist() == [3 * 1 + 0, 3 * 0 + 2]
