"""Test infrastructure only: CPU restatement of diffren's area-weighted
vertex normals (diffren/jax/utils/mesh.py:22-52, transforms.py:26-37), in
numpy (forward) and torch (any dtype, for gradients): face normal
cross(v1 - v0, v2 - v0) scattered to the triangle's three vertices, summed
per corner slot as (c0 + c1) + c2, then x * rsqrt(sum(x^2) + 1e-12)."""
import numpy as np
import torch


def vertex_normals(vertices, triangles, dtype=np.float64):
  v = np.asarray(vertices, dtype)
  t = np.asarray(triangles, np.int64)
  c = v[t]
  n = np.cross(c[:, 1] - c[:, 0], c[:, 2] - c[:, 0])
  slots = []
  for i in range(3):
    acc = np.zeros_like(v)
    np.add.at(acc, t[:, i], n)
    slots.append(acc)
  x = (slots[0] + slots[1]) + slots[2]
  return x / np.sqrt((x * x).sum(1, keepdims=True) + 1e-12)


def vertex_normals_t(vertices, triangles):
  t = triangles.long()
  c = vertices[t]
  n = torch.cross(c[:, 1] - c[:, 0], c[:, 2] - c[:, 0], dim=1)
  x = torch.zeros_like(vertices)
  for i in range(3):
    x = x + torch.zeros_like(vertices).index_add(0, t[:, i], n)
  return x * torch.rsqrt((x * x).sum(1, keepdim=True) + 1e-12)
