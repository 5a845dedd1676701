"""Vertex-normal kernels (mesh.py:22-52) against the CPU restatement, the
reference's own sphere known answers and autograd of the restatement."""
import numpy as np
import pytest
import torch

import helpers
from diffren_gb300 import kernels, mesh
from oracle import mesh as omesh

pytestmark = pytest.mark.gpu

# Normals are unit vectors: 1e-5 of unit length against float64.
NORMAL_ATOL = 1e-5
GRAD_RTOL = 1e-4


def sphere():
  g = helpers.golden("render_goldens.npz")
  return g["sphere_vertices"].astype(np.float32), g["sphere_triangles"].astype(np.int32)


def noisy_grid(n, seed):
  """A bumpy n x n heightfield: every interior vertex in six triangles."""
  rng = np.random.default_rng(seed)
  y, x = np.meshgrid(np.linspace(-1, 1, n), np.linspace(-1, 1, n), indexing="ij")
  z = 0.1 * np.sin(3 * x) * np.cos(2 * y) + rng.normal(0, 0.01, x.shape)
  v = np.stack([x, y, z], -1).reshape(-1, 3).astype(np.float32)
  i = np.arange(n * n).reshape(n, n)
  a, b, c, d = i[:-1, :-1], i[:-1, 1:], i[1:, :-1], i[1:, 1:]
  t = np.concatenate([np.stack([a, b, d], -1).reshape(-1, 3),
                      np.stack([a, d, c], -1).reshape(-1, 3)]).astype(np.int32)
  return v, t


def test_sphere_known_answers(device):
  """mesh_test.py:32-80, unbatched and through the [B, V, 3] form."""
  v, t = sphere()
  out = mesh.compute_vertex_normals(torch.tensor(v, device=device),
                                    torch.tensor(t, device=device))
  np.testing.assert_array_almost_equal(v, out.cpu().numpy(), decimal=2)
  s = v.copy()
  s[:, 2] *= 2.0
  want = v.copy()
  want[:, 2] *= 0.5
  want /= np.linalg.norm(want, axis=1, keepdims=True)
  both = mesh.compute_vertex_normals(torch.tensor(np.stack([v, s]), device=device),
                                     torch.tensor(t, device=device)).cpu().numpy()
  np.testing.assert_array_almost_equal(v, both[0], decimal=2)
  np.testing.assert_array_almost_equal(want, both[1], decimal=2)
  np.testing.assert_allclose(both[1], omesh.vertex_normals(s, t), atol=NORMAL_ATOL)


@pytest.mark.parametrize("n", [2, 17, 300])
def test_grid_matches_oracle(n, device):
  v, t = noisy_grid(n, n)
  out = mesh.compute_vertex_normals(torch.tensor(v, device=device),
                                    torch.tensor(t, device=device))
  np.testing.assert_allclose(out.cpu().numpy(), omesh.vertex_normals(v, t), atol=NORMAL_ATOL)


def test_ragged_batch_matches_per_mesh(device):
  """Meshes of different sizes, unused vertices (normal 0) and an
  out-of-range index (adds nothing) in one call."""
  meshes = [noisy_grid(5, 1), sphere(), noisy_grid(40, 2)]
  v0, t0 = meshes[0]
  v0 = np.concatenate([v0, np.ones((3, 3), np.float32)])  # unreferenced rows
  t0 = np.concatenate([t0, [[0, 1, 10_000]]]).astype(np.int32)
  meshes[0] = (v0, t0)
  batch = kernels.ImageBatch([1] * 3, [1] * 3, [len(m[0]) for m in meshes],
                             [len(m[1]) for m in meshes])
  vs = torch.tensor(np.concatenate([m[0] for m in meshes]), device=device)
  ts = torch.tensor(np.concatenate([m[1] for m in meshes]), device=device)
  out = mesh.vertex_normals_packed(vs, ts, batch).cpu().numpy()
  want = [omesh.vertex_normals(v0, t0[:-1])] + [omesh.vertex_normals(*m) for m in meshes[1:]]
  np.testing.assert_allclose(out, np.concatenate(want), atol=NORMAL_ATOL)
  assert np.all(out[len(v0) - 3:len(v0)] == 0)


@pytest.mark.parametrize("batched", [False, True])
def test_vjp_matches_autograd(batched, device):
  v, t = noisy_grid(24, 7)
  rng = np.random.default_rng(3)
  if batched:
    v = np.stack([v, v * np.float32(1.3) + np.float32(0.1)])
  g = rng.standard_normal(v.shape).astype(np.float32)
  ref_v = torch.tensor(v, dtype=torch.float64, requires_grad=True)
  tt = torch.tensor(t, dtype=torch.int64)
  ref = torch.stack([omesh.vertex_normals_t(x, tt) for x in ref_v.reshape(-1, *v.shape[-2:])])
  (want,) = torch.autograd.grad(ref.reshape(v.shape), ref_v, torch.tensor(g, dtype=torch.float64))
  dv = torch.tensor(v, device=device, requires_grad=True)
  out = mesh.compute_vertex_normals(dv, torch.tensor(t, device=device))
  (got,) = torch.autograd.grad(out, dv, torch.tensor(g, device=device))
  want = want.numpy()
  scale = float(np.abs(want).max())
  np.testing.assert_allclose(got.cpu().numpy(), want, rtol=GRAD_RTOL, atol=GRAD_RTOL * scale)


def test_empty_mesh(device):
  out = mesh.compute_vertex_normals(torch.zeros(0, 3, device=device),
                                    torch.zeros(0, 3, dtype=torch.int32, device=device))
  assert out.shape == (0, 3)
  v, _ = sphere()
  out = mesh.compute_vertex_normals(torch.tensor(v, device=device),
                                    torch.zeros(0, 3, dtype=torch.int32, device=device))
  assert torch.all(out == 0)


def slot_sums_f32(v, t):
  """The kernels' summation in float32: face normal cross(v1 - v0, v2 - v0)
  with every operation rounded, per vertex the slot 0, 1 and 2 sums in
  triangle order, then (s0 + s1) + s2 (three scatter-adds into zeros)."""
  v = v.astype(np.float32)
  c = v[t.astype(np.int64)]
  e1, e2 = (c[:, 1] - c[:, 0]).astype(np.float32), (c[:, 2] - c[:, 0]).astype(np.float32)
  n = np.stack([e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1],
                e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2],
                e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]], 1).astype(np.float32)
  slots = []
  for s in range(3):
    acc = np.zeros_like(v)
    np.add.at(acc, t[:, s].astype(np.int64), n)  # sequential, in triangle order
    slots.append(acc)
  return ((slots[0] + slots[1]) + slots[2]).astype(np.float32)


def test_normals_are_the_same_bits_every_run_and_sum_in_triangle_order(device):
  """The adjacency-based normals: forward and gradient repeat bit for bit,
  and the normals equal the float32 slot-ordered sums normalized (to the
  last bits of the reciprocal square root)."""
  v, t = noisy_grid(40, seed=5)
  vt = torch.tensor(v, device=device)
  tt = torch.tensor(t, device=device)
  g = torch.tensor(np.random.default_rng(1).standard_normal(v.shape).astype(np.float32),
                   device=device)
  outs = []
  for _ in range(2):
    x = vt.clone().requires_grad_(True)
    out = mesh.compute_vertex_normals(x, tt)
    (d,) = torch.autograd.grad(out, (x,), g)
    outs.append((out.detach(), d))
  assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])
  x = slot_sums_f32(v, t).astype(np.float64)
  ref = x / np.sqrt((x * x).sum(1, keepdims=True) + 1e-12)
  np.testing.assert_allclose(outs[0][0].cpu().numpy(), ref, rtol=0, atol=1e-6)


def test_atomic_normals_entry_points_match_the_adjacency_ones(device):
  """dr_vertex_normals_fwd / _bwd (float atomics, kept in the ABI) against
  dr_vertex_normals_csr_fwd / _bwd on a ragged two-mesh batch: normals
  within 1e-6, vertex gradients within 1e-5 of their largest magnitude
  (the two sum in different orders)."""
  import ctypes
  from diffren_gb300 import _lib
  lib = _lib.load()
  v0, t0 = noisy_grid(20, seed=2)
  v1, t1 = sphere()
  batch = kernels.ImageBatch([1, 1], [1, 1], [len(v0), len(v1)], [len(t0), len(t1)])
  v = torch.tensor(np.concatenate([v0, v1]), device=device)
  t = torch.tensor(np.concatenate([t0, t1]), device=device)
  V, T = v.shape[0], t.shape[0]
  P = lambda x: ctypes.c_void_p(x.data_ptr())
  s = ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
  acc = torch.empty(V, 4, device=device)
  n_atomic = torch.empty(V, 3, device=device)
  assert lib.dr_vertex_normals_fwd(P(v), P(t), batch.ptr, 2, P(acc), P(n_atomic), s) == 0
  g = torch.tensor(np.random.default_rng(0).standard_normal((V, 3)).astype(np.float32),
                   device=device)
  d_acc = torch.empty(V, 4, device=device)
  d_atomic = torch.zeros(V, 3, device=device)
  assert lib.dr_vertex_normals_bwd(P(g), P(v), P(t), batch.ptr, 2, P(acc), P(d_acc),
                                   P(d_atomic), s) == 0
  x = v.clone().requires_grad_(True)
  n_csr = mesh.vertex_normals_packed(x, t, batch)
  (d_csr,) = torch.autograd.grad(n_csr, (x,), g)
  torch.testing.assert_close(n_atomic, n_csr.detach(), rtol=0, atol=1e-6)
  scale = float(d_csr.abs().max())
  torch.testing.assert_close(d_atomic, d_csr, rtol=0, atol=1e-5 * scale)
