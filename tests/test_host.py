"""CPU tests of host-side logic: batch tables, validation, workloads,
cameras. No GPU work."""
import math

import numpy as np
import pytest
import torch

import helpers
from diffren_gb300 import camera, constants, kernels, rasterize, render, workloads
from diffren_gb300 import framebuffer as fb


def test_image_batch_offsets_and_views():
  b = kernels.ImageBatch([4, 8, 2], [3, 2, 5], [10, 20, 30], [5, 6, 7])
  assert list(b.pixel_offsets) == [0, 12, 28, 38]
  assert list(b.vertex_offsets) == [0, 10, 30, 60]
  assert list(b.triangle_offsets) == [0, 5, 11, 18]
  assert b.descs[2].pixel_offset == 28 and b.descs[1].vertex_offset == 10
  flat = torch.arange(3 * b.total_pixels * 2).view(-1, 2)
  v = b.layered_view(flat, 1, 3)
  assert v.shape == (3, 2, 8, 2) and int(v[0, 0, 0, 0]) == 3 * 12 * 2
  img = b.image_view(torch.arange(b.total_pixels * 4).view(-1, 4), 2)
  assert img.shape == (5, 2, 4) and int(img[0, 0, 0]) == 28 * 4
  idx = b.vertex_image_index("cpu")
  assert idx.shape[0] == 60 and int(idx[9]) == 0 and int(idx[10]) == 1
  with pytest.raises(ValueError):
    kernels.ImageBatch([0], [1], [1], [1])


def test_render_validates_before_gpu_work():
  v = torch.zeros(3, 3)
  t = torch.zeros(1, 3, dtype=torch.int32)
  with pytest.raises(ValueError, match="Backface culling"):
    render.render_triangles(v, {}, t, torch.eye(4), 8, 8, lambda x: x,
                            face_culling_mode=constants.FaceCullingMode.NONE)
  with pytest.raises(ValueError, match="vertices must have shape"):
    rasterize.rasterize_triangles(torch.zeros(3, 5), t, None, 8, 8)
  with pytest.raises(ValueError, match="triangles must have shape"):
    rasterize.rasterize_triangles(v, torch.zeros(2, 2), torch.eye(4), 8, 8)
  with pytest.raises(ValueError, match="camera must be"):
    rasterize.rasterize_triangles(v, t, torch.eye(3), 8, 8)
  with pytest.raises(ValueError, match="image_width"):
    rasterize.rasterize_triangles(v, t, torch.eye(4), 0, 8)
  with pytest.raises(ValueError, match="num_layers"):
    rasterize.rasterize_triangles(v, t, torch.eye(4), 8, 8, num_layers=0)
  with pytest.raises(ValueError, match="clip coordinates"):
    rasterize.rasterize_triangles(v, t, None, 8, 8)


def test_framebuffer_shape_contract():
  b = torch.zeros(2, 4, 5, 3)
  ids = torch.zeros(2, 4, 5, 1, dtype=torch.int32)
  frame = fb.Framebuffer(b, ids, triangles=torch.zeros(1, 3, dtype=torch.int64),
                         z_buffer=torch.ones(2, 4, 5))
  assert (frame.num_layers, frame.height, frame.width) == (2, 4, 5)
  assert frame.foreground_mask.shape == (2, 4, 5, 1)
  assert float(frame.background_mask.sum()) == 40
  assert frame.layer(1).barycentrics.shape == (4, 5, 3)
  with pytest.raises(ValueError, match="Expected all input shapes"):
    fb.Framebuffer(b, torch.zeros(2, 4, 6, 1), triangles=torch.zeros(1, 3),
                   z_buffer=torch.ones(2, 4, 5))


def test_icosphere_counts_and_orientation():
  for f in (1, 2, 16, 71):
    v, t = workloads.icosphere(f)
    assert len(t) == 20 * f * f and len(v) == 10 * f * f + 2
    a, b, c = v[t[:, 0]], v[t[:, 1]], v[t[:, 2]]
    assert (np.einsum("ij,ij->i", np.cross(b - a, c - a), a) > 0).all()
  assert workloads.frequency_for_triangles(100820) == 71


def test_heightfield_topology_matches_depthmap_split():
  t = workloads.grid_triangles(3)
  # depthmap.py:22-64: per quad (bl, br, tl) and (br, tr, tl), row-major.
  np.testing.assert_array_equal(t[:2], [[0, 1, 3], [1, 4, 3]])
  assert len(t) == 2 * 2 * 2
  m = workloads.heightfield_workload(20, seed=1)
  a, b, c = (m.vertices[m.triangles[:, i]] for i in range(3))
  assert (np.cross(b - a, c - a)[:, 1] > 0).all()  # faces up


def test_camera_matches_reference_formulas():
  # camera.py:23-44: perspective via intrinsics and ortho.
  p = camera.perspective(4 / 3, 40.0, 0.01, 10.0)
  f = 1 / math.tan(40 * math.pi / 360)
  np.testing.assert_allclose(p[0, 0], f / (4 / 3))
  np.testing.assert_allclose(p[1, 1], f)
  np.testing.assert_allclose(p, helpers.make_perspective_matrix(0), rtol=1e-6, atol=1e-9)
  la = camera.look_at((2.0, 3.0, 6.0), (0, 0, 0), (0, 1, 0))
  np.testing.assert_allclose(la, helpers.make_look_at_matrix("view_1"), atol=1e-12)
  with pytest.raises(ValueError):
    camera.look_at((0, 0, 0), (0, 0, 0), (0, 1, 0))


def test_ragged_batch_statistics():
  meshes, cams, sizes = workloads.ragged_batch(64, seed=0)
  counts = np.array([len(m.triangles) for m in meshes])
  assert counts.min() >= 400 and counts.max() <= 520000
  assert set(s[0] for s in sizes) <= {256, 512, 1024}
  assert len(cams) == 64 and all(c.shape == (4, 4) for c in cams)


def test_launch_counter():
  kernels.LAUNCHES.reset()
  with kernels._op("x", 3):
    pass
  assert kernels.LAUNCHES.count == 3


def test_diff_barycentrics_tangent_matches_oracle_forward_mode():
  """The forward-mode rule of the differentiable barycentrics (torch ops,
  runs on the CPU) against torch.func.jvp of the float64 restatement of
  rasterize.py:127-255."""
  import types
  from oracle import raster, torch_ref
  m = workloads.icosphere_workload(4, seed=1)
  W, H, L = 24, 20, 2
  clip = raster.transform(workloads.camera_matrix((0.3, 0.2, 2.5), W, H), m.vertices)
  ids, z, _ = raster.rasterize(clip, m.triangles, W, H, L, 0)
  batch = kernels.ImageBatch.single(W, H, len(m.vertices), len(m.triangles))
  tc = torch.tensor(clip)
  d_clip = torch.randn(tc.shape, generator=torch.Generator().manual_seed(0)) * 0.01
  ctx = types.SimpleNamespace(
      saved_tensors=(tc, torch.tensor(m.triangles), torch.tensor(ids).reshape(-1),
                     torch.tensor(z).reshape(-1)), batch=batch, L=L)
  got = kernels._DiffBary.jvp(ctx, d_clip)

  def bary(c):
    return torch_ref.diff_barycentrics(c, torch.tensor(ids), torch.tensor(z),
                                       torch.tensor(m.triangles).long(), W, H)

  _, want = torch.func.jvp(bary, (tc.double(),), (d_clip.double(),))
  want = want.reshape(-1, 3)
  assert float((got.double() - want).abs().max()) <= 1e-4 * float(want.abs().max())
