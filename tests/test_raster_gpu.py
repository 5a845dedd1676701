"""GPU parity of the CUDA rasterizer, through the C ABI, against the oracle
(bit-exact ids, depth and barycentrics in both depth semantics) and against
the reference CPU rasterizer's recorded outputs."""
import ctypes

import numpy as np
import pytest
import torch

import helpers
from diffren_gb300 import _lib, kernels, workloads
from oracle import raster

pytestmark = pytest.mark.gpu

FIX = helpers.golden("raster_ref.npz")
CASES = sorted({k.split("__")[0] for k in FIX.files})


def _bits(a):
  return np.asarray(a).view(np.uint32)


def run_abi(verts, tris, w, h, layers, cull, mode, device, tile=(0, 0)):
  """Calls dr_rasterize_batch for one image; returns numpy (ids, z, bary)."""
  v = torch.as_tensor(np.asarray(verts, np.float32), device=device).contiguous()
  t = torch.as_tensor(np.asarray(tris, np.int32).reshape(-1, 3), device=device).contiguous()
  batch = kernels.ImageBatch.single(w, h, v.shape[0], t.shape[0])
  cfg = kernels.raster_config(layers, cull, mode, tile)
  ids, z, b = kernels.rasterize_packed(v, t, batch, cfg)
  torch.cuda.synchronize()
  return (ids.view(layers, h, w).cpu().numpy(), z.view(layers, h, w).cpu().numpy(),
          b.view(layers, h, w, 3).cpu().numpy())


def assert_same(ours, ref):
  for a, b, name in zip(ours, ref, ("ids", "z", "bary")):
    a, b = np.asarray(a), np.asarray(b)
    if not np.array_equal(_bits(a), _bits(b)):
      bad = np.argwhere(_bits(a) != _bits(b))
      raise AssertionError("%s differs at %d elements, first %s: %r vs %r" % (
          name, len(bad), bad[0], a[tuple(bad[0])], b[tuple(bad[0])]))


@pytest.mark.parametrize("name", CASES)
def test_float_mode_matches_reference_cpu_fixture(name, device):
  g = lambda k: FIX[name + "__" + k]
  w, h, layers, cull = (int(x) for x in g("meta"))
  ours = run_abi(g("vertices"), g("triangles"), w, h, layers, cull, _lib.DR_DEPTH_FLOAT,
                 device)
  assert_same(ours, (g("ids"), g("z"), g("bary")))


@pytest.mark.parametrize("name", CASES)
def test_discretized_mode_matches_oracle(name, device):
  g = lambda k: FIX[name + "__" + k]
  w, h, layers, cull = (int(x) for x in g("meta"))
  ref = raster.rasterize(g("vertices"), g("triangles"), w, h, layers, cull,
                         raster.DEPTH_DISCRETIZED)
  ours = run_abi(g("vertices"), g("triangles"), w, h, layers, cull,
                 _lib.DR_DEPTH_DISCRETIZED, device)
  assert_same(ours, ref)


RANDOM = [
    # (kind, n, w, h, layers, cull, tile)
    ("soup", 4000, 200, 150, 3, 1, (0, 0)),
    ("soup", 4000, 200, 150, 5, 0, (32, 8)),
    ("soup", 2500, 131, 77, 2, 2, (8, 8)),
    ("soup", 50, 1, 1, 3, 0, (0, 0)),
    ("soup", 300, 17, 13, 4, 0, (16, 16)),
    ("ico", 12, 257, 255, 3, 1, (0, 0)),
    ("ico", 30, 320, 240, 8, 0, (64, 16)),
    ("height", 60, 300, 200, 3, 1, (0, 0)),
    ("near", 3000, 120, 90, 3, 0, (0, 0)),
    ("big", 40, 640, 480, 2, 0, (0, 0)),
]


def _scene(kind, n, w, h, seed):
  if kind == "soup":
    m = workloads.soup_workload(n, seed=seed, mu=-2.5, sigma=0.8)
    eye = workloads.sphere_eyes(1, seed=seed)[0]
  elif kind == "ico":
    m = workloads.icosphere_workload(n, seed=seed)
    eye = workloads.sphere_eyes(1, seed=seed)[0]
  elif kind == "height":
    m = workloads.heightfield_workload(n, seed=seed)
    eye = workloads.sphere_eyes(1, seed=seed, upper_only=True)[0]
  elif kind == "near":  # camera inside the geometry: near-plane clipping
    m = workloads.soup_workload(n, seed=seed, mu=-1.5, sigma=0.5)
    eye = np.array([0.05, 0.1, 0.2])
  else:  # few big triangles spanning many tiles (large-triangle list)
    m = workloads.soup_workload(n, seed=seed, mu=0.0, sigma=0.3)
    eye = workloads.sphere_eyes(1, seed=seed, radius=2.0)[0]
  cam = workloads.camera_matrix(eye, w, h)
  return raster.transform(cam, m.vertices), m.triangles


@pytest.mark.parametrize("mode", [_lib.DR_DEPTH_DISCRETIZED, _lib.DR_DEPTH_FLOAT])
@pytest.mark.parametrize("case", range(len(RANDOM)))
def test_random_scenes_match_oracle(case, mode, device):
  kind, n, w, h, layers, cull, tile = RANDOM[case]
  clip, tris = _scene(kind, n, w, h, seed=case)
  ref = raster.rasterize(clip, tris, w, h, layers, cull, mode)
  ours = run_abi(clip, tris, w, h, layers, cull, mode, device, tile)
  assert_same(ours, ref)


def test_c2_full_size_matches_oracle(device):
  """200k-triangle soup, 512x512, 3 layers, back culling (c2 camera 0)."""
  m = workloads.soup_workload(200000, seed=0)
  cam = workloads.camera_matrix(workloads.sphere_eyes(8, seed=1)[0], 512, 512)
  clip = raster.transform(cam, m.vertices)
  ref = raster.rasterize(clip, m.triangles, 512, 512, 3, 1)
  ours = run_abi(clip, m.triangles, 512, 512, 3, 1, _lib.DR_DEPTH_DISCRETIZED, device)
  assert_same(ours, ref)


def test_depth_codec_matches_double_formulas_exhaustively(device):
  """The integer depth codec equals the reference's double-precision
  DiscretizeZ / UndiscretizeZ on all 2^32 inputs (every float in [-1, 1]
  and NaN for the first)."""
  res = torch.tensor([0, -1, 0, -1, 0, 0, 0], dtype=torch.int64, device=device)
  rc = _lib.load().dr_selftest_depth_codec(ctypes.c_void_p(res.data_ptr()),
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
  assert rc == 0
  r = res.cpu().numpy().view(np.uint64)
  assert r[0] == 0, "discretize mismatches: %d, first input bits %#x" % (r[0], r[1])
  assert r[2] == 0, "undiscretize mismatches: %d, first input %d" % (r[2], r[3])
  # NaN conversions are what the CPU checker assumes.
  got = (int(r[4]), int(r[5]) & 0xffffffff, int(r[6]))
  want = (raster.NAN_TO_U32_FROM_DOUBLE, raster.NAN_TO_I32 & 0xffffffff,
          raster.NAN_TO_I64 & 0xffffffffffffffff)
  assert got == want, [hex(x) for x in got]


def test_empty_and_degenerate_inputs(device):
  # No triangles: every layer is background.
  ids, z, b = run_abi(np.zeros((3, 4), np.float32), np.zeros((0, 3), np.int32), 9, 7, 2,
                      0, 0, device)
  assert (ids == 0).all() and (z == 1).all() and (b == 0).all()
  ids, z, b = run_abi(np.zeros((3, 4), np.float32), np.zeros((0, 3), np.int32), 9, 7, 2,
                      0, 1, device)
  assert (ids == -1).all()
  # Degenerate triangle on a 1x1 image (impl_test.cc:213-225).
  v = np.array([[-1, -1, 0, 1], [1, 1, 0, 1], [0, 0, 0, 1]], np.float32)
  _, _, b = run_abi(v, [[0, 1, 2]], 1, 1, 1, 0, 0, device)
  assert abs(b.sum()) < 1e-6


def test_out_of_range_indices_are_skipped_and_flagged(device):
  v = torch.tensor([[-0.5, -0.5, 0.5, 1], [0.5, -0.5, 0.5, 1], [0, 0.5, 0.5, 1]],
                   device=device)
  t = torch.tensor([[0, 1, 2], [0, 1, 7], [-1, 0, 1]], dtype=torch.int32, device=device)
  batch = kernels.ImageBatch.single(32, 32, 3, 3)
  cfg = kernels.raster_config(1, 0, 0)
  ws = kernels.Workspace(device)
  ids, _, _ = kernels.rasterize_packed(v, t, batch, cfg, workspace=ws)
  flags = kernels.read_error_flags(ws, device)
  assert flags & _lib.DR_FLAG_INDEX_OUT_OF_RANGE
  ref = raster.rasterize(v.cpu().numpy(), np.array([[0, 1, 2]], np.int32), 32, 32, 1, 0)
  np.testing.assert_array_equal(ids.view(1, 32, 32).cpu().numpy(), ref[0])


def test_nonfinite_vertices_are_flagged_and_rasterized_as_the_oracle(device):
  v = np.array([[-0.5, -0.5, 0.5, 1], [0.5, -0.5, 0.5, 1], [0, 0.5, 0.5, 1],
                [0.2, 0.2, np.nan, 1], [0.9, 0.1, 0.5, 1], [0.1, 0.9, 0.5, np.inf]], np.float32)
  t = np.array([[0, 1, 2], [3, 4, 5], [0, 4, 2]], np.int32)
  batch = kernels.ImageBatch.single(32, 32, 6, 3)
  cfg = kernels.raster_config(2, 0, 0)
  ws = kernels.Workspace(device)
  ids, z, _ = kernels.rasterize_packed(torch.tensor(v, device=device),
                                       torch.tensor(t, device=device), batch, cfg, workspace=ws)
  assert kernels.read_error_flags(ws, device) & _lib.DR_FLAG_NONFINITE_VERTEX
  ref = raster.rasterize(v, t, 32, 32, 2, 0)
  np.testing.assert_array_equal(ids.view(2, 32, 32).cpu().numpy(), ref[0])
  # finite input raises no flag
  ws2 = kernels.Workspace(device)
  kernels.rasterize_packed(torch.tensor(v[:3], device=device),
                           torch.tensor(t[:1], device=device),
                           kernels.ImageBatch.single(32, 32, 3, 1), cfg, workspace=ws2)
  assert kernels.read_error_flags(ws2, device) == 0


def test_invalid_arguments_raise(device):
  v = torch.zeros(3, 4, device=device)
  t = torch.zeros(1, 3, dtype=torch.int32, device=device)
  with pytest.raises(_lib.DiffrenError):
    kernels.rasterize_packed(v, t, kernels.ImageBatch.single(8, 8, 3, 1),
                             kernels.raster_config(17, 0, 0))
  with pytest.raises(_lib.DiffrenError):
    kernels.rasterize_packed(v, t, kernels.ImageBatch.single(8, 8, 3, 1),
                             kernels.raster_config(1, 3, 0))
  lib = _lib.load()
  rc = lib.dr_rasterize_triangles(ctypes.c_void_p(v.data_ptr() + 4), 3,
                                  ctypes.c_void_p(t.data_ptr()), 1, 8, 8, 1, 0, 0,
                                  None, None, None, None, 0, None)
  assert rc != 0


def test_ragged_batch_equals_single_images(device):
  """One batched launch over meshes of different sizes and resolutions gives
  exactly the per-image results."""
  meshes, cams, sizes = workloads.ragged_batch(6, seed=3, median_triangles=3000,
                                               resolutions=(64, 96, 160))
  clips = [raster.transform(c, m.vertices) for m, c in zip(meshes, cams)]
  batch = kernels.ImageBatch([s[0] for s in sizes], [s[1] for s in sizes],
                             [len(c) for c in clips], [len(m.triangles) for m in meshes])
  v = torch.as_tensor(np.concatenate(clips), device=device)
  t = torch.as_tensor(np.concatenate([m.triangles for m in meshes]), device=device)
  ids, z, b = kernels.rasterize_packed(v, t, batch, kernels.raster_config(3, 1, 0))
  for i, (m, c, (w, h)) in enumerate(zip(meshes, clips, sizes)):
    ref = raster.rasterize(c, m.triangles, w, h, 3, 1)
    got = (batch.layered_view(ids, i, 3).cpu().numpy(),
           batch.layered_view(z, i, 3).cpu().numpy(),
           batch.layered_view(b, i, 3).cpu().numpy())
    assert_same(got, ref)
