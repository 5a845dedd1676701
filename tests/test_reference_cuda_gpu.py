"""GPU parity of the discretized depth semantics (the default) against the
reference's own CUDA rasterizer, diffren::cuda::RasterizeTrianglesImpl
(diffren/common/kernels/rasterize_triangles_impl_cuda.cu.cc:397-484), built
for sm_103a with nvcc's default flags by oracle/Makefile and run on the same
GPU on the same inputs: triangle ids, depth and barycentrics bit for bit.

Covered: the reference tests' own geometry, seeded scenes, the random scenes
of the rasterizer tests (every tile shape they use), non-power-of-two image
sizes (where the pixel-centre multiply-add of the CUDA build matters), the
200k-triangle 512x512 soup of the plain GPU workload at all eight cameras,
and the whole 64-mesh ragged batch of the benchmark in one batched launch
with the default and a wide tile (and the fused interpolating epilogue).
"""
import numpy as np
import pytest
import torch

import test_raster_gpu as trg
from diffren_gb300 import _lib, kernels, workloads
from golden import make_golden_cuda
from oracle import raster

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ref_built():
  if raster.build_reference_cuda() is None:
    pytest.skip("reference CUDA rasterizer sources not present (DIFFREN_REFERENCE or the "
                "staged copy in oracle/_ref/src)")
  return True


def ref_cuda(clip, tris, w, h, layers, cull, device):
  """Runs the reference CUDA rasterizer; returns numpy (ids, z, bary)."""
  v = torch.as_tensor(np.ascontiguousarray(clip, np.float32), device=device)
  t = torch.as_tensor(np.ascontiguousarray(tris, np.int32).reshape(-1, 3), device=device)
  ids = torch.full((layers, h, w), 7, dtype=torch.int32, device=device)
  z = torch.full((layers, h, w), 7.0, device=device)
  b = torch.full((layers, h, w, 3), 7.0, device=device)
  raster.rasterize_reference_cuda(v.data_ptr(), t.data_ptr(), t.shape[0], w, h, layers, cull,
                                  ids.data_ptr(), z.data_ptr(), b.data_ptr(),
                                  torch.cuda.current_stream(device).cuda_stream)
  torch.cuda.synchronize(device)
  return ids.cpu().numpy(), z.cpu().numpy(), b.cpu().numpy()


def check(clip, tris, w, h, layers, cull, device, tile=(0, 0)):
  ref = ref_cuda(clip, tris, w, h, layers, cull, device)
  ours = trg.run_abi(clip, tris, w, h, layers, cull, _lib.DR_DEPTH_DISCRETIZED, device, tile)
  trg.assert_same(ours, ref)
  return ref


@pytest.mark.parametrize("name", trg.CASES)
def test_reference_test_geometry(name, device, ref_built):
  g = lambda k: trg.FIX[name + "__" + k]
  w, h, layers, cull = (int(x) for x in g("meta"))
  check(g("vertices"), g("triangles"), w, h, layers, cull, device)


@pytest.mark.parametrize("name", sorted(make_golden_cuda.SEEDED))
def test_seeded_scenes(name, device, ref_built):
  _, _, _, w, h, layers, cull = make_golden_cuda.SEEDED[name]
  clip, tris = make_golden_cuda.seeded_scene(name, w, h)
  ref = check(clip, tris, w, h, layers, cull, device)
  # The CPU oracle agrees with the reference build too.
  trg.assert_same(raster.rasterize(clip, tris, w, h, layers, cull, raster.DEPTH_DISCRETIZED),
                  ref)


@pytest.mark.parametrize("case", range(len(trg.RANDOM)))
def test_random_scenes(case, device, ref_built):
  kind, n, w, h, layers, cull, tile = trg.RANDOM[case]
  clip, tris = trg._scene(kind, n, w, h, seed=case)
  check(clip, tris, w, h, layers, cull, device, tile)


@pytest.mark.parametrize("size", [(640, 480), (131, 77), (1000, 600), (333, 517)])
@pytest.mark.parametrize("kind", ["soup_none", "soup_back", "ico"])
def test_non_power_of_two_sizes(size, kind, device, ref_built):
  w, h = size
  seed = w % 7
  cam = workloads.camera_matrix(workloads.sphere_eyes(1, seed=seed)[0], w, h)
  if kind == "ico":
    m = workloads.icosphere_workload(40, seed=seed)
  else:
    m = workloads.soup_workload(20000, seed=seed, mu=-3.0, sigma=0.8)
  check(raster.transform(cam, m.vertices), m.triangles, w, h, 3,
        0 if kind == "soup_none" else 1, device)


def test_c2_soup_all_cameras(device, ref_built):
  """200k-triangle soup, 512x512, 3 layers, back culling, 8 cameras: each
  camera alone and all eight in one batched launch."""
  m = workloads.soup_workload(200000, seed=0)
  eyes = workloads.sphere_eyes(8, seed=1)
  clips, refs = [], []
  for e in eyes:
    clip = raster.transform(workloads.camera_matrix(e, 512, 512), m.vertices)
    refs.append(check(clip, m.triangles, 512, 512, 3, 1, device))
    clips.append(clip)
  batch = kernels.ImageBatch([512] * 8, [512] * 8, [len(m.vertices)] * 8,
                             [len(m.triangles)] * 8)
  v = torch.as_tensor(np.concatenate(clips), device=device)
  t = torch.as_tensor(np.tile(m.triangles, (8, 1)), device=device)
  ids, z, b = kernels.rasterize_packed(v, t, batch,
                                       kernels.raster_config(3, 1, _lib.DR_DEPTH_DISCRETIZED))
  for i, ref in enumerate(refs):
    trg.assert_same((batch.layered_view(ids, i, 3).cpu().numpy(),
                     batch.layered_view(z, i, 3).cpu().numpy(),
                     batch.layered_view(b, i, 3).cpu().numpy()), ref)


@pytest.mark.parametrize("tile", [(0, 0), (32, 32)])
def test_ragged_benchmark_batch(tile, device, ref_built):
  """The benchmark's 64 meshes (256-1024 px, 500-500k triangles) in one
  batched launch of the fused rasterizer (ids, z and barycentrics out of the
  interpolating epilogue), every image against the reference."""
  meshes, cams, sizes = workloads.ragged_batch(64, seed=0)
  clips = [raster.transform(c, mm.vertices) for mm, c in zip(meshes, cams)]
  batch = kernels.ImageBatch([s[0] for s in sizes], [s[1] for s in sizes],
                             [len(c) for c in clips], [len(mm.triangles) for mm in meshes])
  v = torch.as_tensor(np.concatenate(clips), device=device)
  t = torch.as_tensor(np.concatenate([mm.triangles for mm in meshes]), device=device)
  attrs = torch.ones(v.shape[0], 4, device=device)
  cfg = kernels.raster_config(3, 1, _lib.DR_DEPTH_DISCRETIZED, tile)
  ws = kernels.Workspace(device)
  with torch.no_grad():
    _, _, ids, z, b = kernels.rasterize_interpolate_packed(attrs, v, t, batch, cfg, ws)
  for i, (mm, c, (w, h)) in enumerate(zip(meshes, clips, sizes)):
    ref = ref_cuda(c, mm.triangles, w, h, 3, 1, device)
    trg.assert_same((batch.layered_view(ids, i, 3).cpu().numpy(),
                     batch.layered_view(z, i, 3).cpu().numpy(),
                     batch.layered_view(b, i, 3).cpu().numpy()), ref)
