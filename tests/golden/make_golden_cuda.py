"""Records outputs of the reference's own CUDA rasterizer into
tests/golden/raster_ref_cuda.npz (test infrastructure).

Run on a machine with a CUDA GPU (sm_103a) after the reference CUDA
rasterizer has been built (oracle/Makefile `ref_cuda`, from the reference
tree or its staged copy in oracle/_ref/src):
    python tests/golden/make_golden_cuda.py [output.npz]
(the default output is tests/golden/raster_ref_cuda.npz).

It calls diffren::cuda::RasterizeTrianglesImpl
(diffren/common/kernels/rasterize_triangles_impl_cuda.cu.cc:397-484) through
oracle/ref_cuda_shim.cu on (1) every scene of raster_ref.npz (the reference
tests' own geometry and small seeded scenes) and (2) the seeded scenes named
in SEEDED, whose inputs `seeded_scene` regenerates, and keeps ids, z and
barycentrics. The CPU tests compare the oracle's discretized semantics with
these bit for bit.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from diffren_gb300 import workloads  # noqa: E402
from oracle import raster  # noqa: E402

# name -> (kind, triangles or icosphere frequency, seed, width, height, layers, culling).
# Widths that are not powers of two exercise the pixel-centre multiply-add.
SEEDED = {
    "seeded_soup_131x77_none": ("soup", 6000, 1, 131, 77, 3, 0),
    "seeded_soup_200x150_back": ("soup", 4000, 0, 200, 150, 3, 1),
    "seeded_soup_97x61_front": ("soup", 3000, 2, 97, 61, 4, 2),
    "seeded_ico_160x100_back": ("ico", 12, 5, 160, 100, 3, 1),
    "seeded_near_120x90_none": ("near", 3000, 8, 120, 90, 3, 0),
}


def seeded_scene(name, width, height):
  """Clip-space vertices and triangles of SEEDED[name]."""
  kind, n, seed, w, h, _, _ = SEEDED[name]
  assert (w, h) == (width, height), name
  if kind == "soup":
    m = workloads.soup_workload(n, seed=seed, mu=-2.5, sigma=0.8)
    eye = workloads.sphere_eyes(1, seed=seed)[0]
  elif kind == "ico":
    m = workloads.icosphere_workload(n, seed=seed)
    eye = workloads.sphere_eyes(1, seed=seed)[0]
  else:  # camera inside the geometry: near-plane clipping
    m = workloads.soup_workload(n, seed=seed, mu=-1.5, sigma=0.5)
    eye = np.array([0.05, 0.1, 0.2])
  cam = workloads.camera_matrix(eye, w, h)
  return raster.transform(cam, m.vertices), m.triangles


def main():
  import torch
  if raster.build_reference_cuda() is None:
    raise SystemExit("reference CUDA rasterizer sources not found (set DIFFREN_REFERENCE "
                     "or stage them with oracle/Makefile `stage`)")
  dev = torch.device("cuda", 0)
  fix = np.load(os.path.join(HERE, "raster_ref.npz"))
  scenes = []
  for name in sorted({k.split("__")[0] for k in fix.files}):
    w, h, layers, cull = (int(x) for x in fix[name + "__meta"])
    scenes.append((name, fix[name + "__vertices"], fix[name + "__triangles"], w, h, layers,
                   cull))
  for name, (_, _, _, w, h, layers, cull) in SEEDED.items():
    scenes.append((name, *seeded_scene(name, w, h), w, h, layers, cull))
  out = {}
  for name, v, t, w, h, layers, cull in scenes:
    vd = torch.as_tensor(np.ascontiguousarray(v, np.float32), device=dev)
    td = torch.as_tensor(np.ascontiguousarray(t, np.int32), device=dev)
    ids = torch.empty((layers, h, w), dtype=torch.int32, device=dev)
    z = torch.empty((layers, h, w), dtype=torch.float32, device=dev)
    b = torch.empty((layers, h, w, 3), dtype=torch.float32, device=dev)
    raster.rasterize_reference_cuda(vd.data_ptr(), td.data_ptr(), td.shape[0], w, h, layers,
                                    cull, ids.data_ptr(), z.data_ptr(), b.data_ptr(),
                                    torch.cuda.current_stream(dev).cuda_stream)
    torch.cuda.synchronize(dev)
    out[name + "__meta"] = np.array([w, h, layers, cull], np.int32)
    out[name + "__ids"] = ids.cpu().numpy()
    out[name + "__z"] = z.cpu().numpy()
    out[name + "__bary"] = b.cpu().numpy()
  path = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "raster_ref_cuda.npz")
  np.savez_compressed(path, **out)
  print(path, os.path.getsize(path), "bytes,", len(scenes), "scenes")


if __name__ == "__main__":
  main()
