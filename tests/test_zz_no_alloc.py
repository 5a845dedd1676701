"""GPU test of dr_rasterize_triangles_static_scratch, the rasterizer entry
point for callers that cannot allocate device scratch memory (for example an
XLA custom-call handler, which receives only its input and result buffers).

It is called through the C ABI twice in a row, on two different scenes, and
each result must equal, bit for bit, what the workspace-taking
dr_rasterize_triangles returns for the same inputs (the rasterizer's parity
bar). The two calls share the library's static scratch array, so the second
also checks that the first call's leftovers do not leak into its result.
Around the second call the device's free memory and torch's reserved
memory must not move: the entry point exists because its callers cannot
allocate. The error word of the static scratch is read back through
dr_read_static_scratch_error_flags, the only way such a caller can see it.
"""
import ctypes

import numpy as np
import pytest
import torch

from diffren_gb300 import _lib, workloads
from oracle import raster

pytestmark = pytest.mark.gpu


def _p(t):
  return ctypes.c_void_p(t.data_ptr())


def _scene(seed, n, w, h):
  m = workloads.soup_workload(n, seed=seed, mu=-2.5, sigma=0.8)
  cam = workloads.camera_matrix(workloads.sphere_eyes(1, seed=seed)[0], w, h)
  return raster.transform(cam, m.vertices), m.triangles


def _outputs(layers, w, h, device):
  return (torch.full((layers, h, w), 7, dtype=torch.int32, device=device),
          torch.full((layers, h, w), 7.0, device=device),
          torch.full((layers, h, w, 3), 7.0, device=device))


def test_static_scratch_matches_workspace_entry_point_twice():
  assert torch.cuda.is_available(), "needs a CUDA device"
  device = torch.device("cuda", 0)
  lib = _lib.load()
  stream = ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
  scenes = [(0, 6000, 256, 192, 3, 1, 0), (1, 20000, 320, 240, 4, 0, 1)]
  for i, (seed, n, w, h, layers, cull, mode) in enumerate(scenes):
    clip, tris = _scene(seed, n, w, h)
    v = torch.as_tensor(clip, device=device).contiguous()
    t = torch.as_tensor(tris, device=device).contiguous()
    # Existing entry point with a caller-allocated workspace.
    need = lib.dr_rasterize_triangles_workspace_bytes(t.shape[0], w, h, layers)
    ws = torch.empty(need, dtype=torch.uint8, device=device)
    ref = _outputs(layers, w, h, device)
    rc = lib.dr_rasterize_triangles(_p(v), v.shape[0], _p(t), t.shape[0], w, h, layers,
                                    cull, mode, _p(ref[0]), _p(ref[1]), _p(ref[2]),
                                    _p(ws), need, stream)
    assert rc == 0, lib.dr_last_error()
    # Allocation-free entry point.
    out = _outputs(layers, w, h, device)
    torch.cuda.synchronize(device)
    free0, reserved0 = torch.cuda.mem_get_info(device)[0], torch.cuda.memory_reserved(device)
    rc = lib.dr_rasterize_triangles_static_scratch(
        _p(v), v.shape[0], _p(t), t.shape[0], w, h, layers, cull, mode, _p(out[0]),
        _p(out[1]), _p(out[2]), stream)
    assert rc == 0, lib.dr_last_error()
    torch.cuda.synchronize(device)
    if i > 0:  # the first call may load the module (and so take the array)
      assert torch.cuda.mem_get_info(device)[0] == free0, "device memory was allocated"
      assert torch.cuda.memory_reserved(device) == reserved0
    for a, b in zip(out, ref):
      assert torch.equal(a.view(torch.int32), b.view(torch.int32))
    flags = ctypes.c_uint32(99)
    assert lib.dr_read_static_scratch_error_flags(ctypes.byref(flags), stream) == 0
    assert flags.value == 0


def test_static_scratch_rejects_oversized_requests():
  lib = _lib.load()
  # 600k triangles need more scratch than the static array holds; the call
  # must fail before touching any pointer or launching anything.
  rc = lib.dr_rasterize_triangles_static_scratch(None, 3, None, 600000, 512, 512, 3, 1,
                                                 0, None, None, None, None)
  assert rc == 3
  msg = lib.dr_last_error().decode()
  assert "static array" in msg and str(_lib.DR_STATIC_SCRATCH_BYTES) in msg


def test_static_scratch_flags_out_of_range_indices():
  """An out-of-range triangle is skipped on the device and reported through
  dr_read_static_scratch_error_flags; the next clean call clears the flag."""
  device = torch.device("cuda", 0)
  lib = _lib.load()
  stream = ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
  v = torch.tensor([[-0.5, -0.5, 0.5, 1], [0.5, -0.5, 0.5, 1], [0, 0.5, 0.5, 1]],
                   device=device)
  for tris, want in (([[0, 1, 2], [0, 1, 7], [-1, 0, 1]], _lib.DR_FLAG_INDEX_OUT_OF_RANGE),
                     ([[0, 1, 2]], 0)):
    t = torch.tensor(tris, dtype=torch.int32, device=device)
    out = _outputs(1, 32, 32, device)
    rc = lib.dr_rasterize_triangles_static_scratch(_p(v), 3, _p(t), t.shape[0], 32, 32, 1,
                                                   0, 0, _p(out[0]), _p(out[1]),
                                                   _p(out[2]), stream)
    assert rc == 0, lib.dr_last_error()
    flags = ctypes.c_uint32(0)
    assert lib.dr_read_static_scratch_error_flags(ctypes.byref(flags), stream) == 0
    assert flags.value == want
    ref = raster.rasterize(v.cpu().numpy(), np.array([[0, 1, 2]], np.int32), 32, 32, 1, 0)
    np.testing.assert_array_equal(out[0].cpu().numpy(), ref[0])
