"""The torch.library adapter (diffren_gb300/ops.py): operator registration
and fake (shape) implementations on CPU; on the GPU, the ops equal the
Python API bit for bit and pass torch.library.opcheck."""
import numpy as np
import pytest
import torch
from torch._subclasses.fake_tensor import FakeTensorMode

from diffren_gb300 import ops  # noqa: F401  (registers torch.ops.diffren_gb300)


def test_ops_are_registered_with_fake_shapes():
  with FakeTensorMode():
    clip = torch.empty(10, 4)
    tris = torch.empty(5, 3, dtype=torch.int32)
    ids, z, bary = torch.ops.diffren_gb300.rasterize_triangles(clip, tris, 8, 6, 3, 1, 0)
    assert ids.shape == (3, 6, 8) and ids.dtype == torch.int32
    assert z.shape == (3, 6, 8) and bary.shape == (3, 6, 8, 3)
    pos, col, zb = torch.empty(3, 6, 8, 4), torch.empty(3, 6, 8, 4), torch.empty(3, 6, 8)
    out, saved = torch.ops.diffren_gb300.splat_fwd(pos, col, zb)
    assert out.shape == (6, 8, 4) and saved.shape == (17, 48)
    d_pos, d_col = torch.ops.diffren_gb300.splat_bwd(out, pos, col, zb, saved)
    assert d_pos.shape == pos.shape and d_col.shape == col.shape


def _scene(device, size=(40, 32)):
  from diffren_gb300 import workloads
  m = workloads.icosphere_workload(6, seed=2)
  w, h = size
  cam = torch.tensor(workloads.camera_matrix((0.4, 0.3, 2.6), w, h), device=device)
  v = torch.tensor(m.vertices, device=device)
  clip = torch.cat([v, torch.ones_like(v[:, :1])], 1) @ cam.T
  return m, clip.contiguous(), torch.tensor(m.triangles, device=device), w, h


@pytest.mark.gpu
def test_rasterize_op_matches_api(device):
  from diffren_gb300 import kernels
  m, clip, tris, w, h = _scene(device)
  ids, z, bary = torch.ops.diffren_gb300.rasterize_triangles(clip, tris, w, h, 3, 1, 0)
  batch = kernels.ImageBatch.single(w, h, clip.shape[0], tris.shape[0])
  ri, rz, rb = kernels.rasterize_packed(clip, tris.int(), batch, kernels.raster_config(3, 1, 0))
  assert torch.equal(ids.reshape(-1), ri) and torch.equal(z.reshape(-1), rz)
  assert torch.equal(bary.reshape(-1, 3), rb)
  torch.library.opcheck(torch.ops.diffren_gb300.rasterize_triangles.default,
                        (clip, tris.int(), w, h, 3, 1, 0),
                        test_utils=("test_schema", "test_faketensor"))


@pytest.mark.gpu
def test_splat_op_matches_api_and_passes_opcheck(device):
  from diffren_gb300 import kernels
  m, clip, tris, w, h = _scene(device)
  batch = kernels.ImageBatch.single(w, h, clip.shape[0], tris.shape[0])
  ids, z, bary = kernels.rasterize_packed(clip, tris.int(), batch, kernels.raster_config(3, 1, 0))
  vp = kernels.splat_positions_packed(clip, bary, tris.int(), ids, z, batch, 3)
  rng = np.random.default_rng(0)
  colors = torch.tensor(rng.uniform(0, 1, (3 * w * h, 4)), dtype=torch.float32, device=device)
  g = torch.tensor(rng.standard_normal((h, w, 4)), dtype=torch.float32, device=device)
  p1 = vp.detach().clone().requires_grad_(True)
  c1 = colors.clone().requires_grad_(True)
  ref = kernels.splat_packed(p1, c1, batch, 3, z=z)
  rp, rc = torch.autograd.grad(ref, (p1, c1), g.reshape(-1, 4))
  p2 = vp.detach().clone().view(3, h, w, 4).requires_grad_(True)
  c2 = colors.clone().view(3, h, w, 4).requires_grad_(True)
  out = ops.splat(p2, c2, z.view(3, h, w))
  op_p, op_c = torch.autograd.grad(out, (p2, c2), g)
  assert torch.equal(out.reshape(-1, 4), ref)
  assert torch.equal(op_c.reshape(-1, 4), rc)
  fg = (z != 1.0)
  assert torch.equal(op_p.reshape(-1, 4)[fg], rp[fg])
  assert torch.all(op_p.reshape(-1, 4)[~fg] == 0)
  torch.library.opcheck(torch.ops.diffren_gb300.splat_fwd.default,
                        (p2.detach().requires_grad_(True), c2.detach().requires_grad_(True),
                         z.view(3, h, w)),
                        test_utils=("test_schema", "test_autograd_registration",
                                    "test_faketensor"))
