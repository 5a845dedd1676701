"""Clip-space vertex transform (transforms.py:41-79, rasterize.py:90-96) and
its VJP over a ragged batch: four vertices per thread with 16-byte loads
where a run of xyz rows is aligned and inside one mesh, one vertex at a time
elsewhere. The forward is compared bit for bit with the same float order on
the CPU, the VJP with float64."""
import numpy as np
import pytest
import torch

from diffren_gb300 import kernels

pytestmark = pytest.mark.gpu


def cpu_transform(v, M, counts):
  """((m0 x + m1 y) + m2 z) + m3 w per row in float32, products rounded."""
  out = np.empty((v.shape[0], 4), np.float32)
  o = 0
  for i, n in enumerate(counts):
    x = v[o:o + n].astype(np.float32)
    if x.shape[1] == 3:
      x = np.concatenate([x, np.ones((n, 1), np.float32)], 1)
    m = M[i].astype(np.float32)
    for k in range(4):
      r = (m[k, 0] * x[:, 0]).astype(np.float32) + (m[k, 1] * x[:, 1]).astype(np.float32)
      r = r.astype(np.float32) + (m[k, 2] * x[:, 2]).astype(np.float32)
      out[o:o + n, k] = r.astype(np.float32) + (m[k, 3] * x[:, 3]).astype(np.float32)
    o += n
  return out


@pytest.mark.parametrize("dim", [3, 4])
@pytest.mark.parametrize("offset", [0, 1])
def test_transform_matches_cpu(dim, offset, device):
  counts = [5, 0, 13, 4, 1027, 3, 64]  # ragged, an empty mesh, not multiples of 4
  batch = kernels.ImageBatch([8] * len(counts), [8] * len(counts), counts, [1] * len(counts))
  V = sum(counts)
  rng = np.random.default_rng(dim + 10 * offset)
  flat = rng.normal(size=V * dim + offset).astype(np.float32)
  base = torch.tensor(flat, device=device)
  # offset 1 leaves the rows 4 bytes off a 16-byte boundary
  v = base[offset:].view(V, dim).detach().requires_grad_(True)
  M = rng.normal(size=(len(counts), 4, 4)).astype(np.float32)
  clip = kernels.transform(v, torch.tensor(M, device=device), batch)
  ref = cpu_transform(flat[offset:].reshape(V, dim), M, counts)
  assert np.array_equal(clip.detach().cpu().numpy(), ref)
  g = rng.normal(size=(V, 4)).astype(np.float32)
  (dv,) = torch.autograd.grad(clip, (v,), torch.tensor(g, device=device))
  expect = np.empty((V, dim))
  o = 0
  for i, n in enumerate(counts):
    expect[o:o + n] = g[o:o + n].astype(np.float64) @ M[i].astype(np.float64)[:, :dim]
    o += n
  np.testing.assert_allclose(dv.cpu().numpy(), expect, rtol=1e-5, atol=1e-5)
