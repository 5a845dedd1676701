"""OVER compositing kernel (render.py:134-140, composite.py:20-37) against
the float32 restatement (bit-exact) and torch autograd of it (VJP)."""
import numpy as np
import pytest
import torch

from diffren_gb300 import kernels
from oracle import splat as np_splat

pytestmark = pytest.mark.gpu


def masked_layers(L, H, W, C, seed, bg_frac=0.4):
  rng = np.random.default_rng(seed)
  shaded = rng.uniform(-0.2, 1.2, (L, H, W, C)).astype(np.float32)
  z = rng.uniform(-1, 1, (L, H, W)).astype(np.float32)
  z[rng.uniform(size=z.shape) < bg_frac] = 1.0
  return shaded, z


def reference_over(shaded, z):
  """render.py:134-140: mask, then composite.over in float32."""
  fg = (z != 1.0).astype(np.float32)[..., None]
  return np_splat.over((shaded * fg).astype(np.float32))


@pytest.mark.parametrize("L,C", [(1, 4), (3, 4), (3, 1), (2, 7), (5, 3), (16, 4)])
def test_over_forward_bit_exact(L, C, device):
  shaded, z = masked_layers(L, 13, 17, C, L * 10 + C)
  batch = kernels.ImageBatch.single(17, 13, 3, 1)
  out = kernels.over_packed(torch.tensor(shaded.reshape(-1, C), device=device),
                            torch.tensor(z.reshape(-1), device=device), batch, L)
  np.testing.assert_array_equal(out.cpu().numpy().reshape(13, 17, C),
                                reference_over(shaded, z))


def test_over_ragged_batch_matches_per_image(device):
  sizes = [(5, 3), (16, 9), (1, 1), (40, 33)]
  L, C = 3, 4
  data = [masked_layers(L, h, w, C, i) for i, (w, h) in enumerate(sizes)]
  batch = kernels.ImageBatch([w for w, _ in sizes], [h for _, h in sizes], [3] * 4, [1] * 4)
  shaded = np.concatenate([s.reshape(-1, C) for s, _ in data])
  z = np.concatenate([zz.reshape(-1) for _, zz in data])
  out = kernels.over_packed(torch.tensor(shaded, device=device), torch.tensor(z, device=device),
                            batch, L).cpu().numpy()
  want = np.concatenate([reference_over(s, zz).reshape(-1, C) for s, zz in data])
  np.testing.assert_array_equal(out, want)


@pytest.mark.parametrize("L,C", [(3, 4), (2, 1), (4, 6)])
def test_over_backward_matches_autograd(L, C, device):
  shaded, z = masked_layers(L, 11, 9, C, 99 + L)
  g = np.random.default_rng(1).standard_normal((11, 9, C)).astype(np.float32)
  ts = torch.tensor(shaded, dtype=torch.float64, requires_grad=True)
  fg = torch.tensor((z != 1.0).astype(np.float64))[..., None]
  m = ts * fg
  ref = m[-1]
  for i in range(2, L + 1):
    ref = m[-i] + (1.0 - m[-i, ..., -1:]) * ref
  (want,) = torch.autograd.grad(ref, ts, torch.tensor(g, dtype=torch.float64))
  ds = torch.tensor(shaded.reshape(-1, C), device=device, requires_grad=True)
  out = kernels.over_packed(ds, torch.tensor(z.reshape(-1), device=device),
                            kernels.ImageBatch.single(9, 11, 3, 1), L)
  (got,) = torch.autograd.grad(out, ds, torch.tensor(g.reshape(-1, C), device=device))
  want = want.numpy().reshape(-1, C)
  scale = float(np.abs(want).max())
  np.testing.assert_allclose(got.cpu().numpy(), want, rtol=1e-4, atol=1e-4 * scale)
  assert np.all(got.cpu().numpy()[z.reshape(-1) == 1.0] == 0)
