"""CPU tests of the lighting shaders (shaders.py:68-173) against known
answers and the oracle restatement."""
import numpy as np
import torch

from diffren_gb300 import shaders
from oracle import shading


def test_point_light_known_answer():
  """A surface facing a light at distance 2: luma ka + kd = 1.7,
  attenuation 1 / (1 + 0.7 * 2 + 1.8 * 4)."""
  n = torch.tensor([[0.0, 0.0, 1.0]])
  p = torch.zeros(1, 3)
  c = torch.tensor([[1.0, 0.5, 0.25]])
  out = shaders.point_light(c, n, p, (0.0, 0.0, 2.0))
  np.testing.assert_allclose(out.numpy(), c.numpy() * 1.7 / 9.6, rtol=1e-6)
  # Facing away: ambient only.
  out = shaders.point_light(c, -n, p, (0.0, 0.0, 2.0))
  np.testing.assert_allclose(out.numpy(), c.numpy() * 0.3 / 9.6, rtol=1e-6)


def test_point_light_matches_oracle_with_specular():
  rng = np.random.default_rng(2)
  c, n, p = (torch.tensor(rng.uniform(-1, 1, (5, 7, 3))) for _ in range(3))
  kw = dict(eye_position=(0.1, 0.2, 3.0), ks=0.5, ns=8.0)
  ours = shaders.point_light(c, n, p, (2.0, 1.0, 2.0), **kw)
  ref = shading.point_light(c, n, p, (2.0, 1.0, 2.0), eye=(0.1, 0.2, 3.0), ks=0.5, ns=8.0)
  np.testing.assert_allclose(ours.numpy(), ref.numpy(), rtol=1e-12)


def test_diffuse_light_known_answer():
  n = torch.tensor([[0.0, 0.0, 1.0], [0.0, 0.0, -1.0]])
  c = torch.ones(2, 3)
  out = shaders.diffuse_light(c, n)
  cos = 1.0 / np.sqrt(1.5)  # n . normalize(0.5, 0.5, 1)
  np.testing.assert_allclose(out[0].numpy(), 0.5 + 0.5 * cos, rtol=1e-6)
  np.testing.assert_allclose(out[1].numpy(), 0.5, rtol=1e-6)


def test_l2_normalize_matches_reference_formula():
  x = torch.tensor([[3.0, 4.0, 0.0], [0.0, 0.0, 0.0]])
  np.testing.assert_allclose(shaders.l2_normalize(x).numpy(), [[0.6, 0.8, 0.0], [0, 0, 0]],
                             rtol=1e-6)


def test_point_light_row_strides_and_alpha_on_cpu():
  """The fused kernel reads rows evenly spaced in memory (columns of one
  packed buffer); CPU tensors take the torch expressions, and ``alpha``
  appends an alpha of 1 there too."""
  buf = torch.zeros(10, 9)
  assert shaders._row_stride(buf[:, 3:6]) == 9
  assert shaders._row_stride(buf[:, 6:9].view(1, -1, 3)) == 9
  assert shaders._row_stride(torch.zeros(4, 5, 3)) == 3
  assert shaders._row_stride(torch.zeros(3, 4, 3).transpose(0, 1)) is None
  assert shaders._row_stride(torch.zeros(4, 3, dtype=torch.float64)) is None
  rng = np.random.default_rng(4)
  c, n, p = (torch.tensor(rng.uniform(-1, 1, (6, 3)), dtype=torch.float32) for _ in range(3))
  rgb = shaders.point_light(c, n, p, (2.0, 1.0, 2.0))
  rgba = shaders.point_light(c, n, p, (2.0, 1.0, 2.0), alpha=True)
  assert rgba.shape == (6, 4) and torch.equal(rgba[:, :3], rgb) and (rgba[:, 3] == 1).all()
