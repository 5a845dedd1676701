"""GPU parity of interpolation and splat kernels (through the C ABI) against
the numpy oracle (forward, 1e-5 rel / 1e-6 abs) and torch float64 autograd
of the restatement (VJP, 1e-4 rel)."""
import numpy as np
import pytest
import torch

import helpers
from diffren_gb300 import kernels, workloads
from oracle import raster
from oracle import splat as np_splat
from oracle import torch_ref

pytestmark = pytest.mark.gpu

FWD_RTOL, FWD_ATOL = 1e-5, 1e-6
GRAD_RTOL = 1e-4


def assert_grad_close(ours, ref):
  """Gradients within 1e-4 relative to the tensor's largest magnitude, and
  99% of elements within 1e-4 of themselves. Element-wise relative error
  alone is not a usable bound in float32: the (1 - alpha) factors of over
  compositing cancel, and per-vertex sums of many signed float32
  contributions cancel, so near-zero elements carry large relative rounding
  error (in the reference's float32 JAX gradients too)."""
  ours, ref = np.asarray(ours, np.float64), np.asarray(ref, np.float64)
  scale = float(np.abs(ref).max()) or 1.0
  np.testing.assert_allclose(ours, ref, rtol=GRAD_RTOL, atol=GRAD_RTOL * scale)
  strict = np.abs(ours - ref) > GRAD_RTOL * np.abs(ref) + 1e-6 * scale
  assert strict.mean() < 1e-2, strict.mean()


def scene(kind, w, h, layers, C, seed):
  rng = np.random.default_rng(seed)
  if kind == "ico":
    m = workloads.icosphere_workload(4, seed=seed)
    eye = (0.4, 0.5, 2.3)
  elif kind == "soup":
    m = workloads.soup_workload(600, seed=seed, mu=-2.2, sigma=0.5)
    eye = workloads.sphere_eyes(1, seed=seed, radius=2.5)[0]
  else:  # two overlapping shells: several layers everywhere
    a = workloads.icosphere_workload(4, seed=seed)
    b = workloads.icosphere_workload(3, seed=seed + 1)
    v = np.concatenate([a.vertices, b.vertices * 0.6])
    t = np.concatenate([a.triangles, b.triangles + len(a.vertices)])
    m = workloads.Mesh(v, t, np.concatenate([a.colors, b.colors]))
    eye = (0.2, -0.3, 2.2)
  cam = workloads.camera_matrix(eye, w, h)
  clip = raster.transform(cam, m.vertices)
  ids, z, b = raster.rasterize(clip, m.triangles, w, h, layers, 1)
  shaded = rng.uniform(0.0, 1.0, (layers, h, w, C)).astype(np.float32)
  return clip, m.triangles, ids, z, b, shaded, m


def to_dev(device, *arrays):
  return [torch.as_tensor(np.ascontiguousarray(a), device=device) for a in arrays]


CASES = [("ico", 48, 40, 3, 4), ("soup", 37, 29, 3, 4), ("shells", 40, 40, 3, 4),
         ("shells", 33, 31, 5, 2), ("ico", 35, 20, 1, 1), ("soup", 64, 9, 2, 3),
         ("shells", 40, 36, 4, 8)]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_interpolate_forward_matches_oracle(case, device):
  kind, w, h, layers, C = CASES[case]
  clip, tris, ids, z, b, _, m = scene(kind, w, h, layers, C, case)
  attr = np.concatenate([m.colors, m.vertices], axis=1)
  ref = np_splat.interpolate(attr, ids, z, b, tris)
  a, t, i, zz, bb = to_dev(device, attr, tris, ids.reshape(-1), z.reshape(-1),
                           b.reshape(-1, 3))
  batch = kernels.ImageBatch.single(w, h, len(attr), len(tris))
  out = kernels.interpolate_packed(a, bb, t, i, zz, batch, layers)
  np.testing.assert_array_equal(out.view(layers, h, w, -1).cpu().numpy(), ref)


@pytest.mark.parametrize("case", range(len(CASES)))
def test_interpolate_backward_matches_autograd(case, device):
  kind, w, h, layers, C = CASES[case]
  clip, tris, ids, z, b, _, m = scene(kind, w, h, layers, C, case)
  attr = np.concatenate([m.colors, m.vertices], axis=1)
  rng = np.random.default_rng(case)
  g = rng.standard_normal((layers, h, w, attr.shape[1])).astype(np.float32)
  # Reference: float64 autograd of the restatement.
  ta = torch.tensor(attr, dtype=torch.float64, requires_grad=True)
  tb = torch.tensor(b, dtype=torch.float64, requires_grad=True)
  out = torch_ref.interpolate(ta, torch.tensor(ids), torch.tensor(z), tb, torch.tensor(tris))
  ga, gb = torch.autograd.grad(out, (ta, tb), torch.tensor(g, dtype=torch.float64))
  a, t, i, zz, bb = to_dev(device, attr, tris, ids.reshape(-1), z.reshape(-1),
                           b.reshape(-1, 3))
  a.requires_grad_(True)
  bb.requires_grad_(True)
  batch = kernels.ImageBatch.single(w, h, len(attr), len(tris))
  o = kernels.interpolate_packed(a, bb, t, i, zz, batch, layers)
  da, db = torch.autograd.grad(o, (a, bb), torch.as_tensor(g, device=device).view(o.shape))
  assert_grad_close(da.cpu().numpy(), ga.numpy())
  assert_grad_close(db.view(layers, h, w, 3).cpu().numpy(), gb.numpy())


def run_splat(device, clip, tris, ids, z, b, shaded, w, h, layers, accum=False,
              requires_grad=False, with_depth=True):
  """Positions + splat through the C ABI; returns (clip, colors, result).
  ``with_depth`` passes the depth buffer, so background positions are not
  read (the rendering path); otherwise every position is read."""
  c, t, i, zz, bb, s = to_dev(device, clip, tris, ids.reshape(-1), z.reshape(-1),
                              b.reshape(-1, 3), shaded.reshape(-1, shaded.shape[-1]))
  if requires_grad:
    c.requires_grad_(True)
    s.requires_grad_(True)
  batch = kernels.ImageBatch.single(w, h, len(clip), len(tris))
  vp = kernels.splat_positions_packed(c, bb, t, i, zz, batch, layers)
  res = kernels.splat_packed(vp, s, batch, layers, accum, z=zz if with_depth else None)
  return c, s, res


@pytest.mark.parametrize("case", range(len(CASES)))
def test_splat_forward_matches_oracle(case, device):
  kind, w, h, layers, C = CASES[case]
  clip, tris, ids, z, b, shaded, _ = scene(kind, w, h, layers, C, case)
  out, acc, norm = np_splat.splat_shaded_pixels(clip, ids, z, b, tris, shaded, w, h)
  _, _, (o, a, n) = run_splat(device, clip, tris, ids, z, b, shaded, w, h, layers, True)
  np.testing.assert_allclose(o.view(h, w, C).cpu().numpy(), out, rtol=FWD_RTOL,
                             atol=FWD_ATOL)
  np.testing.assert_allclose(a.view(3, h, w, C).cpu().numpy(), acc, rtol=FWD_RTOL,
                             atol=FWD_ATOL)
  np.testing.assert_allclose(n.view(3, h, w, C).cpu().numpy(), norm, rtol=FWD_RTOL,
                             atol=FWD_ATOL)


@pytest.mark.parametrize("case", range(len(CASES)))
def test_splat_backward_matches_autograd(case, device):
  kind, w, h, layers, C = CASES[case]
  clip, tris, ids, z, b, shaded, _ = scene(kind, w, h, layers, C, case)
  rng = np.random.default_rng(10 + case)
  g = rng.standard_normal((h, w, C)).astype(np.float32)
  state = torch_ref.discrete_state(clip, ids, z, b, tris, w, h)
  tc = torch.tensor(clip, dtype=torch.float64, requires_grad=True)
  ts = torch.tensor(shaded, dtype=torch.float64, requires_grad=True)
  out = torch_ref.splat_shaded_pixels(tc, torch.tensor(ids), torch.tensor(z),
                                      torch.tensor(b, dtype=torch.float64),
                                      torch.tensor(tris), ts, w, h, state)[0]
  gc, gs = torch.autograd.grad(out, (tc, ts), torch.tensor(g, dtype=torch.float64))
  c, s, o = run_splat(device, clip, tris, ids, z, b, shaded, w, h, layers,
                      requires_grad=True)
  dc, ds = torch.autograd.grad(o, (c, s), torch.as_tensor(g, device=device).view(o.shape))
  assert_grad_close(ds.view(layers, h, w, C).cpu().numpy(), gs.numpy())
  assert_grad_close(dc.cpu().numpy(), gc.numpy())


@pytest.mark.parametrize("case", [0, 2, 6])
def test_splat_with_and_without_depth_buffer_agree(case, device):
  """Taking background samples from the depth buffer (positions unread)
  gives the same images and gradients as reading every position."""
  kind, w, h, layers, C = CASES[case]
  clip, tris, ids, z, b, shaded, _ = scene(kind, w, h, layers, C, case)
  outs = []
  for with_depth in (True, False):
    c, s, out = run_splat(device, clip, tris, ids, z, b, shaded, w, h, layers,
                          requires_grad=True, with_depth=with_depth)
    g = torch.linspace(-1, 1, out.numel(), device=device).view(out.shape)
    outs.append((out.detach(),) + torch.autograd.grad(out, (c, s), g))
  (o1, dc1, ds1), (o2, dc2, ds2) = outs
  assert torch.equal(o1, o2)
  assert torch.equal(ds1, ds2)
  # d clip sums float atomics, whose order varies between runs.
  assert_grad_close(dc1.cpu().numpy(), dc2.cpu().numpy())


def test_splat_positions_match_oracle(device):
  clip, tris, ids, z, b, shaded, _ = scene("shells", 40, 36, 3, 4, 3)
  ref = np_splat.viewport_xyz(clip, ids, z, b, tris, 40, 36)
  c, t, i, zz, bb = to_dev(device, clip, tris, ids.reshape(-1), z.reshape(-1),
                           b.reshape(-1, 3))
  batch = kernels.ImageBatch.single(40, 36, len(clip), len(tris))
  vp = kernels.splat_positions_packed(c, bb, t, i, zz, batch, 3).view(3, 36, 40, 4)
  np.testing.assert_array_equal(vp[..., :3].cpu().numpy(), ref)
  np.testing.assert_array_equal(vp[..., 3].cpu().numpy(), (z != 1).astype(np.float32))


@pytest.mark.parametrize("case", range(len(CASES)))
def test_interpolate_with_positions_matches_oracle(case, device):
  """The fused pass equals interpolate + viewport_xyz bit for bit, and its
  VJP matches float64 autograd of the restatement."""
  kind, w, h, layers, C = CASES[case]
  clip, tris, ids, z, b, _, m = scene(kind, w, h, layers, C, case)
  attr = np.concatenate([m.colors, m.vertices], axis=1)[:, :C + 2]
  ref_attr = np_splat.interpolate(attr, ids, z, b, tris)
  ref_xyz = np_splat.viewport_xyz(clip, ids, z, b, tris, w, h)
  a, c, t, i, zz, bb = to_dev(device, attr, clip, tris, ids.reshape(-1), z.reshape(-1),
                              b.reshape(-1, 3))
  a.requires_grad_(True)
  c.requires_grad_(True)
  bb.requires_grad_(True)
  batch = kernels.ImageBatch.single(w, h, len(attr), len(tris))
  out, vp = kernels.interpolate_with_positions_packed(a, c, bb, t, i, zz, batch, layers)
  np.testing.assert_array_equal(out.detach().view(layers, h, w, -1).cpu().numpy(), ref_attr)
  np.testing.assert_array_equal(vp.detach()[:, :3].view(layers, h, w, 3).cpu().numpy(),
                                ref_xyz)
  np.testing.assert_array_equal(vp.detach()[:, 3].view(layers, h, w).cpu().numpy(),
                                (z != 1).astype(np.float32))

  rng = np.random.default_rng(case + 7)
  ga = rng.standard_normal((layers, h, w, attr.shape[1])).astype(np.float32)
  gp = rng.standard_normal((layers, h, w, 4)).astype(np.float32)
  ta = torch.tensor(attr, dtype=torch.float64, requires_grad=True)
  tc = torch.tensor(clip, dtype=torch.float64, requires_grad=True)
  tb = torch.tensor(b, dtype=torch.float64, requires_grad=True)
  ti, tz, tt = torch.tensor(ids), torch.tensor(z), torch.tensor(tris)
  ro = torch_ref.interpolate(ta, ti, tz, tb, tt)
  rx = torch_ref.viewport_xyz(tc, ti, tz, tb, tt, w, h)
  # The viewport z and the foreground flag carry no gradient.
  loss = (ro * torch.tensor(ga, dtype=torch.float64)).sum() + \
      (rx[..., :2] * torch.tensor(gp[..., :2], dtype=torch.float64)).sum()
  ra, rc, rb = torch.autograd.grad(loss, (ta, tc, tb))
  da, dc, db = torch.autograd.grad(
      (out, vp), (a, c, bb),
      (torch.as_tensor(ga, device=device).view(out.shape),
       torch.as_tensor(gp, device=device).view(vp.shape)))
  assert_grad_close(da.cpu().numpy(), ra.numpy())
  assert_grad_close(dc.cpu().numpy(), rc.numpy())
  assert_grad_close(db.view(layers, h, w, 3).cpu().numpy(), rb.numpy())


@pytest.mark.parametrize("C", [4, 3])
def test_splat_at_pixel_centers_off_center_positions(C, device):
  """The public splat_at_pixel_centers on samples that sit off the pixel
  centres (so every tap weight differs), forward and VJP w.r.t. xy."""
  from diffren_gb300 import splat as splat_lib
  rng = np.random.default_rng(7)
  L, H, W = 3, 19, 23
  ys, xs = np.meshgrid(np.arange(H) + 0.5, np.arange(W) + 0.5, indexing="ij")
  xyz = np.stack([np.broadcast_to(xs, (L, H, W)), np.broadcast_to(ys, (L, H, W)),
                  np.sort(rng.uniform(0, 1, (L, H, W)), axis=0)], -1).astype(np.float32)
  xyz[..., :2] += rng.uniform(-0.3, 0.3, (L, H, W, 2)).astype(np.float32)
  fg = (rng.uniform(0, 1, (L, H, W, 1)) < 0.8).astype(np.float32)
  col = rng.uniform(0, 1, (L, H, W, C)).astype(np.float32)
  out, acc, norm = np_splat.splat_at_pixel_centers(xyz, col, fg)
  tx = torch.tensor(xyz, device=device, requires_grad=True)
  tc = torch.tensor(col, device=device, requires_grad=True)
  o, a, n = splat_lib.splat_at_pixel_centers(tx, tc, torch.tensor(fg, device=device))
  np.testing.assert_allclose(o.detach().cpu().numpy(), out, rtol=FWD_RTOL, atol=FWD_ATOL)
  np.testing.assert_allclose(a.cpu().numpy(), acc, rtol=FWD_RTOL, atol=FWD_ATOL)
  np.testing.assert_allclose(n.cpu().numpy(), norm, rtol=FWD_RTOL, atol=FWD_ATOL)
  g = rng.standard_normal((H, W, C)).astype(np.float32)
  dx, dc = torch.autograd.grad(o, (tx, tc), torch.tensor(g, device=device))
  # float64 autograd with the float32 discrete decisions held fixed.
  floors = np.floor(xyz[..., :2])
  state = torch_ref.discrete_state_xyz(xyz, fg)
  rx = torch.tensor(xyz, dtype=torch.float64, requires_grad=True)
  rc = torch.tensor(col, dtype=torch.float64, requires_grad=True)
  ro = torch_ref.splat_at_pixel_centers(rx, rc, torch.tensor(fg, dtype=torch.float64),
                                        floors, state)[0]
  gx, gc = torch.autograd.grad(ro, (rx, rc), torch.tensor(g, dtype=torch.float64))
  assert_grad_close(dc.cpu().numpy(), gc.numpy())
  assert_grad_close(dx[..., :2].cpu().numpy(), gx[..., :2].numpy())
  assert float(dx[..., 2].abs().max()) == 0.0


def test_splat_two_triangles_golden(device):
  """splat_test.py:47-82 through the CUDA kernels, vs the reference goldens."""
  g = helpers.golden("splat_two_triangles.npz")
  v = np.array([[-0.2, -0.2, 0, 1], [0.5, -0.2, 0, 1], [0.5, 0.5, 0, 1],
                [0.2, -0.2, 0.5, 1], [-0.5, -0.2, 0.5, 1], [-0.5, 0.5, 0.5, 1]],
               np.float32)
  t = np.array([[0, 1, 2], [3, 5, 4]], np.int32)
  colors = np.array([[0, 1, 0, 1]] * 3 + [[1, 0, 0, 1]] * 3, np.float32)
  ids, z, b = raster.rasterize(v, t, 32, 32, 2, 1)
  shaded = np_splat.interpolate(colors, ids, z, b, t)
  _, _, (o, _, n) = run_splat(device, v, t, ids, z, b, shaded, 32, 32, 2, accum=True)
  ok, msg = helpers.images_near_python(g["Composite"],
                                       helpers.pil_format(o.view(32, 32, 4).cpu().numpy()))
  assert ok, msg
  n = n.view(3, 32, 32, 4).cpu().numpy()
  for i in range(3):
    ok, msg = helpers.images_near_python(g["Layer_%d" % i], helpers.pil_format(n[i]))
    assert ok, (i, msg)
