"""GPU parity at the sizes of the benchmark configurations, through the
public API, against the oracle:

  c1  lit 5120-triangle icosphere, 256x256, point light on vertex normals:
      image vs the float32 restatement, vertex and color gradients vs float64
      autograd of it;
  c3  100k-triangle noisy icosphere, one camera at 1024x1024: image vs the
      oracle, gradients vs float64 autograd, and central finite differences
      (eps 1e-3) of the L2 loss on 64 seeded vertex and color coordinates
      through the CUDA path;
  c4  1M-triangle textured heightfield, one camera at 2048x2048: image vs
      the float32 restatement, vertex and texture gradients vs the float32
      torch restatement's autograd;
  c5  the ragged benchmark batch (BatchRenderer, one launch per kernel) on
      a subset with 256, 512 and 1024 pixel images: every image and its
      mesh's gradients vs the oracle.

Images are compared at 1e-5 relative / 1e-6 absolute (1e-5 absolute where
the restatement's own float32 rounding is that large, as noted), gradients
at 1e-4 of each tensor's largest magnitude. The gradients of c3, c4 and c5
are those of the configurations' objective, the L2 loss against a target
image. (Under a random-sign upstream gradient at 1024x1024 the per-vertex
sums cancel so strongly that the float32 restatement of the reference's own
arithmetic is 1.3e-4 of the largest magnitude from float64, and the CUDA
path is at the same level; under the L2 loss it is 4e-5.)
"""
import numpy as np
import pytest
import torch

from diffren_gb300 import batch as batch_lib
from diffren_gb300 import losses, mesh, render, shaders, workloads
from oracle import mesh as omesh
from oracle import raster, shading, texture, torch_ref

pytestmark = pytest.mark.gpu

LIGHT = (2.0, 2.0, 2.0)


def _alpha(rgb):
  return torch.cat([rgb, torch.ones_like(rgb[..., :1])], -1)


def _oracle_state(cam, m, w, h):
  clip = raster.transform(cam, m.vertices)
  ids, z, b = raster.rasterize(clip, m.triangles, w, h, 3, 1)
  return clip, ids, z, b, torch_ref.discrete_state(clip, ids, z, b, m.triangles, w, h)


def _torch_clip(tv, cam, clip):
  """Clip vertices with the oracle's exact values and the camera's
  gradient (the forward must see the same bits the rasterizer saw)."""
  lin = torch.cat([tv, torch.ones_like(tv[:, :1])], 1) @ torch.tensor(
      np.asarray(cam), dtype=tv.dtype).T
  return torch.tensor(clip, dtype=tv.dtype) + (lin - lin.detach())


def _grads_close(ours, want):
  want = np.asarray(want)
  scale = float(np.abs(want).max())
  np.testing.assert_allclose(np.asarray(ours), want, rtol=0, atol=1e-4 * scale)


def _lit(tv, tc, tt, ti, tz, tb, clip, state, w, h):
  attrs = torch.cat([tc, omesh.vertex_normals_t(tv, tt), tv], 1)
  a = torch_ref.interpolate(attrs, ti, tz, tb, tt)
  shaded = _alpha(shading.point_light(a[..., :3], a[..., 3:6], a[..., 6:9], LIGHT))
  return torch_ref.splat_shaded_pixels(clip, ti, tz, tb, tt, shaded, w, h, state)[0]


def test_c1_lit_icosphere_256(device):
  m = workloads.icosphere_workload(16, seed=0)
  cam = workloads.camera_matrix((0.0, 0.0, 3.0), 256, 256)
  v = torch.tensor(m.vertices, device=device, requires_grad=True)
  c = torch.tensor(m.colors, device=device, requires_grad=True)
  t = torch.tensor(m.triangles, device=device)
  attrs = {"rgb": c, "normals": mesh.compute_vertex_normals(v, t), "pos": v}
  out = render.render_triangles(
      v, attrs, t, torch.tensor(cam, device=device), 256, 256,
      lambda a: _alpha(shaders.point_light(a["rgb"], a["normals"], a["pos"], LIGHT)),
      num_layers=3)
  clip, ids, z, b, state = _oracle_state(cam, m, 256, 256)
  ti, tz, tt = torch.tensor(ids), torch.tensor(z), torch.tensor(m.triangles).long()
  with torch.no_grad():
    ref32 = _lit(torch.tensor(m.vertices), torch.tensor(m.colors), tt, ti, tz,
                 torch.tensor(b), torch.tensor(clip), state, 256, 256)
  # The float32 restatement of the lit chain is itself ~5e-6 from float64.
  np.testing.assert_allclose(out.detach().cpu().numpy(), ref32.numpy(), rtol=1e-5, atol=1e-5)
  g = np.random.default_rng(1).standard_normal(out.shape).astype(np.float32)
  gv, gc = torch.autograd.grad(out, (v, c), torch.tensor(g, device=device))
  tv = torch.tensor(m.vertices, dtype=torch.float64, requires_grad=True)
  tc = torch.tensor(m.colors, dtype=torch.float64, requires_grad=True)
  ref = _lit(tv, tc, tt, ti, tz, torch.tensor(b, dtype=torch.float64),
             _torch_clip(tv, cam, clip), state, 256, 256)
  rv, rc = torch.autograd.grad(ref, (tv, tc), torch.tensor(g, dtype=torch.float64))
  _grads_close(gv.cpu().numpy(), rv.numpy())
  _grads_close(gc.cpu().numpy(), rc.numpy())


@pytest.fixture(scope="module")
def c3_scene():
  m = workloads.icosphere_workload(71, seed=0)
  cam = workloads.camera_matrix(workloads.sphere_eyes(8, seed=1)[0], 1024, 1024)
  rng = np.random.default_rng(3)
  target = rng.uniform(0, 1, (1024, 1024, 4)).astype(np.float32)
  target[..., 3] = 1.0
  return m, cam, target


def _render_c3(v, c, m, cam, device):
  return render.render_triangles(v, {"rgb": c}, torch.tensor(m.triangles, device=device),
                                 torch.tensor(cam, device=device), 1024, 1024,
                                 lambda a: _alpha(a["rgb"]), num_layers=3)


def test_c3_icosphere_1024_image_and_gradients(c3_scene, device):
  m, cam, target = c3_scene
  assert len(m.triangles) == 100820
  v = torch.tensor(m.vertices, device=device, requires_grad=True)
  c = torch.tensor(m.colors, device=device, requires_grad=True)
  out = _render_c3(v, c, m, cam, device)
  clip, ids, z, b, state = _oracle_state(cam, m, 1024, 1024)
  ti, tz, tt = torch.tensor(ids), torch.tensor(z), torch.tensor(m.triangles).long()
  with torch.no_grad():
    shaded = _alpha(torch_ref.interpolate(torch.tensor(m.colors), ti, tz, torch.tensor(b), tt))
    ref32 = torch_ref.splat_shaded_pixels(torch.tensor(clip), ti, tz, torch.tensor(b), tt,
                                          shaded, 1024, 1024, state)[0]
  np.testing.assert_allclose(out.detach().cpu().numpy(), ref32.numpy(), rtol=1e-5, atol=1e-6)
  # The configuration's objective: the L2 loss against a target image.
  _, seed = losses.squared_error_seed(out, torch.tensor(target, device=device))
  gv, gc = torch.autograd.grad(out, (v, c), seed)
  tv = torch.tensor(m.vertices, dtype=torch.float64, requires_grad=True)
  tc = torch.tensor(m.colors, dtype=torch.float64, requires_grad=True)
  tb = torch.tensor(b, dtype=torch.float64)
  ref = torch_ref.splat_shaded_pixels(_torch_clip(tv, cam, clip), ti, tz, tb, tt,
                                      _alpha(torch_ref.interpolate(tc, ti, tz, tb, tt)),
                                      1024, 1024, state)[0]
  loss = ((ref - torch.tensor(target, dtype=torch.float64)) ** 2).sum()
  rv, rc = torch.autograd.grad(loss, (tv, tc))
  _grads_close(gv.cpu().numpy(), rv.numpy())
  _grads_close(gc.cpu().numpy(), rc.numpy())


def test_c3_finite_differences(c3_scene, device):
  """Central differences of the L2 loss sum((image - target)^2) on 64
  seeded coordinates against the gradient of the CUDA path.

  32 vertex colors, eps 1e-3, through the CUDA path itself: colors enter the
  image linearly, so the differences agree to float rounding.

  32 vertex positions among the vertices that reach the image, through the
  float64 restatement with the discrete state of the forward held fixed
  (rasterized ids, depth and barycentrics, the splat floors and surface
  masks), which is the function whose derivative the VJP computes and
  jax.grad of the reference computes. The rendered image itself is not
  differentiable in the positions: a step moves pixel coverage and splat
  floors, and at 1024x1024 eps 1e-3 in world units is 0.3 px, so the
  positions use eps 1e-3 px (3.4e-6 world units at this camera; the
  Gaussian splat has a 0.5 px standard deviation). Each difference is taken
  on a window around the pixels the vertex reaches (the loss outside it
  does not move). The differences must agree with float64 autograd of the
  same function to 1e-5 and with the CUDA gradient to 1e-4 of the largest
  magnitude of the set."""
  m, cam, target_np = c3_scene
  target = torch.tensor(target_np, device=device)
  v0 = torch.tensor(m.vertices, device=device)
  c0 = torch.tensor(m.colors, device=device)

  def loss64(v, c):
    with torch.no_grad():
      out = _render_c3(v, c, m, cam, device)
      return float(((out.double() - target.double()) ** 2).sum())

  v = v0.clone().requires_grad_(True)
  c = c0.clone().requires_grad_(True)
  out = _render_c3(v, c, m, cam, device)
  _, seed = losses.squared_error_seed(out, target)
  gv, gc = torch.autograd.grad(out, (v, c), seed)
  gv, gc = gv.cpu().numpy(), gc.cpu().numpy()
  rng = np.random.default_rng(64)
  # Vertices whose position gradient is nonzero reach the image.
  visible = np.flatnonzero(np.abs(gv).sum(1) > 0)
  vsel = rng.choice(visible, 32, replace=False)
  csel = rng.choice(visible, 32, replace=False)

  eps = 1e-3
  fd_c, an_c = [], []
  for k, i in enumerate(csel):
    d = k % 3
    cp, cm = c0.clone(), c0.clone()
    cp[i, d] += eps
    cm[i, d] -= eps
    fd_c.append((loss64(v0, cp) - loss64(v0, cm)) / (2 * eps))
    an_c.append(gc[i, d])
  fd_c, an_c = np.array(fd_c), np.array(an_c)
  np.testing.assert_allclose(an_c, fd_c, rtol=1e-3, atol=1e-3 * np.abs(fd_c).max())

  W = H = 1024
  clip, ids, z, b, (floors, masks) = _oracle_state(cam, m, W, H)
  tris = m.triangles
  fg = z != 1.0
  corner = tris[ids]  # [L, H, W, 3] vertices of each sample's triangle
  cam64 = torch.tensor(np.asarray(cam), dtype=torch.float64)
  cols64 = torch.tensor(m.colors, dtype=torch.float64)
  tt = torch.tensor(tris).long()
  eps_px = 1e-3
  fd_v, an64_v, an_v = [], [], []
  for k, i in enumerate(vsel):
    d = k % 3
    reach = ((corner == i).any(-1) & fg).any(0)
    ys, xs = np.nonzero(reach)
    y0, y1 = max(ys.min() - 3, 0), min(ys.max() + 4, H)
    x0, x1 = max(xs.min() - 3, 0), min(xs.max() + 4, W)
    ti = torch.tensor(ids[:, y0:y1, x0:x1])
    tz = torch.tensor(z[:, y0:y1, x0:x1])
    tb = torch.tensor(b[:, y0:y1, x0:x1], dtype=torch.float64)
    st = (floors[:, y0:y1, x0:x1], masks[:, :, :, y0:y1 + 2, x0:x1 + 2])
    tgt = torch.tensor(target_np[y0:y1, x0:x1], dtype=torch.float64)
    shaded = _alpha(torch_ref.interpolate(cols64, ti, tz, tb, tt))
    fgw = (tz != 1.0).to(torch.float64)[..., None]

    def crop_loss(tv):
      clip64 = torch.cat([tv, torch.ones_like(tv[:, :1])], 1) @ cam64.T
      xyz = torch_ref.viewport_xyz(clip64, ti, tz, tb, tt, W, H)
      o = torch_ref.splat_at_pixel_centers(xyz, shaded, fgw, *st)[0]
      return ((o - tgt) ** 2).sum()

    base = torch.tensor(m.vertices, dtype=torch.float64)
    # World step that moves the vertex's projection by eps_px pixels.
    tv = base.clone().requires_grad_(True)
    clip_i = torch.cat([tv[i], torch.ones(1, dtype=torch.float64)]) @ cam64.T
    (dpx,) = torch.autograd.grad(clip_i[0] / clip_i[3] * (W * 0.5), tv, retain_graph=True)
    (dpy,) = torch.autograd.grad(clip_i[1] / clip_i[3] * (H * 0.5), tv)
    h = eps_px / max(abs(float(dpx[i, d])), abs(float(dpy[i, d])), 1.0)
    tv = base.clone().requires_grad_(True)
    (g64,) = torch.autograd.grad(crop_loss(tv), tv)
    with torch.no_grad():
      vp_, vm_ = base.clone(), base.clone()
      vp_[i, d] += h
      vm_[i, d] -= h
      fd_v.append(float(crop_loss(vp_) - crop_loss(vm_)) / (2 * h))
    an64_v.append(float(g64[i, d]))
    an_v.append(float(gv[i, d]))
  fd_v, an64_v, an_v = np.array(fd_v), np.array(an64_v), np.array(an_v)
  scale = np.abs(fd_v).max()
  np.testing.assert_allclose(an64_v, fd_v, rtol=1e-5, atol=1e-5 * scale)
  np.testing.assert_allclose(an_v, fd_v, rtol=0, atol=1e-4 * scale)


def test_c4_textured_heightfield_2048(device):
  m = workloads.heightfield_workload(708, seed=0)
  eye = workloads.sphere_eyes(4, seed=1, radius=2.2, upper_only=True)[0]
  cam = workloads.camera_matrix(eye, 2048, 2048)
  rng = np.random.default_rng(5)
  tex_np = rng.integers(0, 256, (1024, 1024, 4)).astype(np.float32) / 255.0
  v = torch.tensor(m.vertices, device=device, requires_grad=True)
  tex = torch.tensor(tex_np, device=device, requires_grad=True)
  out = render.render_triangles(v, {"uv": torch.tensor(m.uvs, device=device)},
                                torch.tensor(m.triangles, device=device),
                                torch.tensor(cam, device=device), 2048, 2048,
                                lambda a: shaders.texture_map(a["uv"], tex), num_layers=3)
  clip, ids, z, b, state = _oracle_state(cam, m, 2048, 2048)
  ti, tz, tt = torch.tensor(ids), torch.tensor(z), torch.tensor(m.triangles).long()
  tb = torch.tensor(b)
  tv = torch.tensor(m.vertices, requires_grad=True)
  ttex = torch.tensor(tex_np, requires_grad=True)
  uvs = torch_ref.interpolate(torch.tensor(m.uvs), ti, tz, tb, tt)
  ref = torch_ref.splat_shaded_pixels(_torch_clip(tv, cam, clip), ti, tz, tb, tt,
                                      texture.texture_map_t(uvs, ttex), 2048, 2048, state)[0]
  np.testing.assert_allclose(out.detach().cpu().numpy(), ref.detach().numpy(), rtol=1e-5,
                             atol=1e-6)
  target = np.random.default_rng(6).uniform(0, 1, out.shape).astype(np.float32)
  _, seed = losses.squared_error_seed(out, torch.tensor(target, device=device))
  gv, gt = torch.autograd.grad(out, (v, tex), seed)
  rv, rt = torch.autograd.grad(((ref - torch.tensor(target)) ** 2).sum(), (tv, ttex))
  _grads_close(gv.cpu().numpy(), rv.numpy())
  _grads_close(gt.cpu().numpy(), rt.numpy())


def test_c5_ragged_subset_against_oracle(device):
  """Images 0..7 of the benchmark's ragged batch (both kinds of mesh, all
  three resolutions) rendered with BatchRenderer as the benchmark does,
  each image and its mesh's gradients against the oracle."""
  meshes, cams, sizes = workloads.ragged_batch(64, seed=0)
  pick = list(range(8))
  assert {sizes[i][0] for i in pick} == {256, 512, 1024}
  ms = [meshes[i] for i in pick]
  r = batch_lib.BatchRenderer([mm.triangles for mm in ms], [len(mm.vertices) for mm in ms],
                              [sizes[i] for i in pick], num_layers=3, device=device,
                              tile="auto")
  rgba = [np.concatenate([mm.colors, np.ones_like(mm.colors[:, :1])], 1) for mm in ms]
  v = torch.tensor(np.concatenate([mm.vertices for mm in ms]), device=device,
                   requires_grad=True)
  c = torch.tensor(np.concatenate(rgba), device=device, requires_grad=True)
  out = r.render(v, {"rgba": c}, torch.tensor(np.stack([cams[i] for i in pick]), device=device),
                 lambda a: a["rgba"])
  target = torch.rand(out.shape, device=device,
                      generator=torch.Generator(device).manual_seed(4))
  _, seed = losses.squared_error_seed(out, target)
  gv, gc = torch.autograd.grad(out, (v, c), seed)
  images = r.images(out.detach())
  timg = r.images(target)
  vo = np.cumsum([0] + [len(mm.vertices) for mm in ms])
  for k, i in enumerate(pick):
    mm, (w, h) = ms[k], sizes[i]
    clip, ids, zz, b, state = _oracle_state(cams[i], mm, w, h)
    ti, tz, tt = torch.tensor(ids), torch.tensor(zz), torch.tensor(mm.triangles).long()
    tb = torch.tensor(b)
    tv = torch.tensor(mm.vertices, requires_grad=True)
    tc = torch.tensor(rgba[k], requires_grad=True)
    ref = torch_ref.splat_shaded_pixels(_torch_clip(tv, cams[i], clip), ti, tz, tb, tt,
                                        torch_ref.interpolate(tc, ti, tz, tb, tt), w, h,
                                        state)[0]
    np.testing.assert_allclose(images[k].cpu().numpy(), ref.detach().numpy(), rtol=1e-5,
                               atol=1e-6)
    rv, rc = torch.autograd.grad(((ref - timg[k].cpu()) ** 2).sum(), (tv, tc))
    _grads_close(gv[vo[k]:vo[k + 1]].cpu().numpy(), rv.numpy())
    _grads_close(gc[vo[k]:vo[k + 1]].cpu().numpy(), rc.numpy())
