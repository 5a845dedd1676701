"""GPU tests of the public API (render_triangles, rasterize_triangles with
differentiable barycentrics), mirroring the reference's own tests:
splat_test.py, render_test.py, interpolate_test.py, rasterize_test.py."""
import numpy as np
import pytest
import torch

import helpers
from diffren_gb300 import constants, rasterize, render, workloads
from oracle import raster
from oracle import splat as np_splat

pytestmark = pytest.mark.gpu

G = helpers.golden("render_goldens.npz")


def test_two_triangle_layers_golden(device):
  """splat_test.py:47-82 through render_triangles."""
  g = helpers.golden("splat_two_triangles.npz")
  v = torch.tensor([[-0.2, -0.2, 0, 1], [0.5, -0.2, 0, 1], [0.5, 0.5, 0, 1],
                    [0.2, -0.2, 0.5, 1], [-0.5, -0.2, 0.5, 1], [-0.5, 0.5, 0.5, 1]],
                   device=device)
  colors = torch.tensor([[0, 1.0, 0, 1.0]] * 3 + [[1.0, 0, 0, 1.0]] * 3, device=device)
  out, _, norm = render.render_triangles(v, {"colors": colors}, [[0, 1, 2], [3, 5, 4]],
                                         None, 32, 32, lambda x: x["colors"],
                                         num_layers=2, return_accum_buffers=True)
  ok, msg = helpers.images_near_python(g["Composite"], helpers.pil_format(out.cpu().numpy()))
  assert ok, msg
  for i in range(3):
    ok, msg = helpers.images_near_python(g["Layer_%d" % i],
                                         helpers.pil_format(norm[i].cpu().numpy()))
    assert ok, (i, msg)


@pytest.mark.parametrize("num_components", [4, 2])
def test_optimize_single_triangle(num_components, device):
  """splat_test.py:84-168: rasterize-only gradient is zero, the splat
  gradient is not, and 15 steps halve the loss."""
  init = torch.tensor([[[0, 0, 0, 1], [0.5, 0, 0, 1], [0.5, 0.5, 0, 1]]], device=device)
  target_v = torch.tensor([[[-0.25, 0, 0, 1], [0.25, 0, 0, 1], [0.25, 0.5, 0, 1]]],
                          device=device)
  tris = torch.tensor([[0, 1, 2]], device=device)
  colors = torch.tensor([[[0, 0.0, 0.8, 1.0], [0, 0.8, 0, 1.0], [0, 0.0, 0.8, 1.0]]],
                        device=device)[..., -num_components:]

  def render_splat(verts, do_splat):
    return render.render_triangles(
        verts, {"colors": colors}, tris, None, 32, 32, lambda x: x["colors"],
        compositing_mode=(constants.CompositingMode.SPLAT_OVER if do_splat else
                          constants.CompositingMode.OVER))

  target = render_splat(target_v, False).detach()
  var = init.clone()
  initial = None
  for i in range(15):
    v = var.clone().requires_grad_(True)
    raster_loss = ((render_splat(v, False) - target) ** 2).mean()
    if raster_loss.requires_grad:
      (rg,) = torch.autograd.grad(raster_loss, v, allow_unused=True)
    else:
      rg = None
    splat_loss = ((render_splat(v, True) - target) ** 2).mean()
    (sg,) = torch.autograd.grad(splat_loss, v)
    if i == 0:
      assert rg is None or float(rg.norm()) == pytest.approx(0.0)
      assert float(sg.norm()) > 0.01
      initial = float(splat_loss.detach())
    var = var - sg
  final = float(((render_splat(var, True) - target) ** 2).mean())
  assert final < 0.5 * initial, (initial, final)


def _cube():
  v = torch.tensor([[-1, -1, 1], [-1, -1, -1], [-1, 1, -1], [-1, 1, 1], [1, -1, 1],
                    [1, -1, -1], [1, 1, -1], [1, 1, 1]], dtype=torch.float32)
  t = torch.tensor([[0, 1, 2], [2, 3, 0], [3, 2, 6], [6, 7, 3], [7, 6, 5], [5, 4, 7],
                    [4, 5, 1], [1, 0, 4], [5, 6, 2], [2, 1, 5], [7, 4, 0], [0, 3, 7]],
                   dtype=torch.int32)
  return v, t


def _projections():
  p = helpers.make_perspective_matrix()
  return torch.tensor(np.stack([p @ helpers.make_look_at_matrix("view_1"),
                                p @ helpers.make_look_at_matrix("view_2")]),
                      dtype=torch.float32)


@pytest.mark.parametrize("num_layers", [1, 2, 3])
def test_renders_colored_cube_layers(num_layers, device):
  """interpolate_test.py:51-75: two views (batched), NONE compositing."""
  v, t = _cube()
  rgba = torch.cat([v * 0.5 + 0.5, torch.ones(8, 1)], 1)
  out = render.render_triangles(
      v.to(device), {"rgba": rgba.to(device)}, t.to(device), _projections().to(device),
      640, 480, lambda x: x["rgba"], num_layers=num_layers,
      face_culling_mode=constants.FaceCullingMode.NONE,
      compositing_mode=constants.CompositingMode.NONE)
  for i in (0, 1):
    for l in range(num_layers):
      ok, msg = helpers.images_near_python(
          G["unlit_cube_%d_%d" % (i, l)], helpers.pil_format(out[i, l].cpu().numpy()))
      assert ok, (i, l, msg)


@pytest.mark.parametrize("mode", ["no batching", "batched vertices", "all batched"])
def test_renders_two_cubes_batch_modes(mode, device):
  """render_test.py:56-98 (OVER compositing)."""
  v, t = _cube()
  rgba = torch.cat([v * 0.5 + 0.5, torch.ones(8, 1)], 1)
  proj = _projections().to(device)
  v, t, rgba = v.to(device), t.to(device), rgba.to(device)
  if mode == "batched vertices":
    v = v[None].expand(2, 8, 3)
  elif mode == "all batched":
    v, t, rgba = v[None].expand(2, 8, 3), t[None].expand(2, 12, 3), rgba[None].expand(2, 8, 4)
  out = render.render_triangles(v, {"rgba": rgba}, t, proj, 640, 480, lambda x: x["rgba"],
                                face_culling_mode=constants.FaceCullingMode.NONE,
                                compositing_mode=constants.CompositingMode.OVER)
  for i in (0, 1):
    ok, msg = helpers.images_near_python(G["unlit_cube_%d_0" % i],
                                         helpers.pil_format(out[i].cpu().numpy()))
    assert ok, (i, msg)


def test_renders_sphere_disparity(device):
  """render_test.py:100-140: a shader that transforms world positions."""
  v = torch.tensor(G["sphere_vertices"], device=device)
  t = torch.tensor(G["sphere_triangles"], device=device)
  look = torch.tensor(helpers.make_look_at_matrix("view_1"), dtype=torch.float32,
                      device=device)

  def shader(a):
    p = a["world_position"]
    flat = p.reshape(-1, 3)
    cam = flat @ look[:3, :3].T + look[:3, 3]
    disp = -1 / cam[:, 2]
    disp = (disp - 0.12523349) / (0.16625337 - 0.12523349)
    disp = disp.reshape(p.shape[:2])
    return torch.stack([disp, torch.ones_like(disp)], -1)

  out = render.render_triangles(v, {"world_position": v}, t, _projections()[0].to(device),
                                640, 480, shader,
                                compositing_mode=constants.CompositingMode.OVER)
  ok, msg = helpers.images_near_python(helpers.to_rgba(G["sphere_disparity"])
                                       if G["sphere_disparity"].shape[2] == 3 else
                                       G["sphere_disparity"],
                                       helpers.pil_format(out[..., 0:1].cpu().numpy()))
  assert ok, msg


def test_diff_barycentrics_known_jacobian(device):
  """rasterize_test.py:169-227: Jacobian of the barycentrics at pixel
  (32, 24) of a 64x48 image w.r.t. the ndc vertex coordinates."""
  expected = helpers.golden("diff_bary_jacobian.npz")["expected"]
  ndc = torch.tensor([[-0.5, -0.5, 0.8], [0.0, 0.5, 0.3], [0.5, -0.5, 0.3]], device=device)
  tris = torch.tensor([[0, 1, 2]], device=device)
  eye = torch.eye(4, device=device)

  def bary(x, diff):
    fb = rasterize.rasterize_triangles(x, tris, eye, 64, 48, compute_diff_barys=diff)
    return fb.barycentrics[0, 24, 32, :]

  jac = torch.zeros(3, 3, 3)
  for i in range(3):
    x = ndc.clone().requires_grad_(True)
    (g,) = torch.autograd.grad(bary(x, True)[i], x)
    jac[i] = g.cpu()
  np.testing.assert_array_almost_equal(jac.numpy(), expected, decimal=6)
  x = ndc.clone().requires_grad_(True)
  assert not bary(x, False).requires_grad


def test_batched_render_matches_per_image(device):
  """A [B, ...] render equals B single renders (forward exactly, gradients
  within tolerance)."""
  m = workloads.icosphere_workload(6, seed=2)
  eyes = workloads.sphere_eyes(3, seed=5)
  cams = torch.tensor(np.stack([workloads.camera_matrix(e, 64, 48) for e in eyes]),
                      device=device)
  v = torch.tensor(m.vertices, device=device)
  t = torch.tensor(m.triangles, device=device)
  col = torch.tensor(m.colors, device=device)

  def shade(a):
    return torch.cat([a["rgb"], torch.ones_like(a["rgb"][..., :1])], -1)

  vb = v[None].repeat(3, 1, 1).requires_grad_(True)
  out_b = render.render_triangles(vb, {"rgb": col}, t, cams, 64, 48, shade, num_layers=3)
  (gb,) = torch.autograd.grad(out_b.square().sum(), vb)
  for i in range(3):
    vi = v.clone().requires_grad_(True)
    out_i = render.render_triangles(vi, {"rgb": col}, t, cams[i], 64, 48, shade,
                                    num_layers=3)
    torch.testing.assert_close(out_b[i], out_i, rtol=0, atol=0)
    (gi,) = torch.autograd.grad(out_i.square().sum(), vi)
    torch.testing.assert_close(gb[i], gi, rtol=1e-4, atol=1e-5)


def test_render_matches_oracle_pipeline(device):
  """c1-like scene end to end: point-light-free pass-through shader,
  forward vs the numpy oracle chain."""
  m = workloads.icosphere_workload(16, seed=0)
  cam = workloads.camera_matrix((0.0, 0.0, 3.0), 128, 128)
  out = render.render_triangles(torch.tensor(m.vertices, device=device),
                                {"rgb": torch.tensor(m.colors, device=device)},
                                torch.tensor(m.triangles, device=device),
                                torch.tensor(cam, device=device), 128, 128,
                                lambda a: torch.cat([a["rgb"], torch.ones_like(
                                    a["rgb"][..., :1])], -1), num_layers=3)
  clip = raster.transform(cam, m.vertices)
  ids, z, b = raster.rasterize(clip, m.triangles, 128, 128, 3, 1)
  rgb = np_splat.interpolate(m.colors, ids, z, b, m.triangles)
  shaded = np.concatenate([rgb, np.ones_like(rgb[..., :1])], -1)
  ref, _, _ = np_splat.splat_shaded_pixels(clip, ids, z, b, m.triangles, shaded, 128, 128)
  np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=1e-5, atol=1e-6)


def test_render_wide_attributes_fall_back_to_separate_kernels(device):
  """More than 16 attribute channels skip the fused rasterizer; the image is
  the same bits as the fused path's."""
  m = workloads.icosphere_workload(6, seed=4)
  cam = torch.tensor(workloads.camera_matrix((0.3, 0.2, 2.5), 48, 40), device=device)
  v = torch.tensor(m.vertices, device=device)
  t = torch.tensor(m.triangles, device=device)
  rgb = torch.tensor(m.colors, device=device)
  extra = torch.rand(len(m.vertices), 14, device=device)

  def shade(a):
    return torch.cat([a["rgb"], torch.ones_like(a["rgb"][..., :1])], -1)

  fused = render.render_triangles(v, {"rgb": rgb}, t, cam, 48, 40, shade, num_layers=3)
  wide = render.render_triangles(v, {"rgb": rgb, "extra": extra}, t, cam, 48, 40, shade,
                                 num_layers=3)
  assert torch.equal(fused, wide)


def _lit_scene(size):
  from diffren_gb300 import workloads as w
  m = w.icosphere_workload(8, seed=3)
  cam = w.camera_matrix((0.4, 0.3, 2.8), size, size)
  return m, cam


def _lit_render(v, c, t, cam, size, device):
  from diffren_gb300 import mesh, shaders
  attrs = {"rgb": c, "normals": mesh.compute_vertex_normals(v, t), "pos": v}

  def shade(a):
    rgb = shaders.point_light(a["rgb"], a["normals"], a["pos"], (2.0, 2.0, 2.0))
    return torch.cat([rgb, torch.ones_like(rgb[..., :1])], -1)

  return render.render_triangles(v, attrs, t, torch.tensor(cam, device=device), size, size,
                                 shade, num_layers=3)


def _lit_oracle(tv, tc, m, ids, z, b, state, size, clip=None):
  from oracle import mesh as omesh
  from oracle import shading, torch_ref
  ti, tz, tt = torch.tensor(ids), torch.tensor(z), torch.tensor(m.triangles).long()
  tb = torch.tensor(b, dtype=tv.dtype)
  attrs = torch.cat([tc, omesh.vertex_normals_t(tv, tt), tv], 1)
  a = torch_ref.interpolate(attrs, ti, tz, tb, tt)
  rgb = shading.point_light(a[..., :3], a[..., 3:6], a[..., 6:9], (2.0, 2.0, 2.0))
  shaded = torch.cat([rgb, torch.ones_like(rgb[..., :1])], -1)
  if clip is None:
    clip = torch.cat([tv, torch.ones_like(tv[:, :1])], 1) @ torch.tensor(
        np.asarray(_lit_scene(size)[1]), dtype=tv.dtype).T
  return torch_ref.splat_shaded_pixels(clip, ti, tz, tb, tt, shaded, size, size, state)[0]


def test_point_light_on_vertex_normals_matches_oracle(device):
  """The c1 shading end to end: vertex normals (mesh.py:22-52), point light
  (shaders.py:100-173), splat; forward against the float32 restatement and
  vertex / color gradients against float64 autograd of it."""
  size = 96
  m, cam = _lit_scene(size)
  v = torch.tensor(m.vertices, device=device, requires_grad=True)
  c = torch.tensor(m.colors, device=device, requires_grad=True)
  t = torch.tensor(m.triangles, device=device)
  out = _lit_render(v, c, t, cam, size, device)
  clip = raster.transform(cam, m.vertices)
  ids, z, b = raster.rasterize(clip, m.triangles, size, size, 3, 1)
  from oracle import torch_ref
  state = torch_ref.discrete_state(clip, ids, z, b, m.triangles, size, size)
  with torch.no_grad():
    ref32 = _lit_oracle(torch.tensor(m.vertices), torch.tensor(m.colors), m, ids, z, b, state,
                        size, torch.tensor(clip))
  # 1e-5 of the image's range [0, 1]: the float32 restatement itself is
  # 5e-6 from a float64 evaluation of the same chain.
  np.testing.assert_allclose(out.detach().cpu().numpy(), ref32.numpy(), rtol=1e-5, atol=1e-5)
  g = np.random.default_rng(0).standard_normal(out.shape).astype(np.float32)
  gv, gc = torch.autograd.grad(out, (v, c), torch.tensor(g, device=device))
  tv = torch.tensor(m.vertices, dtype=torch.float64, requires_grad=True)
  tc = torch.tensor(m.colors, dtype=torch.float64, requires_grad=True)
  ref = _lit_oracle(tv, tc, m, ids, z, b, state, size)
  rv, rc = torch.autograd.grad(ref, (tv, tc), torch.tensor(g, dtype=torch.float64))
  for ours, want in ((gv, rv), (gc, rc)):
    want = want.numpy()
    scale = float(np.abs(want).max())
    np.testing.assert_allclose(ours.cpu().numpy(), want, rtol=1e-4, atol=1e-4 * scale)


def _spike_scene(device):
  v0 = G["sphere_vertices"].astype(np.float32)
  t = torch.tensor(G["sphere_triangles"].astype(np.int32), device=device)
  proj = helpers.make_perspective_matrix() @ helpers.make_look_at_matrix("view_1")
  return v0, t, torch.tensor(proj, dtype=torch.float32, device=device)


def test_spike_derivative_golden(device):
  """splat_test.py:170-224: forward-mode derivative (torch.autograd.forward_ad
  in place of jax.jvp) of render_triangles with respect to the offset of one
  sphere vertex, through the CUDA JVP kernels, against Spike_Derivative.png
  (no pixel may differ beyond the reference's 0.5% outlier allowance)."""
  import torch.autograd.forward_ad as fwAD
  v0, t, proj = _spike_scene(device)
  v = v0.copy()
  v[32] *= 2.0
  tangent = torch.zeros(len(v), 3, device=device)
  tangent[32] = torch.tensor(v0[32], device=device)
  colors = torch.ones(len(v), 4, device=device)
  with fwAD.dual_level():
    vd = fwAD.make_dual(torch.tensor(v, device=device), tangent)
    out = render.render_triangles(vd, {"colors": colors}, t, proj, helpers.IMAGE_WIDTH,
                                  helpers.IMAGE_HEIGHT, lambda a: a["colors"])
    rendered, jac = fwAD.unpack_dual(out)
  image = (jac / jac.abs().max()) * 0.5 + 0.5
  image = image * 0.95 + rendered * 0.05
  ok, msg = helpers.images_near_python(G["spike_derivative"],
                                       helpers.pil_format(image[..., :3].cpu().numpy()),
                                       threshold=0.0)
  assert ok, msg


@pytest.mark.parametrize("wide,diff_barys", [(False, False), (True, False), (False, True)])
def test_jvp_agrees_with_vjp(wide, diff_barys, device):
  """<J t, g> = <t, J^T g> through render_triangles (3 layers, color and
  vertex tangents): the forward-mode kernels and the VJP kernels compute the
  same derivative, on the fused path, on the separate interpolation and
  positions kernels (more than 16 attribute channels) and with
  differentiable barycentrics."""
  import torch.autograd.forward_ad as fwAD
  m = workloads.icosphere_workload(8, seed=6)
  cam = torch.tensor(workloads.camera_matrix((0.5, 0.4, 2.7), 96, 80), device=device)
  v = torch.tensor(m.vertices, device=device)
  c = torch.tensor(m.colors, device=device)
  t = torch.tensor(m.triangles, device=device)
  rng = np.random.default_rng(3)
  tv = torch.tensor(rng.standard_normal(v.shape), dtype=torch.float32, device=device) * 0.01
  tc = torch.tensor(rng.standard_normal(c.shape), dtype=torch.float32, device=device)

  extra = {"pad": torch.zeros(len(m.vertices), 14, device=device)} if wide else {}

  def shade(a):
    return torch.cat([a["rgb"], torch.ones_like(a["rgb"][..., :1])], -1)

  with fwAD.dual_level():
    out = render.render_triangles(fwAD.make_dual(v, tv),
                                  {"rgb": fwAD.make_dual(c, tc), **extra}, t, cam, 96, 80,
                                  shade, num_layers=3, compute_diff_barys=diff_barys)
    _, jt = fwAD.unpack_dual(out)
  g = torch.tensor(rng.standard_normal(tuple(jt.shape)), dtype=torch.float32, device=device)
  vr, cr = v.clone().requires_grad_(True), c.clone().requires_grad_(True)
  out2 = render.render_triangles(vr, {"rgb": cr, **extra}, t, cam, 96, 80, shade, num_layers=3,
                                 compute_diff_barys=diff_barys)
  gv, gc = torch.autograd.grad(out2, (vr, cr), g)
  lhs = float((jt.double() * g.double()).sum())
  rhs = float((tv.double() * gv.double()).sum() + (tc.double() * gc.double()).sum())
  assert abs(lhs - rhs) <= 1e-4 * max(abs(lhs), abs(rhs)), (lhs, rhs)


@pytest.mark.parametrize("w_vector,golden,none_camera,diff_barys", [
    ([1.0, 1.0, 1.0], "simple_triangle", False, False),
    ([1.0, 1.0, 1.0], "simple_triangle", False, True),
    ([1.0, 1.0, 1.0], "simple_triangle", True, False),
    ([0.2, 0.5, 2.0], "perspective_corrected_triangle", False, False),
    ([0.2, 0.5, 2.0], "perspective_corrected_triangle", False, True),
])
def test_rasterize_simple_triangle_goldens(w_vector, golden, none_camera, diff_barys, device):
  """rasterize_test.py:28-152: barycentrics of one triangle through
  rasterize.rasterize_triangles (identity or no camera, w constant or
  varying, with and without differentiable barycentrics)."""
  clip = torch.tensor([[-0.5, -0.5, 0.8, 1.0], [0.0, 0.5, 0.3, 1.0], [0.5, -0.5, 0.3, 1.0]],
                      device=device) * torch.tensor(w_vector, device=device)[:, None]
  camera = None if none_camera else torch.eye(4, device=device)
  fb = rasterize.rasterize_triangles(clip, torch.tensor([[0, 1, 2]], device=device), camera,
                                     helpers.IMAGE_WIDTH, helpers.IMAGE_HEIGHT,
                                     compute_diff_barys=diff_barys)
  b = fb.barycentrics[0].detach().cpu().numpy()
  image = np.concatenate([b, np.ones_like(b[..., :1])], -1)
  ok, msg = helpers.images_near_python(helpers.to_rgba(G[golden]), helpers.pil_format(image))
  assert ok, msg
