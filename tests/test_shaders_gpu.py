"""Texture-map shader kernel (shaders.py:40-65, image.py:21-118) against the
CPU restatement, the reference's own resampling known answers and its
textured-square golden render."""
import numpy as np
import pytest
import torch

import helpers
from diffren_gb300 import render, shaders
from oracle import texture

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-4


def assert_grad_close(ours, ref):
  ours, ref = np.asarray(ours, np.float64), np.asarray(ref, np.float64)
  scale = float(np.abs(ref).max()) or 1.0
  np.testing.assert_allclose(ours, ref, rtol=GRAD_RTOL, atol=GRAD_RTOL * scale)


@pytest.mark.parametrize("shape", [(5, 7, 3), (16, 9, 4), (1, 1, 4), (1, 1, 1), (33, 2, 2),
                                   (8, 8, 16)])
def test_texture_map_forward_matches_oracle(shape, device):
  rng = np.random.default_rng(sum(shape))
  tex = rng.uniform(-1, 1, shape).astype(np.float32)
  uv = rng.uniform(-0.3, 1.3, (3000, 2)).astype(np.float32)
  # texel centers, edges and corners exactly
  h, w = shape[:2]
  cx = (np.arange(w) + 0.5) / w
  cy = (np.arange(h) + 0.5) / h
  gx, gy = np.meshgrid(np.concatenate([cx, [0.0, 1.0]]), np.concatenate([cy, [0.0, 1.0]]))
  uv = np.concatenate([uv, np.stack([gx, gy], -1).reshape(-1, 2).astype(np.float32)])
  ref = texture.texture_map(uv, tex)
  out = shaders.texture_map(torch.tensor(uv, device=device), torch.tensor(tex, device=device))
  np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_bilinear_resample_known_answers(device):
  """image_test.py:26-119 through the kernel (zero padding, texel units)."""
  n = 64
  img = np.arange(3 * n * n).reshape(n, n, 3).astype(np.float32)
  x, y = np.meshgrid(np.arange(n), np.arange(n))
  loc = (np.stack((x, y), -1) + 0.5).astype(np.float32)
  out = shaders.bilinear_resample(torch.tensor(img, device=device),
                                  torch.tensor(loc, device=device))
  np.testing.assert_array_equal(out.cpu().numpy(), img)
  g = helpers.golden("texture_cases.npz")
  h, w = g["shape"]
  ramp = np.repeat(np.arange(1, w + 1, dtype=np.float32)[None], h, 0)[..., None].repeat(3, 2)
  out = shaders.bilinear_resample(torch.tensor(ramp, device=device),
                                  torch.tensor(g["samples"], device=device))
  np.testing.assert_array_almost_equal(out.cpu().numpy(),
                                       g["expected"][:, None].repeat(3, 1), decimal=5)
  ref = texture.bilinear_resample(ramp, g["samples"])
  np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("pad_mode", ["edge", "constant"])
@pytest.mark.parametrize("channels", [3, 4])
def test_texture_map_backward_matches_autograd(pad_mode, channels, device):
  rng = np.random.default_rng(11)
  tex = rng.uniform(-1, 1, (6, 9, channels)).astype(np.float32)
  loc = rng.uniform(-1.5, 10.5, (2000, 2)).astype(np.float32) * np.array([1.0, 6.0 / 9.0],
                                                                          np.float32)
  g = rng.standard_normal((2000, channels)).astype(np.float32)
  g[::7] = 0.0  # points without gradient
  tl = torch.tensor(loc, dtype=torch.float64, requires_grad=True)
  tt = torch.tensor(tex, dtype=torch.float64, requires_grad=True)
  ref = texture.bilinear_resample_t(tt, tl, pad_mode)
  gl, gt = torch.autograd.grad(ref, (tl, tt), torch.tensor(g, dtype=torch.float64))
  dl = torch.tensor(loc, device=device, requires_grad=True)
  dt = torch.tensor(tex, device=device, requires_grad=True)
  out = shaders.bilinear_resample(dt, dl, pad_mode)
  ol, ot = torch.autograd.grad(out, (dl, dt), torch.tensor(g, device=device))
  assert_grad_close(ol.cpu().numpy(), gl.numpy())
  assert_grad_close(ot.cpu().numpy(), gt.numpy())


def test_textured_square_golden(device):
  """shaders_test.py:33-74: a textured square through render_triangles."""
  g = helpers.golden("render_goldens.npz")
  tex = torch.tensor(g["textured_square_texture"], device=device)
  rendered = render.render_triangles(
      torch.tensor(g["textured_square_clip"], device=device),
      {"uv": torch.tensor(g["textured_square_uv"], device=device)},
      torch.tensor(g["textured_square_triangles"], device=device), None, 640, 480,
      lambda a: shaders.texture_map(a["uv"], tex))
  ok, msg = helpers.images_near_python(helpers.to_rgba(g["textured_square"]),
                                       helpers.pil_format(rendered.cpu().numpy()))
  assert ok, msg


@pytest.mark.parametrize("channels", [2, 4])
def test_texture_map_uv_backward_matches_autograd(channels, device):
  """shaders.texture_map's VJP in uv units (edge clamping)."""
  rng = np.random.default_rng(12)
  tex = rng.uniform(0, 1, (7, 5, channels)).astype(np.float32)
  uv = rng.uniform(-0.2, 1.2, (3000, 2)).astype(np.float32)
  g = rng.standard_normal((3000, channels)).astype(np.float32)
  tu = torch.tensor(uv, dtype=torch.float64, requires_grad=True)
  tt = torch.tensor(tex, dtype=torch.float64, requires_grad=True)
  ref = texture.texture_map_t(tu, tt)
  gu, gt = torch.autograd.grad(ref, (tu, tt), torch.tensor(g, dtype=torch.float64))
  du = torch.tensor(uv, device=device, requires_grad=True)
  dt = torch.tensor(tex, device=device, requires_grad=True)
  out = shaders.texture_map(du, dt)
  ou, ot = torch.autograd.grad(out, (du, dt), torch.tensor(g, device=device))
  assert_grad_close(ou.cpu().numpy(), gu.numpy())
  assert_grad_close(ot.cpu().numpy(), gt.numpy())


def test_spot_textured_golden(device):
  """splat_test.py:227-277 ('spot'): the textured, diffusely lit spot with
  normals from mesh.compute_vertex_normals, through render_triangles,
  against the reference's blurred golden render."""
  from diffren_gb300 import mesh
  g = helpers.golden("spot.npz")
  proj = helpers.make_perspective_matrix() @ helpers.make_look_at_matrix("spot")
  pos = torch.tensor(g["positions"], device=device)
  tris = torch.tensor(g["triangles"], device=device)
  # load_texture: float [0, 1], flipped to the lower-left origin.
  tex = torch.tensor(np.flipud(g["texture"]).astype(np.float32) / 255.0, device=device)
  attrs = {"uvs": torch.tensor(g["uvs"], device=device),
           "normals": mesh.compute_vertex_normals(pos, tris)}

  def shade(a):
    lit = shaders.diffuse_light(shaders.texture_map(a["uvs"], tex), a["normals"])
    alpha = (a["uvs"][..., 0:1] > -1.0).float()
    return torch.cat([lit, alpha], -1)

  rendered = render.render_triangles(pos, attrs, tris, torch.tensor(proj, dtype=torch.float32,
                                                                    device=device),
                                     helpers.IMAGE_WIDTH, helpers.IMAGE_HEIGHT, shade)
  ok, msg = helpers.images_near_python(g["target"],
                                       helpers.pil_format(rendered[..., :3].cpu().numpy()))
  assert ok, msg


@pytest.mark.parametrize("lighting", ["diffuse", "point", "phong_point"])
def test_spot_lighting_goldens(lighting, device):
  """shaders_test.py:76-168: the spot with texture and diffuse / point /
  Blinn-Phong point lighting on vertex normals, CompositingMode.OVER (the
  OVER kernel), against the reference's golden renders."""
  from diffren_gb300 import constants, mesh
  g = helpers.golden("spot.npz")
  proj = helpers.make_perspective_matrix() @ helpers.make_look_at_matrix("spot")
  pos = torch.tensor(g["positions"], device=device)
  tris = torch.tensor(g["triangles"], device=device)
  tex = torch.tensor(np.flipud(g["texture"]).astype(np.float32) / 255.0, device=device)
  eye = tuple(float(x) for x in helpers.eye_position("spot")[0])
  attrs = {"uvs": torch.tensor(g["uvs"], device=device), "positions": pos,
           "normals": mesh.compute_vertex_normals(pos, tris)}

  def shade(a):
    textured = shaders.texture_map(a["uvs"], tex)
    if lighting == "diffuse":
      return shaders.diffuse_light(textured, a["normals"])
    kw = dict(eye_position=eye, ks=1.0, ns=50.0) if lighting == "phong_point" else {}
    return shaders.point_light(textured, a["normals"], a["positions"], eye, **kw)

  rendered = render.render_triangles(pos, attrs, tris,
                                     torch.tensor(proj, dtype=torch.float32, device=device),
                                     helpers.IMAGE_WIDTH, helpers.IMAGE_HEIGHT, shade,
                                     compositing_mode=constants.CompositingMode.OVER)
  ok, msg = helpers.images_near_python(g[lighting], helpers.pil_format(rendered.cpu().numpy()))
  assert ok, msg


@pytest.mark.parametrize("kw", [{}, dict(ks=1.0, ns=50.0, eye_position=(0.3, -0.2, 2.5)),
                                dict(ka=0.1, kd=0.9, ks=0.5, ns=3.0, attenuation_constant=0.5,
                                     attenuation_linear=0.2, attenuation_quadratic=0.05)])
@pytest.mark.parametrize("packed", [False, True])
def test_point_light_kernel_matches_oracle(kw, packed, device):
  """dr_point_light_fwd / _bwd (one kernel each way) against the float64
  restatement with autograd: images within 1e-5 relative / 1e-6 absolute,
  gradients of the three inputs within 1e-4 of the largest magnitude; the
  inputs as separate buffers and as columns of one packed buffer, with the
  alpha channel appended."""
  from oracle import shading
  rng = np.random.default_rng(len(kw) + 10 * packed)
  n = 6000
  rgb = rng.uniform(0, 1, (n, 3))
  nrm = rng.normal(size=(n, 3))
  nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
  pos = rng.uniform(-1.5, 1.5, (n, 3))
  light = (2.0, 2.0, 2.0)
  if packed:
    buf = torch.tensor(np.concatenate([rgb, nrm, pos], 1), dtype=torch.float32, device=device,
                       requires_grad=True)
    ins = (buf[:, 0:3], buf[:, 3:6], buf[:, 6:9])
    leaves = (buf,)
  else:
    ins = tuple(torch.tensor(x, dtype=torch.float32, device=device, requires_grad=True)
                for x in (rgb, nrm, pos))
    leaves = ins
  out = shaders.point_light(*ins, light, alpha=True, **kw)
  assert out.shape == (n, 4) and (out[:, 3] == 1).all()
  okw = {{"eye_position": "eye", "attenuation_constant": "att_c", "attenuation_linear": "att_l",
          "attenuation_quadratic": "att_q"}.get(k, k): v for k, v in kw.items()}
  ref_in = tuple(torch.tensor(x, dtype=torch.float64, requires_grad=True) for x in (rgb, nrm, pos))
  ref = shading.point_light(*ref_in, light, **okw)
  np.testing.assert_allclose(out[:, :3].detach().cpu().numpy(), ref.detach().numpy(), rtol=1e-5,
                             atol=1e-6)
  g = rng.standard_normal((n, 4))
  ours = torch.autograd.grad(out, leaves, torch.tensor(g, dtype=torch.float32, device=device))
  refg = torch.autograd.grad(ref, ref_in, torch.tensor(g[:, :3]))
  ours = (torch.cat([x for x in ours], 1) if not packed else ours[0]).cpu().numpy()
  for k in range(3):
    assert_grad_close(ours[:, 3 * k:3 * k + 3], refg[k].numpy())


@pytest.mark.parametrize("C", [4, 3])
def test_deterministic_texture_gradient_repeats_bit_for_bit(C, device):
  """texture_map(..., deterministic=True): the texture gradient summed in
  fixed point is the same bits on two runs and within 1e-6 of the
  float-atomic sum's largest magnitude; the uv gradient and the image are
  unchanged."""
  rng = np.random.default_rng(C)
  tex = torch.tensor(rng.uniform(-1, 1, (37, 53, C)).astype(np.float32), device=device)
  uv = torch.tensor(rng.uniform(-0.1, 1.1, (20000, 2)).astype(np.float32), device=device)
  g = torch.tensor(rng.standard_normal((20000, C)).astype(np.float32), device=device)

  def run(det):
    t = tex.clone().requires_grad_(True)
    u = uv.clone().requires_grad_(True)
    out = shaders.texture_map(u, t, deterministic=det)
    dt, du = torch.autograd.grad(out, (t, u), g)
    return out.detach(), dt, du

  o1, t1, u1 = run(True)
  o2, t2, u2 = run(True)
  o0, t0, u0 = run(False)
  assert torch.equal(o1, o2) and torch.equal(o1, o0)
  assert torch.equal(t1, t2) and torch.equal(u1, u2)
  assert float((t1 - t0).abs().max()) <= 1e-6 * float(t0.abs().max())
  torch.testing.assert_close(u1, u0, rtol=1e-6, atol=1e-6)
