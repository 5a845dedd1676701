"""CPU tests: the oracle against the reference (compiled reference CPU
rasterizer, committed fixtures, the reference tests' golden images and known
answers)."""
import os

import numpy as np
import pytest
import torch

import helpers
from diffren_gb300 import workloads
from golden import png
from oracle import raster
from oracle import splat as np_splat
from oracle import torch_ref

FIX = helpers.golden("raster_ref.npz")
CASES = sorted({k.split("__")[0] for k in FIX.files})


def _case(name):
  g = lambda k: FIX[name + "__" + k]
  w, h, layers, cull = (int(x) for x in g("meta"))
  return g("vertices"), g("triangles"), w, h, layers, cull, g("ids"), g("z"), g("bary")


def _bits(a):
  return np.asarray(a).view(np.uint32)


@pytest.mark.parametrize("name", CASES)
def test_oracle_float_mode_matches_reference_fixture(name):
  v, t, w, h, layers, cull, ids, z, bary = _case(name)
  oi, oz, ob = raster.rasterize(v, t, w, h, layers, cull, raster.DEPTH_FLOAT)
  np.testing.assert_array_equal(oi, ids)
  np.testing.assert_array_equal(_bits(oz), _bits(z))
  np.testing.assert_array_equal(_bits(ob), _bits(bary))


@pytest.mark.parametrize("name", CASES)
def test_discretized_mode_agrees_with_float_mode(name):
  """Reference CUDA vs CPU semantics: the same visible triangles except at
  background (id 0 vs -1), depth near-ties and a few edge pixels. The CUDA
  build fuses the pixel-centre multiply-add, which moves a pixel centre by
  at most one 16.16 fixed-point step (2^-16 in NDC) where the width is not
  a power of two: coverage can change at triangle edges, and barycentrics
  and depth agree to that step times their gradient (closely on most
  samples, loosely on small triangles). Each semantics is pinned bit for bit
  against its own reference build elsewhere."""
  v, t, w, h, layers, cull, ids, z, bary = _case(name)
  gi, gz, gb = raster.rasterize(v, t, w, h, layers, cull, raster.DEPTH_DISCRETIZED)
  fg = ids >= 0
  gfg = gz != 1.0
  np.testing.assert_array_equal(gi[~gfg], 0)
  np.testing.assert_array_equal(gz[~gfg], 1.0)
  limit = max(2, 0.002 * fg.sum())
  assert (gfg != fg).sum() <= limit, (gfg != fg).sum()
  both = fg & gfg
  assert (both & (gi != ids)).sum() <= limit, (both & (gi != ids)).sum()
  same = both & (gi == ids)
  for a, b in ((gz[same], z[same]), (gb[same], bary[same])):
    d = np.abs(a - b)
    if d.size == 0:
      continue
    assert d.max() < 2e-2, d.max()
    assert np.median(d) < 1e-5, np.median(d)


CUDA_FIX = helpers.golden("raster_ref_cuda.npz")
CUDA_CASES = sorted({k.split("__")[0] for k in CUDA_FIX.files})


def _cuda_case(name):
  """Inputs of a recorded reference-CUDA case: a raster_ref.npz scene or a
  seeded scene named by tests/golden/make_golden_cuda.py."""
  g = lambda k: CUDA_FIX[name + "__" + k]
  w, h, layers, cull = (int(x) for x in g("meta"))
  if name in CASES:
    v, t = FIX[name + "__vertices"], FIX[name + "__triangles"]
  else:
    from golden import make_golden_cuda
    v, t = make_golden_cuda.seeded_scene(name, w, h)
  return v, t, w, h, layers, cull, g("ids"), g("z"), g("bary")


@pytest.mark.parametrize("name", CUDA_CASES)
def test_discretized_mode_matches_reference_cuda_fixture(name):
  """The discretized semantics against outputs recorded from the reference's
  own CUDA rasterizer (rasterize_triangles_impl_cuda.cu.cc, built for sm_103a
  with nvcc's defaults): bit-exact ids, depth and barycentrics."""
  v, t, w, h, layers, cull, ids, z, bary = _cuda_case(name)
  oi, oz, ob = raster.rasterize(v, t, w, h, layers, cull, raster.DEPTH_DISCRETIZED)
  np.testing.assert_array_equal(oi, ids)
  np.testing.assert_array_equal(_bits(oz), _bits(z))
  np.testing.assert_array_equal(_bits(ob), _bits(bary))


@pytest.mark.parametrize("seed", range(6))
def test_oracle_matches_compiled_reference_random(seed):
  if raster.build_reference() is None:
    pytest.skip("reference rasterizer sources not present (DIFFREN_REFERENCE or the "
                "staged copy in oracle/_ref/src)")
  rng = np.random.default_rng(100 + seed)
  w, h = int(rng.integers(1, 90)), int(rng.integers(1, 70))
  layers, cull = int(rng.integers(1, 6)), int(rng.integers(0, 3))
  m = workloads.soup_workload(int(rng.integers(1, 800)), seed=seed, mu=-2.0, sigma=1.0)
  eye = workloads.sphere_eyes(1, seed=seed, radius=float(rng.uniform(0.3, 3.0)))[0]
  clip = raster.transform(workloads.camera_matrix(eye, w, h), m.vertices)
  ref = raster.rasterize_reference_cpu(clip, m.triangles, w, h, layers, cull)
  ours = raster.rasterize(clip, m.triangles, w, h, layers, cull, raster.DEPTH_FLOAT)
  for a, b in zip(ref, ours):
    np.testing.assert_array_equal(np.asarray(a).view(np.uint32),
                                  np.asarray(b).view(np.uint32))


PNGS = helpers.golden("raster_pngs.npz")


def _ref_png(name):
  """A golden PNG of the reference's rasterizer tests (kept as file bytes)."""
  return png.decode_png(PNGS[name[:-4]], name)


def _test_case(name):
  return _case("test_" + name)[:2]


@pytest.mark.parametrize("mode", [raster.DEPTH_FLOAT, raster.DEPTH_DISCRETIZED])
@pytest.mark.parametrize("case,golden", [
    ("CanRasterizeTriangle", "Simple_Triangle.png"),
    ("CanRasterizeExternalTriangle", "External_Triangle.png"),
    ("CanRasterizeTetrahedron", "Simple_Tetrahedron.png"),
])
def test_oracle_golden_barycentrics(case, golden, mode):
  """rasterize_triangles_impl_test.cc:125-168 (and the CUDA twin)."""
  v, t = _test_case(case)
  _, _, b = raster.rasterize(v, t, 640, 480, 1, 0, mode)
  ok, msg = helpers.images_near_cpp(_ref_png(golden), helpers.encode_barycentrics(b))
  assert ok, msg


@pytest.mark.parametrize("mode", [raster.DEPTH_FLOAT, raster.DEPTH_DISCRETIZED])
def test_oracle_golden_inside_box(mode):
  v = FIX["inside_box__vertices"]
  t = FIX["inside_box__triangles"]
  _, _, b = raster.rasterize(v, t, 640, 480, 1, 0, mode)
  ok, msg = helpers.images_near_cpp(_ref_png("Inside_Box.png"),
                                    helpers.encode_barycentrics(b))
  assert ok, msg


@pytest.mark.parametrize("mode", [raster.DEPTH_FLOAT, raster.DEPTH_DISCRETIZED])
def test_oracle_golden_cube_two_layers_and_culling(mode):
  """impl_test.cc:227-294: ids and barycentrics of both layers; culling."""
  v = FIX["cube_cull0__vertices"]
  t = FIX["cube_cull0__triangles"]
  # The C++ test harness zero-fills its id buffer (impl_test.cc:36-37); the
  # -1 background of the CPU semantics comes from the XLA handler instead.
  ids, _, b = raster.rasterize(v, t, 640, 480, 2, 0, mode)
  ids = np.maximum(ids, 0)
  for layer, idg, bg in ((0, "Ids_Cube.png", "Barycentrics_Cube.png"),
                         (1, "Ids_Cube_Back.png", "Barycentrics_Cube_Back.png")):
    ok, msg = helpers.images_near_cpp(_ref_png(idg), helpers.encode_ids(ids, layer))
    assert ok, (idg, msg)
    ok, msg = helpers.images_near_cpp(_ref_png(bg), helpers.encode_barycentrics(b, layer))
    assert ok, (bg, msg)
  empty = 0 if mode == raster.DEPTH_DISCRETIZED else -1
  for cull, golden in ((1, "Ids_Cube_Back.png"), (2, "Ids_Cube.png")):
    ids, _, _ = raster.rasterize(v, t, 640, 480, 2, cull, mode)
    ok, msg = helpers.images_near_cpp(_ref_png(golden),
                                      helpers.encode_ids(np.maximum(ids, 0), 0))
    assert ok, (cull, msg)
    assert (ids[1] == empty).all()


def test_oracle_golden_uv_sphere_ids():
  """rasterize_triangles_impl_cuda_test.cc:172-187 (CUDA semantics)."""
  v, t = helpers.uv_sphere(230, 230, 0.9)
  ids, _, _ = raster.rasterize(helpers.homogeneous(v), t, 1600, 1600, 1, 0,
                               raster.DEPTH_DISCRETIZED)
  ok, msg = helpers.images_near_cpp(_ref_png("UV_Sphere_Ids.png"), helpers.encode_ids(ids))
  assert ok, msg


@pytest.mark.parametrize("mode", [raster.DEPTH_FLOAT, raster.DEPTH_DISCRETIZED])
def test_oracle_edge_corner_degenerate(mode):
  """impl_test.cc:170-225: pixel on a shared edge (both windings), image
  corners, degenerate triangle."""
  v = np.array([[0.0, -1.0, 0.5, 1.0], [0.0, 1.0, 0.5, 1.0], [0.5, -1.0, 0.5, 1.0]],
               np.float32)
  for tri in ([0, 1, 2], [2, 1, 0]):
    _, _, b = raster.rasterize(v, np.array([tri], np.int32), 641, 480, 1, 0, mode)
    assert abs(b[0, 5, 320].sum() - 1.0) < 1e-6
  v = np.array([[-1, -1, 0, 1], [1, -1, 0, 1], [1, 1, 0, 1], [-1, 1, 0, 1]], np.float32)
  _, _, b = raster.rasterize(v, np.array([[0, 1, 2], [0, 2, 3]], np.int32), 640, 480, 1,
                             0, mode)
  for x, y in ((0, 0), (639, 0), (639, 479), (0, 479)):
    assert abs(b[0, y, x].sum() - 1.0) < 1e-6
  v = np.array([[-1, -1, 0, 1], [1, 1, 0, 1], [0, 0, 0, 1]], np.float32)
  _, _, b = raster.rasterize(v, np.array([[0, 1, 2]], np.int32), 1, 1, 1, 0, mode)
  assert abs(b.sum()) < 1e-6


def test_oracle_splat_two_triangles_golden():
  """splat_test.py:47-82: composite and the 3 normalized layers."""
  g = helpers.golden("splat_two_triangles.npz")
  v = np.array([[-0.2, -0.2, 0, 1], [0.5, -0.2, 0, 1], [0.5, 0.5, 0, 1],
                [0.2, -0.2, 0.5, 1], [-0.5, -0.2, 0.5, 1], [-0.5, 0.5, 0.5, 1]],
               np.float32)
  t = np.array([[0, 1, 2], [3, 5, 4]], np.int32)
  colors = np.array([[0, 1, 0, 1]] * 3 + [[1, 0, 0, 1]] * 3, np.float32)
  ids, z, b = raster.rasterize(v, t, 32, 32, 2, 1)
  shaded = np_splat.interpolate(colors, ids, z, b, t)
  out, _, norm = np_splat.splat_shaded_pixels(v, ids, z, b, t, shaded, 32, 32)
  ok, msg = helpers.images_near_python(g["Composite"], helpers.pil_format(out))
  assert ok, msg
  for i in range(3):
    ok, msg = helpers.images_near_python(g["Layer_%d" % i], helpers.pil_format(norm[i]))
    assert ok, (i, msg)


def _small_scene(seed=0, w=24, h=20, layers=3):
  m = workloads.icosphere_workload(3, seed=seed)
  cam = workloads.camera_matrix((0.3, 0.4, 2.4), w, h)
  clip = raster.transform(cam, m.vertices)
  ids, z, b = raster.rasterize(clip, m.triangles, w, h, layers, 1)
  rng = np.random.default_rng(seed)
  shaded = rng.uniform(0, 1, (layers, h, w, 4)).astype(np.float32)
  return clip, m.triangles, ids, z, b, shaded, w, h


def test_torch_oracle_matches_numpy_oracle():
  clip, t, ids, z, b, shaded, w, h = _small_scene()
  out, acc, norm = np_splat.splat_shaded_pixels(clip, ids, z, b, t, shaded, w, h)
  state = torch_ref.discrete_state(clip, ids, z, b, t, w, h)
  tout, tacc, tnorm = torch_ref.splat_shaded_pixels(
      torch.tensor(clip), torch.tensor(ids), torch.tensor(z), torch.tensor(b),
      torch.tensor(t), torch.tensor(shaded), w, h, state)
  np.testing.assert_allclose(tout.numpy(), out, rtol=1e-5, atol=1e-6)
  np.testing.assert_allclose(tacc.numpy(), acc, rtol=1e-5, atol=1e-6)


def test_torch_oracle_gradient_matches_finite_differences():
  """Central differences (eps 1e-3, float64) of the frozen-discrete splat."""
  clip, t, ids, z, b, shaded, w, h = _small_scene(seed=1, w=16, h=14)
  state = torch_ref.discrete_state(clip, ids, z, b, t, w, h)
  ti, tz, tb, tt = (torch.tensor(x) for x in (ids, z, b, t))
  target = torch.rand(h, w, 4, dtype=torch.float64, generator=torch.Generator().manual_seed(0))

  def loss(c, s):
    out = torch_ref.splat_shaded_pixels(c, ti, tz, tb.double(), tt, s, w, h, state)[0]
    return ((out - target) ** 2).sum()

  c = torch.tensor(clip, dtype=torch.float64, requires_grad=True)
  s = torch.tensor(shaded, dtype=torch.float64, requires_grad=True)
  gc, gs = torch.autograd.grad(loss(c, s), (c, s))
  rng = np.random.default_rng(3)
  used = np.unique(t[ids[z != 1.0]])
  eps = 1e-3
  for _ in range(16):
    vi, k = int(rng.choice(used)), int(rng.choice([0, 1, 3]))
    cp, cm = c.detach().clone(), c.detach().clone()
    cp[vi, k] += eps
    cm[vi, k] -= eps
    fd = (loss(cp, s) - loss(cm, s)).item() / (2 * eps)
    assert abs(fd - gc[vi, k].item()) <= 1e-4 * max(1.0, abs(fd)) + 1e-5, (vi, k, fd, gc[vi, k])


# ------------------------------------------------------------ texture map
def test_texture_oracle_recovers_input_at_texel_centers():
  """image_test.py:26-41: sampling at (x, y) + 0.5 returns the image."""
  from oracle import texture
  n = 64
  img = np.arange(3 * n * n).reshape(n, n, 3).astype(np.float32)
  x, y = np.meshgrid(np.arange(n), np.arange(n))
  out = texture.bilinear_resample(img, np.stack((x, y), -1) + 0.5)
  np.testing.assert_array_equal(out, img)


def test_texture_oracle_boundary_cases():
  """image_test.py:44-119: the reference's boundary samples (zero padding)
  on its 30 x 10 ramp image."""
  from oracle import texture
  g = np.load(os.path.join(os.path.dirname(__file__), "golden", "texture_cases.npz"))
  h, w = g["shape"]
  img = np.repeat(np.arange(1, w + 1, dtype=np.float32)[None], h, 0)[..., None].repeat(3, 2)
  out = texture.bilinear_resample(img, g["samples"])
  np.testing.assert_array_almost_equal(out, g["expected"][:, None].repeat(3, 1), decimal=5)


def test_texture_oracle_torch_matches_numpy_and_finite_differences():
  import torch
  from oracle import texture
  rng = np.random.default_rng(3)
  tex = rng.uniform(0, 1, (5, 7, 2)).astype(np.float32)
  uv = rng.uniform(-0.2, 1.2, (400, 2)).astype(np.float32)
  a = texture.texture_map(uv, tex)
  b = texture.texture_map_t(torch.tensor(uv), torch.tensor(tex)).numpy()
  np.testing.assert_array_equal(a, b)
  t = torch.tensor(tex, dtype=torch.float64, requires_grad=True)
  u = torch.tensor(uv, dtype=torch.float64, requires_grad=True)
  assert torch.autograd.gradcheck(lambda uu, tt: texture.texture_map_t(uu, tt), (u, t),
                                  eps=1e-6, atol=1e-5)


def _sphere():
  g = helpers.golden("render_goldens.npz")
  return g["sphere_vertices"].astype(np.float32), g["sphere_triangles"].astype(np.int64)


def test_vertex_normals_oracle_sphere_known_answers():
  """mesh_test.py:32-80: a unit sphere's normals are its vertices; stretching
  z by 2 halves the normals' z before renormalizing."""
  from oracle import mesh
  v, t = _sphere()
  np.testing.assert_array_almost_equal(v, mesh.vertex_normals(v, t), decimal=2)
  s = v.copy()
  s[:, 2] *= 2.0
  want = v.copy()
  want[:, 2] *= 0.5
  want /= np.linalg.norm(want, axis=1, keepdims=True)
  np.testing.assert_array_almost_equal(want, mesh.vertex_normals(s, t), decimal=2)


def test_vertex_normals_torch_oracle_matches_numpy_and_finite_differences():
  from oracle import mesh
  v, t = _sphere()
  rng = np.random.default_rng(5)
  v = v + rng.normal(0, 0.05, v.shape).astype(np.float32)
  tv = torch.tensor(v, dtype=torch.float64, requires_grad=True)
  tt = torch.tensor(t)
  np.testing.assert_allclose(mesh.vertex_normals_t(tv, tt).detach().numpy(),
                             mesh.vertex_normals(v, t), rtol=1e-12, atol=1e-12)
  assert torch.autograd.gradcheck(lambda x: mesh.vertex_normals_t(x, tt), (tv,))


def test_oracle_spot_textured_golden():
  """splat_test.py:227-277 ('spot') through the CPU restatement: vertex
  normals, texture map, diffuse light (shaders.py:68-97), splat; pins the
  restated shading chain to the reference's blurred golden render."""
  from oracle import mesh as omesh
  from oracle import splat as np_splat
  from oracle import texture
  g = helpers.golden("spot.npz")
  proj = helpers.make_perspective_matrix() @ helpers.make_look_at_matrix("spot")
  pos, tris, uvs = g["positions"], g["triangles"], g["uvs"]
  clip = raster.transform(proj.astype(np.float32), pos)
  ids, z, b = raster.rasterize(clip, tris, helpers.IMAGE_WIDTH, helpers.IMAGE_HEIGHT, 1, 1)
  normals = omesh.vertex_normals(pos, tris).astype(np.float32)
  uv = np_splat.interpolate(uvs, ids, z, b, tris)
  n = np_splat.interpolate(normals, ids, z, b, tris)
  tex = np.flipud(g["texture"]).astype(np.float32) / np.float32(255.0)
  rgb = texture.texture_map(uv.reshape(-1, 2), tex).reshape(uv.shape[:-1] + (3,))
  d = np.array([0.5, 0.5, 1.0], np.float32)
  d = d / np.sqrt((d * d).sum() + np.float32(1e-12))
  ndl = np.clip((n * d).sum(-1, keepdims=True), 0.0, 1.0)
  lit = rgb * np.float32(0.5) + rgb * np.float32(0.5) * ndl
  rgba = np.concatenate([lit, (uv[..., :1] > -1.0).astype(np.float32)], -1).astype(np.float32)
  out, _, _ = np_splat.splat_shaded_pixels(clip, ids, z, b, tris, rgba, helpers.IMAGE_WIDTH,
                                           helpers.IMAGE_HEIGHT)
  ok, msg = helpers.images_near_python(g["target"], helpers.pil_format(out[..., :3]))
  assert ok, msg


@pytest.mark.parametrize("lighting", ["diffuse", "point", "phong_point"])
def test_oracle_spot_lighting_goldens(lighting):
  """shaders_test.py:76-168 through the CPU restatement: the spot with
  texture and diffuse / point / Blinn-Phong point lighting (shaders.py:68-173)
  on vertex normals (mesh.py:22-52), CompositingMode.OVER, one layer."""
  from oracle import mesh as omesh
  from oracle import shading
  from oracle import splat as np_splat
  from oracle import texture
  g = helpers.golden("spot.npz")
  proj = helpers.make_perspective_matrix() @ helpers.make_look_at_matrix("spot")
  pos, tris, uvs = g["positions"], g["triangles"], g["uvs"]
  clip = raster.transform(proj.astype(np.float32), pos)
  ids, z, b = raster.rasterize(clip, tris, helpers.IMAGE_WIDTH, helpers.IMAGE_HEIGHT, 1, 1)
  normals = omesh.vertex_normals(pos, tris).astype(np.float32)
  uv = np_splat.interpolate(uvs, ids, z, b, tris)
  n = np_splat.interpolate(normals, ids, z, b, tris)
  p = np_splat.interpolate(pos, ids, z, b, tris)
  tex = np.flipud(g["texture"]).astype(np.float32) / np.float32(255.0)
  rgb = texture.texture_map(uv.reshape(-1, 2), tex).reshape(uv.shape[:-1] + (3,))
  eye = helpers.eye_position("spot")[0].astype(np.float32)
  if lighting == "diffuse":
    d = np.array([0.5, 0.5, 1.0], np.float32)
    d = d / np.sqrt((d * d).sum() + np.float32(1e-12))
    ndl = np.clip((n * d).sum(-1, keepdims=True), 0.0, 1.0)
    lit = rgb * np.float32(0.5) + rgb * np.float32(0.5) * ndl
  else:
    kw = dict(eye=tuple(eye), ks=1.0, ns=50.0) if lighting == "phong_point" else {}
    lit = shading.point_light(torch.tensor(rgb), torch.tensor(n), torch.tensor(p),
                              tuple(eye), **kw).numpy()
  out = (lit * (z != 1.0)[..., None])[0]  # OVER of one masked layer
  ok, msg = helpers.images_near_python(g[lighting], helpers.pil_format(out))
  assert ok, msg


@pytest.mark.filterwarnings("ignore::DeprecationWarning")  # torch.func's own imports
def test_oracle_spike_derivative_golden():
  """splat_test.py:170-224: the forward-mode derivative (jax.jvp) of a
  render with respect to the offset of one sphere vertex, through the torch
  restatement (torch.func.jvp in place of jax.jvp, discrete state held
  fixed), equals the reference's Spike_Derivative.png. Pins the derivative
  of the splat chain to the reference's own output."""
  g = helpers.golden("render_goldens.npz")
  v0 = g["sphere_vertices"].astype(np.float32)
  t = g["sphere_triangles"].astype(np.int32)
  v = v0.copy()
  v[32] *= 2.0
  proj = helpers.make_perspective_matrix() @ helpers.make_look_at_matrix("view_1")
  W, H = helpers.IMAGE_WIDTH, helpers.IMAGE_HEIGHT
  clip32 = raster.transform(proj.astype(np.float32), v)
  ids, z, b = raster.rasterize(clip32, t, W, H, 1, 1)
  state = torch_ref.discrete_state(clip32, ids, z, b, t, W, H)
  ti, tz, tt, tb = torch.tensor(ids), torch.tensor(z), torch.tensor(t).long(), torch.tensor(b)
  P = torch.tensor(proj, dtype=torch.float32)
  ones = torch.ones(len(v), 4)

  def render(vv):
    clip = torch.cat([vv, torch.ones_like(vv[:, :1])], 1) @ P.T
    shaded = torch_ref.interpolate(ones, ti, tz, tb, tt)
    return torch_ref.splat_shaded_pixels(clip, ti, tz, tb, tt, shaded, W, H, state)[0]

  tangent = torch.zeros(len(v), 3)
  tangent[32] = torch.tensor(v0[32])  # d vertices / d offset
  rendered, jac = torch.func.jvp(render, (torch.tensor(v),), (tangent,))
  image = (jac / jac.abs().max()) * 0.5 + 0.5
  image = image * 0.95 + rendered * 0.05
  ok, msg = helpers.images_near_python(g["spike_derivative"],
                                       helpers.pil_format(image[..., :3].numpy()),
                                       threshold=0.0)
  assert ok, msg
