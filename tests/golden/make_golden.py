"""Generates the committed golden fixtures of tests/golden from the reference.

Run where the reference tree exists (it is read-only input):
    python tests/golden/make_golden.py --reference <diffren source tree>
(or with DIFFREN_REFERENCE set to that tree).

It (1) compiles the reference's own CPU rasterizer in place
(oracle/Makefile `ref`) and records its outputs on seeded and reference-test
geometry (raster_ref.npz); (2) extracts the reference tests' fixtures and
known answers from their source text (cube vertices, triangle cases, the
differentiable-barycentrics Jacobian of rasterize_test.py:216-224); (3)
decodes the small golden PNGs the GPU tests compare against, (4) keeps
the textured spot mesh, its texture and its blurred target render
(spot.npz), and (5) keeps the file bytes of the rasterizer's golden PNGs
(raster_pngs.npz) that the oracle tests decode. Nothing here is used at run time by the library.
"""
import argparse
import ast
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import raster  # noqa: E402
from diffren_gb300 import workloads  # noqa: E402
import helpers  # noqa: E402
from golden import png  # noqa: E402


def _floats(text):
  return [float(x) for x in re.findall(r"-?\d+(?:\.\d+)?(?:e-?\d+)?", text)]


def cpp_arrays(path):
  """Named constexpr arrays of a C++ header, as numpy arrays."""
  src = open(path).read()
  out = {}
  for m in re.finditer(r"constexpr\s+(float|int32_t)\s+(\w+)\[\]\s*=\s*\{([^}]*)\}", src):
    kind, name, body = m.groups()
    vals = _floats(body)
    out[name] = np.array(vals, np.float32 if kind == "float" else np.int32)
  return out


def cpp_test_cases(path):
  """(name, vertices, triangles) of each TEST_F that declares both inline."""
  src = open(path).read()
  cases = []
  for m in re.finditer(r"TEST_F\(\w+,\s*(\w+)\)\s*\{(.*?)\n\}", src, re.S):
    name, body = m.groups()
    for c, val in re.findall(r"const float (\w+) = ([-\d.]+);", body):
      body = re.sub(r"\b%s\b(?! =)" % c, val, body)
    v = re.search(r"std::vector<float> vertices = \{([^}]*)\}", body)
    t = re.search(r"std::vector<int32_t> triangles = \{([^}]*)\}", body)
    if v and t:
      cases.append((name, np.array(_floats(v.group(1)), np.float32).reshape(-1, 4),
                    np.array(_floats(t.group(1)), np.int32).reshape(-1, 3)))
  return cases


def jacobian_known_answer(path):
  src = open(path).read()
  m = re.search(r"expected_jacobian = np\.array\((\[.*?\])\)", src, re.S)
  return np.array(_floats(m.group(1)), np.float32).reshape(3, 3, 3)


def textured_square_inputs(path):
  """Clip coordinates, uvs and 2x2 texture of shaders_test.py's textured
  square (its 4:3 scaling of x included)."""
  src = open(path).read()
  body = src[src.index("def test_textured_square"):]
  body = body[:body.index("rendered = ")]
  arrays = re.findall(r"jnp\.array\(\s*(\[.*?\])\s*(?:,\s*dtype=[^)]*)?\)", body, re.S)
  clip = np.array(_floats(arrays[0]), np.float32).reshape(4, 4)
  uv = np.array(_floats(arrays[1]), np.float32).reshape(4, 2)
  tex = np.array(_floats(arrays[2]), np.float32).reshape(2, 2, 3)
  m = re.search(r"clip_coordinates\.at\[:, 0\]\.multiply\(([0-9.]+)\)", body)
  clip[:, 0] *= np.float32(float(m.group(1)))
  tris = re.search(r"\{'uv': uv_coordinates\},\s*(\(\(.*?\)\)),", src, re.S)
  tri = np.array(_floats(tris.group(1)), np.int32).reshape(-1, 3)
  return {"textured_square_clip": clip, "textured_square_uv": uv,
          "textured_square_texture": tex, "textured_square_triangles": tri}


def _safe_number(text, names):
  """Value of a small arithmetic expression of the test source: numbers, the
  given names, + - * /, unary minus, parentheses and float('inf')."""
  def ev(node):
    if isinstance(node, ast.Expression):
      return ev(node.body)
    if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)):
      return float(node.value)
    if isinstance(node, ast.Name) and node.id in names:
      return float(names[node.id])
    if isinstance(node, ast.UnaryOp) and isinstance(node.op, (ast.USub, ast.UAdd)):
      v = ev(node.operand)
      return -v if isinstance(node.op, ast.USub) else v
    if isinstance(node, ast.BinOp) and isinstance(node.op, (ast.Add, ast.Sub, ast.Mult,
                                                            ast.Div)):
      a, b = ev(node.left), ev(node.right)
      return {ast.Add: a + b, ast.Sub: a - b, ast.Mult: a * b,
              ast.Div: a / b if b else float("nan")}[type(node.op)]
    if (isinstance(node, ast.Call) and isinstance(node.func, ast.Name) and
        node.func.id == "float" and len(node.args) == 1 and
        isinstance(node.args[0], ast.Constant) and node.args[0].value in ("inf", "-inf")):
      return float(node.args[0].value)
    raise ValueError("unexpected expression in test data: %r" % text)
  return ev(ast.parse(text.strip(), mode="eval"))


def bilinear_boundary_cases(path):
  """(x, y) samples and expected values of image_test.py's boundary test
  on its 30 x 10 ramp image (values 1..10 along x)."""
  src = open(path).read()
  body = src[src.index("test_case_list = [") + len("test_case_list = ["):]
  body = body[:body.index("# pyformat: enable")]
  rows = re.findall(r"\[\[\s*([^\[\]]+?)\s*\],\s*([^\[\]]+?)\]", body)
  names = {"image_width": 10, "image_height": 30}
  samples, expected = [], []
  for pt, val in rows:
    samples.append([_safe_number(t, names) for t in pt.split(",")])
    expected.append(_safe_number(val, names))
  return {"samples": np.array(samples, np.float32), "expected": np.array(expected, np.float32),
          "shape": np.array([30, 10], np.int32)}


RASTER_PNGS = ["Simple_Triangle.png", "External_Triangle.png", "Simple_Tetrahedron.png",
               "Inside_Box.png", "Ids_Cube.png", "Ids_Cube_Back.png", "Barycentrics_Cube.png",
               "Barycentrics_Cube_Back.png", "UV_Sphere_Ids.png"]


def main():
  ap = argparse.ArgumentParser()
  ap.add_argument("--reference", default=os.environ.get("DIFFREN_REFERENCE"),
                  help="root of the diffren source tree (default $DIFFREN_REFERENCE)")
  args = ap.parse_args()
  ref = args.reference
  if not ref:
    raise SystemExit("pass --reference or set DIFFREN_REFERENCE")
  kern = os.path.join(ref, "diffren", "common", "kernels")
  data = os.path.join(ref, "diffren", "common", "test_data")
  if raster.build_reference(ref) is None:
    raise SystemExit("reference tree not found at " + ref)

  fixtures = {}

  def record(name, verts, tris, w, h, layers, cull):
    ids, z, b = raster.rasterize_reference_cpu(verts, tris, w, h, layers, cull)
    fixtures[name + "__vertices"] = np.asarray(verts, np.float32)
    fixtures[name + "__triangles"] = np.asarray(tris, np.int32)
    fixtures[name + "__meta"] = np.array([w, h, layers, cull], np.int32)
    fixtures[name + "__ids"] = ids
    fixtures[name + "__z"] = z
    fixtures[name + "__bary"] = b

  arrays = cpp_arrays(os.path.join(kern, "rasterize_test_utils.h"))
  cube_v = arrays["CUBE_VERTICES"].reshape(-1, 4)
  cube_t = arrays["CUBE_TRIANGLES"].reshape(-1, 3)
  big_v = arrays["LARGE_CUBE_VERTICES"].reshape(-1, 4)
  big_t = arrays["LARGE_CUBE_TRIANGLES"].reshape(-1, 3)
  for name, v, t in cpp_test_cases(os.path.join(kern, "rasterize_triangles_impl_test.cc")):
    record("test_" + name, v, t, 160, 120, 1, 0)
  record("test_SimpleTriangleFull", *cpp_test_cases(
      os.path.join(kern, "rasterize_triangles_impl_test.cc"))[0][1:], 640, 480, 1, 0)
  record("inside_box", big_v, big_t, 160, 120, 1, 0)
  for cull in (0, 1, 2):
    record("cube_cull%d" % cull, cube_v, cube_t, 160, 120, 2, cull)
  for seed, (w, h, layers, cull) in enumerate([(96, 72, 3, 0), (96, 72, 3, 1),
                                              (97, 61, 4, 2), (64, 64, 1, 0)]):
    m = workloads.soup_workload(1500, seed=seed, mu=-2.5, sigma=0.6)
    eye = workloads.sphere_eyes(1, seed=seed + 11, radius=2.0 + seed * 0.4)[0]
    cam = workloads.camera_matrix(eye, w, h)
    record("soup%d" % seed, raster.transform(cam, m.vertices), m.triangles, w, h,
           layers, cull)
  # Camera inside the soup: many near-plane crossings.
  m = workloads.soup_workload(3000, seed=9, mu=-1.8, sigma=0.5)
  cam = workloads.camera_matrix((0.05, 0.1, 0.2), 80, 60)
  record("soup_near", raster.transform(cam, m.vertices), m.triangles, 80, 60, 3, 0)
  m = workloads.icosphere_workload(16, seed=0)
  cam = workloads.camera_matrix((0.0, 0.0, 3.0), 128, 128)
  record("icosphere_c1", raster.transform(cam, m.vertices), m.triangles, 128, 128, 3, 1)
  np.savez_compressed(os.path.join(HERE, "raster_ref.npz"), **fixtures)

  # Known answer of the differentiable-barycentrics Jacobian.
  jac = jacobian_known_answer(os.path.join(ref, "diffren", "jax", "internal",
                                           "rasterize_test.py"))
  np.savez_compressed(os.path.join(HERE, "diff_bary_jacobian.npz"), expected=jac)

  # Splat goldens: 32x32 renders upsampled 16x with nearest; keep 32x32.
  splat = {}
  for name in ["Composite", "Layer_0", "Layer_1", "Layer_2"]:
    im = png.read_png(os.path.join(data, "Two_Triangles_Splat_%s.png" % name))
    blocks = im.reshape(32, 16, 32, 16, -1)
    assert (blocks == blocks[:, :1, :, :1]).all()
    splat[name] = im[::16, ::16]
  np.savez_compressed(os.path.join(HERE, "splat_two_triangles.npz"), **splat)

  # Meshes and 640x480 goldens for the render tests on the GPU.
  sv, st = helpers.load_obj(os.path.join(data, "sphere.obj"))
  imgs = {"sphere_vertices": sv, "sphere_triangles": st}
  for i in (0, 1):
    for l in (0, 1, 2):
      imgs["unlit_cube_%d_%d" % (i, l)] = png.read_png(
          os.path.join(data, "Unlit_Cube_%d_%d.png" % (i, l)))
  imgs["spike_derivative"] = png.read_png(os.path.join(data, "Spike_Derivative.png"))
  imgs["textured_square"] = png.read_png(os.path.join(data, "Textured_Square.png"))
  imgs.update(textured_square_inputs(os.path.join(ref, "diffren", "jax", "utils",
                                                   "shaders_test.py")))
  imgs["sphere_disparity"] = png.read_png(os.path.join(data, "Sphere_Disparity.png"))
  # rasterize_test.py:28-152 (barycentrics of one triangle, w constant or varying)
  imgs["simple_triangle"] = png.read_png(os.path.join(data, "Simple_Triangle.png"))
  imgs["perspective_corrected_triangle"] = png.read_png(
      os.path.join(data, "Perspective_Corrected_Triangle.png"))
  np.savez_compressed(os.path.join(HERE, "render_goldens.npz"), **imgs)

  # The textured spot of splat_test.py:227-277: the mesh flattened and scaled
  # as test_utils.load_test_obj does (positions x 0.2), its texture, and the
  # target image blurred as load_and_blur_image does (gaussian, sigma 0.5,
  # edge mode 'nearest', truncated at 4 sigma, per channel), formatted like
  # get_pil_formatted_image.
  from scipy import ndimage
  pos, uv, nrm, tri = helpers.load_obj_attributes(os.path.join(data, "spot_triangulated.obj"))
  assert uv is not None and nrm is None
  target = png.read_png(os.path.join(data, "Spot_Textured.png"))[..., :3].astype(np.float32)
  blurred = ndimage.gaussian_filter(target / 255.0, sigma=(0.5, 0.5, 0.0), mode="nearest",
                                    truncate=4.0)
  np.savez_compressed(os.path.join(HERE, "spot.npz"), positions=pos * np.float32(0.2),
                      uvs=uv, triangles=tri,
                      texture=png.read_png(os.path.join(data, "spot_texture.png")),
                      target=helpers.pil_format(blurred),
                      # shaders_test.py:76-168: OVER renders of the same spot
                      diffuse=png.read_png(os.path.join(data, "Spot_Textured.png")),
                      point=png.read_png(os.path.join(data, "Spot_Textured_Pt_Light.png")),
                      phong_point=png.read_png(
                          os.path.join(data, "Spot_Textured_Phong_Point.png")))

  # The rasterizer goldens of rasterize_triangles_impl_test.cc and
  # rasterize_triangles_impl_cuda_test.cc, as their PNG file bytes.
  np.savez_compressed(os.path.join(HERE, "raster_pngs.npz"), **{
      name[:-4]: np.frombuffer(open(os.path.join(data, name), "rb").read(), np.uint8)
      for name in RASTER_PNGS})

  # Bilinear resampling known answers (image_test.py boundary cases).
  np.savez_compressed(os.path.join(HERE, "texture_cases.npz"),
                      **bilinear_boundary_cases(os.path.join(ref, "diffren", "jax", "utils",
                                                             "image_test.py")))
  for f in sorted(os.listdir(HERE)):
    if f.endswith(".npz"):
      print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
  main()
