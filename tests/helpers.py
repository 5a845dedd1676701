"""Shared test helpers: the reference tests' cameras, image comparisons and
encoders, restated (test infrastructure)."""
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
# The diffren source tree, where a test wants it (only the fixture generator
# and the reference builds read it; set DIFFREN_REFERENCE to use it).
REFERENCE = os.environ.get("DIFFREN_REFERENCE", "")

IMAGE_WIDTH = 640
IMAGE_HEIGHT = 480


def golden(name):
  return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


# diffren/common/test_utils.py:38-96
def eye_position(view_name):
  if view_name.startswith("view_1"):
    return np.array((2.0, 3.0, 6.0)), np.array((0.0, 1.0, 0.0))
  if view_name.startswith("view_2"):
    return np.array((-3.0, 1.0, 6.0)), np.array((0.0, 1.0, 0.0))
  if view_name.startswith("spot"):
    return np.array((0.2, 0.3, -0.5)), np.array((0.0, -1.0, 0.0))
  raise ValueError(view_name)


def make_look_at_matrix(view_name):
  eye, world_up = eye_position(view_name)
  forward = -eye / np.linalg.norm(eye)
  to_side = np.cross(forward, world_up)
  to_side /= np.linalg.norm(to_side)
  cam_up = np.cross(to_side, forward)
  rot = np.eye(4)
  rot[0, :3], rot[1, :3], rot[2, :3] = to_side, cam_up, -forward
  trans = np.eye(4)
  trans[:3, 3] = -eye
  return rot @ trans


def make_perspective_matrix(index=0):
  fov_y, near, far = [40.0, 60.0][index], [0.01, 0.1][index], [10.0, 20.0][index]
  aspect = IMAGE_WIDTH / IMAGE_HEIGHT
  f = 1.0 / np.tan(fov_y * (math.pi / 360.0))
  a = -(far + near) / (far - near)
  b = -2.0 * (far * near / (far - near))
  return np.array([[f / aspect, 0, 0, 0], [0, f, 0, 0], [0, 0, a, b], [0, 0, -1, 0]])


# diffren/common/compare_images.py:26-70 (Python tests) and
# diffren/common/kernels/rasterize_test_utils.cc:195-230 (C++ tests).
def pil_format(image, add_transparency=True):
  image = np.asarray(image, np.float32)
  if image.ndim == 2:
    image = image[..., None]
  if image.shape[2] == 1:
    image = np.tile(image, (1, 1, 3))
  if image.shape[2] == 3 and add_transparency:
    image = np.concatenate([image, np.ones(image.shape[:2] + (1,), np.float32)], 2)
  return np.clip(255.0 * image, 0.0, 255.0).astype(np.uint8)


def images_near_python(baseline, result, max_outlier_fraction=0.005, threshold=0.04):
  if baseline.shape != result.shape:
    return False, "shapes %s vs %s" % (baseline.shape, result.shape)
  diff = np.abs(baseline.astype(float) / 255 - result.astype(float) / 255) > threshold
  frac = np.count_nonzero(diff.any(axis=2)) / np.prod(baseline.shape[:2])
  return frac <= max_outlier_fraction, "%f outliers" % frac


def to_rgba(image):
  """lodepng::decode's default output: 8-bit RGBA (opaque alpha added)."""
  image = np.asarray(image, np.uint8)
  if image.shape[2] == 3:
    image = np.concatenate([image, np.full(image.shape[:2] + (1,), 255, np.uint8)], 2)
  return image


def images_near_cpp(baseline, result, tolerance=10):
  baseline = to_rgba(baseline)
  if baseline.shape != result.shape:
    return False, "shapes %s vs %s" % (baseline.shape, result.shape)
  outliers = np.count_nonzero(
      np.abs(baseline.astype(int) - result.astype(int)) > tolerance)
  limit = int(0.005 * baseline.shape[0] * baseline.shape[1])
  return outliers <= limit, "%d outlier channels (max %d)" % (outliers, limit)


def encode_barycentrics(bary, layer=0):
  """rasterize_test_utils.cc:150-163: uint8(b * 255), alpha 255."""
  b = np.asarray(bary, np.float32)[layer]
  out = np.empty(b.shape[:2] + (4,), np.uint8)
  out[..., :3] = (b * np.float32(255.0)).astype(np.uint8)
  out[..., 3] = 255
  return out


COLOR_CYCLE = np.array([255, 0, 0, 0, 255, 0, 0, 0, 255, 255, 0, 255, 0, 255, 255, 255,
                        255, 0, 128, 0, 0, 0, 128, 0, 0, 0, 128, 128, 0, 128, 0, 128,
                        128, 128, 128, 0], np.uint8).reshape(12, 3)


def encode_ids(ids, layer=0):
  """rasterize_test_utils.cc:165-193: id % 12 color cycle (C++ '%')."""
  i = np.asarray(ids)[layer].astype(np.int64)
  mod = np.fmod(i, 12)  # C++ remainder keeps the sign
  out = np.empty(i.shape + (4,), np.uint8)
  out[..., :3] = COLOR_CYCLE[np.where(mod < 0, mod + 12, mod)]
  out[..., :3][mod < 0] = 0  # negative index reads outside the table; unused
  out[..., 3] = 255
  return out


def uv_sphere(n_rows, n_cols, radius):
  """rasterize_test_utils.cc:34-118: UV sphere, float32 math."""
  vs = [[0.0, radius, 0.0]]
  for ri in range(n_rows):
    for ci in range(n_cols):
      phi = np.float32(math.pi * (ri + 1) / (n_rows + 1))
      theta = np.float32(2.0 * math.pi * ci / n_cols)
      s = np.float32(radius) * np.sin(phi, dtype=np.float32)
      vs.append([s * np.sin(theta, dtype=np.float32),
                 np.float32(radius) * np.cos(phi, dtype=np.float32),
                 s * np.cos(theta, dtype=np.float32)])
  vs.append([0.0, -radius, 0.0])
  n_verts = len(vs)
  ts = []
  for ci in range(n_cols):
    ts.append([0, 1 + ci, 1 + (ci + 1) % n_cols])
  for ri in range(n_rows - 1):
    for ci in range(n_cols):
      tl = 1 + ri * n_cols + ci
      tr = 1 + ri * n_cols + (ci + 1) % n_cols
      bl = 1 + (ri + 1) * n_cols + ci
      br = 1 + (ri + 1) * n_cols + (ci + 1) % n_cols
      ts += [[tl, bl, br], [tr, tl, br]]
  last = n_verts - 1 - n_cols
  for ci in range(n_cols):
    ts.append([last + ci, n_verts - 1, last + (ci + 1) % n_cols])
  return np.array(vs, np.float32), np.array(ts, np.int32)


def load_obj(path):
  """Wavefront OBJ -> (positions [V,3] float32, triangles [T,3] int32).

  Vertices are numbered in order of first appearance of each face-vertex
  token, and only the first three tokens of a face are used, as
  diffren/common/obj_loader.py:24-104 does (positions only).
  """
  positions, flat, index, tris = [], [], {}, []
  for line in open(path):
    p = line.split()
    if not p:
      continue
    if p[0] == "v":
      positions.append([float(x) for x in p[1:4]])
    elif p[0] == "f":
      tri = []
      for name in p[1:4]:
        if name not in index:
          index[name] = len(flat)
          flat.append(positions[int(name.split("/")[0]) - 1])
        tri.append(index[name])
      tris.append(tri)
  return np.array(flat, np.float32), np.array(tris, np.int32)


def load_obj_attributes(path):
  """Wavefront OBJ -> (positions [N,3], uvs [N,2] or None, normals [N,3] or
  None, triangles [T,3]) flattened as diffren/common/obj_loader.py:24-104
  does: one vertex per distinct face-vertex token ('v', 'v/vt', 'v//vn',
  'v/vt/vn'), numbered in order of first appearance, zeros for an attribute
  a token lacks, and each attribute kept only if some token uses it."""
  lists = {"v": [], "vt": [], "vn": []}
  flat, index, tris, used = [], {}, [], {"vt": False, "vn": False}
  for line in open(path):
    p = line.split()
    if not p:
      continue
    if p[0] in lists:
      lists[p[0]].append([float(x) for x in p[1:]])
    elif p[0] == "f":
      tri = []
      for name in p[1:4]:
        if name not in index:
          parts = (name.split("/") + ["", ""])[:3]
          row = list(lists["v"][int(parts[0]) - 1][:3])
          for kind, idx, width in (("vt", parts[1], 2), ("vn", parts[2], 3)):
            if idx:
              row += lists[kind][int(idx) - 1][:width]
              used[kind] = True
            else:
              row += [0.0] * width
          index[name] = len(flat)
          flat.append(row)
        tri.append(index[name])
      tris.append(tri)
  a = np.array(flat, np.float32)
  return (a[:, :3], a[:, 3:5] if used["vt"] else None, a[:, 5:8] if used["vn"] else None,
          np.array(tris, np.int32))


def homogeneous(v):
  v = np.asarray(v, np.float32)
  return np.concatenate([v, np.ones((len(v), 1), np.float32)], axis=1)
