"""Seeded synthetic meshes and cameras for the rasterize-then-splat workloads.

No dataset is involved: every input is generated from a numpy seed. The
shapes follow the benchmark configurations of the path:

* ``icosphere_workload``: geodesic icosphere of frequency f
  (T = 20 f^2 triangles, V = 10 f^2 + 2 vertices), unit radius plus Gaussian
  radial noise, per-vertex RGB uniform in [0, 1].
* ``soup_workload``: independent triangles, centres uniform in [-1, 1]^3,
  each vertex at centre + random unit direction * lognormal(mu, sigma).
* ``heightfield_workload``: an n x n vertex grid split into 2 (n-1)^2
  triangles with the quad split of diffren/jax/utils/depthmap.py:22-64,
  heights from seeded multi-octave value noise.
* ``ragged_batch``: meshes with lognormal triangle counts, each with its own
  camera and a square resolution from {256, 512, 1024}.

Cameras are perspective (fov_y 60 degrees, near 0.1, far 10) looking at the
origin from a sphere of radius 3 (camera.py:23-44, 126-184).
"""
import dataclasses
import functools

import numpy as np

from . import camera as camera_lib


@dataclasses.dataclass
class Mesh:
  vertices: np.ndarray  # [V, 3] float32 world positions
  triangles: np.ndarray  # [T, 3] int32, counter-clockwise seen from outside
  colors: np.ndarray  # [V, 3] float32 RGB in [0, 1]
  uvs: np.ndarray = None  # [V, 2] float32, heightfields only


def _icosahedron():
  t = (1.0 + 5.0**0.5) / 2.0
  v = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t],
                [0, 1, t], [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1],
                [-t, 0, -1], [-t, 0, 1]], np.float64)
  f = np.array([[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
                [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
                [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
                [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]],
               np.int64)
  return v / np.linalg.norm(v, axis=1, keepdims=True), f


@functools.lru_cache(maxsize=64)
def icosphere(frequency):
  """Geodesic (class I) icosphere: 20 f^2 faces, 10 f^2 + 2 vertices."""
  base_v, base_f = _icosahedron()
  f = int(frequency)
  # Barycentric lattice (i, j), i + j <= f, numbered i-major.
  ii, jj = np.meshgrid(np.arange(f + 1), np.arange(f + 1), indexing="ij")
  keep = ii + jj <= f
  ii, jj = ii[keep], jj[keep]
  idx = lambda i, j: i * (f + 1) - (i * (i - 1)) // 2 + j
  ui, uj = np.meshgrid(np.arange(f), np.arange(f), indexing="ij")
  up = ui + uj < f
  ui, uj = ui[up], uj[up]
  tri_up = np.stack([idx(ui, uj), idx(ui + 1, uj), idx(ui, uj + 1)], 1)
  dn = ui + uj + 1 < f
  di, dj = ui[dn], uj[dn]
  tri_dn = np.stack([idx(di + 1, dj), idx(di + 1, dj + 1), idx(di, dj + 1)], 1)
  tris_local = np.concatenate([tri_up, tri_dn]).astype(np.int64)
  wa, wb, wc = (f - ii - jj) / f, ii / f, jj / f
  pts = np.concatenate([wa[:, None] * base_v[a] + wb[:, None] * base_v[b] +
                        wc[:, None] * base_v[c] for a, b, c in base_f])
  pts /= np.linalg.norm(pts, axis=1, keepdims=True)
  n_local = len(ii)
  # Merge duplicated edge/corner vertices: 21-bit quantized coordinates
  # (resolution ~1e-6, far below the vertex spacing) packed in one int64.
  q = np.round((pts + 1.0) * (2**20 - 1)).astype(np.int64)
  keys = (q[:, 0] << 42) | (q[:, 1] << 21) | q[:, 2]
  _, first, inverse = np.unique(keys, return_index=True, return_inverse=True)
  inverse = inverse.reshape(-1)
  verts = pts[first]
  faces = inverse[np.concatenate([tris_local + k * n_local for k in range(20)])]
  # Orient counter-clockwise seen from outside.
  a, b, c = verts[faces[:, 0]], verts[faces[:, 1]], verts[faces[:, 2]]
  flip = np.einsum("ij,ij->i", np.cross(b - a, c - a), a + b + c) < 0
  faces[flip] = faces[flip][:, [0, 2, 1]]
  assert len(verts) == 10 * f * f + 2 and len(faces) == 20 * f * f
  verts.setflags(write=False)
  faces = faces.astype(np.int32)
  faces.setflags(write=False)
  return verts, faces


def frequency_for_triangles(t):
  return max(1, int(round((t / 20.0)**0.5)))


def icosphere_workload(frequency, seed=0, noise=0.02):
  rng = np.random.default_rng(seed)
  v, f = icosphere(frequency)
  v = v * (1.0 + noise * rng.standard_normal((len(v), 1)))
  colors = rng.uniform(0.0, 1.0, (len(v), 3))
  return Mesh(v.astype(np.float32), np.array(f), colors.astype(np.float32))


def soup_workload(num_triangles, seed=0, mu=-4.0, sigma=0.7):
  rng = np.random.default_rng(seed)
  centers = rng.uniform(-1.0, 1.0, (num_triangles, 1, 3)).astype(np.float32)
  dirs = rng.standard_normal((num_triangles, 3, 3), dtype=np.float32)
  dirs /= np.sqrt((dirs * dirs).sum(-1, keepdims=True))
  lengths = rng.lognormal(mu, sigma, (num_triangles, 3, 1)).astype(np.float32)
  v = (centers + dirs * lengths).reshape(-1, 3)
  f = np.arange(3 * num_triangles, dtype=np.int32).reshape(-1, 3)
  colors = rng.random((len(v), 3), dtype=np.float32)
  return Mesh(v, f, colors)


def value_noise(n, seed, octaves=4, amplitude=0.2):
  """Seeded multi-octave value noise on an n x n grid, range ~[-a, a]."""
  rng = np.random.default_rng(seed)
  out = np.zeros((n, n))
  x = np.linspace(0.0, 1.0, n)
  total = 0.0
  for o in range(octaves):
    cells = 4 * 2**o
    lattice = rng.uniform(-1.0, 1.0, (cells + 1, cells + 1))
    g = x * cells
    i0 = np.minimum(np.floor(g).astype(int), cells - 1)
    t = g - i0
    t = t * t * (3 - 2 * t)
    a = lattice[i0][:, i0] * (1 - t)[None, :] + lattice[i0][:, i0 + 1] * t[None, :]
    b = (lattice[i0 + 1][:, i0] * (1 - t)[None, :] +
         lattice[i0 + 1][:, i0 + 1] * t[None, :])
    layer = a * (1 - t)[:, None] + b * t[:, None]
    weight = 0.5**o
    out += weight * layer
    total += weight
  return amplitude * out / total


def grid_triangles(n):
  """Quad split of depthmap.py:22-64 on an n x n grid (row-major indices)."""
  x, y = np.meshgrid(np.arange(n - 1), np.arange(n - 1))
  bl = y * n + x
  br = y * n + x + 1
  tl = (y + 1) * n + x
  tr = (y + 1) * n + x + 1
  tris = np.stack([bl, br, tl, br, tr, tl], axis=-1).reshape(-1, 3)
  return tris.astype(np.int32)


def heightfield_workload(n, seed=0, amplitude=0.2):
  h = value_noise(n, seed, amplitude=amplitude)
  g = np.linspace(-1.0, 1.0, n)
  gx, gz = np.meshgrid(g, g)
  # Row index runs along -z so that the quad split faces +y (up).
  v = np.stack([gx, h, -gz], axis=-1).reshape(-1, 3)
  uv = np.stack(np.meshgrid(np.linspace(0, 1, n), np.linspace(0, 1, n)),
                axis=-1).reshape(-1, 2)
  rng = np.random.default_rng(seed + 1)
  colors = rng.uniform(0.0, 1.0, (len(v), 3))
  return Mesh(v.astype(np.float32), grid_triangles(n), colors.astype(np.float32),
              uv.astype(np.float32))


def camera_matrix(eye, width, height, fov_y=60.0, near=0.1, far=10.0,
                  up=(0.0, 1.0, 0.0)):
  proj = camera_lib.perspective(width / height, fov_y, near, far)
  view = camera_lib.look_at(eye, (0.0, 0.0, 0.0), up)
  return (proj @ view).astype(np.float32)


def sphere_eyes(num, seed=0, radius=3.0, upper_only=False):
  rng = np.random.default_rng(seed)
  eyes = []
  while len(eyes) < num:
    d = rng.standard_normal(3)
    d /= np.linalg.norm(d)
    if upper_only:
      d[1] = abs(d[1]) + 0.3
      d /= np.linalg.norm(d)
    if abs(d[1]) > 0.995:  # keep look_at well conditioned
      continue
    eyes.append(radius * d)
  return np.array(eyes)


def ragged_batch(num_meshes=64, seed=0, median_triangles=20000, sigma=1.2,
                 t_min=500, t_max=500000, resolutions=(256, 512, 1024)):
  """Meshes (icosphere or soup, 50/50) with lognormal triangle counts."""
  rng = np.random.default_rng(seed)
  counts = np.clip(rng.lognormal(np.log(median_triangles), sigma, num_meshes),
                   t_min, t_max).astype(int)
  kinds = rng.integers(0, 2, num_meshes)
  sizes = rng.choice(np.array(resolutions), num_meshes)
  eyes = sphere_eyes(num_meshes, seed=seed + 7)
  meshes, cams = [], []
  for i in range(num_meshes):
    if kinds[i] == 0:
      m = icosphere_workload(frequency_for_triangles(counts[i]), seed=seed + i)
    else:
      m = soup_workload(int(counts[i]), seed=seed + i)
    meshes.append(m)
    cams.append(camera_matrix(eyes[i], sizes[i], sizes[i]))
  return meshes, cams, [(int(s), int(s)) for s in sizes]
