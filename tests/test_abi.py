"""CPU tests of the C ABI boundary: the library builds and loads, exports
every symbol the header declares with the argument count the header gives,
and rejects bad arguments without touching a GPU."""
import ctypes
import os
import re

import pytest

from diffren_gb300 import _lib, kernels

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                      "include", "diffren_gb300.h")


def declarations():
  with open(HEADER) as f:
    src = f.read()
  src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
  decls = {}
  for m in re.finditer(r"\b(dr_\w+)\s*\(([^)]*)\)\s*;", src):
    name, params = m.groups()
    params = params.strip()
    n = 0 if params in ("", "void") else params.count(",") + 1
    decls[name] = n
  return decls


def test_header_declares_the_boundary():
  d = declarations()
  for name in ("dr_rasterize_triangles", "dr_rasterize_batch", "dr_splat_fwd",
               "dr_splat_bwd", "dr_interpolate_fwd", "dr_interpolate_bwd",
               "dr_diff_barycentrics_fwd", "dr_diff_barycentrics_bwd",
               "dr_transform_vertices", "dr_transform_vertices_bwd", "dr_last_error"):
    assert name in d, name


def test_library_exports_every_declared_symbol():
  lib = _lib.load()
  for name, nargs in declarations().items():
    assert hasattr(lib, name), name
    assert name in _lib.SIGNATURES, name
    assert len(_lib.SIGNATURES[name][1]) == nargs, (name, nargs)


def test_abi_version_and_error_string():
  lib = _lib.load()
  assert lib.dr_abi_version() == 3
  assert isinstance(lib.dr_last_error(), bytes)


def test_workspace_query_rejects_bad_config():
  lib = _lib.load()
  b = kernels.ImageBatch.single(8, 8, 3, 1)
  for cfg in (kernels.raster_config(0, 0, 0), kernels.raster_config(17, 0, 0),
              kernels.raster_config(1, 5, 0), kernels.raster_config(1, 0, 2),
              kernels.raster_config(1, 0, 0, tile=(256, 8)),
              kernels.raster_config(1, 0, 0, flags=4)):
    assert lib.dr_rasterize_batch_workspace_bytes(b.ptr, 1, ctypes.byref(cfg)) == 0
    assert lib.dr_last_error()
  good = kernels.raster_config(3, 1, 0)
  n = lib.dr_rasterize_batch_workspace_bytes(b.ptr, 1, ctypes.byref(good))
  assert n > 0 and n % 256 == 0
  assert lib.dr_rasterize_triangles_workspace_bytes(1000, 64, 64, 3) > 0


def test_workspace_grows_with_triangles_and_tiles():
  lib = _lib.load()
  cfg = kernels.raster_config(3, 1, 0)
  small = kernels.ImageBatch.single(64, 64, 3, 10)
  big = kernels.ImageBatch.single(64, 64, 3, 10000)
  wide = kernels.ImageBatch.single(4096, 64, 3, 10)
  f = lambda b: lib.dr_rasterize_batch_workspace_bytes(b.ptr, 1, ctypes.byref(cfg))
  assert f(big) > f(small) and f(wide) > f(small)


def test_entry_points_reject_bad_arguments_without_gpu_work():
  lib = _lib.load()
  b = kernels.ImageBatch.single(8, 8, 3, 1)
  cfg = kernels.raster_config(1, 0, 0)
  # Null outputs / workspace.
  rc = lib.dr_rasterize_batch(None, None, b.ptr, 1, ctypes.byref(cfg), None, None, None,
                              None, 0, None)
  assert rc == 1 and b"non-null" in lib.dr_last_error()
  # Bad image sizes.
  bad = kernels.ImageBatch.single(8, 8, 3, 1)
  bad.descs[0].width = 0
  rc = lib.dr_rasterize_batch(None, None, bad.ptr, 1, ctypes.byref(cfg), None, None,
                              None, None, 0, None)
  assert rc == 1
  # Too many splat channels, bad layer counts.
  assert lib.dr_splat_fwd(None, None, None, 9, b.ptr, 1, 3, None, None, None, None,
                          None) == 1
  assert lib.dr_splat_fwd(None, None, None, 4, b.ptr, 1, 0, None, None, None, None,
                          None) == 1
  # The backward needs the forward's saved accumulators.
  assert lib.dr_splat_bwd(None, None, None, None, None, 4, b.ptr, 1, 3, None, None,
                          None) == 1
  # Unknown splat flags; foreground-only color gradients need the depth buffer.
  saved = fake = ctypes.c_void_p(256)
  assert lib.dr_splat_bwd_ex(None, None, None, None, saved, 4, b.ptr, 1, 3, 2, None, None,
                             None) == 1
  assert lib.dr_splat_bwd_ex(None, None, None, None, saved, 4, b.ptr, 1, 3,
                             _lib.DR_SPLAT_FOREGROUND_GRADIENTS, None, None, None) == 1
  assert b"depth buffer" in lib.dr_last_error()
  # Samples VJP: unknown flags; the deterministic sums need their scratch.
  assert lib.dr_interpolate_with_positions_bwd_ex(
      None, None, None, 4, None, None, None, None, None, None, None, b.ptr, 1, 3, 2,
      None, saved, None, None, 0, None) == 1
  assert lib.dr_interpolate_with_positions_bwd_ex(
      None, None, None, 4, None, None, None, None, None, None, None, b.ptr, 1, 3,
      _lib.DR_SAMPLES_DETERMINISTIC, None, saved, None, None, 0, None) == 1
  assert b"scratch" in lib.dr_last_error()
  n = lib.dr_interpolate_with_positions_bwd_scratch_bytes(b.ptr, 1, 4)
  assert n >= 256 + 3 * (4 + 4) * 8  # the header, then 3 vertices x (4 + 4) sums
  assert lib.dr_interpolate_with_positions_bwd_scratch_bytes(b.ptr, 1, 17) == 0
  # Texture VJP: the deterministic sums need the _ex entry point and its scratch.
  assert lib.dr_texture_map_bwd(fake, fake, 10, fake, 4, 4, 4, _lib.DR_TEXTURE_DETERMINISTIC,
                                fake, fake, None) == 1
  assert lib.dr_texture_map_bwd_ex(fake, fake, 10, fake, 4, 4, 4,
                                   _lib.DR_TEXTURE_DETERMINISTIC, fake, fake, None, 0,
                                   None) == 1
  assert b"scratch" in lib.dr_last_error()
  assert lib.dr_texture_map_bwd_ex(fake, fake, 10, fake, 4, 4, 4, 8, fake, fake, None, 0,
                                   None) == 1
  assert lib.dr_texture_map_bwd_scratch_bytes(4, 4, 4) == 256 + 4 * 4 * 4 * 8
  assert lib.dr_interpolate_fwd(None, 17, None, None, None, None, None, b.ptr, 1, 3, None,
                                None) == 1
  assert lib.dr_transform_vertices(None, None, 5, b.ptr, 1, None, None) == 1
  # Misaligned positions / clip vertices.
  assert lib.dr_splat_fwd(ctypes.c_void_p(4), None, None, 4, b.ptr, 1, 3, None, None,
                          None, None, None) == 4
  assert lib.dr_splat_positions_fwd(ctypes.c_void_p(4), None, None, None, None, b.ptr, 1,
                                    3, None, None) == 4
  fake = ctypes.c_void_p(256)
  # OVER compositing: layer and channel counts, null buffers.
  assert lib.dr_composite_over_fwd(fake, fake, 4, b.ptr, 1, 0, fake, None) == 1
  assert lib.dr_composite_over_fwd(fake, fake, 0, b.ptr, 1, 3, fake, None) == 1
  assert lib.dr_composite_over_bwd(None, fake, fake, 4, b.ptr, 1, 3, fake, None) == 1
  # Vertex normals: null mesh, negative counts, misaligned scratch.
  assert lib.dr_vertex_normals_fwd(None, None, b.ptr, 1, None, None, None) == 1
  neg = kernels.ImageBatch.single(8, 8, 3, 1)
  neg.descs[0].num_triangles = -1
  assert lib.dr_vertex_normals_fwd(fake, fake, neg.ptr, 1, fake, fake, None) == 1
  assert lib.dr_vertex_normals_fwd(fake, fake, b.ptr, 1, ctypes.c_void_p(260), fake,
                                   None) == 4
  assert lib.dr_vertex_normals_bwd(fake, fake, fake, b.ptr, 1, fake, ctypes.c_void_p(260),
                                   fake, None) == 4


def test_squared_error_rejects_bad_arguments():
  lib = _lib.load()
  fake = ctypes.c_void_p(256)
  assert lib.dr_squared_error(fake, fake, -1, 1.0, fake, fake, fake, None) == 1
  assert lib.dr_squared_error(fake, fake, 4, 1.0, fake, None, fake, None) == 1
  assert lib.dr_squared_error(None, fake, 4, 1.0, fake, fake, fake, None) == 1
  assert lib.dr_squared_error(fake, fake, 4, 1.0, fake, fake, None, None) == 1


def test_squared_error_takes_cuda_tensors():
  import torch
  from diffren_gb300 import losses
  with pytest.raises(ValueError, match="CUDA tensors"):
    losses.squared_error_seed(torch.zeros(4), torch.zeros(4))


def test_python_constants_match_header():
  with open(HEADER) as f:
    src = f.read()
  for name in ("DR_FLAG_INDEX_OUT_OF_RANGE", "DR_FLAG_NONFINITE_VERTEX", "DR_TEXTURE_PAD_ZERO",
               "DR_TEXTURE_TEXEL_UNITS",
               "DR_MAX_LAYERS", "DR_MAX_CHANNELS", "DR_MAX_BATCH_INLINE", "DR_MAX_IMAGE_DIM",
               "DR_MAX_SPLAT_CHANNELS", "DR_OK", "DR_SQUARED_ERROR_PARTIALS",
               "DR_CULL_NONE", "DR_CULL_BACK", "DR_CULL_FRONT", "DR_DEPTH_DISCRETIZED",
               "DR_DEPTH_FLOAT"):
    m = re.search(r"#define %s (\d+)u?" % name, src)
    assert m and int(m.group(1)) == getattr(_lib, name), name
  assert kernels._groups(kernels.ImageBatch([1] * 129, [1] * 129, [0] * 129,
                                            [0] * 129)) == 2


def test_oversized_image_is_rejected():
  lib = _lib.load()
  cfg = kernels.raster_config(1, 0, 0)
  ok = kernels.ImageBatch.single(_lib.DR_MAX_IMAGE_DIM, 1, 3, 1)
  assert lib.dr_rasterize_batch_workspace_bytes(ok.ptr, 1, ctypes.byref(cfg)) > 0
  big = kernels.ImageBatch.single(_lib.DR_MAX_IMAGE_DIM + 1, 1, 3, 1)
  assert lib.dr_rasterize_batch_workspace_bytes(big.ptr, 1, ctypes.byref(cfg)) == 0
  assert b"32768" in lib.dr_last_error()


def test_status_raises_with_message():
  lib = _lib.load()
  b = kernels.ImageBatch.single(8, 8, 3, 1)
  lib.dr_transform_vertices(None, None, 5, b.ptr, 1, None, None)
  with pytest.raises(_lib.DiffrenError, match="dim"):
    _lib.check(1, "dr_transform_vertices")
