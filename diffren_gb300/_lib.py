"""ctypes binding of libdiffren_gb300.so (the C ABI in include/diffren_gb300.h).

The library is built in-tree by ``diffren_gb300.build``; ``load()`` builds it
on first use when nvcc is available and raises otherwise. There is no CPU or
PyTorch fallback: every op of this package runs through this library.
"""
import ctypes
import os
import threading

from . import build as _build

DR_OK = 0
DR_CULL_NONE, DR_CULL_BACK, DR_CULL_FRONT = 0, 1, 2
DR_DEPTH_DISCRETIZED, DR_DEPTH_FLOAT = 0, 1
DR_FLAG_INDEX_OUT_OF_RANGE = 1
DR_FLAG_NONFINITE_VERTEX = 2
DR_RASTER_FOREGROUND_ONLY = 1
DR_RASTER_FOREGROUND_ATTRIBUTES = 2
DR_SPLAT_FOREGROUND_GRADIENTS = 1
DR_SAMPLES_DETERMINISTIC = 1
DR_MAX_LAYERS = 16
DR_MAX_CHANNELS = 16
DR_MAX_SPLAT_CHANNELS = 8
DR_MAX_BATCH_INLINE = 128
DR_TEXTURE_PAD_ZERO = 1
DR_TEXTURE_TEXEL_UNITS = 2
DR_TEXTURE_DETERMINISTIC = 4
DR_MAX_IMAGE_DIM = 32768
DR_STATIC_SCRATCH_BYTES = 64 << 20
DR_SQUARED_ERROR_PARTIALS = 1216

# Every symbol the header declares, with (restype, argtypes).
_P = ctypes.c_void_p
_I = ctypes.c_int32
_S = ctypes.c_size_t
_L = ctypes.c_int64
_F = ctypes.c_float


class ImageDesc(ctypes.Structure):
  _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32),
              ("num_vertices", ctypes.c_int32), ("num_triangles", ctypes.c_int32),
              ("vertex_offset", ctypes.c_int64),
              ("triangle_offset", ctypes.c_int64),
              ("pixel_offset", ctypes.c_int64)]


class RasterConfig(ctypes.Structure):
  _fields_ = [("num_layers", ctypes.c_int32),
              ("face_culling_mode", ctypes.c_int32),
              ("depth_mode", ctypes.c_int32), ("tile_width", ctypes.c_int32),
              ("tile_height", ctypes.c_int32), ("large_tiles", ctypes.c_int32),
              ("flags", ctypes.c_uint32)]


class PointLight(ctypes.Structure):
  _fields_ = [("light", ctypes.c_float * 3), ("eye", ctypes.c_float * 3),
              ("ka", ctypes.c_float), ("kd", ctypes.c_float), ("ks", ctypes.c_float),
              ("ns", ctypes.c_float), ("attenuation_constant", ctypes.c_float),
              ("attenuation_linear", ctypes.c_float),
              ("attenuation_quadratic", ctypes.c_float)]


SIGNATURES = {
    "dr_last_error": (ctypes.c_char_p, []),
    "dr_abi_version": (_I, []),
    "dr_rasterize_batch_workspace_bytes": (_S, [_P, _I, _P]),
    "dr_rasterize_batch": (_I, [_P, _P, _P, _I, _P, _P, _P, _P, _P, _S, _P]),
    "dr_rasterize_batch_interpolate": (_I, [_P, _P, _P, _I, _P, _P, _P, _P, _P, _I, _P, _P,
                                           _P, _P, _S, _P]),
    "dr_rasterize_triangles_workspace_bytes": (_S, [_I, _I, _I, _I]),
    "dr_rasterize_triangles": (_I, [_P, _I, _P, _I, _I, _I, _I, _I, _I, _P, _P,
                                    _P, _P, _S, _P]),
    "dr_rasterize_triangles_static_scratch": (_I, [_P, _I, _P, _I, _I, _I, _I, _I,
                                                   _I, _P, _P, _P, _P]),
    "dr_read_error_flags": (_I, [_P, _P, _P]),
    "dr_read_static_scratch_error_flags": (_I, [_P, _P]),
    "dr_selftest_depth_codec": (_I, [_P, _P]),
    "dr_transform_vertices": (_I, [_P, _P, _I, _P, _I, _P, _P]),
    "dr_transform_vertices_bwd": (_I, [_P, _P, _I, _P, _I, _P, _P]),
    "dr_interpolate_fwd": (_I, [_P, _I, _P, _P, _P, _P, _P, _P, _I, _I, _P, _P]),
    "dr_interpolate_bwd": (_I, [_P, _P, _I, _P, _P, _P, _P, _P, _I, _I, _P, _P,
                                _P, _P]),
    "dr_diff_barycentrics_fwd": (_I, [_P, _P, _P, _P, _P, _I, _I, _P, _P]),
    "dr_diff_barycentrics_bwd": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _P, _P]),
    "dr_interpolate_with_positions_fwd": (_I, [_P, _I, _P, _P, _P, _P, _P, _P, _I, _I,
                                              _P, _P, _P]),
    "dr_interpolate_with_positions_bwd": (_I, [_P, _P, _P, _I, _P, _P, _P, _P, _P, _P, _P,
                                              _P, _I, _I, _P, _P, _P, _P]),
    "dr_interpolate_with_positions_bwd_ex": (_I, [_P, _P, _P, _I, _P, _P, _P, _P, _P, _P,
                                                 _P, _P, _I, _I, ctypes.c_uint32, _P, _P,
                                                 _P, _P, _S, _P]),
    "dr_interpolate_with_positions_bwd_scratch_bytes": (_S, [_P, _I, _I]),
    "dr_splat_positions_fwd": (_I, [_P, _P, _P, _P, _P, _P, _I, _I, _P, _P]),
    "dr_splat_positions_bwd": (_I, [_P, _P, _P, _P, _P, _P, _P, _I, _I, _P, _P, _P]),
    "dr_texture_map_fwd": (_I, [_P, _L, _P, _I, _I, _I, _I, _P, _P]),
    "dr_texture_map_bwd": (_I, [_P, _P, _L, _P, _I, _I, _I, _I, _P, _P, _P]),
    "dr_texture_map_bwd_ex": (_I, [_P, _P, _L, _P, _I, _I, _I, _I, _P, _P, _P, _S, _P]),
    "dr_texture_map_bwd_scratch_bytes": (_S, [_I, _I, _I]),
    "dr_point_light_fwd": (_I, [_P, _P, _P, _L, _I, _I, _I, _P, _P, _I, _P]),
    "dr_point_light_bwd": (_I, [_P, _I, _P, _P, _P, _L, _I, _I, _I, _P, _P, _P, _P, _I,
                                _P]),
    "dr_composite_over_fwd": (_I, [_P, _P, _I, _P, _I, _I, _P, _P]),
    "dr_composite_over_bwd": (_I, [_P, _P, _P, _I, _P, _I, _I, _P, _P]),
    "dr_squared_error": (_I, [_P, _P, _L, _F, _P, _P, _P, _P]),
    "dr_vertex_normals_fwd": (_I, [_P, _P, _P, _I, _P, _P, _P]),
    "dr_vertex_normals_bwd": (_I, [_P, _P, _P, _P, _I, _P, _P, _P, _P]),
    "dr_vertex_normals_csr_fwd": (_I, [_P, _P, _P, _I, _P, _P, _P, _P, _P, _P]),
    "dr_vertex_normals_csr_bwd": (_I, [_P, _P, _P, _P, _I, _P, _P, _P, _P, _P, _P, _P]),
    "dr_splat_fwd": (_I, [_P, _P, _P, _I, _P, _I, _I, _P, _P, _P, _P, _P]),
    "dr_splat_jvp": (_I, [_P, _P, _P, _P, _P, _I, _P, _I, _I, _P, _P]),
    "dr_splat_bwd": (_I, [_P, _P, _P, _P, _P, _I, _P, _I, _I, _P, _P, _P]),
    "dr_splat_bwd_ex": (_I, [_P, _P, _P, _P, _P, _I, _P, _I, _I, ctypes.c_uint32, _P, _P,
                             _P]),
}

_lib = None
_lock = threading.Lock()


class DiffrenError(RuntimeError):
  pass


def library_path():
  """The in-tree build, or DIFFREN_GB300_LIBRARY when set (a prebuilt
  library elsewhere; it is then never rebuilt)."""
  return os.environ.get("DIFFREN_GB300_LIBRARY") or _build.LIB


def load():
  """Returns the loaded library, building it first if needed."""
  global _lib
  if _lib is not None:
    return _lib
  with _lock:
    if _lib is None:
      path = library_path()
      if path == _build.LIB and not os.path.exists(path):
        try:
          _build.build()
        except Exception as e:  # no nvcc, compile error
          raise DiffrenError(
              "libdiffren_gb300.so is missing and could not be built: %s" % e)
      lib = ctypes.CDLL(path)
      for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
      _lib = lib
  return _lib


def check(rc, what):
  if rc != DR_OK:
    msg = load().dr_last_error().decode("utf-8", "replace")
    raise DiffrenError("%s failed (status %d): %s" % (what, rc, msg))
