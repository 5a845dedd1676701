"""Test infrastructure only: ctypes access to the CPU rasterizer checkers.

``rasterize`` runs this repo's C restatement (``raster_oracle.c``);
``rasterize_reference_cpu`` runs the reference's own CPU rasterizer
(``diffren/common/kernels/rasterize_triangles_impl.cc:27-118``) compiled in
place into ``oracle/_ref`` where the reference tree exists.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ORACLE_SO = os.path.join(_HERE, "_build", "libraster_oracle.so")
_REF_SO = os.path.join(_HERE, "_ref", "libref_raster.so")

DEPTH_DISCRETIZED = 0  # reference CUDA rasterizer semantics
DEPTH_FLOAT = 1  # reference CPU rasterizer semantics
# What the GPU's toward-zero conversions give a NaN input (the rules
# raster_oracle.c implements; checked by the GPU depth-codec self-test).
NAN_TO_U32_FROM_DOUBLE = 0x80000000
NAN_TO_I32 = 0
NAN_TO_I64 = -0x8000000000000000

_lib = None
_ref = None


def build(force=False):
  """Compiles raster_oracle.c (needs only gcc); returns the .so path."""
  if force or not os.path.exists(_ORACLE_SO) or (
      os.path.getmtime(_ORACLE_SO) <
      os.path.getmtime(os.path.join(_HERE, "raster_oracle.c"))):
    subprocess.run(["make", "-s", "-C", _HERE, "oracle"], check=True)
  return _ORACLE_SO


def build_reference(reference_root="/root/reference"):
  """Compiles the reference CPU rasterizer in place; None if unavailable."""
  src = os.path.join(reference_root, "diffren", "common", "kernels",
                     "rasterize_triangles_impl.cc")
  if not os.path.exists(src):
    return None
  subprocess.run(["make", "-s", "-C", _HERE, "ref",
                  "REFERENCE=" + reference_root], check=True)
  return _REF_SO


def _load():
  global _lib
  if _lib is None:
    build()
    _lib = ctypes.CDLL(_ORACLE_SO)
    _lib.oracle_rasterize.restype = ctypes.c_int
    _lib.oracle_transform.restype = None
  return _lib


def reference_available():
  return os.path.exists(_REF_SO)


def _load_ref():
  global _ref
  if _ref is None:
    if not os.path.exists(_REF_SO):
      raise RuntimeError("reference CPU rasterizer not built (needs the "
                         "reference tree; see oracle/Makefile)")
    _ref = ctypes.CDLL(_REF_SO)
    _ref.ref_rasterize_cpu.restype = ctypes.c_int
  return _ref


def _ptr(a):
  return a.ctypes.data_as(ctypes.c_void_p)


def _prep(vertices, triangles):
  v = np.ascontiguousarray(vertices, dtype=np.float32)
  t = np.ascontiguousarray(triangles, dtype=np.int32)
  assert v.ndim == 2 and v.shape[1] == 4, v.shape
  assert t.ndim == 2 and t.shape[1] == 3, t.shape
  return v, t


def rasterize(vertices, triangles, width, height, num_layers, culling,
              depth_mode=DEPTH_DISCRETIZED):
  """C restatement. Returns (ids [L,H,W] i32, z [L,H,W] f32, bary [L,H,W,3])."""
  v, t = _prep(vertices, triangles)
  ids = np.empty((num_layers, height, width), np.int32)
  z = np.empty((num_layers, height, width), np.float32)
  b = np.empty((num_layers, height, width, 3), np.float32)
  rc = _load().oracle_rasterize(_ptr(v), _ptr(t), ctypes.c_int32(t.shape[0]),
                                ctypes.c_int32(width), ctypes.c_int32(height),
                                ctypes.c_int32(num_layers),
                                ctypes.c_int32(int(culling)),
                                ctypes.c_int32(depth_mode), _ptr(ids), _ptr(z),
                                _ptr(b))
  if rc != 0:
    raise ValueError("oracle_rasterize failed")
  return ids, z, b


def rasterize_reference_cpu(vertices, triangles, width, height, num_layers,
                            culling):
  """The reference's own compiled CPU rasterizer (ids -1 on background)."""
  v, t = _prep(vertices, triangles)
  ids = np.empty((num_layers, height, width), np.int32)
  z = np.empty((num_layers, height, width), np.float32)
  b = np.empty((num_layers, height, width, 3), np.float32)
  _load_ref().ref_rasterize_cpu(_ptr(v), _ptr(t), ctypes.c_int32(t.shape[0]),
                                ctypes.c_int32(width), ctypes.c_int32(height),
                                ctypes.c_int32(num_layers),
                                ctypes.c_int32(int(culling)), _ptr(ids), _ptr(z),
                                _ptr(b))
  return ids, z, b


def transform(matrix, vertices):
  """Clip-space transform with a fixed left-to-right float32 order."""
  m = np.ascontiguousarray(matrix, dtype=np.float32).reshape(4, 4)
  v = np.ascontiguousarray(vertices, dtype=np.float32)
  out = np.empty((v.shape[0], 4), np.float32)
  _load().oracle_transform(_ptr(m), _ptr(v), ctypes.c_int64(v.shape[0]),
                           ctypes.c_int32(v.shape[1]), _ptr(out))
  return out
