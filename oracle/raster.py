"""Test infrastructure only: ctypes access to the rasterizer checkers.

``rasterize`` runs this repo's C restatement (``raster_oracle.c``);
``rasterize_reference_cpu`` runs the reference's own CPU rasterizer
(``diffren/common/kernels/rasterize_triangles_impl.cc:27-118``) and
``rasterize_reference_cuda`` the reference's own CUDA rasterizer
(``diffren/common/kernels/rasterize_triangles_impl_cuda.cu.cc:397-484``),
both compiled by ``oracle/Makefile`` into ``oracle/_ref`` from the reference
tree (``DIFFREN_REFERENCE`` or an explicit root) or from the git-ignored
staged copy of its sources in ``oracle/_ref/src``.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_ORACLE_SO = os.path.join(_HERE, "_build", "libraster_oracle.so")
_REF_SO = os.path.join(_HERE, "_ref", "libref_raster.so")
_REF_CUDA_SO = os.path.join(_HERE, "_ref", "libref_raster_cuda.so")
_STAGED = os.path.join(_HERE, "_ref", "src")
_KERNELS = os.path.join("diffren", "common", "kernels")

DEPTH_DISCRETIZED = 0  # reference CUDA rasterizer semantics
DEPTH_FLOAT = 1  # reference CPU rasterizer semantics
# What the GPU's toward-zero conversions give a NaN input (the rules
# raster_oracle.c implements; checked by the GPU depth-codec self-test).
NAN_TO_U32_FROM_DOUBLE = 0x80000000
NAN_TO_I32 = 0
NAN_TO_I64 = -0x8000000000000000

_lib = None
_ref = None
_ref_cuda = None


def build(force=False):
  """Compiles raster_oracle.c (needs only gcc); returns the .so path."""
  if force or not os.path.exists(_ORACLE_SO) or (
      os.path.getmtime(_ORACLE_SO) <
      os.path.getmtime(os.path.join(_HERE, "raster_oracle.c"))):
    subprocess.run(["make", "-s", "-C", _HERE, "oracle"], check=True)
  return _ORACLE_SO


def reference_root(root=None):
  """The reference tree to build from: `root`, else $DIFFREN_REFERENCE, else
  None (the staged copy is used when present)."""
  return root or os.environ.get("DIFFREN_REFERENCE") or None


def stage_reference(root=None):
  """Copies the reference rasterizer sources into oracle/_ref/src
  (git-ignored), so the reference builds where its tree is absent. Returns
  False when no reference tree is given."""
  root = reference_root(root)
  if root is None or not os.path.exists(os.path.join(root, _KERNELS)):
    return False
  subprocess.run(["make", "-s", "-C", _HERE, "stage", "REFERENCE=" + root], check=True)
  return True


def _reference_make(target, source, root):
  root = reference_root(root)
  if root is not None and os.path.exists(os.path.join(root, _KERNELS, source)):
    args = ["REFERENCE=" + root]
  elif os.path.exists(os.path.join(_STAGED, _KERNELS, source)):
    args = ["REFERENCE="]
  else:
    return False
  subprocess.run(["make", "-s", "-C", _HERE, target] + args, check=True)
  return True


def build_reference(root=None):
  """Compiles the reference CPU rasterizer; None if its sources are absent."""
  if not _reference_make("ref", "rasterize_triangles_impl.cc", root):
    return None
  return _REF_SO


def build_reference_cuda(root=None):
  """Compiles the reference CUDA rasterizer for sm_103a with nvcc's default
  flags; None if its sources are absent."""
  if not _reference_make("ref_cuda", "rasterize_triangles_impl_cuda.cu.cc", root):
    return None
  return _REF_CUDA_SO


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


def reference_cuda_available():
  return os.path.exists(_REF_CUDA_SO)


def _load_ref():
  global _ref
  if _ref is None:
    if not os.path.exists(_REF_SO):
      raise RuntimeError("reference CPU rasterizer not built (needs the "
                         "reference tree; see oracle/Makefile)")
    _ref = ctypes.CDLL(_REF_SO)
    _ref.ref_rasterize_cpu.restype = ctypes.c_int
  return _ref


def _load_ref_cuda():
  global _ref_cuda
  if _ref_cuda is None:
    if not os.path.exists(_REF_CUDA_SO):
      raise RuntimeError("reference CUDA rasterizer not built (see oracle/Makefile)")
    _ref_cuda = ctypes.CDLL(_REF_CUDA_SO)
    _ref_cuda.ref_rasterize_cuda.restype = ctypes.c_int
    _ref_cuda.ref_rasterize_cuda.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [
        ctypes.c_int32] * 5 + [ctypes.c_void_p] * 4 + [ctypes.c_char_p, ctypes.c_int32]
  return _ref_cuda


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


def rasterize_reference_cuda(vertices, triangles, triangle_count, width, height,
                             num_layers, culling, triangle_ids, z_buffer, barycentrics,
                             stream=0):
  """The reference's own CUDA rasterizer on device buffers given as integer
  addresses (vertices [V,4] f32, triangles [T,3] i32, outputs [L,H,W] i32,
  [L,H,W] f32, [L,H,W,3] f32), launched on `stream`. Raises on a failed
  launch. Background samples get id 0 and z 1."""
  msg = ctypes.create_string_buffer(512)
  rc = _load_ref_cuda().ref_rasterize_cuda(vertices, triangles, triangle_count, width,
                                           height, num_layers, int(culling), triangle_ids,
                                           z_buffer, barycentrics, stream, msg, 512)
  if rc != 0:
    raise RuntimeError("reference CUDA rasterizer: " + msg.value.decode())


def transform(matrix, vertices):
  """Clip-space transform with a fixed left-to-right float32 order."""
  m = np.ascontiguousarray(matrix, dtype=np.float32).reshape(4, 4)
  v = np.ascontiguousarray(vertices, dtype=np.float32)
  out = np.empty((v.shape[0], 4), np.float32)
  _load().oracle_transform(_ptr(m), _ptr(v), ctypes.c_int64(v.shape[0]),
                           ctypes.c_int32(v.shape[1]), _ptr(out))
  return out
