"""Enums of the public API (diffren/jax/constants.py:20-30); the integer
values are the C ABI values (DR_CULL_*)."""
import enum


class FaceCullingMode(enum.IntEnum):
  NONE = 0
  BACK = 1
  FRONT = 2


class CompositingMode(enum.IntEnum):
  NONE = 0
  OVER = 1
  SPLAT_OVER = 2


class DepthSemantics(enum.IntEnum):
  """Which reference rasterizer the results reproduce bit for bit.

  CUDA: diffren's CUDA rasterizer (packed 32-bit discretized depth keys,
  background id 0). CPU: diffren's CPU rasterizer (exact float depth order,
  background id -1). The reference picks one by platform
  (rasterize_triangles_xla.py:77-78); the default here is CUDA.
  """
  CUDA = 0
  CPU = 1
