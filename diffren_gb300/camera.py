"""Camera matrices, numerically following diffren/jax/camera.py.

``perspective`` follows camera.py:23-44 (gluPerspective through
perspective_from_intrinsics and ortho, camera.py:47-125) and ``look_at``
follows camera.py:126-184 (gluLookAt). Everything is float64 numpy; callers
cast to float32 when building clip-space vertices. These are host-side
helpers for building inputs; they are not on the device path.
"""
import math

import numpy as np


def ortho(left, right, bottom, top, near, far):
  depth_range = far - near
  return np.array([
      [2.0 / (right - left), 0.0, 0.0, -(right + left) / (right - left)],
      [0.0, 2.0 / (top - bottom), 0.0, -(top + bottom) / (top - bottom)],
      [0.0, 0.0, -2.0 / depth_range, -(far + near) / depth_range],
      [0.0, 0.0, 0.0, 1.0],
  ])


def perspective_from_intrinsics(focal_x, focal_y, center_offset_x,
                                center_offset_y, near_clip, far_clip,
                                image_width, image_height):
  a = near_clip + far_clip
  b = near_clip * far_clip
  persp = np.array([
      [focal_x, 0.0, -center_offset_x, 0.0],
      [0.0, focal_y, -center_offset_y, 0.0],
      [0.0, 0.0, a, b],
      [0.0, 0.0, -1.0, 0.0],
  ])
  ndc = ortho(image_width * -0.5, image_width * 0.5, image_height * -0.5,
              image_height * 0.5, near_clip, far_clip)
  return ndc @ persp


def perspective(aspect_ratio, fov_y, near_clip, far_clip):
  focal_y = 1.0 / math.tan(fov_y * (math.pi / 360.0))
  return perspective_from_intrinsics(focal_y / aspect_ratio, focal_y, 0.0, 0.0,
                                     near_clip, far_clip, 2, 2)


def look_at(eye, center, world_up):
  eye = np.asarray(eye, np.float64)
  center = np.asarray(center, np.float64)
  world_up = np.asarray(world_up, np.float64)
  forward = center - eye
  n = np.linalg.norm(forward)
  if n < 1e-6:
    raise ValueError(
        "Camera matrix is degenerate because eye and center are close.")
  forward = forward / n
  to_side = np.cross(forward, world_up)
  n = np.linalg.norm(to_side)
  if n < 1e-6:
    raise ValueError("Camera matrix is degenerate because up and gaze are "
                     "close or up is degenerate.")
  to_side = to_side / n
  cam_up = np.cross(to_side, forward)
  rot = np.eye(4)
  rot[:3, :3] = np.stack([to_side, cam_up, -forward])
  trans = np.eye(4)
  trans[:3, 3] = -eye
  return rot @ trans
