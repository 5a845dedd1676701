"""Tile and bin size autotuner for the rasterizer.

The fine rasterizer's tile (the block's shared-memory z-buffer) and the
large-triangle threshold (how many tiles a triangle may span before it goes
to its image's shared list instead of per-tile bins) trade binning work,
shared memory per block (and so occupancy) and load balance against each
other; the best choice depends on the batch's resolutions and triangle
sizes. Every choice gives the same bits (ids, depth and barycentrics are
per-pixel exact), so tuning only changes speed.

``tune`` times each candidate on the caller's actual inputs with CUDA events
and keeps the fastest; results are cached in memory and in a JSON file keyed
by the device, the layer count, the culling and depth modes, the attribute
width and the batch's size class (image count, log2 of pixels and of
triangles), so a later process with a similar batch skips the search.
"""
import json
import math
import os
import threading

import torch

from . import _lib
from . import kernels

# (tile_width, tile_height, large_tiles); tile_width * tile_height <= 1024.
CANDIDATES = [
    (16, 16, 16), (16, 16, 8), (16, 16, 32),
    (32, 16, 16), (16, 8, 16), (32, 32, 16), (8, 8, 16), (32, 8, 16),
]

_lock = threading.Lock()
_memory = {}


def cache_path():
  """JSON file of tuned configurations (DIFFREN_GB300_TUNE_CACHE overrides)."""
  p = os.environ.get("DIFFREN_GB300_TUNE_CACHE")
  if p:
    return p
  root = os.environ.get("XDG_CACHE_HOME", os.path.join(os.path.expanduser("~"), ".cache"))
  return os.path.join(root, "diffren_gb300", "autotune.json")


def signature(device_name, batch, config, channels):
  """Cache key: device, layers, culling, depth mode, attribute width and the
  batch's size class."""
  px = max(1, batch.total_pixels)
  tris = max(1, batch.total_triangles)
  return "%s|L%d|c%d|d%d|k%d|n%d|p%d|t%d" % (
      device_name, config.num_layers, config.face_culling_mode, config.depth_mode,
      int(channels), batch.n, round(math.log2(px)), round(math.log2(tris)))


def _load(path):
  try:
    with open(path) as f:
      data = json.load(f)
    return data if isinstance(data, dict) else {}
  except (OSError, ValueError):
    return {}


def lookup(key, path=None):
  with _lock:
    if key in _memory:
      return tuple(_memory[key])
    entry = _load(path or cache_path()).get(key)
    if entry is not None and len(entry) == 3:
      _memory[key] = tuple(int(v) for v in entry)
      return _memory[key]
  return None


def store(key, choice, path=None):
  path = path or cache_path()
  with _lock:
    _memory[key] = tuple(int(v) for v in choice)
    data = _load(path)
    data[key] = list(_memory[key])
    try:
      os.makedirs(os.path.dirname(path), exist_ok=True)
      tmp = path + ".%d.tmp" % os.getpid()
      with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
      os.replace(tmp, path)
    except OSError:
      pass  # an unwritable cache only costs a re-tune


def clear_memory():
  with _lock:
    _memory.clear()


def time_candidates(run, candidates, repeats=3, timer=None):
  """{candidate: best time} of ``run(candidate)``; ``timer(fn)`` returns
  one call's duration (CUDA events by default). Candidates that the
  rasterizer rejects are skipped."""
  timer = timer or _cuda_time
  times = {}
  for cand in candidates:
    try:
      run(cand)  # warm-up (and the kernels' one-time attribute setup)
      times[cand] = min(timer(lambda: run(cand)) for _ in range(repeats))
    except _lib.DiffrenError:
      continue
  return times


def _cuda_time(fn):
  s = torch.cuda.current_stream()
  e0 = torch.cuda.Event(enable_timing=True)
  e1 = torch.cuda.Event(enable_timing=True)
  e0.record(s)
  fn()
  e1.record(s)
  e1.synchronize()
  return e0.elapsed_time(e1)


def tune(clip, triangles, batch, config, attributes=None, workspace=None,
         candidates=None, repeats=3, path=None, timer=None, use_cache=True):
  """Fastest (tile_width, tile_height, large_tiles) for rasterizing this
  batch (with the fused interpolation when ``attributes`` is given)."""
  channels = 0 if attributes is None else attributes.shape[1]
  dev = clip.device
  key = signature(torch.cuda.get_device_name(dev) if dev.type == "cuda" else dev.type,
                  batch, config, channels)
  if use_cache:
    hit = lookup(key, path)
    if hit is not None:
      return hit
  ws = workspace or kernels.Workspace(dev)

  def run(cand):
    cfg = kernels.raster_config(config.num_layers, config.face_culling_mode,
                                config.depth_mode, cand[:2], cand[2])
    with torch.no_grad():
      if attributes is None:
        kernels.rasterize_packed(clip, triangles, batch, cfg, workspace=ws)
      else:
        kernels.rasterize_interpolate_packed(attributes, clip, triangles, batch, cfg, ws)

  times = time_candidates(run, candidates or CANDIDATES, repeats, timer)
  if not times:
    raise _lib.DiffrenError("no tile configuration could be launched")
  best = min(times, key=times.get)
  store(key, best, path)
  return best
