"""Autotuner host logic on CPU: cache keys, the JSON cache and candidate
selection with a fake timer (the GPU test times real launches)."""
import json

from diffren_gb300 import _lib, autotune, kernels


def batch_and_config():
  b = kernels.ImageBatch([256, 512], [256, 512], [100, 200], [1000, 3000])
  c = kernels.raster_config(3, 1, 0)
  return b, c


def test_signature_groups_similar_batches():
  b, c = batch_and_config()
  k1 = autotune.signature("GB300", b, c, 4)
  b2 = kernels.ImageBatch([256, 512], [256, 512], [100, 210], [1000, 3100])
  assert autotune.signature("GB300", b2, c, 4) == k1
  assert autotune.signature("GB300", b, c, 3) != k1
  assert autotune.signature("B200", b, c, 4) != k1
  c5 = kernels.raster_config(5, 1, 0)
  assert autotune.signature("GB300", b, c5, 4) != k1


def test_cache_round_trip(tmp_path):
  path = str(tmp_path / "tune.json")
  autotune.clear_memory()
  assert autotune.lookup("k", path) is None
  autotune.store("k", (32, 16, 8), path)
  autotune.clear_memory()
  assert autotune.lookup("k", path) == (32, 16, 8)
  with open(path) as f:
    assert json.load(f) == {"k": [32, 16, 8]}
  autotune.store("k2", (16, 16, 16), path)
  with open(path) as f:
    assert set(json.load(f)) == {"k", "k2"}
  autotune.clear_memory()


def test_corrupt_cache_is_ignored(tmp_path):
  path = tmp_path / "tune.json"
  path.write_text("not json")
  autotune.clear_memory()
  assert autotune.lookup("k", str(path)) is None
  autotune.store("k", (8, 8, 16), str(path))
  assert json.loads(path.read_text()) == {"k": [8, 8, 16]}
  autotune.clear_memory()


def test_time_candidates_picks_fastest_and_skips_rejected():
  cost = {(16, 16, 16): 3.0, (32, 16, 16): 1.5, (8, 8, 16): 2.0, (32, 32, 16): None}
  current = {}

  def run(cand):
    if cost[cand] is None:
      raise _lib.DiffrenError("rejected")
    current["c"] = cand

  def timer(fn):
    fn()
    return cost[current["c"]]

  times = autotune.time_candidates(run, list(cost), repeats=2, timer=timer)
  assert set(times) == {(16, 16, 16), (32, 16, 16), (8, 8, 16)}
  assert min(times, key=times.get) == (32, 16, 16)


def test_candidates_fit_the_rasterizer_limits():
  for w, h, large in autotune.CANDIDATES:
    assert 0 < w <= 128 and 0 < h <= 128 and w * h <= 1024 and large > 0
