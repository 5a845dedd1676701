"""Ragged batches through BatchRenderer (the benchmarked path): every image
equals its own render_triangles call, the rasterizer's fused interpolation
equals the separate kernels bit for bit, and a CUDA-graph replay of a
forward+backward step equals the eager step."""
import ctypes

import numpy as np
import pytest
import torch

from diffren_gb300 import _lib
from diffren_gb300 import batch as batch_lib
from diffren_gb300 import constants, kernels, render, workloads

pytestmark = pytest.mark.gpu


def rgba_shader(a):
  return a["rgba"]


def rgba(colors):
  return torch.cat([colors, torch.ones_like(colors[:, :1])], 1)


def ragged_scene(seed=0):
  meshes = [workloads.icosphere_workload(5, seed=seed),
            workloads.soup_workload(700, seed=seed + 1, mu=-2.2, sigma=0.5),
            workloads.icosphere_workload(3, seed=seed + 2),
            workloads.soup_workload(300, seed=seed + 3, mu=-2.0, sigma=0.5)]
  sizes = [(48, 40), (64, 64), (33, 57), (70, 18)]
  eyes = workloads.sphere_eyes(len(meshes), seed=seed + 5, radius=2.6)
  cams = [workloads.camera_matrix(e, w, h) for e, (w, h) in zip(eyes, sizes)]
  return meshes, cams, sizes


def test_batch_renderer_matches_per_image(device):
  meshes, cams, sizes = ragged_scene()
  r = batch_lib.BatchRenderer([m.triangles for m in meshes], [len(m.vertices) for m in meshes],
                              sizes, num_layers=3, device=device)
  v = torch.tensor(np.concatenate([m.vertices for m in meshes]), device=device,
                   requires_grad=True)
  c = torch.tensor(np.concatenate([m.colors for m in meshes]), device=device,
                   requires_grad=True)
  cam = torch.tensor(np.stack(cams), device=device)
  out = r.render(v, {"rgba": rgba(c)}, cam, rgba_shader)
  rng = np.random.default_rng(0)
  g = torch.tensor(rng.standard_normal(tuple(out.shape)).astype(np.float32), device=device)
  gv, gc = torch.autograd.grad(out, (v, c), g)
  imgs = r.images(out)
  gimgs = r.images(g)
  voff = np.cumsum([0] + [len(m.vertices) for m in meshes])
  for i, (m, cm, (w, h)) in enumerate(zip(meshes, cams, sizes)):
    vi = torch.tensor(m.vertices, device=device, requires_grad=True)
    ci = torch.tensor(m.colors, device=device, requires_grad=True)
    oi = render.render_triangles(vi, {"rgba": rgba(ci)}, torch.tensor(m.triangles, device=device),
                                 torch.tensor(cm, device=device), w, h, rgba_shader,
                                 num_layers=3)
    torch.testing.assert_close(imgs[i], oi, rtol=0, atol=0)
    gvi, gci = torch.autograd.grad(oi, (vi, ci), gimgs[i])
    sl = slice(int(voff[i]), int(voff[i + 1]))
    torch.testing.assert_close(gv[sl], gvi, rtol=1e-4, atol=1e-4 * float(gvi.abs().max()))
    torch.testing.assert_close(gc[sl], gci, rtol=1e-4, atol=1e-4 * float(gci.abs().max()))


@pytest.mark.parametrize("K", [4, 3, 6])
@pytest.mark.parametrize("depth_mode", [constants.DepthSemantics.CUDA,
                                        constants.DepthSemantics.CPU])
def test_fused_raster_interpolation_matches_separate_kernels(K, depth_mode, device):
  meshes, cams, sizes = ragged_scene(seed=3)
  r = batch_lib.BatchRenderer([m.triangles for m in meshes], [len(m.vertices) for m in meshes],
                              sizes, num_layers=3, device=device, depth_semantics=depth_mode)
  v = torch.tensor(np.concatenate([m.vertices for m in meshes]), device=device)
  clip = kernels.transform(v, torch.tensor(np.stack(cams), device=device), r.batch)
  rng = np.random.default_rng(K)
  attr = torch.tensor(rng.uniform(-1, 1, (len(v), K)).astype(np.float32), device=device)
  out, vp, ids, z, bary = kernels.rasterize_interpolate_packed(attr, clip, r.triangles, r.batch,
                                                               r.config, r.workspace)
  ids2, z2, bary2 = kernels.rasterize_packed(clip, r.triangles, r.batch, r.config)
  out2, vp2 = kernels.interpolate_with_positions_packed(attr, clip, bary2, r.triangles, ids2,
                                                        z2, r.batch, 3)
  for a, b in [(ids, ids2), (z, z2), (bary, bary2), (out, out2)]:
    assert torch.equal(a, b)
  # The fused pass writes positions of foreground samples only, with the
  # interpolated clip w in place of the foreground flag.
  fg = z != 1.0
  assert torch.equal(vp[fg][:, :3], vp2[fg][:, :3])
  assert (vp2[~fg][:, 3] == 0).all() and (vp2[fg][:, 3] == 1).all()
  img = torch.as_tensor(np.repeat(np.arange(r.batch.n), 3 * np.array(
      [w * h for w, h in sizes])), device=device)
  toff = torch.as_tensor(r.batch.triangle_offsets[:-1], device=device)
  voff = torch.as_tensor(r.batch.vertex_offsets[:-1], device=device)
  tri = r.triangles.long()[toff[img] + ids.long()]  # local vertex indices
  vfg = voff[img][fg]
  w_ref = (clip[vfg[:, None] + tri[fg]][..., 3] * bary[fg]).sum(-1)
  torch.testing.assert_close(vp[fg][:, 3], w_ref, rtol=1e-6, atol=1e-6)
  # The vertex indices it stores for the VJP are the triangles' rows.
  vids = torch.full((ids.shape[0], 3), -7, dtype=torch.int32, device=device)
  bufs = [torch.empty_like(t) for t in (ids, z, bary, out, vp)]
  ws = kernels.Workspace(device).get(kernels.raster_workspace_bytes(r.batch, r.config))
  p = kernels._p
  rc = _lib.load().dr_rasterize_batch_interpolate(
      p(clip), p(r.triangles), r.batch.ptr, r.batch.n, ctypes.byref(r.config), p(bufs[0]),
      p(bufs[1]), p(bufs[2]), p(attr), K, p(bufs[3]), p(bufs[4]), p(vids), p(ws), ws.numel(),
      ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
  assert rc == 0
  torch.cuda.synchronize()
  assert torch.equal(vids[fg].long(), tri[fg])
  assert (vids[~fg] == -7).all()


def test_graph_replay_matches_eager(device):
  meshes, cams, sizes = ragged_scene(seed=7)
  r = batch_lib.BatchRenderer([m.triangles for m in meshes], [len(m.vertices) for m in meshes],
                              sizes, num_layers=3, device=device)
  verts = torch.tensor(np.concatenate([m.vertices for m in meshes]), device=device)
  cols = torch.tensor(np.concatenate([m.colors for m in meshes]), device=device)
  cams_t = torch.tensor(np.stack(cams), device=device)
  target = torch.rand(r.total_pixels, 4, device=device)
  g_v = torch.empty_like(verts)
  loss_out = torch.empty((), device=device)

  def step():
    v = verts.detach().requires_grad_(True)
    out = r.render(v, {"rgba": rgba(cols)}, cams_t, rgba_shader)
    loss = (out - target).square().sum()
    (gv,) = torch.autograd.grad(loss, (v,))
    g_v.copy_(gv)
    loss_out.copy_(loss.detach())

  s = torch.cuda.Stream(device)
  s.wait_stream(torch.cuda.current_stream(device))
  with torch.cuda.stream(s):
    for _ in range(3):
      step()
  torch.cuda.current_stream(device).wait_stream(s)
  torch.cuda.synchronize(device)
  eager_loss, eager_g = loss_out.clone(), g_v.clone()
  graph = torch.cuda.CUDAGraph()
  with torch.cuda.graph(graph):
    step()
  graph.replay()
  torch.cuda.synchronize(device)
  torch.testing.assert_close(loss_out, eager_loss, rtol=1e-6, atol=0)
  torch.testing.assert_close(g_v, eager_g, rtol=1e-4, atol=1e-4 * float(eager_g.abs().max()))


def test_every_tile_configuration_gives_the_same_bits(device):
  """Tile and bin sizes only change speed: every autotuner candidate
  rasterizes (and interpolates) the ragged batch to the same bits."""
  from diffren_gb300 import autotune
  meshes, cams, sizes = ragged_scene(seed=11)
  r = batch_lib.BatchRenderer([m.triangles for m in meshes], [len(m.vertices) for m in meshes],
                              sizes, num_layers=4, device=device)
  v = torch.tensor(np.concatenate([m.vertices for m in meshes]), device=device)
  clip = kernels.transform(v, torch.tensor(np.stack(cams), device=device), r.batch)
  attr = torch.tensor(np.concatenate([m.colors for m in meshes]), device=device)
  ref = None
  for w, h, large in autotune.CANDIDATES:
    cfg = kernels.raster_config(4, constants.FaceCullingMode.BACK, 0, (w, h), large)
    res = kernels.rasterize_interpolate_packed(attr, clip, r.triangles, r.batch, cfg,
                                               kernels.Workspace(device))
    out, vp, ids, z, bary = res
    fg = z != 1.0
    res = (out, vp[fg], ids, z, bary)  # positions are written for foreground only
    if ref is None:
      ref = res
    else:
      for a, b in zip(res, ref):
        assert torch.equal(a, b), (w, h, large)


def test_autotuned_renderer_matches_default(device, tmp_path, monkeypatch):
  from diffren_gb300 import autotune
  monkeypatch.setenv("DIFFREN_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
  autotune.clear_memory()
  meshes, cams, sizes = ragged_scene(seed=13)
  args = ([m.triangles for m in meshes], [len(m.vertices) for m in meshes], sizes)
  v = torch.tensor(np.concatenate([m.vertices for m in meshes]), device=device)
  c = torch.tensor(np.concatenate([m.colors for m in meshes]), device=device)
  cam = torch.tensor(np.stack(cams), device=device)
  r0 = batch_lib.BatchRenderer(*args, num_layers=3, device=device)
  r1 = batch_lib.BatchRenderer(*args, num_layers=3, device=device, tile="auto")
  out0 = r0.render(v, {"rgba": rgba(c)}, cam, rgba_shader)
  out1 = r1.render(v, {"rgba": rgba(c)}, cam, rgba_shader)
  assert torch.equal(out0, out1)
  chosen = (r1.config.tile_width, r1.config.tile_height, r1.config.large_tiles)
  assert chosen in autotune.CANDIDATES
  # A second renderer for the same batch class reuses the cached choice.
  autotune.clear_memory()
  r2 = batch_lib.BatchRenderer(*args, num_layers=3, device=device, tile="auto")
  r2.render(v, {"rgba": rgba(c)}, cam, rgba_shader)
  assert (r2.config.tile_width, r2.config.tile_height, r2.config.large_tiles) == chosen
  autotune.clear_memory()


@pytest.mark.parametrize("mode", [constants.CompositingMode.OVER, constants.CompositingMode.NONE])
def test_batch_renderer_over_and_none_match_per_image(mode, device):
  """BatchRenderer's OVER (the OVER kernel over the ragged batch) and NONE
  modes equal each image's own render_triangles call, forward and backward."""
  meshes, cams, sizes = ragged_scene(seed=4)
  r = batch_lib.BatchRenderer([m.triangles for m in meshes], [len(m.vertices) for m in meshes],
                              sizes, num_layers=3, device=device,
                              face_culling_mode=constants.FaceCullingMode.NONE)
  c = torch.tensor(np.concatenate([m.colors for m in meshes]), device=device,
                   requires_grad=True)
  v = torch.tensor(np.concatenate([m.vertices for m in meshes]), device=device)
  cam = torch.tensor(np.stack(cams), device=device)

  def shade(a):  # semi-transparent, so that OVER mixes the layers
    return a["rgba"] * 0.6

  out = r.render(v, {"rgba": rgba(c)}, cam, shade, compositing_mode=mode)
  g = torch.tensor(np.random.default_rng(1).standard_normal(tuple(out.shape)).astype(np.float32),
                   device=device)
  (gc,) = torch.autograd.grad(out, c, g)
  coff = np.cumsum([0] + [len(m.vertices) for m in meshes])
  poff = np.cumsum([0] + [w * h * (3 if mode == constants.CompositingMode.NONE else 1)
                          for w, h in sizes])
  for i, (m, cm, (w, h)) in enumerate(zip(meshes, cams, sizes)):
    ci = torch.tensor(m.colors, device=device, requires_grad=True)
    oi = render.render_triangles(torch.tensor(m.vertices, device=device), {"rgba": rgba(ci)},
                                 torch.tensor(m.triangles, device=device),
                                 torch.tensor(cm, device=device), w, h, shade, num_layers=3,
                                 face_culling_mode=constants.FaceCullingMode.NONE,
                                 compositing_mode=mode)
    mine = out[int(poff[i]):int(poff[i + 1])].reshape(oi.shape)
    assert torch.equal(mine, oi)
    (gci,) = torch.autograd.grad(oi, ci, g[int(poff[i]):int(poff[i + 1])].reshape(oi.shape))
    sl = slice(int(coff[i]), int(coff[i + 1]))
    scale = float(gci.abs().max()) or 1.0
    torch.testing.assert_close(gc[sl], gci, rtol=1e-4, atol=1e-5 * scale)


@pytest.mark.parametrize("use_batch", [True, False])
def test_recompute_raster_gives_the_same_gradients(use_batch, device):
  """recompute_raster reruns the rasterizer in the backward instead of
  keeping its per-sample ids, barycentrics and vertex ids: same image and
  same gradients (the vertex-gradient atomics may reorder float sums, so
  within 1e-6 of the largest magnitude), and fewer bytes kept for the VJP."""
  meshes, cams, sizes = workloads.ragged_batch(5, seed=7, median_triangles=3000,
                                               resolutions=(64, 96, 128))

  def run(recompute):
    torch.cuda.synchronize(device)
    base = torch.cuda.memory_allocated(device)
    if use_batch:
      r = batch_lib.BatchRenderer([m.triangles for m in meshes],
                                  [len(m.vertices) for m in meshes], sizes, num_layers=3,
                                  device=device, recompute_raster=recompute)
      v = torch.tensor(np.concatenate([m.vertices for m in meshes]), device=device,
                       requires_grad=True)
      c = torch.tensor(np.concatenate([m.colors for m in meshes]), device=device,
                       requires_grad=True)
      out = r.render(v, {"rgb": c}, torch.tensor(np.stack(cams), device=device),
                     lambda a: torch.cat([a["rgb"], torch.ones_like(a["rgb"][..., :1])], -1))
    else:
      m, cam, (w, h) = meshes[0], cams[0], sizes[0]
      v = torch.tensor(m.vertices, device=device, requires_grad=True)
      c = torch.tensor(m.colors, device=device, requires_grad=True)
      out = render.render_triangles(
          v, {"rgb": c}, torch.tensor(m.triangles, device=device), torch.tensor(cam, device=device),
          w, h, lambda a: torch.cat([a["rgb"], torch.ones_like(a["rgb"][..., :1])], -1),
          num_layers=3, recompute_raster=recompute)
    kept = torch.cuda.memory_allocated(device) - base
    gv, gc = torch.autograd.grad(out.square().sum(), (v, c))
    return out.detach(), gv, gc, kept

  o0, gv0, gc0, kept0 = run(False)
  o1, gv1, gc1, kept1 = run(True)
  assert torch.equal(o0, o1)
  for a, b in ((gv0, gv1), (gc0, gc1)):
    assert float((a - b).abs().max()) <= 1e-6 * float(b.abs().max())
  assert kept1 < kept0


def test_foreground_only_flag_writes_the_same_foreground(device):
  """DR_RASTER_FOREGROUND_ONLY leaves background ids and barycentrics
  unwritten; depth, foreground ids / barycentrics, attributes (background
  0) and foreground positions are the same bits as without it."""
  meshes, cams, sizes = workloads.ragged_batch(6, seed=11, median_triangles=4000,
                                               resolutions=(64, 128, 160))
  from oracle import raster
  clips = [raster.transform(c, m.vertices) for m, c in zip(meshes, cams)]
  batch = kernels.ImageBatch([s[0] for s in sizes], [s[1] for s in sizes],
                             [len(c) for c in clips], [len(m.triangles) for m in meshes])
  v = torch.as_tensor(np.concatenate(clips), device=device)
  t = torch.as_tensor(np.concatenate([m.triangles for m in meshes]), device=device)
  attrs = torch.rand(v.shape[0], 4, device=device)
  outs = []
  for cfg in (kernels.raster_config(3, 1, 0),
              kernels.foreground_only(kernels.raster_config(3, 1, 0))):
    with torch.no_grad():
      outs.append(kernels.rasterize_interpolate_packed(attrs, v, t, batch, cfg,
                                                       kernels.Workspace(device)))
  (a0, p0, i0, z0, b0), (a1, p1, i1, z1, b1) = outs
  fg = z0 != 1.0
  assert torch.equal(z0, z1) and torch.equal(a0, a1)
  assert torch.equal(i0[fg], i1[fg]) and torch.equal(b0[fg], b1[fg])
  assert torch.equal(p0[fg], p1[fg])
  assert (a1[~fg] == 0).all()


@pytest.mark.parametrize("recompute", [False, True])
def test_passthrough_shader_gives_the_same_image_and_gradients(recompute, device):
  """shading_function=None, under which background samples' attributes and
  color gradients are not written, renders what lambda a: a["rgba"] renders
  and gives the same gradients (the gradient atomics may reorder float sums:
  within 1e-6 of the largest magnitude), through BatchRenderer and
  render_triangles."""
  meshes, cams, sizes = workloads.ragged_batch(5, seed=13, median_triangles=3000,
                                               resolutions=(64, 96, 128))
  r = batch_lib.BatchRenderer([m.triangles for m in meshes], [len(m.vertices) for m in meshes],
                              sizes, num_layers=3, device=device, recompute_raster=recompute)
  cam = torch.tensor(np.stack(cams), device=device)
  rng = np.random.default_rng(1)

  def grads(out, leaves):
    g = torch.tensor(rng.standard_normal(tuple(out.shape)).astype(np.float32), device=device)
    return torch.autograd.grad(out, leaves, g)

  def batched(shader):
    v = torch.tensor(np.concatenate([m.vertices for m in meshes]), device=device,
                     requires_grad=True)
    c = rgba(torch.tensor(np.concatenate([m.colors for m in meshes]), device=device))
    c = c.detach().requires_grad_(True)
    out = r.render(v, {"rgba": c}, cam, shader)
    return (out.detach(),) + grads(out, (v, c))

  def single(shader):
    m, cm, (w, h) = meshes[1], cams[1], sizes[1]
    v = torch.tensor(m.vertices, device=device, requires_grad=True)
    c = rgba(torch.tensor(m.colors, device=device)).detach().requires_grad_(True)
    out = render.render_triangles(v, {"rgba": c}, torch.tensor(m.triangles, device=device),
                                  torch.tensor(cm, device=device), w, h, shader, num_layers=3,
                                  recompute_raster=recompute)
    return (out.detach(),) + grads(out, (v, c))

  for run in (batched, single):
    rng = np.random.default_rng(1)
    o0, gv0, gc0 = run(rgba_shader)
    rng = np.random.default_rng(1)
    o1, gv1, gc1 = run(None)
    assert torch.equal(o0, o1)
    for a, b in ((gv0, gv1), (gc0, gc1)):
      assert float((a - b).abs().max()) <= 1e-6 * float(b.abs().max())
  with pytest.raises(ValueError):
    r.render(torch.zeros(r.batch.total_vertices, 3, device=device),
             {"a": torch.zeros(r.batch.total_vertices, 2, device=device),
              "b": torch.zeros(r.batch.total_vertices, 2, device=device)}, cam, None)


def test_foreground_flags_leave_background_rows_untouched(device):
  """DR_RASTER_FOREGROUND_ATTRIBUTES and DR_SPLAT_FOREGROUND_GRADIENTS
  (through the C ABI, into buffers prefilled with NaN): background rows keep
  their contents, foreground rows are the same bits as without the flags."""
  meshes, cams, sizes = workloads.ragged_batch(6, seed=17, median_triangles=4000,
                                               resolutions=(64, 128, 160))
  from oracle import raster
  lib = _lib.load()
  clips = [raster.transform(c, m.vertices) for m, c in zip(meshes, cams)]
  batch = kernels.ImageBatch([s[0] for s in sizes], [s[1] for s in sizes],
                             [len(c) for c in clips], [len(m.triangles) for m in meshes])
  v = torch.as_tensor(np.concatenate(clips), device=device)
  t = torch.as_tensor(np.concatenate([m.triangles for m in meshes]), device=device)
  attrs = torch.rand(v.shape[0], 4, device=device)
  n = 3 * batch.total_pixels
  P = lambda x: ctypes.c_void_p(x.data_ptr())
  stream = ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)
  outs = []
  for flags in (_lib.DR_RASTER_FOREGROUND_ONLY,
                _lib.DR_RASTER_FOREGROUND_ONLY | _lib.DR_RASTER_FOREGROUND_ATTRIBUTES):
    cfg = kernels.raster_config(3, 1, 0, flags=flags)
    ws = torch.empty(kernels.raster_workspace_bytes(batch, cfg), dtype=torch.uint8,
                     device=device)
    ids = torch.empty(n, dtype=torch.int32, device=device)
    z = torch.empty(n, device=device)
    bary = torch.empty(n, 3, device=device)
    out = torch.full((n, 4), float("nan"), device=device)
    vp = torch.empty(n, 4, device=device)
    rc = lib.dr_rasterize_batch_interpolate(P(v), P(t), batch.ptr, batch.n, ctypes.byref(cfg),
                                            P(ids), P(z), P(bary), P(attrs), 4, P(out), P(vp),
                                            None, P(ws), ws.numel(), stream)
    assert rc == 0, lib.dr_last_error()
    outs.append((z, out, vp))
  (z0, a0, p0), (z1, a1, p1) = outs
  fg = z0 != 1.0
  assert torch.equal(z0, z1) and torch.equal(a0[fg], a1[fg]) and torch.equal(p0[fg], p1[fg])
  assert (a0[~fg] == 0).all() and torch.isnan(a1[~fg]).all()
  # Splat forward, then the backward with and without the flag.
  C = 4
  img = torch.empty(batch.total_pixels, C, device=device)
  saved = torch.empty(3 * (C + 1) + 2, batch.total_pixels, device=device)
  rc = lib.dr_splat_fwd(P(p0), P(z0), P(a0), C, batch.ptr, batch.n, 3, P(img), P(saved), None,
                        None, stream)
  assert rc == 0, lib.dr_last_error()
  d_out = torch.rand(batch.total_pixels, C, device=device) - 0.5
  res = []
  for flags in (0, _lib.DR_SPLAT_FOREGROUND_GRADIENTS):
    d_col = torch.full((n, C), float("nan"), device=device)
    d_pos = torch.full((n, 4), float("nan"), device=device)
    rc = lib.dr_splat_bwd_ex(P(d_out), P(p0), P(z0), P(a0), P(saved), C, batch.ptr, batch.n, 3,
                             flags, P(d_col), P(d_pos), stream)
    assert rc == 0, lib.dr_last_error()
    res.append((d_col, d_pos))
  (c0, q0), (c1, q1) = res
  assert torch.equal(c0[fg], c1[fg]) and torch.equal(q0[fg], q1[fg])
  assert (c0[~fg] == 0).all() and torch.isnan(c1[~fg]).all()


@pytest.mark.parametrize("recompute", [False, True])
def test_deterministic_gradients_repeat_bit_for_bit(recompute, device):
  """deterministic_gradients sums the vertex and color gradients in 64-bit
  fixed point: two backward passes give the same bits, and they agree with
  the float-atomic sums within 1e-6 of the largest magnitude (both round the
  same exact sum, the fixed-point one once). The image is the same bits."""
  meshes, cams, sizes = workloads.ragged_batch(6, seed=21, median_triangles=3000,
                                               resolutions=(64, 96, 128))
  cam = torch.tensor(np.stack(cams), device=device)

  def run(det):
    r = batch_lib.BatchRenderer([m.triangles for m in meshes], [len(m.vertices) for m in meshes],
                                sizes, num_layers=3, device=device, recompute_raster=recompute,
                                deterministic_gradients=det)
    v = torch.tensor(np.concatenate([m.vertices for m in meshes]), device=device,
                     requires_grad=True)
    c = rgba(torch.tensor(np.concatenate([m.colors for m in meshes]), device=device))
    c = c.detach().requires_grad_(True)
    out = r.render(v, {"rgba": c}, cam, rgba_shader)
    g = torch.tensor(np.random.default_rng(3).standard_normal(tuple(out.shape)).astype(np.float32),
                     device=device)
    gv, gc = torch.autograd.grad(out, (v, c), g)
    return out.detach(), gv, gc

  o1, gv1, gc1 = run(True)
  o2, gv2, gc2 = run(True)
  o0, gv0, gc0 = run(False)
  assert torch.equal(o1, o2) and torch.equal(o1, o0)
  assert torch.equal(gv1, gv2) and torch.equal(gc1, gc2)
  for a, b in ((gv1, gv0), (gc1, gc0)):
    assert float((a - b).abs().max()) <= 1e-6 * float(b.abs().max())


def test_batches_over_the_inline_limit_match_per_image(device):
  """131 images (more than DR_MAX_BATCH_INLINE = 128): every kernel splits
  its launches into groups of images and the splat runs one block per tile
  instead of the tile list. Each image still equals its own
  render_triangles call bit for bit, gradients within 1e-4, and the
  deterministic mode (fixed-point sums spanning both groups) repeats its
  bits."""
  n = _lib.DR_MAX_BATCH_INLINE + 3
  meshes = [workloads.icosphere_workload(2, seed=i) if i % 2 == 0 else
            workloads.soup_workload(40, seed=i, mu=-1.5, sigma=0.4) for i in range(n)]
  rng = np.random.default_rng(11)
  sizes = [(int(rng.integers(8, 41)), int(rng.integers(8, 41))) for _ in range(n)]
  eyes = workloads.sphere_eyes(n, seed=13, radius=2.6)
  cams = [workloads.camera_matrix(e, w, h) for e, (w, h) in zip(eyes, sizes)]
  cam = torch.tensor(np.stack(cams), device=device)
  voff = np.cumsum([0] + [len(m.vertices) for m in meshes])

  def run(det):
    r = batch_lib.BatchRenderer([m.triangles for m in meshes], [len(m.vertices) for m in meshes],
                                sizes, num_layers=3, device=device, deterministic_gradients=det)
    v = torch.tensor(np.concatenate([m.vertices for m in meshes]), device=device,
                     requires_grad=True)
    c = torch.tensor(np.concatenate([m.colors for m in meshes]), device=device,
                     requires_grad=True)
    out = r.render(v, {"rgba": rgba(c)}, cam, rgba_shader)
    g = torch.tensor(np.random.default_rng(5).standard_normal(tuple(out.shape))
                     .astype(np.float32), device=device)
    gv, gc = torch.autograd.grad(out, (v, c), g)
    return r, out.detach(), g, gv, gc

  r, out, g, gv, gc = run(False)
  _, out1, _, gv1, gc1 = run(True)
  _, out2, _, gv2, gc2 = run(True)
  assert torch.equal(out1, out) and torch.equal(out2, out)
  assert torch.equal(gv1, gv2) and torch.equal(gc1, gc2)
  for a, b in ((gv1, gv), (gc1, gc)):
    assert float((a - b).abs().max()) <= 1e-6 * float(b.abs().max())
  imgs, gimgs = r.images(out), r.images(g)
  assert sum(int((im[..., 3] > 0).any()) for im in imgs) > n // 2
  for i in range(n):
    m, (w, h) = meshes[i], sizes[i]
    vi = torch.tensor(m.vertices, device=device, requires_grad=True)
    ci = torch.tensor(m.colors, device=device, requires_grad=True)
    oi = render.render_triangles(vi, {"rgba": rgba(ci)}, torch.tensor(m.triangles, device=device),
                                 cam[i], w, h, rgba_shader, num_layers=3)
    torch.testing.assert_close(imgs[i], oi, rtol=0, atol=0)
    gvi, gci = torch.autograd.grad(oi, (vi, ci), gimgs[i])
    sl = slice(int(voff[i]), int(voff[i + 1]))
    torch.testing.assert_close(gv[sl], gvi, rtol=1e-4, atol=1e-4 * float(gvi.abs().max()) + 1e-12)
    torch.testing.assert_close(gc[sl], gci, rtol=1e-4, atol=1e-4 * float(gci.abs().max()) + 1e-12)
