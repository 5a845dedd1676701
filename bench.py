"""Benchmark: rasterize-then-splat forward+backward throughput (Mpix/s).

Workload (default `c5`): a ragged batch of 64 seeded meshes (noisy
icospheres or triangle soups, 50/50), triangle counts lognormal (median 20k,
sigma 1.2) clipped to [500, 500k], one camera per mesh on a sphere of radius
3, square resolutions drawn from {256, 512, 1024}, 3 depth layers, back-face
culling, RGBA vertex colors (RGB seeded, alpha 1) interpolated as an
attribute and passed through by the deferred shader (`lambda a: a['rgba']`,
as the reference's render tests shade). One step = forward
render of every image + L2 loss against fixed target images + backward to
vertex positions and vertex colors (the optimized color parameter is the
RGBA vertex color; the RGB gradients are its first three columns).

Reported (one JSON line on rank 0):
  value      batched path: all images in one launch per kernel, the step
             captured in a CUDA graph and replayed; inputs resident in HBM.
  plain      the same work as 64 per-mesh render_triangles calls (the
             reference's vmap 'sequential_unrolled' structure), eager.
  e2e        the batched step through the public API with pinned host
             inputs copied in and loss + gradients copied out every step.
  roofline   dominant kernel: algorithmic bytes / CUDA-event duration vs the
             measured HBM copy bandwidth.
  cpu_baseline  the reference path on the host cores, on a sample of the
             workload: the reference's own C++ CPU rasterizer (built from
             the reference sources by oracle/Makefile) + the torch CPU
             restatement of the JAX interpolate/splat/composite and its
             autodiff (JAX is not installed).
  parity     the first images of the benchmarked step and their vertex and
             color gradients against the CPU path in the same depth
             semantics (1e-5 rel / 1e-6 abs images, 1e-4 gradients).

`--impl reference` times that CPU path alone, one image per step.
Multi-GPU: replicas only (each rank renders the full batch independently).
"""
import argparse
import concurrent.futures
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_BYTES = 129 * 1024 * 1024


def parse():
  ap = argparse.ArgumentParser()
  ap.add_argument("--gpus", type=int, default=1)
  ap.add_argument("--steps", type=int, default=100)
  ap.add_argument("--warmup", type=int, default=3)
  ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
  ap.add_argument("--workload", default="c5", choices=["c5", "c2", "c3", "c4", "c1"])
  ap.add_argument("--num-meshes", type=int, default=64)
  ap.add_argument("--no-cpu-baseline", action="store_true")
  ap.add_argument("--no-plain", action="store_true")
  ap.add_argument("--no-parity", action="store_true",
                  help="skip the CPU comparison of the first images and gradients")
  ap.add_argument("--recompute-raster", action="store_true",
                  help="the VJP reruns the rasterizer instead of keeping its ids, "
                       "barycentrics and vertex ids (memory-tight mode)")
  ap.add_argument("--deterministic-gradients", action="store_true",
                  help="sum the vertex, color and texture gradients in fixed point (same "
                       "bits on every run)")
  ap.add_argument("--cpu-budget", type=float, default=20.0,
                  help="seconds of CPU work per reference-arm step / baseline")
  return ap.parse_args()


# --------------------------------------------------------------- workload
class Workload:
  """Seeded meshes, cameras, resolutions and target images."""

  def __init__(self, name, num_meshes, seed=0):
    from diffren_gb300 import workloads as wl
    self.name = name
    if name == "c5":
      meshes, cams, sizes = wl.ragged_batch(num_meshes, seed=seed)
      desc = ("ragged batch of %d meshes (icosphere|soup), T lognormal median 20k "
              "in [500, 500k], square res in {256,512,1024}, L=3, fwd+bwd L2 loss "
              "wrt vertices and RGBA vertex colors" % num_meshes)
    elif name == "c2":
      m = wl.soup_workload(200000, seed=seed)
      eyes = wl.sphere_eyes(8, seed=seed + 1)
      meshes = [m] * 8
      cams = [wl.camera_matrix(e, 512, 512) for e in eyes]
      sizes = [(512, 512)] * 8
      desc = "200k-triangle soup, 8 cameras, 512x512, L=3, fwd+bwd"
    elif name == "c3":
      m = wl.icosphere_workload(71, seed=seed)
      eyes = wl.sphere_eyes(8, seed=seed + 1)
      meshes = [m] * 8
      cams = [wl.camera_matrix(e, 1024, 1024) for e in eyes]
      sizes = [(1024, 1024)] * 8
      desc = "100k-triangle noisy icosphere, 8 cameras, 1024x1024, L=3, fwd+bwd"
    elif name == "c4":
      m = wl.heightfield_workload(708, seed=seed)
      eyes = wl.sphere_eyes(4, seed=seed + 1, radius=2.2, upper_only=True)
      k = max(1, min(4, num_meshes))  # fewer cameras for small profiling runs
      meshes = [m] * k
      cams = [wl.camera_matrix(e, 2048, 2048) for e in eyes[:k]]
      sizes = [(2048, 2048)] * k
      rng = np.random.default_rng(seed + 5)
      self.texture = rng.integers(0, 256, (1024, 1024, 4)).astype(np.float32) / 255.0
      desc = ("708x708 heightfield (999,698 triangles) with uv, 1024^2 RGBA texture "
              "(bilinear, edge clamp), %d cameras, 2048x2048, L=3, fwd+bwd L2 loss wrt "
              "vertices and texture" % k)
    else:
      m = wl.icosphere_workload(16, seed=seed)
      meshes, cams, sizes = [m], [wl.camera_matrix((0, 0, 3.0), 256, 256)], [(256, 256)]
      desc = ("5120-triangle icosphere, 256x256, L=3, point light (2,2,2) on area-weighted "
              "vertex normals, fwd+bwd L2 loss wrt vertices and RGB")
    if name != "c4":
      self.texture = None
    # Lit workloads shade with shaders.point_light on vertex normals
    # recomputed from the vertices every step.
    self.lit = name == "c1"
    self.meshes, self.cams, self.sizes, self.desc = meshes, cams, sizes, desc
    self.num_layers = 3
    self.pixels = int(sum(w * h for w, h in sizes))
    self.triangles = int(sum(len(m.triangles) for m in meshes))
    self.vertices = int(sum(len(m.vertices) for m in meshes))
    rng = np.random.default_rng(seed + 99)
    self.targets = [rng.uniform(0, 1, (h, w, 4)).astype(np.float32) for w, h in sizes]
    for t in self.targets:
      t[..., 3] = 1.0


def shader(a):
  """Pass-through of the interpolated RGBA vertex colors (the reference's
  render tests shade with `lambda x: x['rgba']` the same way)."""
  return a["rgba"]


LIGHT = (2.0, 2.0, 2.0)


def lit_shader(a):
  """point_light (shaders.py:100-173) with default coefficients on the
  interpolated RGB, normals and world positions; alpha 1 (appended by the
  shader kernel itself on the GPU)."""
  from diffren_gb300 import shaders
  return shaders.point_light(a["rgb"], a["normals"], a["pos"], LIGHT, alpha=True)


def rgba(colors):
  """Per-vertex RGBA from RGB with alpha 1 (differentiable w.r.t. RGB)."""
  import torch
  return torch.cat([colors, torch.ones_like(colors[:, :1])], 1)


def l2_loss_grads(out, target, params):
  """L2 loss sum((out - target)^2) and its gradients w.r.t. params.

  One fused CUDA pass over the images gives the loss and d loss / d out =
  2 (out - target) (`losses.squared_error_seed`), which seeds the renderer's
  VJP directly: the gradients are the same bits as autograd of the loss.
  """
  import torch
  from diffren_gb300 import losses
  loss, seed = losses.squared_error_seed(out, target)
  return loss, torch.autograd.grad(out, params, grad_outputs=seed)


_L2 = []


def l2_loss(out, target):
  """sum((out - target)^2), with the residual kept for the gradient
  2 (out - target): one pass each way over the images (torch's mse_loss
  zero-fills its gradient and re-reads both images in the backward)."""
  if not _L2:
    import torch

    class L2(torch.autograd.Function):

      @staticmethod
      def forward(ctx, o, t):
        diff = o - t
        ctx.save_for_backward(diff)
        flat = diff.reshape(-1)
        return torch.linalg.vecdot(flat, flat)

      @staticmethod
      def backward(ctx, g):
        (diff,) = ctx.saved_tensors
        return diff * (2.0 * g), None

    _L2.append(L2)
  return _L2[0].apply(out, target)


# ----------------------------------------------------------------- clocks
class ClockSampler:
  """nvidia-smi sampling during the timed region."""
  Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
       "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
       "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

  def __init__(self, gpu_index):
    self.gpu = gpu_index
    self.proc = None
    self.lines = []

  def __enter__(self):
    try:
      self.proc = subprocess.Popen(
          ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
           "--format=csv,noheader,nounits", "-lms", "200"],
          stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
      self.thread = threading.Thread(target=self._read, daemon=True)
      self.thread.start()
    except (OSError, FileNotFoundError):
      self.proc = None
    return self

  def _read(self):
    for line in self.proc.stdout:
      self.lines.append(line.strip())

  def wait_for_samples(self, n=2, timeout=5.0):
    """Blocks until the sampler has produced n lines (or timeout)."""
    t0 = time.time()
    while self.proc is not None and len(self.lines) < n and time.time() - t0 < timeout:
      time.sleep(0.05)

  def mark(self):
    """Index of the next sample; samples from here on are in the region."""
    return len(self.lines)

  def __exit__(self, *a):
    if self.proc is not None:
      self.proc.terminate()
      try:
        self.proc.wait(timeout=5)
      except subprocess.TimeoutExpired:
        self.proc.kill()

  def summary(self, start=0):
    sm, mx, reasons = [], [], set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    lines = self.lines[start:] or self.lines[-1:]
    for ln in lines:
      p = [x.strip() for x in ln.split(",")]
      if len(p) < 9:
        continue
      try:
        sm.append(float(p[1]))
        mx.append(float(p[2]))
      except ValueError:
        continue
      for n, v in zip(names, p[5:9]):
        if v.lower().startswith("active"):
          reasons.add(n)
    if not sm:
      return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
            "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- our arm
# DRAM bytes (read + write) per layer sample of each op, from the ncu
# capture of the 8-mesh subset of the ragged workload (the summaries under
# profiles/): setup + tile scan + binning + fine raster;
# splat forward; splat backward; samples VJP. Traffic grows with the layer
# samples, so the full workload's traffic is this times its samples.
TRAFFIC_PER_SAMPLE = {"raster": 32.98, "splat_fwd": 22.61, "splat_bwd": 31.73,
                      "samples_bwd": 22.92}


def kernel_bytes(wl, fg, near=None, C=4, K=4, fg_attributes=False, fg_color_grads=False,
                 vids=True):
  """Algorithmic (compulsory) HBM bytes per launch of each kernel: every
  input read and every output written once. `fg` = foreground layer samples
  among the L * P; work on background samples stops after their depth.
  `near` = pixels within one pixel of a foreground sample (the only ones
  whose splat accumulators the backward needs); all pixels if None.
  `fg_attributes`: background attributes are not written (shading_function
  None); `fg_color_grads`: nor background color gradients (the splat colors
  are the interpolated attributes). `vids`: the rasterizer stores vertex ids
  (no recompute)."""
  L, P, T, V = wl.num_layers, wl.pixels, wl.triangles, wl.vertices
  S = L * P
  near = P if near is None else near
  attr_written = fg if fg_attributes else S  # samples whose attributes are written
  grad_written = fg if fg_color_grads else S  # samples whose d colors are written
  return {
      # rasterizer with the fused interpolation epilogue: the mesh (indices,
      # clip vertices, attributes) in; z of every sample, ids, barycentrics,
      # viewport position (and vertex ids) of every foreground sample and K
      # attributes of the written samples out
      "raster": (T * 12 + V * (16 + 4 * K) + 4 * S + fg * (16 + 16 + (12 if vids else 0))
                 + 4 * K * attr_written),
      # depth of every sample, position and color of every foreground
      # sample in; composited color per pixel, saved accumulators (3 (C + 1))
      # and the surface code per pixel near foreground out
      "splat_fwd": 4 * S + (16 + 4 * C) * fg + 4 * C * P + (12 * (C + 1) + 4) * near,
      # saved accumulators, surface code and d color per pixel near
      # foreground, depth of every sample, position and color of the
      # foreground ones in; d color of the written samples and d position of
      # every foreground sample out
      "splat_bwd": (near * (12 * (C + 1) + 4 + 4 * C) + 4 * S + (16 + 4 * C) * fg
                    + 4 * C * grad_written + 16 * fg),
      # z of every sample; ids, bary, d position and d attributes of the
      # depth of every sample; barycentrics, vertex indices, d position,
      # position and d attributes of the foreground ones; vertex gradients
      # (clip + attributes) read and written once
      "samples_bwd": 4 * S + fg * (12 + 12 + 8 + 16 + 4 * K) + V * (16 + 4 * K) * 3,
      # texture shader on every sample: uv in, C channels out (texels from L2)
      "texture_fwd": S * (8 + 4 * C),
      # its VJP: d color and uv in, d uv out (texture gradient atomics in L2)
      "texture_bwd": S * (4 * C + 8 + 8),
      # L2 loss: image and target in, the VJP's seed out
      "squared_error": 12 * C * P,
  }


def max_over_ranks(ms, world, device):
  """The slowest rank's time: every rank's N replicas must finish a step."""
  if world <= 1:
    return ms
  import torch
  import torch.distributed as dist
  t = torch.tensor([ms], dtype=torch.float64, device=device)
  dist.all_reduce(t, op=dist.ReduceOp.MAX)
  return float(t)


def whole_job_mpix(world, pixels_per_rank, ms):
  """Aggregate throughput of N replicas, each rendering its own batch."""
  return world * pixels_per_rank / ms / 1e3


def run_ours(args, rank, world, device):
  import torch
  import torch.distributed as dist
  from diffren_gb300 import batch as batch_lib
  from diffren_gb300 import kernels, render

  wl = Workload(args.workload, args.num_meshes)
  r = batch_lib.BatchRenderer([m.triangles for m in wl.meshes],
                              [len(m.vertices) for m in wl.meshes], wl.sizes,
                              num_layers=wl.num_layers, device=device, tile="auto",
                              recompute_raster=args.recompute_raster,
                              deterministic_gradients=args.deterministic_gradients)
  from diffren_gb300 import shaders
  textured = wl.texture is not None
  verts_h = torch.from_numpy(np.concatenate([m.vertices for m in wl.meshes])).pin_memory()
  # The optimized parameters besides the vertices: per-vertex RGB, or the
  # texture of a textured workload (whose uvs are a fixed input).
  if textured:
    cols_h = torch.from_numpy(wl.texture).pin_memory()
    uv = torch.from_numpy(np.concatenate([m.uvs for m in wl.meshes])).to(device)
  else:
    rgb = np.concatenate([m.colors for m in wl.meshes])
    cols_h = torch.from_numpy(rgb if wl.lit else np.concatenate(
        [rgb, np.ones_like(rgb[:, :1])], 1)).pin_memory()
  cams_h = torch.from_numpy(np.stack(wl.cams)).pin_memory()
  target = torch.from_numpy(np.concatenate([t.reshape(-1, 4) for t in wl.targets])).to(device)
  # Two sets of device inputs and outputs: the end-to-end loop below runs
  # one step on each set in turn while the other set's copies are in flight.
  sets = [dict(verts=verts_h.to(device), cols=cols_h.to(device), cams=cams_h.to(device))
          for _ in range(2)]
  verts, cams = sets[0]["verts"], sets[0]["cams"]

  def step(b=sets[0]):
    v = b["verts"].detach().requires_grad_(True)
    c = b["cols"].detach().requires_grad_(True)
    cams = b["cams"]
    if textured:
      out = r.render(v, {"uv": uv}, cams, lambda a: shaders.texture_map(
          a["uv"], c, deterministic=args.deterministic_gradients))
    elif wl.lit:
      out = r.render(v, {"rgb": c, "normals": r.vertex_normals(v), "pos": v}, cams,
                     lit_shader)
    else:
      out = r.render(v, {"rgba": c}, cams, shader)
    loss, (gv, gc) = l2_loss_grads(out, target, (v, c))
    return dict(g_v=gv, g_c=gc.contiguous(), loss=loss, out=out.detach())

  # Eager warm-up on a side stream, then capture the step.
  s = torch.cuda.Stream(device)
  s.wait_stream(torch.cuda.current_stream(device))
  with torch.cuda.stream(s):
    for _ in range(max(args.warmup, 3)):
      step()
  torch.cuda.current_stream(device).wait_stream(s)
  # Launch count of our kernels in one step (eager), and the step's results
  # on the first images for the parity check.
  kernels.LAUNCHES.reset()
  torch.cuda.synchronize(device)
  mem0 = torch.cuda.memory_allocated(device)
  torch.cuda.reset_peak_memory_stats(device)
  res0 = step()
  torch.cuda.synchronize(device)
  step_peak_bytes = torch.cuda.max_memory_allocated(device) - mem0
  launches_per_step = kernels.LAUNCHES.count
  gpu = None
  if rank == 0 and not args.no_parity:
    nck = min(16, r.batch.n)
    vo = np.cumsum([0] + [len(m.vertices) for m in wl.meshes])
    gpu = {"images": [x.cpu().numpy() for x in r.images(res0["out"])[:nck]],
           "g_v": [res0["g_v"][vo[i]:vo[i + 1]].cpu().numpy() for i in range(nck)],
           "g_c": [None if textured else res0["g_c"][vo[i]:vo[i + 1], :3].cpu().numpy()
                   for i in range(nck)]}
  del res0
  # Foreground layer samples of the workload, and pixels within one pixel
  # of one (for the algorithmic bytes).
  with torch.no_grad():
    _, z_fg, _ = r.rasterize(kernels.transform(verts, cams, r.batch))
    fg = int((z_fg != 1.0).sum())
    near = 0
    for i in range(r.batch.n):
      m = (r.batch.layered_view(z_fg, i, wl.num_layers) != 1.0).any(0).float()
      near += int(torch.nn.functional.max_pool2d(m[None, None], 3, 1, 1).sum())
  del z_fg
  # One graph per buffer set, each with its own memory pool: a graph's
  # outputs (loss and gradients, read back while the other graph runs) live
  # in its pool and are rewritten in place by every replay.
  graphs = []
  for b in sets:
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
      outs = step(b)
    b.update(outs)
    graphs.append(g)
  graph = graphs[0]
  for _ in range(args.warmup):
    graph.replay()
  torch.cuda.synchronize(device)

  def timed(fn, k):
    if world > 1:
      dist.barrier()
    torch.cuda.synchronize(device)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(k):
      fn()
    e1.record()
    torch.cuda.synchronize(device)
    return max_over_ranks(e0.elapsed_time(e1) / k, world, device)

  with ClockSampler(device.index) as clocks:
    clocks.wait_for_samples()
    start = clocks.mark()
    ms = timed(graph.replay, args.steps)
    time.sleep(0.25)  # let the sample that covers the region's end arrive
  clock = clocks.summary(start)
  loss_val = float(sets[0]["loss"])

  # e2e: public API with host buffers. Every step copies its inputs from
  # pinned host memory and its loss and gradients back. Steps alternate
  # between the two buffer sets (and their graphs), so that step i+1's
  # inputs arrive and step i's gradients leave on two copy streams while
  # the next step computes; the timed region runs from before the first
  # input copy to the end of the last gradient copy.
  gv_h = torch.empty_like(verts_h).pin_memory()
  gc_h = torch.empty_like(cols_h).pin_memory()
  loss_h = torch.empty((), pin_memory=True)
  h2d_s = torch.cuda.Stream(device)
  d2h_s = torch.cuda.Stream(device)

  def e2e_steps(k):
    cur = torch.cuda.current_stream(device)
    in_ready = [torch.cuda.Event(), torch.cuda.Event()]
    done = [torch.cuda.Event(), torch.cuda.Event()]
    out_free = [torch.cuda.Event(), torch.cuda.Event()]

    def upload(j):
      with torch.cuda.stream(h2d_s):
        b = sets[j]
        for name, src in (("verts", verts_h), ("cols", cols_h), ("cams", cams_h)):
          b[name].copy_(src, non_blocking=True)
        in_ready[j].record(h2d_s)

    h2d_s.wait_stream(cur)
    upload(0)
    for i in range(k):
      j = i % 2
      cur.wait_event(in_ready[j])
      if i >= 2:
        cur.wait_event(out_free[j])  # step i-2's gradients have left set j
      graphs[j].replay()
      done[j].record(cur)
      if i + 1 < k:
        if i >= 1:
          h2d_s.wait_event(done[1 - j])  # step i-1 has finished with set 1-j
        upload(1 - j)
      d2h_s.wait_event(done[j])
      with torch.cuda.stream(d2h_s):
        b = sets[j]
        for dst, name in ((gv_h, "g_v"), (gc_h, "g_c"), (loss_h, "loss")):
          dst.copy_(b[name], non_blocking=True)
        out_free[j].record(d2h_s)
    cur.wait_stream(d2h_s)

  e2e_steps(2)
  torch.cuda.synchronize(device)
  ms_e2e = timed(lambda: e2e_steps(args.steps), 1) / args.steps
  if abs(float(loss_h) - loss_val) > 1e-4 * abs(loss_val):
    print("warning: e2e loss %r differs from the graph's %r" % (float(loss_h), loss_val),
          file=sys.stderr)
  h2d = verts_h.numel() * 4 + cols_h.numel() * 4 + cams_h.numel() * 4
  d2h = gv_h.numel() * 4 + gc_h.numel() * 4 + 4

  # Per-kernel CUDA-event durations on the launching stream (eager step with
  # events around each op), for the roofline of the dominant kernel.
  per_kernel = kernels.profile_step(step, args.steps, device)
  plain = None
  if not args.no_plain and rank == 0:
    plain = run_plain(wl, device, args)
  tile = [r.config.tile_width, r.config.tile_height, r.config.large_tiles]
  return dict(wl=wl, fg=fg, near=near, tile=tile, ms=ms, ms_e2e=ms_e2e, h2d=h2d, d2h=d2h, clock=clock,
              loss=loss_val, launches=launches_per_step, per_kernel=per_kernel,
              plain=plain, renderer=r, gpu=gpu, step_peak_bytes=step_peak_bytes)


def run_plain(wl, device, args):
  """64 separate per-mesh renders (eager), same loss and gradients."""
  import torch
  from diffren_gb300 import mesh, render
  from diffren_gb300 import shaders
  textured = wl.texture is not None
  tex = torch.tensor(wl.texture, device=device) if textured else None
  data = []
  for m, cam, (w, h), t in zip(wl.meshes, wl.cams, wl.sizes, wl.targets):
    data.append((torch.tensor(m.vertices, device=device),
                 tex if textured else torch.tensor(
                     m.colors if wl.lit else np.concatenate(
                         [m.colors, np.ones_like(m.colors[:, :1])], 1), device=device),
                 torch.tensor(m.uvs, device=device) if textured else None,
                 torch.tensor(m.triangles, device=device),
                 torch.tensor(cam, device=device), w, h,
                 torch.tensor(t, device=device)))

  def step():
    for v0, c0, uv, tri, cam, w, h, tgt in data:
      v = v0.detach().requires_grad_(True)
      c = c0.detach().requires_grad_(True)
      if textured:
        out = render.render_triangles(v, {"uv": uv}, tri, cam, w, h,
                                      lambda a: shaders.texture_map(a["uv"], c),
                                      num_layers=wl.num_layers)
      elif wl.lit:
        attrs = {"rgb": c, "normals": mesh.compute_vertex_normals(v, tri), "pos": v}
        out = render.render_triangles(v, attrs, tri, cam, w, h, lit_shader,
                                      num_layers=wl.num_layers)
      else:
        out = render.render_triangles(v, {"rgba": c}, tri, cam, w, h, shader,
                                      num_layers=wl.num_layers)
      l2_loss_grads(out, tgt, (v, c))

  for _ in range(2):
    step()
  torch.cuda.synchronize(device)
  k = max(10, min(args.steps, 20))
  e0 = torch.cuda.Event(enable_timing=True)
  e1 = torch.cuda.Event(enable_timing=True)
  e0.record()
  for _ in range(k):
    step()
  e1.record()
  torch.cuda.synchronize(device)
  ms = e0.elapsed_time(e1) / k
  return {"ms_per_step": ms, "value": wl.pixels / ms / 1e3, "steps": k}


# -------------------------------------------------------- CPU (reference)
def cpu_rasterize(wl, i, kind):
  """Clip vertices and (ids, z, bary) of image i on the CPU. kind
  "reference": the reference's own C++ CPU rasterizer
  (rasterize_triangles_impl.cc:27-118, compiled by oracle/Makefile; float
  depth, single-threaded per image, as the reference runs it); "oracle": the
  C restatement in the discretized semantics of the reference's CUDA
  rasterizer, which the GPU path computes (checked bit for bit against the
  reference's CUDA build by the tests)."""
  from oracle import raster
  m, cam, (w, h) = wl.meshes[i], wl.cams[i], wl.sizes[i]
  clip = raster.transform(cam, m.vertices)
  if kind == "reference":
    return clip, raster.rasterize_reference_cpu(clip, m.triangles, w, h, wl.num_layers, 1)
  return clip, raster.rasterize(clip, m.triangles, w, h, wl.num_layers, 1,
                                raster.DEPTH_DISCRETIZED)


def cpu_render(wl, i, clip, rast, ttex=None):
  """Interpolate, shade, splat, normalize, composite, L2 loss and the
  backward of image i on the CPU: the torch float32 restatement of the
  reference's JAX code (oracle/torch_ref.py) with torch autograd standing in
  for jax.grad. The forward uses the exact clip vertices the rasterizer saw;
  gradients flow to the world vertices through the camera matrix. Returns
  (image [H, W, C], d vertices [V, 3], d colors [V, 3] or None)."""
  import torch
  from oracle import mesh as omesh
  from oracle import texture, torch_ref
  ids, z, b = rast
  m, (w, h), tgt = wl.meshes[i], wl.sizes[i], wl.targets[i]
  state = torch_ref.discrete_state(clip, ids, z, b, m.triangles, w, h)
  ti, tz, tb, tt = (torch.tensor(x) for x in (ids, z, b, m.triangles))
  tv = torch.tensor(m.vertices, requires_grad=True)
  cam = torch.tensor(wl.cams[i], dtype=torch.float32)
  lin = torch.cat([tv, torch.ones_like(tv[:, :1])], 1) @ cam.T
  tc = torch.tensor(clip) + (lin - lin.detach())  # exact values, camera gradient
  tparam = None
  if ttex is not None:
    uvs = torch_ref.interpolate(torch.tensor(m.uvs), ti, tz, tb, tt)
    shaded = texture.texture_map_t(uvs, ttex)
  elif wl.lit:
    tparam = torch.tensor(m.colors, requires_grad=True)
    attrs = torch.cat([tparam, omesh.vertex_normals_t(tv, tt), tv], 1)
    a = torch_ref.interpolate(attrs, ti, tz, tb, tt)
    shaded = lit_shader({"rgb": a[..., :3], "normals": a[..., 3:6], "pos": a[..., 6:9]})
  else:
    tparam = torch.tensor(m.colors, requires_grad=True)
    shaded = torch_ref.interpolate(rgba(tparam), ti, tz, tb, tt)
  out = torch_ref.splat_shaded_pixels(tc, ti, tz, tb, tt, shaded, w, h, state)[0]
  loss = l2_loss(out, torch.tensor(tgt))
  params = [tv] + ([tparam] if tparam is not None else []) + (
      [ttex] if ttex is not None else [])
  grads = torch.autograd.grad(loss, params)
  return (out.detach().numpy(), grads[0].numpy(),
          grads[1].numpy() if tparam is not None else None)


def cpu_port_sample(wl, budget_s, threads, images=None, kind="reference", keep=False):
  """Times the CPU path on images of the workload until `budget_s` of work
  (or on exactly the given `images`): rasterization (`cpu_rasterize`), a
  group of `threads` images at a time on `threads` host threads, then
  `cpu_render` of each on `threads` torch threads. Returns (pixels, seconds,
  images used, {image: (image, d vertices, d colors)} if keep)."""
  import concurrent.futures
  import torch
  torch.set_num_threads(threads)
  ttex = None if wl.texture is None else torch.tensor(wl.texture, requires_grad=True)
  order = list(images) if images is not None else list(range(len(wl.meshes)))
  px = used = 0
  t_total = 0.0
  kept = {}
  with concurrent.futures.ThreadPoolExecutor(threads) as pool:
    for g0 in range(0, len(order), threads):
      group = order[g0:g0 + threads]
      t0 = time.perf_counter()
      # ctypes calls release the GIL: the rasterizers run in parallel.
      rasters = list(pool.map(lambda i: cpu_rasterize(wl, i, kind), group))
      for i, (clip, rast) in zip(group, rasters):
        res = cpu_render(wl, i, clip, rast, ttex)
        if keep:
          kept[i] = res
        px += wl.sizes[i][0] * wl.sizes[i][1]
        used += 1
      t_total += time.perf_counter() - t0
      if images is None and t_total >= budget_s:
        break
  return px, t_total, used, kept


def parity_check(wl, gpu, budget_s, threads):
  """Compares the benchmarked GPU step with the CPU path on the first images
  of the workload (until `budget_s` of CPU work, at most 16 images): the
  rasterizer in the same (discretized) semantics, the torch restatement of
  the splat and its autograd. Images: elementwise against 1e-5 relative /
  1e-6 absolute (`image_tol_ratio` <= 1 passes). Gradients of each mesh:
  max abs difference over the largest magnitude (`max_rel_err_grad`, bar
  1e-4). Vertex gradients are compared per image only where every image has
  its own mesh."""
  n = min(16, len(wl.meshes), len(gpu["images"]))
  t0 = time.perf_counter()
  res = {}
  for i in range(n):
    res.update(cpu_port_sample(wl, 0.0, threads, images=[i], kind="oracle", keep=True)[3])
    if time.perf_counter() - t0 >= budget_s:
      break
  per_mesh = len({id(m) for m in wl.meshes}) == len(wl.meshes)
  img_ratio = img_abs = img_rel = grad_rel = 0.0
  for i, (out, gv, gc) in res.items():
    a, b = gpu["images"][i], out
    d = np.abs(a - b)
    img_abs = max(img_abs, float(d.max()))
    img_ratio = max(img_ratio, float((d / (1e-6 + 1e-5 * np.abs(b))).max()))
    big = np.abs(b) >= 1e-3
    if big.any():
      img_rel = max(img_rel, float((d[big] / np.abs(b[big])).max()))
    if per_mesh:
      for g_gpu, g_cpu in ((gpu["g_v"][i], gv), (gpu["g_c"][i], gc)):
        if g_cpu is None:
          continue
        scale = float(np.abs(g_cpu).max()) or 1.0
        grad_rel = max(grad_rel, float(np.abs(g_gpu - g_cpu).max()) / scale)
  return {"images_checked": len(res), "max_abs_err_image": img_abs,
          "max_rel_err_image": img_rel, "image_tol_ratio": img_ratio,
          "max_rel_err_grad": grad_rel if per_mesh else None,
          "within_tolerance": bool(img_ratio <= 1.0 and (not per_mesh or grad_rel <= 1e-4)),
          "cpu_side": "C restatement of the reference CUDA rasterizer (bit-exact) + torch "
                      "float32 restatement of the JAX splat with autograd"}


def bench_config(wl):
  """The `config` both arms print: the workload and its sizes."""
  return {"workload": wl.desc, "num_images": len(wl.meshes), "total_mpix": wl.pixels / 1e6,
          "total_triangles": wl.triangles, "num_layers": wl.num_layers,
          "l2": "per-step working set of several GB > 129 MB L2"}


def run_reference(args):
  """The reference arm, on the machine's host cores: the reference's own C++
  CPU rasterizer for the raster stage (built from the reference sources by
  oracle/Makefile) and the torch CPU restatement of the reference's JAX
  splat and its autodiff (JAX is not installed). Step i renders image
  i mod N of the workload forward and backward; the value is the timed
  steps' pixels over their time."""
  from oracle import raster
  wl = Workload(args.workload, args.num_meshes)
  if raster.build_reference() is None:
    print(json.dumps({"impl": "reference", "unavailable": "the reference CPU rasterizer's "
                      "sources are not present (oracle/_ref/src or DIFFREN_REFERENCE)"}))
    return
  threads = os.cpu_count() or 1
  n = len(wl.meshes)
  px_t = secs_t = 0.0
  for it in range(args.warmup + args.steps):
    px, secs, _, _ = cpu_port_sample(wl, 0.0, threads, images=[it % n], kind="reference")
    if it >= args.warmup:
      px_t += px
      secs_t += secs
  value = px_t / secs_t / 1e6
  sample = ("one image of the workload per step (images %d..%d of %d, cycling), %d px in "
            "%.1f s; rasterizer: the reference's own C++ CPU rasterizer, one thread per "
            "image; splat fwd+bwd: torch float32 restatement of the JAX path on %d threads"
            % (args.warmup % n, (args.warmup + args.steps - 1) % n, n, px_t, secs_t, threads))
  line = {
      "metric": "RtS fwd+bwd Mpix/s on 1 GB300, batched vs plain, at 1e-5 rel err",
      "value": value, "unit": "Mpix/s", "n_gpus": args.gpus, "steps": args.steps,
      "warmup": args.warmup, "ms_per_step": secs_t * 1e3 / args.steps,
      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
      "data": "synthetic (seeded meshes, cameras and targets)", "impl": "reference",
      "config": bench_config(wl),
      "cpu_baseline": {"value": value, "unit": "Mpix/s", "cores": threads, "kind": "reference",
                       "sample": sample},
      "e2e": {"value": value, "unit": "Mpix/s", "h2d_bytes_per_step": 0,
              "d2h_bytes_per_step": 0},
  }
  print(json.dumps(line))


def measured_peaks():
  path = os.path.join(ROOT, "MEASURED_PEAKS.json")
  try:
    with open(path) as f:
      d = json.load(f)
    return float(d["hbm_gbs"]), "measured"
  except (OSError, KeyError, ValueError):
    return 6800.0, "fallback"


def main():
  args = parse()
  rank = int(os.environ.get("RANK", "0"))
  world = int(os.environ.get("WORLD_SIZE", "1"))
  local = int(os.environ.get("LOCAL_RANK", "0"))
  if args.impl == "reference":
    if rank == 0:
      run_reference(args)
    return
  import torch
  import torch.distributed as dist
  device = torch.device("cuda", local)
  torch.cuda.set_device(device)
  if world > 1:
    dist.init_process_group("nccl", device_id=device)
  res = run_ours(args, rank, world, device)
  wl = res["wl"]
  cpu = None
  parity = None
  if rank == 0 and not args.no_cpu_baseline:
    from oracle import raster
    threads = os.cpu_count() or 1
    kind = "reference" if raster.build_reference() is not None else "port"
    px, secs, used, _ = cpu_port_sample(wl, args.cpu_budget, threads,
                                        kind="reference" if kind == "reference" else "oracle")
    cpu = {"value": px / secs / 1e6, "unit": "Mpix/s", "cores": threads, "kind": kind,
           "sample": "first %d of %d images of the workload (%d px), fwd+bwd, %.1f s; "
                     "rasterizer: %s, one image per thread; splat fwd+bwd: torch float32 "
                     "restatement of the JAX path (JAX is not installed) on all threads"
                     % (used, len(wl.meshes), px, secs,
                        "the reference's own C++ CPU rasterizer" if kind == "reference"
                        else "the C restatement")}
  if rank == 0 and res["gpu"] is not None:
    parity = parity_check(wl, res["gpu"], args.cpu_budget, os.cpu_count() or 1)
  if rank != 0:
    if world > 1:
      dist.destroy_process_group()
    return
  peak, peak_kind = measured_peaks()
  pk = res["per_kernel"]
  nbytes = kernel_bytes(wl, res["fg"], res["near"], K=2 if wl.texture is not None else 4,
                        fg_color_grads=wl.texture is None and not wl.lit,
                        vids=not args.recompute_raster)
  dom = max((k for k in pk if k in nbytes), key=lambda k: pk[k])
  achieved = nbytes[dom] / (pk[dom] * 1e-3) / 1e9
  value = whole_job_mpix(world, wl.pixels, res["ms"])
  line = {
      "metric": "RtS fwd+bwd Mpix/s on 1 GB300, batched vs plain, at 1e-5 rel err",
      "value": value, "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
      "warmup": args.warmup, "ms_per_step": res["ms"], "higher_is_better": True,
      "scaling": "weak", "vs_baseline": None, "dtype": "f32",
      "data": "synthetic (seeded meshes, cameras and targets)",
      "config": bench_config(wl),
      "details": {"foreground_samples": res["fg"], "pixels_near_foreground": res["near"],
                  "parallelism": "replicas" if world > 1 else "1 GPU",
                  "cuda_graph": True, "raster_tile_autotuned": res["tile"],
                  "depth_semantics": "discretized (the reference CUDA rasterizer's)",
                  "recompute_raster": bool(args.recompute_raster),
                  "deterministic_gradients": bool(args.deterministic_gradients),
                  "step_peak_device_bytes": res["step_peak_bytes"]},
      "parity": parity,
      "e2e": {"value": whole_job_mpix(world, wl.pixels, res["ms_e2e"]), "unit": "Mpix/s",
              "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"]},
      "plain": None if res["plain"] is None else {
          "value": res["plain"]["value"], "unit": "Mpix/s",
          "ms_per_step": res["plain"]["ms_per_step"], "steps": res["plain"]["steps"],
          "batched_over_plain": value / world / res["plain"]["value"]},
      "gpu_launches": res["launches"] * args.steps,
      "kernels_ms": {k: round(v, 4) for k, v in pk.items()},
      "kernels_gbs": {k: round(nbytes[k] / (pk[k] * 1e-3) / 1e9, 1)
                      for k in pk if k in nbytes},
      "raster_rates": None if "raster" not in pk else {
          "mpix_per_s": wl.pixels / (pk["raster"] * 1e-3) / 1e6,
          "mtriangles_per_s": wl.triangles / (pk["raster"] * 1e-3) / 1e6},
      "roofline": {"kernel": dom, "bound": "hbm", "achieved": achieved, "peak": peak,
                   "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                   "algorithmic_bytes": nbytes[dom],
                   "traffic": (TRAFFIC_PER_SAMPLE[dom] * wl.num_layers * wl.pixels
                               if dom in TRAFFIC_PER_SAMPLE else None),
                   "traffic_source": "ncu DRAM bytes of the 8-mesh subset, scaled by "
                                     "layer samples"},
      "cpu_baseline": cpu,
      "clocks": res["clock"],
      "loss": res["loss"],
  }
  print(json.dumps(line))
  if world > 1:
    dist.destroy_process_group()


if __name__ == "__main__":
  main()
