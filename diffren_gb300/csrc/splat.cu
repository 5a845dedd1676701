// Rasterize-then-splat for GB300 (diffren/jax/internal/splat.py:26-229,
// diffren/jax/composite.py:20-37) and its VJP:
//
//   positions_fwd  per layer sample: clip xyzw interpolated with the
//                  rasterized barycentrics (background (0, 0, 1, 1)),
//                  projected to viewport xyz, plus the foreground flag
//                  (splat.py:207-221) -> float4 per sample.
//   samples_fwd    the same pass fused with the interpolation of the vertex
//                  attributes (interpolate.py:24-63): one triangle lookup and
//                  one set of vertex gathers feed both outputs.
//   splat_fwd      screen tiles with a 1-pixel halo of samples in shared
//                  memory; each output pixel gathers the splats of its 3x3
//                  neighbours and every layer with the per-tap surface test,
//                  normalizes and composites; optionally saves its
//                  fg/surface/bg accumulators for the VJP.
//   splat_bwd      gather form of the adjoint: the adjoints of the saved
//                  accumulators on the tile plus a 1-pixel ring go to shared
//                  memory, then each sample of the tile reads those of the 9
//                  pixels it reached -> d colors and d viewport xy. No atomics.
//   positions_bwd  d viewport -> d clip vertices (float atomics over the
//                  triangle's three vertices) and d barycentrics.
//   samples_bwd    positions_bwd fused with the attribute VJP.
//
// With positions computed once, neither splat kernel gathers triangle data,
// and the backward never recomputes the forward accumulation.
#include <algorithm>
#include <cmath>
#include <initializer_list>
#include <string>

#include "common.cuh"
#include "internal.h"

namespace dr {
namespace {

constexpr int kTX = 32;  // tile width (one warp per row)
constexpr int kTY = 8;   // tile height (256 threads)

// ---------------------------------------------------------------- positions
struct PosArgs {
  const float4* clip;
  const int32_t* tris;
  const int32_t* ids;
  const float* z;
  const float* bary;
  int L;
  float4* vp;         // forward output
  const float4* dvp;  // backward input
  float4* d_clip;     // backward outputs
  float* d_bary;
};

struct Interp {
  float4 c;  // interpolated clip xyzw
  int vid[3];
  float4 V[3];
  float b[3];
};

// A layer sample's triangle id and barycentrics, loaded together with its
// depth so that the three loads overlap.
struct SampleRef {
  float z;
  int id;
  float b[3];
};

__device__ __forceinline__ SampleRef load_sample(const PosArgs& a, int64_t e) {
  SampleRef s;
  s.z = __ldg(a.z + e);
  s.id = __ldg(a.ids + e);
#pragma unroll
  for (int i = 0; i < 3; ++i) s.b[i] = __ldg(a.bary + 3 * e + i);
  return s;
}

__device__ __forceinline__ Interp interpolate_clip(const PosArgs& a, const Batch& B,
                                                   int img, const SampleRef& sr) {
  Interp r;
  const int32_t* t = a.tris + 3 * (B.triangle_offset[img] + sr.id);
  const float4* vb = a.clip + B.vertex_offset[img];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    r.vid[i] = __ldg(t + i);
    r.V[i] = __ldg(vb + r.vid[i]);
    r.b[i] = sr.b[i];
  }
  // (c0 b0 + c1 b1) + c2 b2 per coordinate (interpolate.py:24-63).
  r.c.x = __fadd_rn(__fadd_rn(__fmul_rn(r.V[0].x, r.b[0]), __fmul_rn(r.V[1].x, r.b[1])),
                    __fmul_rn(r.V[2].x, r.b[2]));
  r.c.y = __fadd_rn(__fadd_rn(__fmul_rn(r.V[0].y, r.b[0]), __fmul_rn(r.V[1].y, r.b[1])),
                    __fmul_rn(r.V[2].y, r.b[2]));
  r.c.z = __fadd_rn(__fadd_rn(__fmul_rn(r.V[0].z, r.b[0]), __fmul_rn(r.V[1].z, r.b[1])),
                    __fmul_rn(r.V[2].z, r.b[2]));
  r.c.w = __fadd_rn(__fadd_rn(__fmul_rn(r.V[0].w, r.b[0]), __fmul_rn(r.V[1].w, r.b[1])),
                    __fmul_rn(r.V[2].w, r.b[2]));
  return r;
}

__global__ void __launch_bounds__(256) positions_fwd_kernel(PosArgs a, Batch B) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= int64_t(a.L) * B.pix_prefix[B.n]) return;
  const PixelRef r = decode(B, a.L, q);
  const float W = __int2float_rn(B.width[r.img]), H = __int2float_rn(B.height[r.img]);
  float4 c = make_float4(0.0f, 0.0f, 1.0f, 1.0f);
  float fg = 0.0f;
  const SampleRef sr = load_sample(a, r.e);
  if (sr.z != 1.0f) {
    fg = 1.0f;
    c = interpolate_clip(a, B, r.img, sr).c;
  }
  a.vp[r.e] = viewport_of(c, W, H, fg);
}

__global__ void __launch_bounds__(256) positions_bwd_kernel(PosArgs a, Batch B) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= int64_t(a.L) * B.pix_prefix[B.n]) return;
  const PixelRef r = decode(B, a.L, q);
  const float4 g = a.dvp[r.e];
  const SampleRef sr = load_sample(a, r.e);
  if (sr.z == 1.0f || (g.x == 0.0f && g.y == 0.0f)) {
    if (a.d_bary) {
      a.d_bary[3 * r.e] = 0.0f;
      a.d_bary[3 * r.e + 1] = 0.0f;
      a.d_bary[3 * r.e + 2] = 0.0f;
    }
    return;
  }
  const Interp it = interpolate_clip(a, B, r.img, sr);
  const float W = __int2float_rn(B.width[r.img]), H = __int2float_rn(B.height[r.img]);
  // viewport z carries no gradient (it only enters comparisons).
  const float dnx = g.x * W * 0.5f, dny = g.y * H * 0.5f;
  const float cw = it.c.w;
  const float4 dcl = make_float4(dnx / cw, dny / cw, 0.0f,
                                 -(dnx * it.c.x + dny * it.c.y) / (cw * cw));
  float4* dv = a.d_clip + B.vertex_offset[r.img];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float b = it.b[i];
    atomicAdd(dv + it.vid[i], make_float4(b * dcl.x, b * dcl.y, 0.0f, b * dcl.w));
    if (a.d_bary)
      a.d_bary[3 * r.e + i] = it.V[i].x * dcl.x + it.V[i].y * dcl.y + it.V[i].w * dcl.w;
  }
}

// ------------------------------------------- fused attributes + positions
// One pass per layer sample that both interpolates vertex attributes
// (interpolate.py:24-63, background 0) and computes the splat position: the
// triangle lookup, barycentrics and vertex gathers are shared. The render
// paths use it; results equal interp_fwd_kernel and positions_fwd_kernel.
struct SampleArgs {
  PosArgs pos;
  const float4* vp;    // backward: stored positions, w = clip w (nullable)
  const int32_t* vid;  // backward: stored vertex indices [L*P, 3] (nullable)
  const float* attr;  // [V, K]
  int K;
  float* attr_out;         // [L*P, K]
  const float* d_attr_out;  // backward input (nullable)
  float* d_attr;            // [V, K] accumulated
  // DR_SAMPLES_DETERMINISTIC: the vertex gradients are summed in 64-bit
  // fixed point, 2^e units per unit with e chosen from the largest value
  // added, so that the sums do not depend on the order of the atomics.
  unsigned* fx_max;              // [1] float bits of the largest |value| added
  unsigned long long* fx_clip;   // [V, 4] fixed-point sums
  unsigned long long* fx_attr;   // [V, K]
  int fx_log2_count;             // ceil(log2(bound on the additions per sum))
};

// Exponent e of the fixed-point sums from the bound on what the run sums add
// (see fixed_exponent_of): a run sum adds at most 32 lanes' values, and one
// more bit covers their rounding.
constexpr int kRunBits = 6;

__device__ __forceinline__ int fixed_exponent(const SampleArgs& a) {
  return fixed_exponent_of(__ldg(a.fx_max), kRunBits + a.fx_log2_count);
}


__device__ __forceinline__ void add_chunk(float* p, float4 v, int n, bool vec) {
  if (vec) {
    atomicAdd(reinterpret_cast<float4*>(p), v);
    return;
  }
  atomicAdd(p, v.x);
  if (n > 1) atomicAdd(p + 1, v.y);
  if (n > 2) atomicAdd(p + 2, v.z);
  if (n > 3) atomicAdd(p + 3, v.w);
}

__global__ void __launch_bounds__(256) samples_fwd_kernel(SampleArgs a, Batch B) {
  const PosArgs& p = a.pos;
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= int64_t(p.L) * B.pix_prefix[B.n]) return;
  const PixelRef r = decode(B, p.L, q);
  const float W = __int2float_rn(B.width[r.img]), H = __int2float_rn(B.height[r.img]);
  const int K = a.K;
  const bool vec_rows = (K & 3) == 0;
  float4 c = make_float4(0.0f, 0.0f, 1.0f, 1.0f);
  float fg = 0.0f;
  float* o = a.attr_out + r.e * K;
  const SampleRef sr = load_sample(p, r.e);
  if (sr.z != 1.0f) {
    fg = 1.0f;
    const Interp it = interpolate_clip(p, B, r.img, sr);
    c = it.c;
    const float* ab = a.attr + B.vertex_offset[r.img] * K;
    const float* a0 = ab + int64_t(it.vid[0]) * K;
    const float* a1 = ab + int64_t(it.vid[1]) * K;
    const float* a2 = ab + int64_t(it.vid[2]) * K;
    for (int k = 0; k < K; k += 4) {
      const int n = min(4, K - k);
      const float4 x = load_chunk(a0 + k, n, vec_rows), y = load_chunk(a1 + k, n, vec_rows),
                   z = load_chunk(a2 + k, n, vec_rows);
      store_chunk(o + k,
                  make_float4(lerp3(x.x, y.x, z.x, it.b), lerp3(x.y, y.y, z.y, it.b),
                              lerp3(x.z, y.z, z.z, it.b), lerp3(x.w, y.w, z.w, it.b)),
                  n, vec_rows);
    }
  } else {
    for (int k = 0; k < K; k += 4)
      store_chunk(o + k, make_float4(0.0f, 0.0f, 0.0f, 0.0f), min(4, K - k), vec_rows);
  }
  p.vp[r.e] = viewport_of(c, W, H, fg);
}

// Sum of v over lanes lane..last of the calling lane's run (runs are
// contiguous lanes; `last` is the run's final lane): afterwards each run's
// first lane holds its total. Every lane of the warp must call it. kSteps
// shuffle steps (d = 1, 2, 4, ...) cover runs of up to 2^kSteps lanes: steps
// with d above every lane's last - lane add nothing, so a warp whose runs
// are short takes fewer steps and gets the same bits.
template <int kSteps>
__device__ __forceinline__ float run_sum(float v, int lane, int last) {
#pragma unroll
  for (int k = 0; k < kSteps; ++k) {
    const int d = 1 << k;
    const float t = __shfl_down_sync(0xffffffffu, v, d);
    if (lane + d <= last) v += t;
  }
  return v;
}

template <int kSteps>
__device__ __forceinline__ float4 run_sum4(float4 v, int lane, int last) {
  return make_float4(run_sum<kSteps>(v.x, lane, last), run_sum<kSteps>(v.y, lane, last),
                     run_sum<kSteps>(v.z, lane, last), run_sum<kSteps>(v.w, lane, last));
}

constexpr int kVjpThreads = 512;
constexpr int kVjpPerThread = 8;  // samples whose depth each thread tests
constexpr int kVjpBlock = kVjpThreads * kVjpPerThread;

// The run-summed scatter of one compacted foreground sample per lane into
// the vertex gradients (clip and attributes) and its barycentric adjoint
// db; kSteps as in run_sum. Every lane of the warp calls it.
// kMode 0 adds with float atomics; kMode 2 adds in fixed point at exponent
// `scale` (float atomics for kFixedFloat; nothing for kFixedZero, as only
// zeros would be added). The first deterministic pass (kMode 1) does not
// get here.
template <int kSteps, int kMode>
__device__ __forceinline__ void scatter_runs(const SampleArgs& a, const PosArgs& p,
                                             const Batch& B, int lane, int last, bool leader,
                                             bool on, int im, int64_t el, const float (&b)[3],
                                             const int (&vid)[3], const float4 (&V)[3],
                                             float4 dcl, float (&db)[3], float& mx,
                                             int scale) {
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float bi = b[i];
    float4 cv = make_float4(bi * dcl.x, bi * dcl.y, 0.0f, bi * dcl.w);
    cv.x = run_sum<kSteps>(cv.x, lane, last);
    cv.y = run_sum<kSteps>(cv.y, lane, last);
    cv.w = run_sum<kSteps>(cv.w, lane, last);
    if (kMode == 2 && scale != kFixedFloat) {
      if (leader && on && scale != kFixedZero) {
        unsigned long long* q = a.fx_clip + 4 * (B.vertex_offset[im] + vid[i]);
        add_fixed(q, cv.x, scale);
        add_fixed(q + 1, cv.y, scale);
        add_fixed(q + 3, cv.w, scale);
      }
    } else if (leader && on && (cv.x != 0.0f || cv.y != 0.0f || cv.w != 0.0f)) {
      atomicAdd(p.d_clip + B.vertex_offset[im] + vid[i], cv);
    }
    db[i] = on ? V[i].x * dcl.x + V[i].y * dcl.y + V[i].w * dcl.w : 0.0f;
  }
  if (a.d_attr_out) {
    const int K = a.K;
    const bool vec_rows = (K & 3) == 0;
    const float* src = a.d_attr_out + el * K;
    const int64_t aoff = on ? B.vertex_offset[im] * K : 0;
    for (int kk = 0; kk < K; kk += 4) {
      const int nc = min(4, K - kk);
      const float4 ga = on ? load_chunk(src + kk, nc, vec_rows) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
#pragma unroll
      for (int i = 0; i < 3; ++i) {
        const float bi = b[i];
        float4 av = make_float4(bi * ga.x, bi * ga.y, bi * ga.z, bi * ga.w);
        av = run_sum4<kSteps>(av, lane, last);
        const int64_t row = aoff + int64_t(vid[i]) * K + kk;
        if (kMode == 2 && scale != kFixedFloat) {
          if (leader && on && scale != kFixedZero) {
            const float vv[4] = {av.x, av.y, av.z, av.w};
            for (int c = 0; c < nc; ++c) add_fixed(a.fx_attr + row + c, vv[c], scale);
          }
        } else if (leader && on) {
          add_chunk(a.d_attr + row, av, nc, vec_rows);
        }
        if (on && p.d_bary) {
          const float4 at = load_chunk(a.attr + row, nc, vec_rows);
          db[i] += at.x * ga.x + at.y * ga.y + at.z * ga.z + at.w * ga.w;
        }
      }
    }
  }
}

// VJP of the interpolation and the splat positions. A block takes kVjpBlock
// consecutive layer samples: each thread tests the depth of kVjpPerThread of
// them, the foreground ones (z != 1) are compacted in shared memory in
// sample order, and the block's threads then work on those densely (for
// mostly-background images most samples cost one depth read). Consecutive
// lanes then hold consecutive foreground samples, which mostly share a
// triangle, and every sample of a triangle adds into the same three vertex
// rows: contributions are summed over each run of lanes with the same
// triangle and only the run's first lane issues the atomics (same-address
// atomics serialize in L2).
template <int kMode>
__global__ void __launch_bounds__(kVjpThreads) samples_bwd_kernel(SampleArgs a, Batch B) {
  __shared__ int64_t s_e[kVjpBlock];
  __shared__ unsigned char s_img[kVjpBlock];
  __shared__ int s_warp[kVjpThreads / 32];
  const PosArgs& p = a.pos;
  const int lane = threadIdx.x & 31;
  const int scale = kMode == 2 ? fixed_exponent(a) : 0;
  float mx = 0.0f;  // kMode 1: largest magnitude this thread would add
  const int64_t total = int64_t(p.L) * B.pix_prefix[B.n];
  const int64_t q0 = int64_t(blockIdx.x) * kVjpBlock + int64_t(threadIdx.x) * kVjpPerThread;
  int img[kVjpPerThread];
  int64_t e[kVjpPerThread];
  bool fg[kVjpPerThread];
  int nfg = 0;
  // The thread's samples are consecutive: find the first one's image, then
  // step to the next image only where a sample crosses into it.
  int cur = 0;
  int64_t cur_end = 0, local0 = 0;
  if (q0 < total) {
    cur = locate(B, p.L, q0, local0);
    cur_end = int64_t(p.L) * B.pix_prefix[cur + 1];
  }
#pragma unroll
  for (int u = 0; u < kVjpPerThread; ++u) {
    const int64_t q = q0 + u;
    img[u] = 0;
    e[u] = 0;
    fg[u] = false;
    if (q < total) {
      while (q >= cur_end) {
        ++cur;
        cur_end = int64_t(p.L) * B.pix_prefix[cur + 1];
      }
      img[u] = cur;
      e[u] = int64_t(p.L) * B.pix_off[cur] + (q - int64_t(p.L) * B.pix_prefix[cur]);
    }
  }
#pragma unroll
  for (int u = 0; u < kVjpPerThread; ++u) {
    if (q0 + u < total) {
      fg[u] = __ldg(p.z + e[u]) != 1.0f;
      nfg += fg[u];
    }
  }
  if (p.d_bary) {
#pragma unroll
    for (int u = 0; u < kVjpPerThread; ++u)
      if (q0 + u < total && !fg[u]) {
        p.d_bary[3 * e[u]] = 0.0f;
        p.d_bary[3 * e[u] + 1] = 0.0f;
        p.d_bary[3 * e[u] + 2] = 0.0f;
      }
  }
  int slot;
  const int n = block_exclusive_scan<kVjpThreads>(nfg, s_warp, slot);
  if (n == 0) return;
#pragma unroll
  for (int u = 0; u < kVjpPerThread; ++u)
    if (fg[u]) {
      s_e[slot] = e[u];
      s_img[slot] = (unsigned char)img[u];
      ++slot;
    }
  __syncthreads();

  for (int k0 = 0; k0 < n; k0 += kVjpThreads) {
    const int k = k0 + threadIdx.x;
    const bool on = k < n;
    const int im = on ? s_img[k] : 0;
    const int64_t el = on ? s_e[k] : 0;
    int id = -1;
    float b[3] = {0.0f, 0.0f, 0.0f};
    int vid[3] = {0, 0, 0};
    float4 V[3] = {make_float4(0.0f, 0.0f, 0.0f, 1.0f), make_float4(0.0f, 0.0f, 0.0f, 1.0f),
                   make_float4(0.0f, 0.0f, 0.0f, 1.0f)};
    float4 dcl = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (on) {
#pragma unroll
      for (int i = 0; i < 3; ++i) b[i] = __ldg(p.bary + 3 * el + i);
      const float2 g =
          p.dvp ? __ldg(reinterpret_cast<const float2*>(p.dvp + el)) : make_float2(0.0f, 0.0f);
      if (a.vid) {
        // Vertex indices stored by the rasterizer: no triangle gather.
#pragma unroll
        for (int i = 0; i < 3; ++i) vid[i] = __ldg(a.vid + 3 * el + i);
        id = vid[0];
      } else {
        id = __ldg(p.ids + el);
        const int32_t* t = p.tris + 3 * (B.triangle_offset[im] + id);
#pragma unroll
        for (int i = 0; i < 3; ++i) vid[i] = __ldg(t + i);
      }
      const float W = __int2float_rn(B.width[im]), H = __int2float_rn(B.height[im]);
      const float dnx = g.x * W * 0.5f, dny = g.y * H * 0.5f;
      const bool moved = g.x != 0.0f || g.y != 0.0f;
      if (a.vp && !p.d_bary) {
        // From the stored position: ndc = 2 viewport / (W, H) - 1, and the
        // clip w it carries (no vertex gathers).
        if (moved) {
          const float4 q = __ldg(a.vp + el);
          const float nx = q.x * (2.0f / W) - 1.0f, ny = q.y * (2.0f / H) - 1.0f;
          dcl = make_float4(dnx / q.w, dny / q.w, 0.0f, -(dnx * nx + dny * ny) / q.w);
        }
      } else {
        const float4* vb = p.clip + B.vertex_offset[im];
#pragma unroll
        for (int i = 0; i < 3; ++i) V[i] = __ldg(vb + vid[i]);
        if (moved) {
          // (c0 b0 + c1 b1) + c2 b2 of the clip coordinates
          // (interpolate.py:24-63); viewport z carries no gradient (it only
          // enters comparisons).
          const float4 c = lerp_clip(V[0], V[1], V[2], b);
          dcl = make_float4(dnx / c.w, dny / c.w, 0.0f, -(dnx * c.x + dny * c.y) / (c.w * c.w));
        }
      }
    }
    if (kMode == 1) {
      // First deterministic pass: a bound on what the run sums add. A run
      // sum adds at most 32 lanes' values (each |b_i x| <= |x| max b), so
      // 2^kRunBits times the largest per-sample value bounds it.
      if (on) {
        const float bm = fmaxf(fabsf(b[0]), fmaxf(fabsf(b[1]), fabsf(b[2])));
        float m = fmaxf(fixed_mag(dcl.x), fmaxf(fixed_mag(dcl.y), fixed_mag(dcl.w)));
        if (a.d_attr_out) {
          const float* src = a.d_attr_out + el * a.K;
          for (int c = 0; c < a.K; ++c) m = fmaxf(m, fixed_mag(__ldg(src + c)));
        }
        mx = fmaxf(mx, m * fixed_mag(bm));
      }
      continue;
    }
    // Runs of lanes with the same image and the same three vertex rows are
    // summed by shuffles and only each run's first lane issues the atomics
    // (measured faster than atomics from every lane even for warps of many
    // short runs). All four shuffles run on every lane before any comparison.
    const int kim = on ? im : -1;
    const int p_im = __shfl_up_sync(0xffffffffu, kim, 1);
    const int p_v0 = __shfl_up_sync(0xffffffffu, vid[0], 1);
    const int p_v1 = __shfl_up_sync(0xffffffffu, vid[1], 1);
    const int p_v2 = __shfl_up_sync(0xffffffffu, vid[2], 1);
    const bool differs = (kim != p_im) | (vid[0] != p_v0) | (vid[1] != p_v1) | (vid[2] != p_v2);
    (void)id;
    const unsigned heads = __ballot_sync(0xffffffffu, lane == 0 || differs);
    const unsigned later = heads & ~((2u << lane) - 1u);  // heads after this lane
    const int last = later ? __ffs(later) - 2 : 31;
    const bool leader = ((heads >> lane) & 1u) != 0;
    // Shuffle steps for the warp's longest run (warp-uniform).
    const unsigned span = __reduce_max_sync(0xffffffffu, unsigned(last - lane));
    float db[3];
    if (span == 0)
      scatter_runs<0, kMode>(a, p, B, lane, last, leader, on, im, el, b, vid, V, dcl, db, mx,
                             scale);
    else if (span < 2)
      scatter_runs<1, kMode>(a, p, B, lane, last, leader, on, im, el, b, vid, V, dcl, db, mx,
                             scale);
    else if (span < 4)
      scatter_runs<2, kMode>(a, p, B, lane, last, leader, on, im, el, b, vid, V, dcl, db, mx,
                             scale);
    else if (span < 8)
      scatter_runs<3, kMode>(a, p, B, lane, last, leader, on, im, el, b, vid, V, dcl, db, mx,
                             scale);
    else
      scatter_runs<5, kMode>(a, p, B, lane, last, leader, on, im, el, b, vid, V, dcl, db, mx,
                             scale);
    if (on && p.d_bary) {
      p.d_bary[3 * el] = db[0];
      p.d_bary[3 * el + 1] = db[1];
      p.d_bary[3 * el + 2] = db[2];
    }
  }
  if (kMode == 1) {
    // magnitudes are >= 0 (or +inf), so their bits order as the values do
    const unsigned wm = __reduce_max_sync(0xffffffffu, __float_as_uint(mx));
    if (lane == 0 && wm != 0u) atomicMax(a.fx_max, wm);
  }
}

// Deterministic sums back to float, added to the gradients (one thread per
// vertex).
__global__ void __launch_bounds__(256) fixed_finalize_kernel(SampleArgs a, int64_t nv) {
  const int64_t v = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int e = fixed_exponent(a);
  if (e == kFixedZero || e == kFixedFloat) return;  // zeros, or float atomics took over
  // the sum rounded to float, then scaled by 2^-e (exact unless subnormal)
  const auto back = [e](unsigned long long q) { return fixed_back(q, e); };
  const unsigned long long* q = a.fx_clip + 4 * v;
  float4 d = a.pos.d_clip[v];
  d.x += back(q[0]);
  d.y += back(q[1]);
  d.w += back(q[3]);
  a.pos.d_clip[v] = d;
  if (a.d_attr)
    for (int k = 0; k < a.K; ++k) a.d_attr[v * a.K + k] += back(a.fx_attr[v * a.K + k]);
}

// -------------------------------------------------------------------- splat
struct SplatArgs {
  const float4* vp;  // [L*P] viewport xyz + foreground flag
  const float* zb;   // [L*P] rasterizer depth (nullable): 1 = background
  const float* colors;
  int L;
  int64_t P;     // pixels covered by the call: plane stride of `saved`
  float coef;
  float* out;
  float* saved;  // [3 (C+1) + 2, P] planar accumulators, surface codes and
                 // the tile list (forward out; the backward reads it and
                 // resets its own work counter in it)
  float* accum;
  float* normalized;
  const float* d_out;
  float* d_colors;
  float4* d_vp;
  bool fg_grads;  // DR_SPLAT_FOREGROUND_GRADIENTS: background d_colors unwritten
};

// A block covers a kTX x kTY tile of pixels, one per thread; the samples it
// reads are the tile plus a 1-pixel halo: kRS x (kTY + 2) per layer.
constexpr int kRS = kTX + 2;
constexpr int kRR = kRS * (kTY + 2);

// Colors travel through shared memory as float4 groups, zero padded to a
// multiple of 4 channels, so that one 128-bit load fetches four channels.
template <int C>
struct Groups {
  static constexpr int Q = (C + 3) / 4;
};

// Separable tap weights of a sample (splat.py:106-115): tap (u, v) weighs
// ex[u+1] * ey[v+1] with ex = fg * coef * exp(-2 dx^2), ey = exp(-2 dy^2),
// dx = floor(x) + 0.5 - x + u. Equal to the reference's
// fg * coef * exp(-2 (dx^2 + dy^2)) up to float rounding: the fast
// exponential's relative error is below 1e-6 for these arguments
// (|2 dx^2| <= 4.5), well inside the path's 1e-5 tolerance. The forward and
// the VJP use this same function, so they see identical weights.
struct Taps {
  float ex[3], ey[3];
  float d0, d1;
};

// `fg` is the foreground weight of the sample (the mask value; 1 for
// positions from the rasterizer, whose w holds the clip w instead).
__device__ __forceinline__ Taps taps_of(float4 q, float fg, float coef) {
  Taps t;
  t.d0 = __fsub_rn(__fadd_rn(floorf(q.x), 0.5f), q.x);
  t.d1 = __fsub_rn(__fadd_rn(floorf(q.y), 0.5f), q.y);
  const float fc = __fmul_rn(fg, coef);
#pragma unroll
  for (int u = 0; u < 3; ++u) {
    const float dx = __fadd_rn(t.d0, float(u - 1)), dy = __fadd_rn(t.d1, float(u - 1));
    t.ex[u] = fg != 0.0f ? __fmul_rn(fc, __expf(__fmul_rn(-2.0f, __fmul_rn(dx, dx)))) : 0.0f;
    t.ey[u] = fg != 0.0f ? __expf(__fmul_rn(-2.0f, __fmul_rn(dy, dy))) : 0.0f;
  }
  return t;
}

// Foreground weight of a loaded sample: from the depth buffer when there is
// one (the position's w is then the clip w), else the position's w.
__device__ __forceinline__ float fg_weight(bool zb, bool fg_bit, float4 q) {
  return zb ? (fg_bit ? 1.0f : 0.0f) : q.w;
}

template <int C>
__device__ __forceinline__ void load_row(const float* p, float* v) {
  if constexpr (C % 4 == 0) {
#pragma unroll
    for (int c = 0; c < C; c += 4) {
      const float4 q = __ldg(reinterpret_cast<const float4*>(p + c));
      v[c] = q.x; v[c + 1] = q.y; v[c + 2] = q.z; v[c + 3] = q.w;
    }
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c) v[c] = __ldg(p + c);
  }
}

template <int C>
__device__ __forceinline__ void store_row(float* p, const float* v) {
  if constexpr (C % 4 == 0) {
#pragma unroll
    for (int c = 0; c < C; c += 4)
      *reinterpret_cast<float4*>(p + c) = make_float4(v[c], v[c + 1], v[c + 2], v[c + 3]);
  } else {
#pragma unroll
    for (int c = 0; c < C; ++c) p[c] = v[c];
  }
}

// A color row as zero-padded float4 groups.
template <int C>
__device__ __forceinline__ void load_groups(const float* p, float4* g) {
  constexpr int Q = Groups<C>::Q;
  float v[4 * Q];
#pragma unroll
  for (int c = C; c < 4 * Q; ++c) v[c] = 0.0f;
  load_row<C>(p, v);
#pragma unroll
  for (int q = 0; q < Q; ++q) g[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
}

// Position of the (r + 1)-th set bit of m (r < popc(m)), by halving
// (measured a little faster than __fns here).
__device__ __forceinline__ int nth_set_bit(unsigned m, int r) {
  int pos = 0, c;
  c = __popc(m & 0xffffu); if (r >= c) { r -= c; pos += 16; m >>= 16; }
  c = __popc(m & 0xffu); if (r >= c) { r -= c; pos += 8; m >>= 8; }
  c = __popc(m & 0xfu); if (r >= c) { r -= c; pos += 4; m >>= 4; }
  c = __popc(m & 0x3u); if (r >= c) { r -= c; pos += 2; m >>= 2; }
  c = int(m & 1u); if (r >= c) pos += 1;
  return pos;
}

struct TileRef {
  int img, x0, y0;
};

__device__ __forceinline__ TileRef tile_at(const Batch& B, int item) {
  TileRef t;
  t.img = find_segment(B.tile_start, B.n, item);
  const int local = item - B.tile_start[t.img];
  const int ntx = B.tiles_x[t.img];
  t.x0 = (local % ntx) * kTX;
  t.y0 = (local / ntx) * kTY;
  return t;
}

__device__ __forceinline__ TileRef tile_of(const Batch& B) { return tile_at(B, blockIdx.x); }

// The tiles of a splat call whose sample region (tile + 1-pixel halo) holds
// a foreground sample, listed by splat_classify_kernel; the heavy splat
// kernels then run only on those, and the empty tiles' outputs are zeros.
struct TileList {
  unsigned* count;      // [0] tiles listed, [1] / [2] work counters of the
                        // forward / backward kernels over the list
  int* list;            // listed tile items (in any order)
  unsigned char* flag;  // per tile: 1 when listed
};

// Surface index of the splat from sample s reaching pixel p
// (splat.py:131-145): c = argmin_k |zS_k - zD_0|, t = argmin_k |zD_k - zS_0|
// (first index on ties); -t if the tap match is strictly better, else c.
// z holds every layer's depth, layer k at z[k * kRR + i].
__device__ __forceinline__ int surface_index(const float* z, int s, int p, int L) {
  const float zD0 = z[p], zS0 = z[s];
  float minc = fabsf(__fsub_rn(zS0, zD0));
  float mint = minc;
  int c = 0, t = 0;
  for (int k = 1; k < L; ++k) {
    const float dc = fabsf(__fsub_rn(z[k * kRR + s], zD0));
    if (dc < minc) { minc = dc; c = k; }
    const float dt = fabsf(__fsub_rn(z[k * kRR + p], zS0));
    if (dt < mint) { mint = dt; t = k; }
  }
  return mint < minc ? -t : c;
}

// normalization_scales = 1 / (max(W - 1, 0) + 1)   (splat.py:168-169);
// __frcp_rn is the correctly rounded reciprocal, the same value as the
// division.
__device__ __forceinline__ float norm_scale(float w) {
  return __frcp_rn(__fadd_rn(fmaxf(__fsub_rn(w, 1.0f), 0.0f), 1.0f));
}

// acc += w * color over the float4 groups, two channels per packed f32x2 FMA.
template <int Q>
__device__ __forceinline__ void accumulate(float2 (&acc)[2 * Q], float& wacc, const float4* c,
                                           float w) {
  const float2 w2 = make_float2(w, w);
#pragma unroll
  for (int q = 0; q < Q; ++q) {
    acc[2 * q] = __ffma2_rn(w2, make_float2(c[q].x, c[q].y), acc[2 * q]);
    acc[2 * q + 1] = __ffma2_rn(w2, make_float2(c[q].z, c[q].w), acc[2 * q + 1]);
  }
  wacc = __fadd_rn(wacc, w);
}

// Forward: per halo sample, every layer's depth and a mask of its
// foreground layers, and for foreground layers the separable tap weights and
// the color go to shared memory,
//   z[l][i], wx[l][u][i], wy[l][v][i] (floats), col[l][q][i] (float4),
//   fgm[i] (bit l set when layer l of sample i is foreground),
// every array indexed by the region sample i so that a warp reads
// consecutive words; then each pixel gathers the 9 taps of every layer with
// the per-tap surface test, normalizes, composites and stores. Background
// samples weigh nothing, so their weights and colors are never written or
// read, and a tile whose region holds no foreground sample writes zeros.
// LT > 0 fixes the layer count at compile time (the common L = 3 case), so
// the layer loops unroll; LT = 0 reads it from the arguments.
template <int C, int LT>
__device__ __forceinline__ void splat_fwd_tile(const SplatArgs& a, const Batch& B, int item,
                                               float* smem, unsigned& s_layers) {
  constexpr int Q = Groups<C>::Q;
  const TileRef tr = tile_at(B, item);
  const int L = LT > 0 ? LT : a.L;
  float* zs = smem;
  float* wx = zs + L * kRR;
  float* wy = wx + 3 * L * kRR;
  float4* col = reinterpret_cast<float4*>(wy + 3 * L * kRR);
  // 8-bit masks while L <= 8 (keeps five 256-thread blocks per SM at C = 4).
  unsigned char* fgm8 = reinterpret_cast<unsigned char*>(col + Q * L * kRR);
  unsigned short* fgm16 = reinterpret_cast<unsigned short*>(fgm8);
  const bool wide = L > 8;
  const int W = B.width[tr.img], H = B.height[tr.img];
  if (threadIdx.x == 0) s_layers = 0u;
  __syncthreads();
  {
    const int64_t HW = int64_t(W) * H;
    const int64_t base = int64_t(L) * B.pix_off[tr.img];
    unsigned any = 0;
    // Every depth of the thread's region samples is in flight at once; then
    // only the positions and colors of foreground layers are read.
    constexpr int kIt = (kRR + kTX * kTY - 1) / (kTX * kTY);
    unsigned mk[kIt];
#pragma unroll
    for (int k = 0; k < kIt; ++k) {
      const int i = threadIdx.x + k * kTX * kTY;
      const int ry = i / kRS;
      const int x = tr.x0 - 1 + (i - ry * kRS), y = tr.y0 - 1 + ry;
      const bool in = i < kRR && x >= 0 && y >= 0 && x < W && y < H;
      const int64_t e0 = base + int64_t(y) * W + x;
      mk[k] = 0;
      if (in && a.zb)
        for (int l = 0; l < L; ++l) mk[k] |= unsigned(__ldg(a.zb + e0 + l * HW) != 1.0f) << l;
    }
    if (LT > 0 && a.zb) {
      // The warp's foreground (sample, layer) pairs are spread over its
      // lanes: lane t takes the t-th set bit of the per-layer ballots, so
      // the position and color loads and the tap weights run on full warps.
      const int lane = threadIdx.x & 31;
#pragma unroll
      for (int k = 0; k < kIt; ++k) {
        const int i = threadIdx.x + k * kTX * kTY;
        const bool valid = i < kRR;
        const unsigned m = valid ? mk[k] : 0u;
        if (valid) {
          for (int l = 0; l < L; ++l)
            if (!((m >> l) & 1u)) zs[l * kRR + i] = 1.0f;
          fgm8[i] = (unsigned char)m;
        }
        any |= m;
        unsigned masks[LT > 0 ? LT : 1];
        int total = 0;
#pragma unroll
        for (int l = 0; l < (LT > 0 ? LT : 1); ++l) {
          masks[l] = __ballot_sync(0xffffffffu, (m >> l) & 1u);
          total += __popc(masks[l]);
        }
        const int wbase = (threadIdx.x & ~31) + k * kTX * kTY;
        for (int t = lane; t < total; t += 32) {
          int l = 0, r = t;
#pragma unroll
          for (int ll = 0; ll < (LT > 0 ? LT : 1) - 1; ++ll)
            if (l == ll && r >= __popc(masks[ll])) { r -= __popc(masks[ll]); l = ll + 1; }
          unsigned ml = masks[0];
#pragma unroll
          for (int ll = 1; ll < (LT > 0 ? LT : 1); ++ll)
            if (l == ll) ml = masks[ll];
          const int src = nth_set_bit(ml, r);
          const int ii = wbase + src;
          const int ry = ii / kRS;
          const int x = tr.x0 - 1 + (ii - ry * kRS), y = tr.y0 - 1 + ry;
          const int64_t e = base + int64_t(y) * W + x + l * HW;
          const float4 q = __ldg(a.vp + e);
          float4 c[Q];
          load_groups<C>(a.colors + e * C, c);
          zs[l * kRR + ii] = q.z;
          const Taps tp = taps_of(q, 1.0f, a.coef);
#pragma unroll
          for (int u = 0; u < 3; ++u) {
            wx[(l * 3 + u) * kRR + ii] = tp.ex[u];
            wy[(l * 3 + u) * kRR + ii] = tp.ey[u];
          }
#pragma unroll
          for (int g = 0; g < Q; ++g) col[(l * Q + g) * kRR + ii] = c[g];
        }
      }
    } else
#pragma unroll
    for (int k = 0; k < kIt; ++k) {
      const int i = threadIdx.x + k * kTX * kTY;
      if (i >= kRR) break;
      unsigned m = mk[k];
      const int ry = i / kRS;
      const int x = tr.x0 - 1 + (i - ry * kRS), y = tr.y0 - 1 + ry;
      const bool in = x >= 0 && y >= 0 && x < W && y < H;
      const int64_t e0 = base + int64_t(y) * W + x;
      for (int l = 0; l < L; ++l) {
        float4 q = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
        const bool fgbit = in && ((m >> l) & 1u);
        if (in && (!a.zb || fgbit)) q = __ldg(a.vp + e0 + l * HW);
        float4 c[Q];
        // with a depth buffer the color load need not wait for the position
        if (a.zb && fgbit) load_groups<C>(a.colors + (e0 + l * HW) * C, c);
        zs[l * kRR + i] = q.z;
        const float fgw = fg_weight(a.zb != nullptr, fgbit, q);
        if (fgw != 0.0f) {
          m |= 1u << l;
          const Taps t = taps_of(q, fgw, a.coef);
#pragma unroll
          for (int u = 0; u < 3; ++u) {
            wx[(l * 3 + u) * kRR + i] = t.ex[u];
            wy[(l * 3 + u) * kRR + i] = t.ey[u];
          }
          if (!a.zb) load_groups<C>(a.colors + (e0 + l * HW) * C, c);
#pragma unroll
          for (int g = 0; g < Q; ++g) col[(l * Q + g) * kRR + i] = c[g];
        }
      }
      if (wide)
        fgm16[i] = (unsigned short)m;
      else
        fgm8[i] = (unsigned char)m;
      any |= m;
    }
    any = __reduce_or_sync(0xffffffffu, any);
    if ((threadIdx.x & 31) == 0 && any) atomicOr(&s_layers, any);
  }
  __syncthreads();
  const unsigned layers = s_layers;

  const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
  const int px = tr.x0 + tx, py = tr.y0 + ty;
  if (px >= W || py >= H) return;
  const int p = (ty + 1) * kRS + tx + 1;
  const int64_t pix = B.pix_off[tr.img] + int64_t(py) * W + px;

  float acc[3][4 * Q];
  float wacc[3] = {0.0f, 0.0f, 0.0f};
  unsigned code = 0;  // surface codes of the 9 taps (three layers only)
  if (layers == 0) {
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int c = 0; c < 4 * Q; ++c) acc[k][c] = 0.0f;
  } else {
    // Per tap: the foreground layers of the sample behind it (bits 0-15, 0
    // outside the image) and, where it carries any weight, its surface
    // index + 16 (bits 16+). Tap j = (u + 1) * 3 + (v + 1) comes from the
    // sample at p - (u, v).
    unsigned tap[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) {
      const int u = j / 3 - 1, v = j % 3 - 1;
      const int sx = px - u, sy = py - v;
      const bool in = sx >= 0 && sy >= 0 && sx < W && sy < H;
      const int s = p - v * kRS - u;
      const unsigned m = in ? (wide ? unsigned(fgm16[s]) : unsigned(fgm8[s])) : 0u;
      // The center tap (s == p) always has surface index 0: both argmins
      // start at a zero (or NaN) difference that no layer beats.
      tap[j] = m ? m | (unsigned((j == 4 ? 0 : surface_index(zs, s, p, L)) + 16) << 16) : 0u;
      // Surface index + 2 in 3 bits per tap (three layers: -2..2) for the
      // VJP, which then needs no depths.
      if (LT == 3 && tap[j]) code |= ((tap[j] >> 16) - 14u) << (3 * j);
    }
    // Class 0 = in front of the surface, 1 = at it, 2 = behind it
    // (splat.py:149-162), accumulated layer by layer.
    float2 acc0[2 * Q], acc1[2 * Q], acc2[2 * Q];
#pragma unroll
    for (int h = 0; h < 2 * Q; ++h) {
      acc0[h] = make_float2(0.0f, 0.0f);
      acc1[h] = acc0[h];
      acc2[h] = acc0[h];
    }
    for (int l = 0; l < L; ++l) {
      if (!((layers >> l) & 1u)) continue;
#pragma unroll
      for (int j = 0; j < 9; ++j) {
        if (!((tap[j] >> l) & 1u)) continue;
        const int sj = int(tap[j] >> 16) - 16;
        const int u = j / 3 - 1, v = j % 3 - 1;
        const int s = p - v * kRS - u;
        const float w = __fmul_rn(wx[(l * 3 + u + 1) * kRR + s], wy[(l * 3 + v + 1) * kRR + s]);
        float4 c[Q];
#pragma unroll
        for (int g = 0; g < Q; ++g) c[g] = col[(l * Q + g) * kRR + s];
        if (sj > l)
          accumulate<Q>(acc0, wacc[0], c, w);
        else if (sj == l)
          accumulate<Q>(acc1, wacc[1], c, w);
        else
          accumulate<Q>(acc2, wacc[2], c, w);
      }
    }
#pragma unroll
    for (int h = 0; h < 2 * Q; ++h) {
      acc[0][2 * h] = acc0[h].x; acc[0][2 * h + 1] = acc0[h].y;
      acc[1][2 * h] = acc1[h].x; acc[1][2 * h + 1] = acc1[h].y;
      acc[2][2 * h] = acc2[h].x; acc[2][2 * h + 1] = acc2[h].y;
    }
  }

  float n[3][C];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float sc = norm_scale(wacc[k]);
#pragma unroll
    for (int c = 0; c < C; ++c) n[k][c] = __fmul_rn(acc[k][c], sc);
  }
  // over: out = n2; out = n1 + (1 - a1) out; out = n0 + (1 - a0) out
  const float t1 = __fsub_rn(1.0f, n[1][C - 1]), t0 = __fsub_rn(1.0f, n[0][C - 1]);
  float o[C];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const float mid = __fadd_rn(n[1][c], __fmul_rn(t1, n[2][c]));
    o[c] = __fadd_rn(n[0][c], __fmul_rn(t0, mid));
  }
  store_row<C>(a.out + pix * C, o);
  // The backward reads a pixel's accumulators only through taps of
  // foreground samples next to it, and every such sample lies in this
  // tile's region: a region without foreground leaves them unwritten.
  if (a.saved && layers != 0) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
#pragma unroll
      for (int c = 0; c < C; ++c) a.saved[(k * (C + 1) + c) * a.P + pix] = acc[k][c];
      a.saved[(k * (C + 1) + C) * a.P + pix] = wacc[k];
    }
    if (LT == 3) reinterpret_cast<unsigned*>(a.saved)[3 * (C + 1) * a.P + pix] = code;
  }
  if (a.accum || a.normalized) {
    const int64_t HW = int64_t(W) * H;
    const int64_t base = 3 * B.pix_off[tr.img] * C + (int64_t(py) * W + px) * C;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      if (a.accum) store_row<C>(a.accum + base + k * HW * C, acc[k]);
      if (a.normalized) store_row<C>(a.normalized + base + k * HW * C, n[k]);
    }
  }
}

// One block per tile.
template <int C, int LT>
__global__ void __launch_bounds__(256, C <= 4 ? 5 : 3) splat_fwd_kernel(SplatArgs a, Batch B) {
  extern __shared__ __align__(16) float smem[];
  __shared__ unsigned s_layers;
  splat_fwd_tile<C, LT>(a, B, blockIdx.x, smem, s_layers);
}

// Persistent blocks over the listed tiles; a work counter hands them out.
template <int C, int LT>
__global__ void __launch_bounds__(256, C <= 4 ? 5 : 3)
    splat_fwd_list_kernel(SplatArgs a, Batch B, TileList t) {
  extern __shared__ __align__(16) float smem[];
  __shared__ unsigned s_layers;
  __shared__ int s_item;
  const int n = int(t.count[0]);
  for (;;) {
    if (threadIdx.x == 0) s_item = int(atomicAdd(t.count + 1, 1u));
    __syncthreads();
    const int w = s_item;
    if (w >= n) break;
    splat_fwd_tile<C, LT>(a, B, t.list[w], smem, s_layers);
    __syncthreads();
  }
}

// One warp per tile: lists the tiles whose region holds a foreground
// sample (its layer 0 is foreground: layers fill front to back, so a
// background layer 0 has only background behind it) and writes zeros to
// the image of the others.
template <int C>
__global__ void __launch_bounds__(256) splat_classify_kernel(SplatArgs a, Batch B, TileList t,
                                                             int tiles) {
  const int item = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (item >= tiles) return;
  const int lane = threadIdx.x & 31;
  const TileRef tr = tile_at(B, item);
  const int W = B.width[tr.img], H = B.height[tr.img];
  const int64_t base = int64_t(a.L) * B.pix_off[tr.img];
  bool fg = false;
#pragma unroll 4
  for (int i = lane; i < kRR; i += 32) {
    const int ry = i / kRS;
    const int x = tr.x0 - 1 + (i - ry * kRS), y = tr.y0 - 1 + ry;
    if (x >= 0 && y >= 0 && x < W && y < H) fg |= __ldg(a.zb + base + int64_t(y) * W + x) != 1.0f;
  }
  fg = __any_sync(0xffffffffu, fg);
  if (lane == 0) {
    t.flag[item] = fg ? 1 : 0;
    if (fg) t.list[atomicAdd(t.count, 1u)] = item;
  }
  if (fg) return;
  float zero[C];
#pragma unroll
  for (int c = 0; c < C; ++c) zero[c] = 0.0f;
  for (int p = lane; p < kTX * kTY; p += 32) {
    const int px = tr.x0 + p % kTX, py = tr.y0 + p / kTX;
    if (px < W && py < H) store_row<C>(a.out + (B.pix_off[tr.img] + int64_t(py) * W + px) * C, zero);
  }
}

// Adjoints of the accumulators at one pixel, from d_out through the over
// compositing and the normalization (jnp.maximum splits its gradient 0.5 /
// 0.5 at equality, as lax.max does).
template <int C>
__device__ __forceinline__ void accum_adjoint(const float acc[3][C], const float wacc[3],
                                              const float* dO, float g[3][C], float h[3]) {
  float s[3], n[3][C];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    s[k] = norm_scale(wacc[k]);
#pragma unroll
    for (int c = 0; c < C; ++c) n[k][c] = acc[k][c] * s[k];
  }
  const float a0 = n[0][C - 1], a1 = n[1][C - 1];
  float dn[3][C];
  float d_a0 = 0.0f, d_a1 = 0.0f;
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const float mid = n[1][c] + (1.0f - a1) * n[2][c];
    d_a0 -= dO[c] * mid;
    dn[0][c] = dO[c];
    const float dmid = (1.0f - a0) * dO[c];
    d_a1 -= dmid * n[2][c];
    dn[1][c] = dmid;
    dn[2][c] = (1.0f - a1) * dmid;
  }
  dn[0][C - 1] += d_a0;
  dn[1][C - 1] += d_a1;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    float ds = 0.0f;
#pragma unroll
    for (int c = 0; c < C; ++c) {
      g[k][c] = dn[k][c] * s[k];
      ds += dn[k][c] * acc[k][c];
    }
    const float x = wacc[k] - 1.0f;
    const float gate = x > 0.0f ? 1.0f : (x == 0.0f ? 0.5f : 0.0f);
    h[k] = -ds * s[k] * s[k] * gate;
  }
}

// d color (dcol, float2 pairs) and d viewport xy of one foreground sample
// from the adjoints of the 9 pixels it reached: tap (u, v) with weight
// ex[u+1] ey[v+1] lands at ring pixel s1 + (u, v) in the class its surface
// index picks.
template <int Q>
__device__ __forceinline__ void sample_adjoint(const Taps& tp, const float4* col,
                                               const int (&surf)[9], unsigned ok, int l,
                                               int s1, const float4* gs, const float* hs,
                                               float2 (&dcol)[2 * Q], float& dvx,
                                               float& dvy) {
#pragma unroll
  for (int j = 0; j < 9; ++j) {
    if (!((ok >> j) & 1)) continue;
    const int u = j / 3 - 1, v = j % 3 - 1;
    const float w = __fmul_rn(tp.ex[u + 1], tp.ey[v + 1]);
    const int k = surf[j] > l ? 0 : (surf[j] == l ? 1 : 2);
    const int at = s1 + v * kRS + u;
    const float4* gk = gs + k * Q * kRR + at;
    float dw = hs[k * kRR + at];
    const float2 w2 = make_float2(w, w);
#pragma unroll
    for (int g = 0; g < Q; ++g) {
      const float4 gv = gk[g * kRR];
      dcol[2 * g] = __ffma2_rn(w2, make_float2(gv.x, gv.y), dcol[2 * g]);
      dcol[2 * g + 1] = __ffma2_rn(w2, make_float2(gv.z, gv.w), dcol[2 * g + 1]);
      dw = fmaf(gv.x, col[g].x, fmaf(gv.y, col[g].y,
                fmaf(gv.z, col[g].z, fmaf(gv.w, col[g].w, dw))));
    }
    // d w / d (x, y) = 4 w (dx, dy): the floor carries no gradient.
    const float f = 4.0f * w * dw;
    dvx = fmaf(f, tp.d0 + float(u), dvx);
    dvy = fmaf(f, tp.d1 + float(v), dvy);
  }
}

// Backward, gather form: the adjoints of the saved accumulators of the tile
// plus a 1-pixel ring go to shared memory, g[k][q][i] (float4 groups of the
// color adjoint of class k) and h[k][i] (weight adjoint), next to every
// layer's depth z[l][i]; each sample of the tile then reads those of the 9
// pixels it reached, in the class its surface test picked, and writes
// d color and d viewport xy. No atomics. For up to four channels and three
// layers the register bound lets five blocks share an SM, the count the
// shared memory allows (a few bytes of spills, measured faster than four).
template <int C, int LT>
__device__ __forceinline__ void splat_bwd_tile(const SplatArgs& a, const Batch& B, int item,
                                               float* smem) {
  constexpr int Q = Groups<C>::Q;
  const TileRef tr = tile_at(B, item);
  const int L = LT > 0 ? LT : a.L;
  const int W = B.width[tr.img], H = B.height[tr.img];
  const int64_t HW = int64_t(W) * H;
  float* zs = smem;
  float4* gs = reinterpret_cast<float4*>(zs + L * kRR);
  float* hs = reinterpret_cast<float*>(gs + 3 * Q * kRR);
  const int64_t lbase = int64_t(L) * B.pix_off[tr.img];
  const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
  const int sx = tr.x0 + tx, sy = tr.y0 + ty;
  const bool mine = sx < W && sy < H;
  const int64_t ebase = lbase + int64_t(sy) * W + sx;
  // Background samples have no splat and so no gradient: a tile without a
  // foreground sample only writes zeros.
  // Foreground layers of this thread's own sample (bit l).
  unsigned own = 0;
  if (mine) {
    if (a.zb) {
      for (int l = 0; l < L; ++l) own |= unsigned(__ldg(a.zb + ebase + l * HW) != 1.0f) << l;
    } else {
      for (int l = 0; l < L; ++l) own |= unsigned(__ldg(&a.vp[ebase + l * HW].w) != 0.0f) << l;
    }
  }
  if (!__syncthreads_or(own != 0)) {
    if (mine && !a.fg_grads) {
      float dc[4 * Q];
#pragma unroll
      for (int c = 0; c < 4 * Q; ++c) dc[c] = 0.0f;
      for (int l = 0; l < L; ++l) {
        const int64_t e = ebase + l * HW;
        store_row<C>(a.d_colors + e * C, dc);
        if (!a.zb) a.d_vp[e] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      }
    }
    return;
  }
  for (int i = threadIdx.x; i < kRR; i += blockDim.x) {
    const int ry = i / kRS;
    const int qx = tr.x0 - 1 + (i - ry * kRS), qy = tr.y0 - 1 + ry;
    float g[3][C], h[3];
    if (qx >= 0 && qy >= 0 && qx < W && qy < H) {
      const int64_t pix = B.pix_off[tr.img] + int64_t(qy) * W + qx;
      float acc[3][C], wacc[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
#pragma unroll
        for (int c = 0; c < C; ++c) acc[k][c] = __ldg(a.saved + (k * (C + 1) + c) * a.P + pix);
        wacc[k] = __ldg(a.saved + (k * (C + 1) + C) * a.P + pix);
      }
      float d[C];
      load_row<C>(a.d_out + pix * C, d);
      accum_adjoint<C>(acc, wacc, d, g, h);
      const int64_t eq = lbase + int64_t(qy) * W + qx;
      if (LT == 3 && a.zb) {
        // The forward's surface codes of this pixel's taps replace the
        // depths (the zs area holds them).
        reinterpret_cast<unsigned*>(zs)[i] =
            __ldg(reinterpret_cast<const unsigned*>(a.saved) + 3 * (C + 1) * a.P + pix);
      } else if (a.zb) {
        unsigned m = 0;
        for (int l = 0; l < L; ++l) m |= unsigned(__ldg(a.zb + eq + l * HW) != 1.0f) << l;
        for (int l = 0; l < L; ++l)
          zs[l * kRR + i] = ((m >> l) & 1u) ? __ldg(&a.vp[eq + l * HW].z) : 1.0f;
      } else {
        for (int l = 0; l < L; ++l) zs[l * kRR + i] = __ldg(&a.vp[eq + l * HW].z);
      }
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        h[k] = 0.0f;
#pragma unroll
        for (int c = 0; c < C; ++c) g[k][c] = 0.0f;
      }
      for (int l = 0; l < L; ++l) zs[l * kRR + i] = 1.0f;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      float v[4 * Q];
#pragma unroll
      for (int c = 0; c < 4 * Q; ++c) v[c] = c < C ? g[k][c] : 0.0f;
#pragma unroll
      for (int q = 0; q < Q; ++q)
        gs[(k * Q + q) * kRR + i] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
      hs[k * kRR + i] = h[k];
    }
  }
  __syncthreads();
  if (LT > 0 && a.zb) {
    // Surface indexes of this thread's sample at the 9 pixels it reaches,
    // then the warp's foreground (sample, layer) pairs spread over its lanes
    // (lane t takes the t-th set bit of the per-layer ballots and the
    // sample's surface indexes by shuffle); background pairs get zeros from
    // their own thread.
    const int lane = threadIdx.x & 31;
    const int s1 = (ty + 1) * kRS + tx + 1;
    int surf[9];
    unsigned ok = 0;
#pragma unroll
    for (int j = 0; j < 9; ++j) {
      const int u = j / 3 - 1, v = j % 3 - 1;
      const int px = sx + u, py = sy + v;
      const bool in = mine && px >= 0 && py >= 0 && px < W && py < H;
      ok |= unsigned(in) << j;
      if (LT == 3)  // pixel s1 + (u, v) saw this sample as its tap j
        surf[j] = in ? int((reinterpret_cast<const unsigned*>(zs)[s1 + v * kRS + u] >>
                            (3 * j)) & 7u) - 2
                     : 0;
      else
        surf[j] = in && j != 4 ? surface_index(zs, s1, s1 + v * kRS + u, L) : 0;  // center: 0
    }
    constexpr int kL = LT > 0 ? LT : 1;
    unsigned masks[kL];
    int total = 0;
#pragma unroll
    for (int l = 0; l < kL; ++l) {
      const bool fg = mine && ((own >> l) & 1u);
      if (mine && !fg && !a.fg_grads) {
        float dz[4 * Q];
#pragma unroll
        for (int c = 0; c < 4 * Q; ++c) dz[c] = 0.0f;
        store_row<C>(a.d_colors + (ebase + l * HW) * C, dz);
      }
      masks[l] = __ballot_sync(0xffffffffu, fg);
      total += __popc(masks[l]);
    }
    for (int t0 = 0; t0 < total; t0 += 32) {
      const int t = t0 + lane;
      const bool active = t < total;
      int l = 0, src = lane;
      if (active) {
        int r = t;
#pragma unroll
        for (int ll = 0; ll < kL - 1; ++ll)
          if (l == ll && r >= __popc(masks[ll])) { r -= __popc(masks[ll]); l = ll + 1; }
        unsigned ml = masks[0];
#pragma unroll
        for (int ll = 1; ll < kL; ++ll)
          if (l == ll) ml = masks[ll];
        src = nth_set_bit(ml, r);
      }
      int ss[9];
#pragma unroll
      for (int j = 0; j < 9; ++j) ss[j] = __shfl_sync(0xffffffffu, surf[j], src);
      const unsigned okv = __shfl_sync(0xffffffffu, ok, src);
      if (!active) continue;
      const int64_t e = lbase + int64_t(sy) * W + (tr.x0 + src) + l * HW;
      const int s1s = (ty + 1) * kRS + src + 1;
      const float4 q = __ldg(a.vp + e);
      float2 dcol[2 * Q];
#pragma unroll
      for (int hh = 0; hh < 2 * Q; ++hh) dcol[hh] = make_float2(0.0f, 0.0f);
      float dvx = 0.0f, dvy = 0.0f;
      const Taps tp = taps_of(q, 1.0f, a.coef);
      float4 col[Q];
      load_groups<C>(a.colors + e * C, col);
      sample_adjoint<Q>(tp, col, ss, okv, l, s1s, gs, hs, dcol, dvx, dvy);
      float dc[4 * Q];
#pragma unroll
      for (int hh = 0; hh < 2 * Q; ++hh) {
        dc[2 * hh] = dcol[hh].x;
        dc[2 * hh + 1] = dcol[hh].y;
      }
      store_row<C>(a.d_colors + e * C, dc);
      a.d_vp[e] = make_float4(dvx, dvy, 0.0f, 0.0f);
    }
    return;
  }
  if (!mine) return;
  const int s1 = (ty + 1) * kRS + tx + 1;  // this sample's pixel in the ring grid
  // Surface index of this sample's splat at each of the 9 pixels it reaches:
  // pixel s1 + (u, v) sees this sample as its tap (u, v).
  int surf[9];
  unsigned ok = 0;
#pragma unroll
  for (int j = 0; j < 9; ++j) {
    const int u = j / 3 - 1, v = j % 3 - 1;
    const int px = sx + u, py = sy + v;
    const bool in = px >= 0 && py >= 0 && px < W && py < H;
    ok |= unsigned(in) << j;
    surf[j] = in && j != 4 ? surface_index(zs, s1, s1 + v * kRS + u, L) : 0;  // center: 0
  }
  for (int l = 0; l < L; ++l) {
    const int64_t e = ebase + l * HW;
    const float4 q = ((own >> l) & 1u) ? __ldg(a.vp + e) : make_float4(0.0f, 0.0f, 1.0f, 0.0f);
    float2 dcol[2 * Q];
#pragma unroll
    for (int hh = 0; hh < 2 * Q; ++hh) dcol[hh] = make_float2(0.0f, 0.0f);
    float dvx = 0.0f, dvy = 0.0f;
    const float fgw = fg_weight(a.zb != nullptr, (own >> l) & 1u, q);
    if (fgw != 0.0f) {
      const Taps t = taps_of(q, fgw, a.coef);
      float4 col[Q];
      load_groups<C>(a.colors + e * C, col);
      sample_adjoint<Q>(t, col, surf, ok, l, s1, gs, hs, dcol, dvx, dvy);
    }
    float dc[4 * Q];
#pragma unroll
    for (int hh = 0; hh < 2 * Q; ++hh) {
      dc[2 * hh] = dcol[hh].x;
      dc[2 * hh + 1] = dcol[hh].y;
    }
    if (fgw != 0.0f || !a.fg_grads) store_row<C>(a.d_colors + e * C, dc);
    if (fgw != 0.0f || !a.zb) a.d_vp[e] = make_float4(dvx, dvy, 0.0f, 0.0f);
  }
}

template <int C, int LT>
__global__ void __launch_bounds__(256, (C <= 4 && LT == 3) ? 5 : 4)
    splat_bwd_kernel(SplatArgs a, Batch B) {
  extern __shared__ __align__(16) float smem[];
  splat_bwd_tile<C, LT>(a, B, blockIdx.x, smem);
}

// Persistent blocks over the tiles the forward listed, handed out by the
// backward's work counter (reset by splat_bwd_zero_kernel, which runs first).
template <int C, int LT>
__global__ void __launch_bounds__(256, (C <= 4 && LT == 3) ? 5 : 4)
    splat_bwd_list_kernel(SplatArgs a, Batch B, TileList t) {
  extern __shared__ __align__(16) float smem[];
  __shared__ int s_item;
  const int n = int(t.count[0]);
  for (;;) {
    if (threadIdx.x == 0) s_item = int(atomicAdd(t.count + 2, 1u));
    __syncthreads();
    const int w = s_item;
    if (w >= n) break;
    splat_bwd_tile<C, LT>(a, B, t.list[w], smem);
    __syncthreads();
  }
}

// One warp per tile that the forward did not list: no foreground sample in
// the region, so every sample of the tile gets a zero color gradient (with
// a depth buffer their position gradients stay unwritten). Also resets the
// backward's work counter.
template <int C>
__global__ void __launch_bounds__(256) splat_bwd_zero_kernel(SplatArgs a, Batch B, TileList t,
                                                             int tiles) {
  if (blockIdx.x == 0 && threadIdx.x == 0) t.count[2] = 0u;
  const int item = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (a.fg_grads || item >= tiles || t.flag[item]) return;
  const int lane = threadIdx.x & 31;
  const TileRef tr = tile_at(B, item);
  const int W = B.width[tr.img], H = B.height[tr.img];
  const int64_t HW = int64_t(W) * H;
  const int64_t lbase = int64_t(a.L) * B.pix_off[tr.img];
  float zero[C];
#pragma unroll
  for (int c = 0; c < C; ++c) zero[c] = 0.0f;
  for (int p = lane; p < kTX * kTY; p += 32) {
    const int px = tr.x0 + p % kTX, py = tr.y0 + p / kTX;
    if (px >= W || py >= H) continue;
    const int64_t e = lbase + int64_t(py) * W + px;
    for (int l = 0; l < a.L; ++l) store_row<C>(a.d_colors + (e + l * HW) * C, zero);
  }
}


// Forward-mode derivative (JVP) of splat + normalize + over for tangents of
// the sample positions (x, y) and, optionally, of the colors, with the
// discrete state (floors, surface classes, foreground) held fixed, as
// jax.jvp through splat.py:26-175 and composite.py:20-37 gives. A tap's
// weight w = ex ey moves by d w = 4 w (dx tx + dy ty) for the sample's
// position tangent (tx, ty) (dx, dy its tap offsets); each pixel carries the
// accumulators and their tangents through the normalization (lax.max's
// 0.5 tie rule) and the over compositing. Same tiling as the forward, one
// pixel per thread; used by the forward-mode API, not on the benchmark path.
template <int C>
__global__ void __launch_bounds__(256) splat_jvp_kernel(SplatArgs a, const float4* d_vp,
                                                       const float* d_colors, float* d_image,
                                                       Batch B) {
  constexpr int Q = Groups<C>::Q;
  extern __shared__ __align__(16) float smem[];
  const TileRef tr = tile_of(B);
  const int L = a.L;
  const int W = B.width[tr.img], H = B.height[tr.img];
  float* zs = smem;                                         // [L][kRR]
  float* wx = zs + L * kRR;                                 // [L][3][kRR]
  float* wy = wx + 3 * L * kRR;                             // [L][3][kRR]
  float4* tg = reinterpret_cast<float4*>(wy + 3 * L * kRR);  // [L][kRR] (d0, d1, tx, ty)
  float4* col = tg + L * kRR;                               // [L][Q][kRR]
  float4* dcol = col + Q * L * kRR;                         // [L][Q][kRR]
  unsigned short* fgm = reinterpret_cast<unsigned short*>(dcol + Q * L * kRR);
  const int64_t HW = int64_t(W) * H;
  const int64_t base = int64_t(L) * B.pix_off[tr.img];
  for (int i = threadIdx.x; i < kRR; i += blockDim.x) {
    const int ry = i / kRS;
    const int x = tr.x0 - 1 + (i - ry * kRS), y = tr.y0 - 1 + ry;
    const bool in = x >= 0 && y >= 0 && x < W && y < H;
    const int64_t e0 = base + int64_t(y) * W + x;
    unsigned m = 0;
    for (int l = 0; l < L; ++l) {
      const int64_t e = e0 + l * HW;
      const bool fgbit = in && (a.zb ? __ldg(a.zb + e) != 1.0f : true);
      float4 q = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
      if (fgbit) q = __ldg(a.vp + e);
      zs[l * kRR + i] = q.z;
      const float fgw = fg_weight(a.zb != nullptr, fgbit, q);
      if (fgw != 0.0f) {
        m |= 1u << l;
        const Taps t = taps_of(q, fgw, a.coef);
#pragma unroll
        for (int u = 0; u < 3; ++u) {
          wx[(l * 3 + u) * kRR + i] = t.ex[u];
          wy[(l * 3 + u) * kRR + i] = t.ey[u];
        }
        const float4 dq = d_vp ? __ldg(d_vp + e) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        tg[l * kRR + i] = make_float4(t.d0, t.d1, dq.x, dq.y);
        float4 c[Q], dc[Q];
        load_groups<C>(a.colors + e * C, c);
        if (d_colors) {
          load_groups<C>(d_colors + e * C, dc);
        } else {
#pragma unroll
          for (int g = 0; g < Q; ++g) dc[g] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
#pragma unroll
        for (int g = 0; g < Q; ++g) {
          col[(l * Q + g) * kRR + i] = c[g];
          dcol[(l * Q + g) * kRR + i] = dc[g];
        }
      }
    }
    fgm[i] = (unsigned short)m;
  }
  __syncthreads();

  const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
  const int px = tr.x0 + tx, py = tr.y0 + ty;
  if (px >= W || py >= H) return;
  const int p = (ty + 1) * kRS + tx + 1;
  float acc[3][4 * Q], dacc[3][4 * Q], wacc[3], dwacc[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    wacc[k] = dwacc[k] = 0.0f;
#pragma unroll
    for (int c = 0; c < 4 * Q; ++c) acc[k][c] = dacc[k][c] = 0.0f;
  }
  for (int l = 0; l < L; ++l) {
#pragma unroll
    for (int j = 0; j < 9; ++j) {
      const int u = j / 3 - 1, v = j % 3 - 1;
      const int sx = px - u, sy = py - v;
      if (sx < 0 || sy < 0 || sx >= W || sy >= H) continue;
      const int s = p - v * kRS - u;
      if (!((fgm[s] >> l) & 1u)) continue;
      const int sj = surface_index(zs, s, p, L);
      const int k = sj > l ? 0 : (sj == l ? 1 : 2);
      const float w = __fmul_rn(wx[(l * 3 + u + 1) * kRR + s], wy[(l * 3 + v + 1) * kRR + s]);
      const float4 t = tg[l * kRR + s];
      const float dw = 4.0f * w * ((t.x + float(u)) * t.z + (t.y + float(v)) * t.w);
#pragma unroll
      for (int g = 0; g < Q; ++g) {
        const float4 c = col[(l * Q + g) * kRR + s], dc = dcol[(l * Q + g) * kRR + s];
        const float cv[4] = {c.x, c.y, c.z, c.w}, dcv[4] = {dc.x, dc.y, dc.z, dc.w};
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          acc[k][4 * g + h] = fmaf(w, cv[h], acc[k][4 * g + h]);
          dacc[k][4 * g + h] = fmaf(dw, cv[h], fmaf(w, dcv[h], dacc[k][4 * g + h]));
        }
      }
      wacc[k] += w;
      dwacc[k] += dw;
    }
  }
  float n[3][C], dn[3][C];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float sc = norm_scale(wacc[k]);
    const float x = wacc[k] - 1.0f;
    const float gate = x > 0.0f ? 1.0f : (x == 0.0f ? 0.5f : 0.0f);
    const float dsc = -sc * sc * gate * dwacc[k];
#pragma unroll
    for (int c = 0; c < C; ++c) {
      n[k][c] = acc[k][c] * sc;
      dn[k][c] = dacc[k][c] * sc + acc[k][c] * dsc;
    }
  }
  // out = n0 + (1 - a0) (n1 + (1 - a1) n2), a_k = n_k[C - 1]
  const float a0 = n[0][C - 1], a1 = n[1][C - 1];
  const float da0 = dn[0][C - 1], da1 = dn[1][C - 1];
  float o[4 * Q];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const float mid = n[1][c] + (1.0f - a1) * n[2][c];
    const float dmid = dn[1][c] - da1 * n[2][c] + (1.0f - a1) * dn[2][c];
    o[c] = dn[0][c] - da0 * mid + (1.0f - a0) * dmid;
  }
  const int64_t pix = B.pix_off[tr.img] + int64_t(py) * W + px;
  store_row<C>(d_image + pix * C, o);
}

float gaussian_coef() {
  // (1 + 0.05) / sum_{u,v in {-1,0,1}} exp(-2 (u^2 + v^2)), in double then
  // rounded to float as the reference's weakly typed constant (splat.py:63-78).
  double sum = 0.0;
  for (int u = -1; u <= 1; ++u)
    for (int v = -1; v <= 1; ++v) sum += std::exp(-2.0 * (u * u + v * v));
  return float((1.0 + 0.05) / sum);
}

// Shared memory per block: z, 3 + 3 weights and the padded color groups per
// layer sample (forward); every layer's z, the padded color adjoints and the
// weight adjoint of the 3 classes per ring pixel (backward).
size_t fwd_smem(int L, int C) {
  return size_t(L) * kRR * 4 * (7 + 4 * ((C + 3) / 4)) + size_t(kRR) * (L > 8 ? 2 : 1);
}
size_t bwd_smem(int L, int C) {
  return size_t(L + 3 * 4 * ((C + 3) / 4) + 3) * kRR * 4;
}

// The tile list lives in the last plane of the saved buffer (plane
// 3 (C + 1) + 1): the counters, the list, then one flag byte per tile.
constexpr size_t kListHeader = 16;
size_t list_bytes(int tiles) {
  return kListHeader + ((size_t(tiles) * 4 + 15) & ~size_t(15)) + size_t(tiles);
}

template <int C>
TileList tile_list(const SplatArgs& a, int tiles) {
  unsigned char* p = reinterpret_cast<unsigned char*>(a.saved + size_t(3 * (C + 1) + 1) * a.P);
  TileList t;
  t.count = reinterpret_cast<unsigned*>(p);
  t.list = reinterpret_cast<int*>(p + kListHeader);
  t.flag = p + kListHeader + ((size_t(tiles) * 4 + 15) & ~size_t(15));
  return t;
}

// With saved accumulators and a depth buffer (the training path) a call is
// split: a light kernel classifies the tiles (forward) or zeros the
// gradients of the empty ones (backward), and the heavy kernel runs
// persistent blocks over the listed tiles only. Otherwise one block per
// tile.
template <int C, int LT>
int run_splat(bool bwd, SplatArgs a, const dr_image_desc* images, int n,
              cudaStream_t stream, std::string& err) {
  const size_t smem = bwd ? bwd_smem(a.L, C) : fwd_smem(a.L, C);
  auto kern = bwd ? splat_bwd_kernel<C, LT> : splat_fwd_kernel<C, LT>;
  auto list_kern = bwd ? splat_bwd_list_kernel<C, LT> : splat_fwd_list_kernel<C, LT>;
  // Dynamic shared-memory limits (host-side attributes, raised once per
  // device and size) and the persistent grid of the list kernel.
  static LaunchCache cache[2], list_cache[2];
  const char* too_big = "layers x channels need more shared memory than the device has";
  int sms = 0, per_sm = 0, list_sms = 0, list_per_sm = 0;
  if (!prepare_launch(cache[bwd], kern, kTX * kTY, smem, sms, per_sm, too_big, err) ||
      !prepare_launch(list_cache[bwd], list_kern, kTX * kTY, smem, list_sms, list_per_sm,
                      too_big, err))
    return DR_ERR_INVALID_ARGUMENT;
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    if (!make_batch(images + g0, cnt, a.L, kTX, kTY, b, err)) return DR_ERR_INVALID_ARGUMENT;
    const int tiles = b.tile_start[cnt];
    if (tiles <= 0) continue;
    const bool listed = a.saved && a.zb && !a.accum && !a.normalized &&
                        n <= DR_MAX_BATCH_INLINE && list_bytes(tiles) <= size_t(a.P) * 4;
    if (!listed) {
      kern<<<tiles, kTX * kTY, smem, stream>>>(a, b);
      continue;
    }
    const TileList t = tile_list<C>(a, tiles);
    const int grid = std::min(tiles, list_sms * list_per_sm);
    const unsigned light = unsigned((tiles + 7) / 8);
    if (!bwd) {
      if (cudaMemsetAsync(t.count, 0, kListHeader, stream) != cudaSuccess) {
        err = std::string("cudaMemsetAsync: ") + cudaGetErrorString(cudaGetLastError());
        return DR_ERR_CUDA;
      }
      splat_classify_kernel<C><<<light, 256, 0, stream>>>(a, b, t, tiles);
    } else {
      splat_bwd_zero_kernel<C><<<light, 256, 0, stream>>>(a, b, t, tiles);
    }
    list_kern<<<grid, kTX * kTY, smem, stream>>>(a, b, t);
  }
  return launch_status(bwd ? "splat backward" : "splat", err);
}


size_t jvp_smem(int L, int C) {
  return size_t(L) * kRR * 4 * (7 + 4 + 8 * ((C + 3) / 4)) + size_t(kRR) * 2;
}

template <int C>
int run_splat_jvp(const SplatArgs& a, const float4* d_vp, const float* d_colors,
                  float* d_image, const dr_image_desc* images, int n, cudaStream_t stream,
                  std::string& err) {
  const size_t smem = jvp_smem(a.L, C);
  static LaunchCache cache;
  int sms = 0, per_sm = 0;
  if (!prepare_launch(cache, splat_jvp_kernel<C>, kTX * kTY, smem, sms, per_sm,
                      "layers x channels need more shared memory than the device has", err))
    return DR_ERR_INVALID_ARGUMENT;
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    if (!make_batch(images + g0, cnt, a.L, kTX, kTY, b, err)) return DR_ERR_INVALID_ARGUMENT;
    const int tiles = b.tile_start[cnt];
    if (tiles > 0)
      splat_jvp_kernel<C><<<tiles, kTX * kTY, smem, stream>>>(a, d_vp, d_colors, d_image, b);
  }
  return launch_status("splat jvp", err);
}

int dispatch(bool bwd, int C, const SplatArgs& a, const dr_image_desc* images, int n,
             cudaStream_t stream, std::string& err) {
  if (C == 4 && a.L == 3) return run_splat<4, 3>(bwd, a, images, n, stream, err);
  if (C == 4 && a.L == 1) return run_splat<4, 1>(bwd, a, images, n, stream, err);
  switch (C) {
    case 1: return run_splat<1, 0>(bwd, a, images, n, stream, err);
    case 2: return run_splat<2, 0>(bwd, a, images, n, stream, err);
    case 3: return run_splat<3, 0>(bwd, a, images, n, stream, err);
    case 4: return run_splat<4, 0>(bwd, a, images, n, stream, err);
    case 5: return run_splat<5, 0>(bwd, a, images, n, stream, err);
    case 6: return run_splat<6, 0>(bwd, a, images, n, stream, err);
    case 7: return run_splat<7, 0>(bwd, a, images, n, stream, err);
    case 8: return run_splat<8, 0>(bwd, a, images, n, stream, err);
    default:
      err = "splat supports 1 to 8 channels";
      return DR_ERR_INVALID_ARGUMENT;
  }
}

bool aligned16(std::initializer_list<const void*> ptrs) {
  for (const void* p : ptrs)
    if (p && (reinterpret_cast<uintptr_t>(p) & 15) != 0) return false;
  return true;
}

// Pixels spanned by the images of one call: the plane stride of the saved
// accumulators.
int64_t call_pixels(const dr_image_desc* images, int n) {
  int64_t P = 0;
  for (int i = 0; i < n; ++i)
    P = std::max(P, images[i].pixel_offset + int64_t(images[i].width) * images[i].height);
  return P;
}

bool check_batch(int L, int n, const dr_image_desc* images, std::string& err, int& rc) {
  rc = DR_OK;
  if (n < 0 || (n > 0 && !images)) { err = "invalid image table"; rc = DR_ERR_INVALID_ARGUMENT; return false; }
  if (L < 1 || L > DR_MAX_LAYERS) { err = "num_layers must be in [1, 16]"; rc = DR_ERR_INVALID_ARGUMENT; return false; }
  return n > 0;
}

template <typename K>
int run_positions(K kern, const PosArgs& a, const dr_image_desc* images, int n, int L,
                  cudaStream_t stream, std::string& err, const char* what) {
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    if (!make_batch(images + g0, cnt, L, kTX, kTY, b, err)) return DR_ERR_INVALID_ARGUMENT;
    const int64_t total = int64_t(L) * b.pix_prefix[cnt];
    if (total > 0) kern<<<unsigned((total + 255) / 256), 256, 0, stream>>>(a, b);
  }
  return launch_status(what, err);
}

}  // namespace

int samples_fwd_launch(const float* attributes, int K, const float* clip,
                       const int32_t* tris, const int32_t* ids, const float* z,
                       const float* bary, const dr_image_desc* images, int n, int L,
                       float* attr_out, float* positions, cudaStream_t stream,
                       std::string& err) {
  int rc;
  if (!check_batch(L, n, images, err, rc)) return rc;
  if (K < 1 || K > DR_MAX_CHANNELS) { err = "channels must be in [1, 16]"; return DR_ERR_INVALID_ARGUMENT; }
  if (!aligned16({clip, positions}) ||
      (K % 4 == 0 && !aligned16({attributes, attr_out}))) {
    err = "clip_vertices, positions (and, with a multiple of 4 channels, the attribute "
          "buffers) must be 16-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  SampleArgs a{};
  a.pos.clip = reinterpret_cast<const float4*>(clip);
  a.pos.tris = tris; a.pos.ids = ids; a.pos.z = z; a.pos.bary = bary; a.pos.L = L;
  a.pos.vp = reinterpret_cast<float4*>(positions);
  a.attr = attributes; a.K = K; a.attr_out = attr_out;
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    if (!make_batch(images + g0, cnt, L, kTX, kTY, b, err)) return DR_ERR_INVALID_ARGUMENT;
    const int64_t total = int64_t(L) * b.pix_prefix[cnt];
    if (total > 0) samples_fwd_kernel<<<unsigned((total + 255) / 256), 256, 0, stream>>>(a, b);
  }
  return launch_status("interpolate + splat positions", err);
}

// Scratch of the deterministic samples VJP: the largest magnitude, then the
// fixed-point sums of the clip and attribute gradients of every vertex the
// images span.
int64_t spanned_vertices(const dr_image_desc* images, int n) {
  int64_t nv = 0;
  for (int i = 0; i < n; ++i)
    nv = std::max<int64_t>(nv, images[i].vertex_offset + images[i].num_vertices);
  return nv;
}

size_t samples_fixed_bytes(const dr_image_desc* images, int n, int K) {
  const size_t nv = size_t(spanned_vertices(images, n));
  return 256 + ((nv * 4 * 8 + 255) & ~size_t(255)) + nv * size_t(K) * 8;
}

int samples_bwd_launch(const float* d_attr_out, const float* d_positions,
                       const float* attributes, int K, const float* clip,
                       const int32_t* tris, const int32_t* ids, const float* z,
                       const float* bary, const float* positions,
                       const int32_t* vertex_ids, const dr_image_desc* images, int n,
                       int L, float* d_attributes, float* d_clip, float* d_bary,
                       uint32_t flags, void* scratch, size_t scratch_bytes,
                       cudaStream_t stream, std::string& err) {
  int rc;
  if (!check_batch(L, n, images, err, rc)) return rc;
  if (K < 1 || K > DR_MAX_CHANNELS) { err = "channels must be in [1, 16]"; return DR_ERR_INVALID_ARGUMENT; }
  if ((flags & ~DR_SAMPLES_DETERMINISTIC) != 0) {
    err = "unknown samples backward flags";
    return DR_ERR_INVALID_ARGUMENT;
  }
  if (!d_clip || (d_attr_out && !d_attributes)) {
    err = "d_clip_vertices (and d_attributes with d_attr_out) must be non-null";
    return DR_ERR_INVALID_ARGUMENT;
  }
  const bool det = (flags & DR_SAMPLES_DETERMINISTIC) != 0;
  if (det && (!scratch || (reinterpret_cast<uintptr_t>(scratch) & 255) != 0 ||
              scratch_bytes < samples_fixed_bytes(images, n, K))) {
    err = "DR_SAMPLES_DETERMINISTIC needs a 256-byte aligned scratch of "
          "dr_interpolate_with_positions_bwd_scratch_bytes bytes";
    return DR_ERR_INVALID_ARGUMENT;
  }
  if (!aligned16({d_positions, clip, d_clip, positions}) ||
      (K % 4 == 0 && !aligned16({d_attr_out, attributes, d_attributes}))) {
    err = "d_positions, clip_vertices, d_clip_vertices, positions (and, with a multiple "
          "of 4 channels, the attribute buffers) must be 16-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  SampleArgs a{};
  a.pos.clip = reinterpret_cast<const float4*>(clip);
  a.pos.tris = tris; a.pos.ids = ids; a.pos.z = z; a.pos.bary = bary; a.pos.L = L;
  a.vp = reinterpret_cast<const float4*>(positions);
  a.vid = vertex_ids;
  a.pos.dvp = reinterpret_cast<const float4*>(d_positions);
  a.pos.d_clip = reinterpret_cast<float4*>(d_clip);
  a.pos.d_bary = d_bary;
  a.attr = attributes; a.K = K;
  a.d_attr_out = d_attr_out; a.d_attr = d_attributes;
  int64_t samples = 0;
  for (int i = 0; i < n; ++i) samples += int64_t(L) * images[i].width * images[i].height;
  const int64_t nv = spanned_vertices(images, n);
  if (det) {
    unsigned char* base = static_cast<unsigned char*>(scratch);
    a.fx_max = reinterpret_cast<unsigned*>(base);
    a.fx_clip = reinterpret_cast<unsigned long long*>(base + 256);
    a.fx_attr = reinterpret_cast<unsigned long long*>(
        base + 256 + ((size_t(nv) * 4 * 8 + 255) & ~size_t(255)));
    int lc = 0;
    while ((int64_t(1) << lc) < std::max<int64_t>(samples, 1)) ++lc;
    a.fx_log2_count = lc;
    if (cudaMemsetAsync(scratch, 0, samples_fixed_bytes(images, n, K), stream) != cudaSuccess) {
      err = std::string("cudaMemsetAsync: ") + cudaGetErrorString(cudaGetLastError());
      return DR_ERR_CUDA;
    }
  }
  // Deterministic: a pass that finds the largest magnitude (no outputs), then
  // the fixed-point pass, then the sums back to float.
  for (int mode = det ? 1 : 0; mode <= (det ? 2 : 0); ++mode) {
    SampleArgs am = a;
    if (mode == 1) am.pos.d_bary = nullptr;
    for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
      const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
      Batch b;
      if (!make_batch(images + g0, cnt, L, kTX, kTY, b, err)) return DR_ERR_INVALID_ARGUMENT;
      const int64_t total = int64_t(L) * b.pix_prefix[cnt];
      if (total <= 0) continue;
      const unsigned grid = unsigned((total + kVjpBlock - 1) / kVjpBlock);
      if (mode == 0)
        samples_bwd_kernel<0><<<grid, kVjpThreads, 0, stream>>>(am, b);
      else if (mode == 1)
        samples_bwd_kernel<1><<<grid, kVjpThreads, 0, stream>>>(am, b);
      else
        samples_bwd_kernel<2><<<grid, kVjpThreads, 0, stream>>>(am, b);
    }
  }
  if (det && nv > 0)
    fixed_finalize_kernel<<<unsigned((nv + 255) / 256), 256, 0, stream>>>(a, nv);
  return launch_status("interpolate + splat positions backward", err);
}

int positions_fwd_launch(const float* clip, const int32_t* tris, const int32_t* ids,
                         const float* z, const float* bary, const dr_image_desc* images,
                         int n, int L, float* positions, cudaStream_t stream,
                         std::string& err) {
  int rc;
  if (!check_batch(L, n, images, err, rc)) return rc;
  if (!aligned16({clip, positions})) {
    err = "clip_vertices and positions must be 16-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  PosArgs a{};
  a.clip = reinterpret_cast<const float4*>(clip);
  a.tris = tris; a.ids = ids; a.z = z; a.bary = bary; a.L = L;
  a.vp = reinterpret_cast<float4*>(positions);
  return run_positions(positions_fwd_kernel, a, images, n, L, stream, err, "splat positions");
}

int positions_bwd_launch(const float* d_positions, const float* clip, const int32_t* tris,
                         const int32_t* ids, const float* z, const float* bary,
                         const dr_image_desc* images, int n, int L, float* d_clip,
                         float* d_bary, cudaStream_t stream, std::string& err) {
  int rc;
  if (!check_batch(L, n, images, err, rc)) return rc;
  if (!aligned16({d_positions, clip, d_clip})) {
    err = "d_positions, clip_vertices and d_clip_vertices must be 16-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  PosArgs a{};
  a.clip = reinterpret_cast<const float4*>(clip);
  a.tris = tris; a.ids = ids; a.z = z; a.bary = bary; a.L = L;
  a.dvp = reinterpret_cast<const float4*>(d_positions);
  a.d_clip = reinterpret_cast<float4*>(d_clip);
  a.d_bary = d_bary;
  return run_positions(positions_bwd_kernel, a, images, n, L, stream, err,
                       "splat positions backward");
}

int splat_fwd_launch(const float* positions, const float* z_buffer, const float* colors, int C,
                     const dr_image_desc* images, int n, int L, float* out, float* saved,
                     float* accum, float* normalized, cudaStream_t stream,
                     std::string& err) {
  int rc;
  if (!check_batch(L, n, images, err, rc)) return rc;
  if (!aligned16({positions}) ||
      (C % 4 == 0 && !aligned16({colors, out, accum, normalized}))) {
    err = "positions (and, with a multiple of 4 channels, colors and outputs) must be "
          "16-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  SplatArgs a{};
  a.vp = reinterpret_cast<const float4*>(positions);
  a.zb = z_buffer;
  a.colors = colors;
  a.L = L;
  a.P = call_pixels(images, n);
  a.coef = gaussian_coef();
  a.out = out; a.saved = saved; a.accum = accum; a.normalized = normalized;
  return dispatch(false, C, a, images, n, stream, err);
}

int splat_bwd_launch(const float* d_out, const float* positions, const float* z_buffer,
                     const float* colors, const float* saved, int C,
                     const dr_image_desc* images, int n, int L, uint32_t flags,
                     float* d_colors, float* d_positions, cudaStream_t stream,
                     std::string& err) {
  int rc;
  if (!check_batch(L, n, images, err, rc)) return rc;
  if ((flags & ~DR_SPLAT_FOREGROUND_GRADIENTS) != 0) {
    err = "unknown splat flags";
    return DR_ERR_INVALID_ARGUMENT;
  }
  if ((flags & DR_SPLAT_FOREGROUND_GRADIENTS) && !z_buffer) {
    err = "DR_SPLAT_FOREGROUND_GRADIENTS needs the depth buffer";
    return DR_ERR_INVALID_ARGUMENT;
  }
  if (!saved) {
    err = "splat backward needs the accumulators saved by the forward pass";
    return DR_ERR_INVALID_ARGUMENT;
  }
  if (!aligned16({positions, d_positions}) ||
      (C % 4 == 0 && !aligned16({colors, d_out, d_colors}))) {
    err = "positions, d_positions (and, with a multiple of 4 channels, colors, d_out "
          "and d_colors) must be 16-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  SplatArgs a{};
  a.vp = reinterpret_cast<const float4*>(positions);
  a.zb = z_buffer;
  a.colors = colors;
  a.L = L;
  a.P = call_pixels(images, n);
  a.coef = gaussian_coef();
  a.saved = const_cast<float*>(saved);
  a.d_out = d_out; a.d_colors = d_colors;
  a.d_vp = reinterpret_cast<float4*>(d_positions);
  a.fg_grads = (flags & DR_SPLAT_FOREGROUND_GRADIENTS) != 0;
  return dispatch(true, C, a, images, n, stream, err);
}


int splat_jvp_launch(const float* positions, const float* z_buffer, const float* colors,
                     const float* d_positions, const float* d_colors, int C,
                     const dr_image_desc* images, int n, int L, float* d_image,
                     cudaStream_t stream, std::string& err) {
  int rc;
  if (!check_batch(L, n, images, err, rc)) return rc;
  if (!positions || !colors || !d_image) {
    err = "positions, colors and d_image must be non-null";
    return DR_ERR_INVALID_ARGUMENT;
  }
  if (jvp_smem(L, C) > 227 * 1024) {
    err = "layers x channels need more shared memory than the device has";
    return DR_ERR_INVALID_ARGUMENT;
  }
  if (!aligned16({positions, d_positions}) ||
      (C % 4 == 0 && !aligned16({colors, d_colors, d_image}))) {
    err = "positions, d_positions (and, with a multiple of 4 channels, colors, d_colors "
          "and d_image) must be 16-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  SplatArgs a{};
  a.vp = reinterpret_cast<const float4*>(positions);
  a.zb = z_buffer;
  a.colors = colors;
  a.L = L;
  a.P = call_pixels(images, n);
  a.coef = gaussian_coef();
  const float4* dvp = reinterpret_cast<const float4*>(d_positions);
  switch (C) {
    case 1: return run_splat_jvp<1>(a, dvp, d_colors, d_image, images, n, stream, err);
    case 2: return run_splat_jvp<2>(a, dvp, d_colors, d_image, images, n, stream, err);
    case 3: return run_splat_jvp<3>(a, dvp, d_colors, d_image, images, n, stream, err);
    case 4: return run_splat_jvp<4>(a, dvp, d_colors, d_image, images, n, stream, err);
    case 5: return run_splat_jvp<5>(a, dvp, d_colors, d_image, images, n, stream, err);
    case 6: return run_splat_jvp<6>(a, dvp, d_colors, d_image, images, n, stream, err);
    case 7: return run_splat_jvp<7>(a, dvp, d_colors, d_image, images, n, stream, err);
    case 8: return run_splat_jvp<8>(a, dvp, d_colors, d_image, images, n, stream, err);
    default:
      err = "splat supports 1 to 8 channels";
      return DR_ERR_INVALID_ARGUMENT;
  }
}

}  // namespace dr
