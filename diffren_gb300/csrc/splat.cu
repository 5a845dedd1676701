// Rasterize-then-splat for GB300 (diffren/jax/internal/splat.py:26-229,
// diffren/jax/composite.py:20-37) and its VJP, as four kernels:
//
//   positions_fwd  per layer sample: clip xyzw interpolated with the
//                  rasterized barycentrics (background (0, 0, 1, 1)),
//                  projected to viewport xyz, plus the foreground flag
//                  (splat.py:207-221) -> float4 per sample.
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

__device__ __forceinline__ Interp interpolate_clip(const PosArgs& a, const Batch& B,
                                                   int img, int64_t e) {
  Interp r;
  const int32_t* t = a.tris + 3 * (B.triangle_offset[img] + __ldg(a.ids + e));
  const float4* vb = a.clip + B.vertex_offset[img];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    r.vid[i] = __ldg(t + i);
    r.V[i] = __ldg(vb + r.vid[i]);
    r.b[i] = __ldg(a.bary + 3 * e + i);
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
  if (__ldg(a.z + r.e) != 1.0f) {
    fg = 1.0f;
    c = interpolate_clip(a, B, r.img, r.e).c;
  }
  // viewport = ((xyz / w + 1) * (W, H, 1)) * 0.5
  const float nx = __fdiv_rn(c.x, c.w), ny = __fdiv_rn(c.y, c.w), nz = __fdiv_rn(c.z, c.w);
  a.vp[r.e] = make_float4(__fmul_rn(__fmul_rn(__fadd_rn(nx, 1.0f), W), 0.5f),
                          __fmul_rn(__fmul_rn(__fadd_rn(ny, 1.0f), H), 0.5f),
                          __fmul_rn(__fmul_rn(__fadd_rn(nz, 1.0f), 1.0f), 0.5f), fg);
}

__global__ void __launch_bounds__(256) positions_bwd_kernel(PosArgs a, Batch B) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= int64_t(a.L) * B.pix_prefix[B.n]) return;
  const PixelRef r = decode(B, a.L, q);
  const float4 g = a.dvp[r.e];
  const bool fg = __ldg(a.z + r.e) != 1.0f;
  if (!fg || (g.x == 0.0f && g.y == 0.0f)) {
    if (a.d_bary) {
      a.d_bary[3 * r.e] = 0.0f;
      a.d_bary[3 * r.e + 1] = 0.0f;
      a.d_bary[3 * r.e + 2] = 0.0f;
    }
    return;
  }
  const Interp it = interpolate_clip(a, B, r.img, r.e);
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

// -------------------------------------------------------------------- splat
struct SplatArgs {
  const float4* vp;  // [L*P] viewport xyz + foreground flag
  const float* colors;
  int L, TY;
  float coef;
  float* out;
  float* saved;  // [P, 3, C+1] accumulators (forward output, backward input)
  float* accum;
  float* normalized;
  const float* d_out;
  float* d_colors;
  float4* d_vp;
};

// Separable tap weights of a sample (splat.py:106-115): tap (u, v) weighs
// ex[u+1] * ey[v+1] with ex = fg * coef * exp(-2 dx^2), ey = exp(-2 dy^2),
// dx = floor(x) + 0.5 - x + u. Equal to the reference's
// fg * coef * exp(-2 (dx^2 + dy^2)) up to float rounding.
struct Taps {
  float ex[3], ey[3];
  float d0, d1;
};

__device__ __forceinline__ Taps taps_of(float4 q, float coef) {
  Taps t;
  t.d0 = __fsub_rn(__fadd_rn(floorf(q.x), 0.5f), q.x);
  t.d1 = __fsub_rn(__fadd_rn(floorf(q.y), 0.5f), q.y);
  const float fc = __fmul_rn(q.w, coef);
#pragma unroll
  for (int u = 0; u < 3; ++u) {
    const float dx = __fadd_rn(t.d0, float(u - 1)), dy = __fadd_rn(t.d1, float(u - 1));
    t.ex[u] = q.w != 0.0f ? __fmul_rn(fc, expf(__fmul_rn(-2.0f, __fmul_rn(dx, dx)))) : 0.0f;
    t.ey[u] = q.w != 0.0f ? expf(__fmul_rn(-2.0f, __fmul_rn(dy, dy))) : 0.0f;
  }
  return t;
}

// Shared-memory region of R samples per layer, row stride `stride`:
//   z[l*R + i], wx[(l*3 + u+1)*R + i], wy[(l*3 + v+1)*R + i],
//   col[(l*C + c)*R + i]; every array indexed by i so warps read
// consecutive words.
struct Region {
  float* z;
  float* wx;
  float* wy;
  float* col;
  int R, stride;
};

__device__ __forceinline__ Region region_at(float* base, int L, int R, int stride) {
  Region r;
  r.R = R;
  r.stride = stride;
  r.z = base;
  r.wx = r.z + L * R;
  r.wy = r.wx + 3 * L * R;
  r.col = r.wy + 3 * L * R;
  return r;
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

struct TileRef {
  int img, x0, y0;
};

__device__ __forceinline__ TileRef tile_of(const Batch& B, int TY) {
  TileRef t;
  const int item = blockIdx.x;
  t.img = find_segment(B.tile_start, B.n, item);
  const int local = item - B.tile_start[t.img];
  const int ntx = B.tiles_x[t.img];
  t.x0 = (local % ntx) * kTX;
  t.y0 = (local / ntx) * TY;
  return t;
}

// Loads samples of the region with image origin (x0, y0), all layers.
// Samples outside the image have fg = 0 (no weight).
template <int C>
__device__ void load_region(const SplatArgs& a, const Batch& B, int img, int x0, int y0,
                            Region r) {
  const int W = B.width[img], H = B.height[img];
  const int64_t HW = int64_t(W) * H;
  const int64_t base = int64_t(a.L) * B.pix_off[img];
  const int n = a.L * r.R;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int l = k / r.R, i = k - l * r.R;
    const int y = y0 + i / r.stride, x = x0 + i % r.stride;
    float4 q = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
    float col[C];
#pragma unroll
    for (int c = 0; c < C; ++c) col[c] = 0.0f;
    if (x >= 0 && y >= 0 && x < W && y < H) {
      const int64_t e = base + l * HW + int64_t(y) * W + x;
      q = __ldg(a.vp + e);
      load_row<C>(a.colors + e * C, col);
    }
    const Taps t = taps_of(q, a.coef);
    r.z[l * r.R + i] = q.z;
#pragma unroll
    for (int u = 0; u < 3; ++u) {
      r.wx[(l * 3 + u) * r.R + i] = t.ex[u];
      r.wy[(l * 3 + u) * r.R + i] = t.ey[u];
    }
#pragma unroll
    for (int c = 0; c < C; ++c) r.col[(l * C + c) * r.R + i] = col[c];
  }
}

// Surface index of the splat from sample s reaching pixel p
// (splat.py:131-145): c = argmin_k |zS_k - zD_0|, t = argmin_k |zD_k - zS_0|
// (first index on ties); -t if the tap match is strictly better, else c.
__device__ __forceinline__ int surface_index(const float* z, int R, int s, int p, int L) {
  const float zD0 = z[p], zS0 = z[s];
  float minc = fabsf(__fsub_rn(zS0, zD0));
  float mint = minc;
  int c = 0, t = 0;
  for (int k = 1; k < L; ++k) {
    const float dc = fabsf(__fsub_rn(z[k * R + s], zD0));
    if (dc < minc) { minc = dc; c = k; }
    const float dt = fabsf(__fsub_rn(z[k * R + p], zS0));
    if (dt < mint) { mint = dt; t = k; }
  }
  return mint < minc ? -t : c;
}

// normalization_scales = 1 / (max(W - 1, 0) + 1)   (splat.py:168-169)
__device__ __forceinline__ float norm_scale(float w) {
  return __fdiv_rn(1.0f, __fadd_rn(fmaxf(__fsub_rn(w, 1.0f), 0.0f), 1.0f));
}

template <int C>
__global__ void __launch_bounds__(256) splat_fwd_kernel(SplatArgs a, Batch B) {
  extern __shared__ __align__(16) float smem[];
  const TileRef tr = tile_of(B, a.TY);
  const int TY = a.TY, L = a.L;
  const int stride = kTX + 2, R = stride * (TY + 2);
  const Region r = region_at(smem, L, R, stride);
  load_region<C>(a, B, tr.img, tr.x0 - 1, tr.y0 - 1, r);
  __syncthreads();

  const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
  const int W = B.width[tr.img], H = B.height[tr.img];
  const int px = tr.x0 + tx, py = tr.y0 + ty;
  if (px >= W || py >= H) return;
  const int p = (ty + 1) * stride + tx + 1;

  // Surface index of each of the 9 taps reaching p (independent of layer).
  int surf[9];
  unsigned ok = 0;
#pragma unroll
  for (int j = 0; j < 9; ++j) {
    const int u = j / 3 - 1, v = j % 3 - 1;
    const int sx = px - u, sy = py - v;
    const bool in = sx >= 0 && sy >= 0 && sx < W && sy < H;
    ok |= unsigned(in) << j;
    surf[j] = in ? surface_index(r.z, R, p - v * stride - u, p, L) : 0;
  }
  // Accumulate in the reference's order (layer, u, v); class 0 = in front
  // of the surface, 1 = at it, 2 = behind it.
  float acc[3][C], wacc[3] = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int k = 0; k < 3; ++k)
#pragma unroll
    for (int c = 0; c < C; ++c) acc[k][c] = 0.0f;
  for (int l = 0; l < L; ++l) {
#pragma unroll
    for (int j = 0; j < 9; ++j) {
      if (!((ok >> j) & 1)) continue;
      const int u = j / 3 - 1, v = j % 3 - 1;
      const int s = p - v * stride - u;
      const float wxv = r.wx[(l * 3 + u + 1) * R + s];
      if (wxv == 0.0f) continue;
      const float w = __fmul_rn(wxv, r.wy[(l * 3 + v + 1) * R + s]);
      float t[C];
#pragma unroll
      for (int c = 0; c < C; ++c) t[c] = __fmul_rn(w, r.col[(l * C + c) * R + s]);
      if (surf[j] > l) {
#pragma unroll
        for (int c = 0; c < C; ++c) acc[0][c] = __fadd_rn(acc[0][c], t[c]);
        wacc[0] = __fadd_rn(wacc[0], w);
      } else if (surf[j] == l) {
#pragma unroll
        for (int c = 0; c < C; ++c) acc[1][c] = __fadd_rn(acc[1][c], t[c]);
        wacc[1] = __fadd_rn(wacc[1], w);
      } else {
#pragma unroll
        for (int c = 0; c < C; ++c) acc[2][c] = __fadd_rn(acc[2][c], t[c]);
        wacc[2] = __fadd_rn(wacc[2], w);
      }
    }
  }

  float n[3][C];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float sc = norm_scale(wacc[k]);
#pragma unroll
    for (int c = 0; c < C; ++c) n[k][c] = __fmul_rn(acc[k][c], sc);
  }
  const int64_t pix = B.pix_off[tr.img] + int64_t(py) * W + px;
  // over: out = n2; out = n1 + (1 - a1) out; out = n0 + (1 - a0) out
  const float t1 = __fsub_rn(1.0f, n[1][C - 1]), t0 = __fsub_rn(1.0f, n[0][C - 1]);
  float o[C];
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const float mid = __fadd_rn(n[1][c], __fmul_rn(t1, n[2][c]));
    o[c] = __fadd_rn(n[0][c], __fmul_rn(t0, mid));
  }
  store_row<C>(a.out + pix * C, o);
  if (a.saved) {
    float* sv = a.saved + pix * (3 * (C + 1));
#pragma unroll
    for (int k = 0; k < 3; ++k) {
#pragma unroll
      for (int c = 0; c < C; ++c) sv[k * (C + 1) + c] = acc[k][c];
      sv[k * (C + 1) + C] = wacc[k];
    }
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

template <int C>
__global__ void __launch_bounds__(256) splat_bwd_kernel(SplatArgs a, Batch B) {
  extern __shared__ __align__(16) float smem[];
  const TileRef tr = tile_of(B, a.TY);
  const int TY = a.TY, L = a.L;
  const int W = B.width[tr.img], H = B.height[tr.img];
  const int64_t HW = int64_t(W) * H;
  // Tile + 1-pixel ring: every layer's depth (for the surface tests) and the
  // adjoints of the accumulators, [3*(C+1)][R1] (g[k][c], then h[k]).
  const int S1 = kTX + 2, R1 = S1 * (TY + 2);
  float* zs = smem;
  float* adj = zs + L * R1;
  const int64_t lbase = int64_t(L) * B.pix_off[tr.img];
  for (int i = threadIdx.x; i < R1; i += blockDim.x) {
    const int qx = tr.x0 - 1 + i % S1, qy = tr.y0 - 1 + i / S1;
    float g[3][C], h[3];
    if (qx >= 0 && qy >= 0 && qx < W && qy < H) {
      const int64_t pix = B.pix_off[tr.img] + int64_t(qy) * W + qx;
      const float* sv = a.saved + pix * (3 * (C + 1));
      float acc[3][C], wacc[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
#pragma unroll
        for (int c = 0; c < C; ++c) acc[k][c] = __ldg(sv + k * (C + 1) + c);
        wacc[k] = __ldg(sv + k * (C + 1) + C);
      }
      float d[C];
      load_row<C>(a.d_out + pix * C, d);
      accum_adjoint<C>(acc, wacc, d, g, h);
      for (int l = 0; l < L; ++l)
        zs[l * R1 + i] = __ldg(&a.vp[lbase + l * HW + int64_t(qy) * W + qx].z);
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        h[k] = 0.0f;
#pragma unroll
        for (int c = 0; c < C; ++c) g[k][c] = 0.0f;
      }
      for (int l = 0; l < L; ++l) zs[l * R1 + i] = 1.0f;
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
#pragma unroll
      for (int c = 0; c < C; ++c) adj[(k * (C + 1) + c) * R1 + i] = g[k][c];
      adj[(k * (C + 1) + C) * R1 + i] = h[k];
    }
  }
  __syncthreads();

  const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
  const int sx = tr.x0 + tx, sy = tr.y0 + ty;
  if (sx >= W || sy >= H) return;
  const int s1 = (ty + 1) * S1 + tx + 1;  // this sample's pixel in the ring grid
  int surf[9];
  unsigned ok = 0;
#pragma unroll
  for (int j = 0; j < 9; ++j) {
    const int u = j / 3 - 1, v = j % 3 - 1;
    const int px = sx + u, py = sy + v;
    const bool in = px >= 0 && py >= 0 && px < W && py < H;
    ok |= unsigned(in) << j;
    surf[j] = in ? surface_index(zs, R1, s1, s1 + v * S1 + u, L) : 0;
  }
  const int64_t ebase = lbase + int64_t(sy) * W + sx;
  for (int l = 0; l < L; ++l) {
    const int64_t e = ebase + l * HW;
    const float4 q = __ldg(a.vp + e);
    float dcol[C];
#pragma unroll
    for (int c = 0; c < C; ++c) dcol[c] = 0.0f;
    float dvx = 0.0f, dvy = 0.0f;
    if (q.w != 0.0f) {
      const Taps t = taps_of(q, a.coef);
      float col[C];
      load_row<C>(a.colors + e * C, col);
#pragma unroll
      for (int j = 0; j < 9; ++j) {
        if (!((ok >> j) & 1)) continue;
        const int u = j / 3 - 1, v = j % 3 - 1;
        const float w = __fmul_rn(t.ex[u + 1], t.ey[v + 1]);
        const int k = surf[j] > l ? 0 : (surf[j] == l ? 1 : 2);
        const float* ak = adj + k * (C + 1) * R1 + s1 + v * S1 + u;
        float dw = ak[C * R1];
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const float gc = ak[c * R1];
          dcol[c] += w * gc;
          dw += gc * col[c];
        }
        // d w / d (x, y) = 4 w (dx, dy): the floor carries no gradient.
        const float f = 4.0f * w * dw;
        dvx += f * (t.d0 + float(u));
        dvy += f * (t.d1 + float(v));
      }
    }
    store_row<C>(a.d_colors + e * C, dcol);
    a.d_vp[e] = make_float4(dvx, dvy, 0.0f, 0.0f);
  }
}

float gaussian_coef() {
  // (1 + 0.05) / sum_{u,v in {-1,0,1}} exp(-2 (u^2 + v^2)), in double then
  // rounded to float as the reference's weakly typed constant (splat.py:63-78).
  double sum = 0.0;
  for (int u = -1; u <= 1; ++u)
    for (int v = -1; v <= 1; ++v) sum += std::exp(-2.0 * (u * u + v * v));
  return float((1.0 + 0.05) / sum);
}

size_t fwd_smem(int L, int C) { return size_t(L) * (kTX + 2) * (kTY + 2) * 4 * (7 + C); }
size_t bwd_smem(int L, int C) {
  return size_t(L + 3 * (C + 1)) * (kTX + 2) * (kTY + 2) * 4;
}

template <int C>
int run_splat(bool bwd, SplatArgs a, const dr_image_desc* images, int n,
              cudaStream_t stream, std::string& err) {
  a.TY = kTY;
  const size_t smem = bwd ? bwd_smem(a.L, C) : fwd_smem(a.L, C);
  auto kern = bwd ? splat_bwd_kernel<C> : splat_fwd_kernel<C>;
  // Raise the dynamic shared-memory limit once per kernel and size (host-side
  // attribute only; later calls skip it).
  static size_t reserved[2] = {0, 0};
  if (smem > 48 * 1024 && smem > reserved[bwd]) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem)) != cudaSuccess) {
      err = "layers x channels need more shared memory than the device has";
      return DR_ERR_INVALID_ARGUMENT;
    }
    reserved[bwd] = smem;
  }
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    if (!make_batch(images + g0, cnt, a.L, kTX, kTY, b, err)) return DR_ERR_INVALID_ARGUMENT;
    const int tiles = b.tile_start[cnt];
    if (tiles > 0) kern<<<tiles, kTX * kTY, smem, stream>>>(a, b);
  }
  return launch_status(bwd ? "splat backward" : "splat", err);
}

int dispatch(bool bwd, int C, const SplatArgs& a, const dr_image_desc* images, int n,
             cudaStream_t stream, std::string& err) {
  switch (C) {
    case 1: return run_splat<1>(bwd, a, images, n, stream, err);
    case 2: return run_splat<2>(bwd, a, images, n, stream, err);
    case 3: return run_splat<3>(bwd, a, images, n, stream, err);
    case 4: return run_splat<4>(bwd, a, images, n, stream, err);
    case 5: return run_splat<5>(bwd, a, images, n, stream, err);
    case 6: return run_splat<6>(bwd, a, images, n, stream, err);
    case 7: return run_splat<7>(bwd, a, images, n, stream, err);
    case 8: return run_splat<8>(bwd, a, images, n, stream, err);
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

int splat_fwd_launch(const float* positions, const float* colors, int C,
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
  a.colors = colors;
  a.L = L;
  a.coef = gaussian_coef();
  a.out = out; a.saved = saved; a.accum = accum; a.normalized = normalized;
  return dispatch(false, C, a, images, n, stream, err);
}

int splat_bwd_launch(const float* d_out, const float* positions, const float* colors,
                     const float* saved, int C, const dr_image_desc* images, int n, int L,
                     float* d_colors, float* d_positions, cudaStream_t stream,
                     std::string& err) {
  int rc;
  if (!check_batch(L, n, images, err, rc)) return rc;
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
  a.colors = colors;
  a.L = L;
  a.coef = gaussian_coef();
  a.saved = const_cast<float*>(saved);
  a.d_out = d_out; a.d_colors = d_colors;
  a.d_vp = reinterpret_cast<float4*>(d_positions);
  return dispatch(true, C, a, images, n, stream, err);
}

}  // namespace dr
