// Rasterize-then-splat for GB300: viewport positions from the clip-space
// interpolation of the rasterized triangles, 3x3 Gaussian splats with the
// per-tap surface test, normalization and over compositing
// (diffren/jax/internal/splat.py:26-229, diffren/jax/composite.py:20-37),
// and the VJP of all of it.
//
// Both kernels work on screen tiles with shared-memory halos. The forward
// kernel gathers, for each output pixel, the splats of its 3x3 neighbours
// from a 1-pixel halo tile. The backward kernel is the gather form of the
// adjoint: it recomputes the accumulation of the tile plus a 1-pixel ring
// from a 2-pixel halo of sources, forms the adjoints of the accumulators
// there, and lets every source splat read the adjoints of the 9 pixels it
// reached. No image buffer is written with atomics; only the per-vertex
// clip-space gradient (a scatter over triangles) uses float atomics.
#include <algorithm>
#include <cmath>
#include <string>

#include "common.cuh"
#include "internal.h"

namespace dr {
namespace {

constexpr int kTX = 32;  // tile width (one warp per row)

struct SplatArgs {
  const float4* clip;
  const int32_t* tris;
  const int32_t* ids;
  const float* z;
  const float* bary;
  const float* colors;
  int L, TY;
  float coef;
  // forward outputs
  float* out;
  float* accum;
  float* normalized;
  // backward
  const float* d_out;
  float* d_colors;
  float4* d_clip;
  float* d_bary;
};

// Viewport position and foreground flag of one (layer, pixel) element:
// clip xyzw interpolated with background (0, 0, 1, 1), ndc = xyz / w,
// viewport = ((ndc + 1) * (W, H, 1)) * 0.5    (splat.py:207-221).
__device__ __forceinline__ float4 source_point(const SplatArgs& a, const Batch& B,
                                               int img, int64_t e) {
  const float W = __int2float_rn(B.width[img]), H = __int2float_rn(B.height[img]);
  float4 c = make_float4(0.0f, 0.0f, 1.0f, 1.0f);
  float fg = 0.0f;
  if (__ldg(a.z + e) != 1.0f) {
    fg = 1.0f;
    const int32_t* t = a.tris + 3 * (B.triangle_offset[img] + __ldg(a.ids + e));
    const float4* vb = a.clip + B.vertex_offset[img];
    const float4 v0 = __ldg(vb + __ldg(t)), v1 = __ldg(vb + __ldg(t + 1)),
                 v2 = __ldg(vb + __ldg(t + 2));
    const float b0 = __ldg(a.bary + 3 * e), b1 = __ldg(a.bary + 3 * e + 1),
                b2 = __ldg(a.bary + 3 * e + 2);
    c.x = __fadd_rn(__fadd_rn(__fmul_rn(v0.x, b0), __fmul_rn(v1.x, b1)), __fmul_rn(v2.x, b2));
    c.y = __fadd_rn(__fadd_rn(__fmul_rn(v0.y, b0), __fmul_rn(v1.y, b1)), __fmul_rn(v2.y, b2));
    c.z = __fadd_rn(__fadd_rn(__fmul_rn(v0.z, b0), __fmul_rn(v1.z, b1)), __fmul_rn(v2.z, b2));
    c.w = __fadd_rn(__fadd_rn(__fmul_rn(v0.w, b0), __fmul_rn(v1.w, b1)), __fmul_rn(v2.w, b2));
  }
  const float nx = __fdiv_rn(c.x, c.w), ny = __fdiv_rn(c.y, c.w), nz = __fdiv_rn(c.z, c.w);
  return make_float4(__fmul_rn(__fmul_rn(__fadd_rn(nx, 1.0f), W), 0.5f),
                     __fmul_rn(__fmul_rn(__fadd_rn(ny, 1.0f), H), 0.5f),
                     __fmul_rn(__fmul_rn(__fadd_rn(nz, 1.0f), 1.0f), 0.5f), fg);
}

// Shared-memory view of a source region of R pixels (row stride `stride`):
// sp[l*R + i] = (viewport xyz, fg); col[(l*C + c)*R + i] = color channel c.
struct Region {
  float4* sp;
  float* col;
  int R, stride, x0, y0;  // image coordinates of region pixel 0
};

// Loads the region [x0, x0 + stride) x [y0, y0 + rows) of image `img`, all
// layers. Pixels outside the image get fg = 0 (they never splat).
template <int C>
__device__ void load_region(const SplatArgs& a, const Batch& B, int img, Region r) {
  const int W = B.width[img], H = B.height[img];
  const int64_t HW = int64_t(W) * H;
  const int64_t base = int64_t(a.L) * B.pix_off[img];
  const int n = a.L * r.R;
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int l = k / r.R, i = k - l * r.R;
    const int y = r.y0 + i / r.stride, x = r.x0 + i % r.stride;
    float4 sp = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
    float col[C];
#pragma unroll
    for (int c = 0; c < C; ++c) col[c] = 0.0f;
    if (x >= 0 && y >= 0 && x < W && y < H) {
      const int64_t e = base + l * HW + int64_t(y) * W + x;
      sp = source_point(a, B, img, e);
      const float* cp = a.colors + e * C;
#pragma unroll
      for (int c = 0; c < C; ++c) col[c] = __ldg(cp + c);
    }
    r.sp[l * r.R + i] = sp;
#pragma unroll
    for (int c = 0; c < C; ++c) r.col[(l * C + c) * r.R + i] = col[c];
  }
}

// Surface index of the splat from source s reaching pixel p
// (splat.py:131-145): c = argmin_k |zS_k - zD_0|, t = argmin_k |zD_k - zS_0|
// (first index on ties); -t if the tap match is strictly better, else c.
__device__ __forceinline__ int surface_index(const Region& r, int s, int p, int L) {
  const float zD0 = r.sp[p].z, zS0 = r.sp[s].z;
  float minc = fabsf(__fsub_rn(r.sp[s].z, zD0));
  float mint = fabsf(__fsub_rn(r.sp[p].z, zS0));
  int c = 0, t = 0;
  for (int k = 1; k < L; ++k) {
    const float dc = fabsf(__fsub_rn(r.sp[k * r.R + s].z, zD0));
    if (dc < minc) { minc = dc; c = k; }
    const float dt = fabsf(__fsub_rn(r.sp[k * r.R + p].z, zS0));
    if (dt < mint) { mint = dt; t = k; }
  }
  return mint < minc ? -t : c;
}

// Tap offset (splat.py:106-113) and weight (splat.py:114-115).
__device__ __forceinline__ void tap(float4 q, int u, int v, float coef, float& dx,
                                    float& dy, float& w) {
  dx = __fadd_rn(__fsub_rn(__fadd_rn(floorf(q.x), 0.5f), q.x), float(u));
  dy = __fadd_rn(__fsub_rn(__fadd_rn(floorf(q.y), 0.5f), q.y), float(v));
  const float d2 = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
  w = __fmul_rn(__fmul_rn(q.w, coef), expf(__fmul_rn(-2.0f, d2)));
}

// Accumulators of pixel p (region index p; image coordinates px, py) over
// the 3x3 sources of every layer, in the reference's order (layer, u, v).
template <int C>
__device__ void accumulate(const Region& r, int p, int px, int py, int W, int H, int L,
                           float coef, float acc[3][C], float wacc[3]) {
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    wacc[k] = 0.0f;
#pragma unroll
    for (int c = 0; c < C; ++c) acc[k][c] = 0.0f;
  }
  int surf[9];
  bool ok[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) {
    const int u = j / 3 - 1, v = j % 3 - 1;
    const int sx = px - u, sy = py - v;
    ok[j] = sx >= 0 && sy >= 0 && sx < W && sy < H;
    surf[j] = ok[j] ? surface_index(r, p - v * r.stride - u, p, L) : 0;
  }
  for (int l = 0; l < L; ++l) {
#pragma unroll
    for (int j = 0; j < 9; ++j) {
      if (!ok[j]) continue;
      const int u = j / 3 - 1, v = j % 3 - 1;
      const int s = p - v * r.stride - u;
      const float4 q = r.sp[l * r.R + s];
      if (q.w == 0.0f) continue;
      float dx, dy, w;
      tap(q, u, v, coef, dx, dy, w);
      const float m0 = surf[j] > l ? 1.0f : 0.0f;
      const float m1 = surf[j] == l ? 1.0f : 0.0f;
      const float m2 = surf[j] < l ? 1.0f : 0.0f;
#pragma unroll
      for (int c = 0; c < C; ++c) {
        const float tc = __fmul_rn(w, r.col[(l * C + c) * r.R + s]);
        acc[0][c] = __fadd_rn(acc[0][c], __fmul_rn(tc, m0));
        acc[1][c] = __fadd_rn(acc[1][c], __fmul_rn(tc, m1));
        acc[2][c] = __fadd_rn(acc[2][c], __fmul_rn(tc, m2));
      }
      wacc[0] = __fadd_rn(wacc[0], __fmul_rn(w, m0));
      wacc[1] = __fadd_rn(wacc[1], __fmul_rn(w, m1));
      wacc[2] = __fadd_rn(wacc[2], __fmul_rn(w, m2));
    }
  }
}

// normalization_scales = 1 / (max(W - 1, 0) + 1)   (splat.py:168-169)
__device__ __forceinline__ float norm_scale(float w) {
  return __fdiv_rn(1.0f, __fadd_rn(fmaxf(__fsub_rn(w, 1.0f), 0.0f), 1.0f));
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

template <int C>
__global__ void __launch_bounds__(256) splat_fwd_kernel(SplatArgs a, Batch B) {
  extern __shared__ __align__(16) unsigned char smem[];
  const TileRef tr = tile_of(B, a.TY);
  const int TY = a.TY, L = a.L;
  Region r;
  r.stride = kTX + 2;
  r.R = r.stride * (TY + 2);
  r.x0 = tr.x0 - 1;
  r.y0 = tr.y0 - 1;
  r.sp = reinterpret_cast<float4*>(smem);
  r.col = reinterpret_cast<float*>(r.sp + L * r.R);
  load_region<C>(a, B, tr.img, r);
  __syncthreads();

  const int tx = threadIdx.x % kTX, ty = threadIdx.x / kTX;
  const int W = B.width[tr.img], H = B.height[tr.img];
  const int px = tr.x0 + tx, py = tr.y0 + ty;
  if (px >= W || py >= H) return;
  float acc[3][C], wacc[3];
  accumulate<C>(r, (ty + 1) * r.stride + tx + 1, px, py, W, H, L, a.coef, acc, wacc);

  float n[3][C];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float s = norm_scale(wacc[k]);
#pragma unroll
    for (int c = 0; c < C; ++c) n[k][c] = __fmul_rn(acc[k][c], s);
  }
  const int64_t pix = B.pix_off[tr.img] + int64_t(py) * W + px;
  const int64_t HW = int64_t(W) * H;
  // over: out = n2; out = n1 + (1 - a1) out; out = n0 + (1 - a0) out
  const float t1 = __fsub_rn(1.0f, n[1][C - 1]), t0 = __fsub_rn(1.0f, n[0][C - 1]);
  float* o = a.out + pix * C;
#pragma unroll
  for (int c = 0; c < C; ++c) {
    const float mid = __fadd_rn(n[1][c], __fmul_rn(t1, n[2][c]));
    o[c] = __fadd_rn(n[0][c], __fmul_rn(t0, mid));
  }
  if (a.accum || a.normalized) {
    const int64_t base = 3 * B.pix_off[tr.img] * C + (int64_t(py) * W + px) * C;
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int c = 0; c < C; ++c) {
        if (a.accum) a.accum[base + k * HW * C + c] = acc[k][c];
        if (a.normalized) a.normalized[base + k * HW * C + c] = n[k][c];
      }
  }
}

// Adjoints of the accumulators at one pixel, from d_out through the over
// compositing and the normalization (jnp.maximum splits its gradient 0.5 /
// 0.5 at equality, as lax.max does).
template <int C>
__device__ __forceinline__ void accum_adjoint(const float acc[3][C], const float wacc[3],
                                              const float* d_out, float g[3][C],
                                              float h[3]) {
  float s[3], n[3][C];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    s[k] = norm_scale(wacc[k]);
#pragma unroll
    for (int c = 0; c < C; ++c) n[k][c] = acc[k][c] * s[k];
  }
  const float a0 = n[0][C - 1], a1 = n[1][C - 1];
  float dO[C], dn[3][C];
  float d_a0 = 0.0f, d_a1 = 0.0f;
#pragma unroll
  for (int c = 0; c < C; ++c) {
    dO[c] = d_out[c];
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
  extern __shared__ __align__(16) unsigned char smem[];
  const TileRef tr = tile_of(B, a.TY);
  const int TY = a.TY, L = a.L;
  const int W = B.width[tr.img], H = B.height[tr.img];
  // Sources: tile + 2-pixel ring. Adjoints: tile + 1-pixel ring.
  Region r;
  r.stride = kTX + 4;
  r.R = r.stride * (TY + 4);
  r.x0 = tr.x0 - 2;
  r.y0 = tr.y0 - 2;
  r.sp = reinterpret_cast<float4*>(smem);
  r.col = reinterpret_cast<float*>(r.sp + L * r.R);
  const int S1 = kTX + 2, R1 = S1 * (TY + 2);
  float* adj = r.col + L * C * r.R;  // [3*(C+1)][R1]: g[k][c] then h[k]
  load_region<C>(a, B, tr.img, r);
  __syncthreads();

  for (int i = threadIdx.x; i < R1; i += blockDim.x) {
    const int qx = tr.x0 - 1 + i % S1, qy = tr.y0 - 1 + i / S1;
    float g[3][C], h[3];
    if (qx >= 0 && qy >= 0 && qx < W && qy < H) {
      float acc[3][C], wacc[3];
      const int p = (i / S1 + 1) * r.stride + (i % S1) + 1;
      accumulate<C>(r, p, qx, qy, W, H, L, a.coef, acc, wacc);
      const float* dO = a.d_out + (B.pix_off[tr.img] + int64_t(qy) * W + qx) * C;
      float d[C];
#pragma unroll
      for (int c = 0; c < C; ++c) d[c] = __ldg(dO + c);
      accum_adjoint<C>(acc, wacc, d, g, h);
    } else {
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        h[k] = 0.0f;
#pragma unroll
        for (int c = 0; c < C; ++c) g[k][c] = 0.0f;
      }
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
  const int s = (ty + 2) * r.stride + tx + 2;  // source in the region
  const int s1 = (ty + 1) * S1 + tx + 1;       // same pixel in the adjoint grid
  int surf[9];
  bool ok[9];
#pragma unroll
  for (int j = 0; j < 9; ++j) {
    const int u = j / 3 - 1, v = j % 3 - 1;
    const int px = sx + u, py = sy + v;
    ok[j] = px >= 0 && py >= 0 && px < W && py < H;
    surf[j] = ok[j] ? surface_index(r, s, s + v * r.stride + u, L) : 0;
  }
  const int64_t HW = int64_t(W) * H;
  const int64_t ebase = int64_t(L) * B.pix_off[tr.img] + int64_t(sy) * W + sx;
  const float Wf = __int2float_rn(W), Hf = __int2float_rn(H);
  for (int l = 0; l < L; ++l) {
    const int64_t e = ebase + l * HW;
    const float4 q = r.sp[l * r.R + s];
    float dcol[C];
#pragma unroll
    for (int c = 0; c < C; ++c) dcol[c] = 0.0f;
    float dvx = 0.0f, dvy = 0.0f;
    if (q.w != 0.0f) {
#pragma unroll
      for (int j = 0; j < 9; ++j) {
        if (!ok[j]) continue;
        const int u = j / 3 - 1, v = j % 3 - 1;
        float dx, dy, w;
        tap(q, u, v, a.coef, dx, dy, w);
        const int k = surf[j] > l ? 0 : (surf[j] == l ? 1 : 2);
        const int p1 = s1 + v * S1 + u;
        float dw = adj[(k * (C + 1) + C) * R1 + p1];
#pragma unroll
        for (int c = 0; c < C; ++c) {
          const float gc = adj[(k * (C + 1) + c) * R1 + p1];
          dcol[c] += w * gc;
          dw += gc * r.col[(l * C + c) * r.R + s];
        }
        const float f = 4.0f * w * dw;
        dvx += f * dx;
        dvy += f * dy;
      }
    }
    float* dc = a.d_colors + e * C;
#pragma unroll
    for (int c = 0; c < C; ++c) dc[c] = dcol[c];
    if (q.w == 0.0f) {
      if (a.d_bary) {
        a.d_bary[3 * e] = 0.0f;
        a.d_bary[3 * e + 1] = 0.0f;
        a.d_bary[3 * e + 2] = 0.0f;
      }
      continue;
    }
    // Through viewport = ((xyz / w + 1) * (W, H)) * 0.5 and the
    // interpolation clip = sum_i b_i V_i (viewport z carries no gradient).
    const int32_t* t = a.tris + 3 * (B.triangle_offset[tr.img] + __ldg(a.ids + e));
    const int vid[3] = {__ldg(t), __ldg(t + 1), __ldg(t + 2)};
    const float4* vb = a.clip + B.vertex_offset[tr.img];
    const float4 V[3] = {__ldg(vb + vid[0]), __ldg(vb + vid[1]), __ldg(vb + vid[2])};
    const float b[3] = {__ldg(a.bary + 3 * e), __ldg(a.bary + 3 * e + 1),
                        __ldg(a.bary + 3 * e + 2)};
    const float cx = V[0].x * b[0] + V[1].x * b[1] + V[2].x * b[2];
    const float cy = V[0].y * b[0] + V[1].y * b[1] + V[2].y * b[2];
    const float cw = V[0].w * b[0] + V[1].w * b[1] + V[2].w * b[2];
    const float dnx = dvx * Wf * 0.5f, dny = dvy * Hf * 0.5f;
    const float4 dcl = make_float4(dnx / cw, dny / cw, 0.0f, -(dnx * cx + dny * cy) / (cw * cw));
    float4* dv = a.d_clip + B.vertex_offset[tr.img];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      atomicAdd(dv + vid[i], make_float4(b[i] * dcl.x, b[i] * dcl.y, 0.0f, b[i] * dcl.w));
      if (a.d_bary) a.d_bary[3 * e + i] = V[i].x * dcl.x + V[i].y * dcl.y + V[i].w * dcl.w;
    }
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

size_t fwd_smem(int L, int C, int TY) {
  const size_t R = size_t(kTX + 2) * (TY + 2);
  return size_t(L) * R * (16 + 4 * C);
}

size_t bwd_smem(int L, int C, int TY) {
  const size_t R = size_t(kTX + 4) * (TY + 4);
  const size_t R1 = size_t(kTX + 2) * (TY + 2);
  return size_t(L) * R * (16 + 4 * C) + 3 * size_t(C + 1) * R1 * 4;
}

constexpr size_t kSmemBudget = 200 * 1024;

int pick_ty(int L, int C, bool bwd) {
  for (int ty : {8, 4, 2, 1}) {
    const size_t need = bwd ? bwd_smem(L, C, ty) : fwd_smem(L, C, ty);
    if (need <= kSmemBudget) return ty;
  }
  return 0;
}

template <int C>
int run_splat(bool bwd, SplatArgs a, const dr_image_desc* images, int n,
              cudaStream_t stream, std::string& err) {
  const int TY = pick_ty(a.L, C, bwd);
  if (!TY) { err = "layers x channels too large for shared memory"; return DR_ERR_INVALID_ARGUMENT; }
  a.TY = TY;
  const size_t smem = bwd ? bwd_smem(a.L, C, TY) : fwd_smem(a.L, C, TY);
  auto kern = bwd ? splat_bwd_kernel<C> : splat_fwd_kernel<C>;
  // Raise the dynamic shared-memory limit once per kernel and size (host-side
  // attribute only; later calls, e.g. under stream capture, skip it).
  static size_t reserved[2] = {0, 0};
  if (smem > 48 * 1024 && smem > reserved[bwd]) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(smem)) != cudaSuccess) {
      err = "cannot reserve shared memory for the splat kernel";
      return DR_ERR_CUDA;
    }
    reserved[bwd] = smem;
  }
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    if (!make_batch(images + g0, cnt, a.L, kTX, TY, b, err)) return DR_ERR_INVALID_ARGUMENT;
    const int tiles = b.tile_start[cnt];
    if (tiles > 0) kern<<<tiles, kTX * TY, smem, stream>>>(a, b);
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

bool check_common(const float* clip, int L, int n, const dr_image_desc* images,
                  std::string& err, int& rc) {
  rc = DR_OK;
  if (n < 0 || (n > 0 && !images)) { err = "invalid image table"; rc = DR_ERR_INVALID_ARGUMENT; return false; }
  if (L < 1 || L > DR_MAX_LAYERS) { err = "num_layers must be in [1, 16]"; rc = DR_ERR_INVALID_ARGUMENT; return false; }
  if ((reinterpret_cast<uintptr_t>(clip) & 15) != 0) {
    err = "clip_vertices must be 16-byte aligned";
    rc = DR_ERR_MISALIGNED;
    return false;
  }
  return n > 0;
}

}  // namespace

int splat_fwd_launch(const float* clip, const int32_t* tris, const int32_t* ids,
                     const float* z, const float* bary, const float* colors, int C,
                     const dr_image_desc* images, int n, int L, float* out, float* accum,
                     float* normalized, cudaStream_t stream, std::string& err) {
  int rc;
  if (!check_common(clip, L, n, images, err, rc)) return rc;
  SplatArgs a{};
  a.clip = reinterpret_cast<const float4*>(clip);
  a.tris = tris; a.ids = ids; a.z = z; a.bary = bary; a.colors = colors;
  a.L = L;
  a.coef = gaussian_coef();
  a.out = out; a.accum = accum; a.normalized = normalized;
  return dispatch(false, C, a, images, n, stream, err);
}

int splat_bwd_launch(const float* d_out, const float* clip, const int32_t* tris,
                     const int32_t* ids, const float* z, const float* bary,
                     const float* colors, int C, const dr_image_desc* images, int n, int L,
                     float* d_colors, float* d_clip, float* d_bary, cudaStream_t stream,
                     std::string& err) {
  int rc;
  if (!check_common(clip, L, n, images, err, rc)) return rc;
  if ((reinterpret_cast<uintptr_t>(d_clip) & 15) != 0) {
    err = "d_clip_vertices must be 16-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  SplatArgs a{};
  a.clip = reinterpret_cast<const float4*>(clip);
  a.tris = tris; a.ids = ids; a.z = z; a.bary = bary; a.colors = colors;
  a.L = L;
  a.coef = gaussian_coef();
  a.d_out = d_out; a.d_colors = d_colors;
  a.d_clip = reinterpret_cast<float4*>(d_clip);
  a.d_bary = d_bary;
  return dispatch(true, C, a, images, n, stream, err);
}

}  // namespace dr
