// Shared device code of the diffren_gb300 kernels: the batch table passed by
// value in kernel parameters, and the exact triangle arithmetic of diffren's
// rasterizer written with explicitly rounded intrinsics so that nvcc cannot
// contract or reorder any float operation. Where the reference's CUDA build
// fuses a multiply and an add (nvcc's default contraction), the discretized
// depth semantics use an explicit fused multiply-add at that place.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "diffren_gb300.h"

namespace dr {

// Triangles, images and tiles of one launch. Passed by value as a kernel
// parameter so a launch needs no device-side table and is graph-capturable.
struct Batch {
  int32_t n;
  int32_t num_layers;
  int64_t tri_start[DR_MAX_BATCH_INLINE + 1];   // prefix of num_triangles
  int64_t pix_prefix[DR_MAX_BATCH_INLINE + 1];  // prefix of width*height
  int64_t pix_off[DR_MAX_BATCH_INLINE];         // caller's pixel_offset
  int32_t tile_start[DR_MAX_BATCH_INLINE + 1];  // prefix of tiles per image
  int32_t width[DR_MAX_BATCH_INLINE];
  int32_t height[DR_MAX_BATCH_INLINE];
  int32_t num_vertices[DR_MAX_BATCH_INLINE];
  int32_t tiles_x[DR_MAX_BATCH_INLINE];
  int64_t vertex_offset[DR_MAX_BATCH_INLINE];
  int64_t triangle_offset[DR_MAX_BATCH_INLINE];
};

// Largest i in [0, n) with start[i] <= key (start[0] == 0, start ascending).
template <typename T>
__device__ __forceinline__ int find_segment(const T* start, int n, T key) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (start[mid] <= key) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// One (layer, pixel) element of a packed layered batch buffer: flat index q
// runs over every image's L x H x W elements in image order.
struct PixelRef {
  int img;
  int64_t e;    // element index in the packed layered buffers
  int64_t pix;  // pixel index inside its image (y * W + x)
  int x, y;
};

// Image of flat element q, found by comparing L * pix_prefix (no 64-bit
// division), and its element index in the packed buffers.
__device__ __forceinline__ int locate(const Batch& B, int L, int64_t q, int64_t& local) {
  int lo = 0, hi = B.n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (int64_t(L) * B.pix_prefix[mid] <= q) lo = mid; else hi = mid - 1;
  }
  local = q - int64_t(L) * B.pix_prefix[lo];
  return lo;
}

__device__ __forceinline__ PixelRef decode(const Batch& B, int L, int64_t q) {
  PixelRef r;
  int64_t local;
  r.img = locate(B, L, q, local);
  r.e = int64_t(L) * B.pix_off[r.img] + local;
  // Image sides are at most DR_MAX_IMAGE_DIM, so a layer has < 2^30 pixels:
  // strip whole layers, then 32-bit arithmetic.
  const uint32_t W = uint32_t(B.width[r.img]);
  const int64_t hw = int64_t(W) * B.height[r.img];
  while (local >= hw) local -= hw;
  const uint32_t pix = uint32_t(local);
  r.pix = pix;
  r.y = int(pix / W);
  r.x = int(pix - uint32_t(r.y) * W);
  return r;
}

// Optional outputs of the rasterizer's epilogue: per layer sample the splat
// position (viewport xyz + foreground flag) and the interpolated attributes.
struct SampleOutputs {
  const float* attr;  // [V, K] packed per mesh (nullable)
  int K;
  float* attr_out;    // [L * P, K]
  float4* positions;  // [L * P] viewport xyz + clip w; null = no fused outputs
  int32_t* vertex_ids;  // [L * P, 3] (nullable)
};

// ------------------------------------------------------- sample helpers
// Channels k0 .. k0 + n - 1 (n <= 4) of a row; `vec` when the row is
// 16-byte aligned and holds 4 channels from k0.
__device__ __forceinline__ float4 load_chunk(const float* p, int n, bool vec) {
  if (vec) return __ldg(reinterpret_cast<const float4*>(p));
  float4 v = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  v.x = __ldg(p);
  if (n > 1) v.y = __ldg(p + 1);
  if (n > 2) v.z = __ldg(p + 2);
  if (n > 3) v.w = __ldg(p + 3);
  return v;
}

__device__ __forceinline__ void store_chunk(float* p, float4 v, int n, bool vec) {
  if (vec) {
    *reinterpret_cast<float4*>(p) = v;
    return;
  }
  p[0] = v.x;
  if (n > 1) p[1] = v.y;
  if (n > 2) p[2] = v.z;
  if (n > 3) p[3] = v.w;
}

// (a0 b0 + a1 b1) + a2 b2 per channel (interpolate.py:24-63).
__device__ __forceinline__ float lerp3(float a0, float a1, float a2, const float b[3]) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a0, b[0]), __fmul_rn(a1, b[1])), __fmul_rn(a2, b[2]));
}

// Splat position of a layer sample (splat.py:207-221): viewport
// ((xyz / w + 1) * (W, H, 1)) * 0.5 of the interpolated clip coordinates c
// ((0, 0, 1, 1) on background), with the foreground flag in w.
__device__ __forceinline__ float4 viewport_of(float4 c, float W, float H, float fg) {
  const float nx = __fdiv_rn(c.x, c.w), ny = __fdiv_rn(c.y, c.w), nz = __fdiv_rn(c.z, c.w);
  return make_float4(__fmul_rn(__fmul_rn(__fadd_rn(nx, 1.0f), W), 0.5f),
                     __fmul_rn(__fmul_rn(__fadd_rn(ny, 1.0f), H), 0.5f),
                     __fmul_rn(__fmul_rn(__fadd_rn(nz, 1.0f), 1.0f), 0.5f), fg);
}

// (c0 b0 + c1 b1) + c2 b2 per coordinate of three clip vertices.
__device__ __forceinline__ float4 lerp_clip(float4 v0, float4 v1, float4 v2, const float b[3]) {
  return make_float4(lerp3(v0.x, v1.x, v2.x, b), lerp3(v0.y, v1.y, v2.y, b),
                     lerp3(v0.z, v1.z, v2.z, b), lerp3(v0.w, v1.w, v2.w, b));
}

// ------------------------------------------------------------ exact math
// Float-to-integer conversions round toward zero, saturate and map NaN to 0
// (cvt.rzi); int64-to-float rounds to nearest. The CPU checker implements
// the same rules explicitly.
__device__ __forceinline__ long long wmul(long long a, long long b) {
  return (long long)((unsigned long long)a * (unsigned long long)b);
}
__device__ __forceinline__ long long wadd(long long a, long long b) {
  return (long long)((unsigned long long)a + (unsigned long long)b);
}
__device__ __forceinline__ long long wsub(long long a, long long b) {
  return (long long)((unsigned long long)a - (unsigned long long)b);
}
__device__ __forceinline__ long long shl16(long long a) {
  return (long long)((unsigned long long)a << 16);
}

// ToFixedPoint (rasterize_utils.h:57-59): 16 fractional bits.
__device__ __forceinline__ long long to_fixed(float f) {
  const float s = __fmul_rn(f, 65536.0f);
  // Below 2^31 the 32-bit conversion truncates to the same value (NaN fails
  // the test and takes the 64-bit conversion, which maps it to INT64_MIN).
  if (fabsf(s) < 2147483648.0f) return (long long)__float2int_rz(s);
  return __float2ll_rz(s);
}

// AddPoint (rasterize_utils.h:75-84) on the running box {l, r, b, t}.
__device__ __forceinline__ void box_add_point(float x, float y, float w, int W,
                                              int H, int& l, int& r, int& b,
                                              int& t) {
  const float px = __fmul_rn(__fmul_rn(0.5f, __fadd_rn(__fdiv_rn(x, w), 1.0f)),
                             __int2float_rn(W));
  const float py = __fmul_rn(__fmul_rn(0.5f, __fadd_rn(__fdiv_rn(y, w), 1.0f)),
                             __int2float_rn(H));
  l = min(W, max(0, __float2int_rz(floorf(fminf(__int2float_rn(l), px)))));
  r = min(W, max(0, __float2int_rz(ceilf(fmaxf(__int2float_rn(r), px)))));
  b = min(H, max(0, __float2int_rz(floorf(fminf(__int2float_rn(b), py)))));
  t = min(H, max(0, __float2int_rz(ceilf(fmaxf(__int2float_rn(t), py)))));
}

// AddNearPoint (rasterize_utils.h:86-99): where edge p0->p1 meets z/w = -1.
// `fused`: p0 + s (p1 - p0) as one fused multiply-add per coordinate, as
// nvcc's default contraction compiles it in the reference's CUDA build (the
// CPU build rounds the product first). The box edge this point sets bounds
// the visible part of the triangle, so pixels that the two forms' boxes
// disagree on lie beyond the near plane and never produce a fragment.
__device__ __forceinline__ void box_add_near(float4 p0, float4 p1, int W, int H,
                                             int& l, int& r, int& b, int& t, bool fused) {
  const float denom =
      __fsub_rn(__fadd_rn(__fsub_rn(p0.z, p1.z), p0.w), p1.w);
  if (denom != 0.0f) {
    const float s = __fdiv_rn(__fadd_rn(p0.z, p0.w), denom);
    const float dx = __fsub_rn(p1.x, p0.x), dy = __fsub_rn(p1.y, p0.y);
    const float dw = __fsub_rn(p1.w, p0.w);
    const float x = fused ? __fmaf_rn(s, dx, p0.x) : __fadd_rn(p0.x, __fmul_rn(s, dx));
    const float y = fused ? __fmaf_rn(s, dy, p0.y) : __fadd_rn(p0.y, __fmul_rn(s, dy));
    const float w = fused ? __fmaf_rn(s, dw, p0.w) : __fadd_rn(p0.w, __fmul_rn(s, dw));
    box_add_point(x, y, w, W, H, l, r, b, t);
  }
}

__device__ __forceinline__ bool clip_visible(float4 p) {
  return p.w > 0.0f && p.z >= -p.w;
}

// ComputeTriangleBoundingBox (rasterize_utils.h:111-161). box = {l, r, b, t}
// with l, b inclusive and r, t exclusive. `fused`: see box_add_near.
__device__ __forceinline__ bool triangle_box(float4 v0, float4 v1, float4 v2,
                                             int W, int H, int4& box, bool fused) {
  int l = W, r = 0, b = H, t = 0;
  const bool s0 = clip_visible(v0), s1 = clip_visible(v1), s2 = clip_visible(v2);
  if (s0) {
    box_add_point(v0.x, v0.y, v0.w, W, H, l, r, b, t);
    if (!s1) box_add_near(v0, v1, W, H, l, r, b, t, fused);
    if (!s2) box_add_near(v0, v2, W, H, l, r, b, t, fused);
  }
  if (s1) {
    box_add_point(v1.x, v1.y, v1.w, W, H, l, r, b, t);
    if (!s2) box_add_near(v1, v2, W, H, l, r, b, t, fused);
    if (!s0) box_add_near(v1, v0, W, H, l, r, b, t, fused);
  }
  if (s2) {
    box_add_point(v2.x, v2.y, v2.w, W, H, l, r, b, t);
    if (!s0) box_add_near(v2, v0, W, H, l, r, b, t, fused);
    if (!s1) box_add_near(v2, v1, W, H, l, r, b, t, fused);
  }
  box = make_int4(l, r, b, t);
  return (r > l) && (t > b);
}

// ComputeUnnormalizedMatrixInverse (rasterize_utils.h:176-206) of the matrix
// with columns (x_i, y_i, w_i) in 16.16 fixed point. Row i of m holds the
// coefficients (a, b, c) of edge function i. For NONE and FRONT the reference
// scales each int64 entry by a float sign, which rounds it to float
// precision; that rounding is part of the result.
__device__ __forceinline__ void edge_matrix(float4 v0, float4 v1, float4 v2,
                                            int culling, long long m[9]) {
  const long long x0 = to_fixed(v0.x), x1 = to_fixed(v1.x), x2 = to_fixed(v2.x);
  const long long y0 = to_fixed(v0.y), y1 = to_fixed(v1.y), y2 = to_fixed(v2.y);
  const long long w0 = to_fixed(v0.w), w1 = to_fixed(v1.w), w2 = to_fixed(v2.w);
  m[0] = wsub(wmul(y1, w2), wmul(w1, y2));
  m[1] = wsub(wmul(x2, w1), wmul(w2, x1));
  m[2] = wsub(wmul(x1, y2), wmul(y1, x2));
  m[3] = wsub(wmul(y2, w0), wmul(w2, y0));
  m[4] = wsub(wmul(x0, w2), wmul(w0, x2));
  m[5] = wsub(wmul(x2, y0), wmul(y2, x0));
  m[6] = wsub(wmul(y0, w1), wmul(w0, y1));
  m[7] = wsub(wmul(x1, w0), wmul(w1, x0));
  m[8] = wsub(wmul(x0, y1), wmul(y0, x1));
  if (culling == DR_CULL_NONE || culling == DR_CULL_FRONT) {
    const long long det_i = wadd(wadd(wmul(x0, m[0]), wmul(x1, m[3])), wmul(x2, m[6]));
    const float det = __ll2float_rn(det_i);
    const float sign = culling == DR_CULL_NONE ? copysignf(1.0f, det) : -1.0f;
#pragma unroll
    for (int i = 0; i < 9; ++i) m[i] = __float2ll_rz(__fmul_rn(__ll2float_rn(m[i]), sign));
  }
}

// Fixed-point NDC coordinate of the center of pixel i of n
// (rasterize_utils.h:225-228). `fused`: (2/n) (i + 0.5) - 1 as one fused
// multiply-add, which is how nvcc's default contraction compiles the
// reference's CUDA rasterizer (checked bit for bit against that build); the
// CPU rasterizer rounds the product first. The two differ only where 2/n is
// not a power of two.
__device__ __forceinline__ long long pixel_center_fixed(int i, int n, bool fused) {
  const float scale = __fdiv_rn(2.0f, __int2float_rn(n));
  const float c = __fadd_rn(__int2float_rn(i), 0.5f);
  const float p = fused ? __fmaf_rn(scale, c, -1.0f) : __fsub_rn(__fmul_rn(scale, c), 1.0f);
  return to_fixed(p);
}

// Edge functions at a pixel (rasterize_utils.h:220-238).
__device__ __forceinline__ void edge_values(const long long m[9], long long px,
                                            long long py, long long e[3]) {
#pragma unroll
  for (int i = 0; i < 3; ++i)
    e[i] = wadd(wadd(wmul(m[3 * i], px), wmul(m[3 * i + 1], py)), shl16(m[3 * i + 2]));
}

// PixelIsInsideTriangle (rasterize_utils.h:243-248).
__device__ __forceinline__ bool inside(const long long e[3]) {
  return (e[0] >= 0 && e[1] >= 0 && e[2] >= 0) && (e[0] > 0 || e[1] > 0 || e[2] > 0);
}

// Perspective-correct barycentrics (rasterize_triangles_impl.cc:79-82).
__device__ __forceinline__ void barycentrics_of(const long long e[3], float b[3]) {
  const float sum = __ll2float_rn(wadd(wadd(e[0], e[1]), e[2]));
  b[0] = __fdiv_rn(__ll2float_rn(e[0]), sum);
  b[1] = __fdiv_rn(__ll2float_rn(e[1]), sum);
  b[2] = __fdiv_rn(__ll2float_rn(e[2]), sum);
}

// b0 a0 + b1 a1 + b2 a2 as the reference's CUDA build computes it
// (rasterize_triangles_impl_cuda.cu.cc:300-302 under nvcc's default
// contraction, checked bit for bit against that build): the first product
// fused into the sum with the second, then the third fused in.
__device__ __forceinline__ float dot3_fused(const float b[3], float a0, float a1, float a2) {
  return __fmaf_rn(b[2], a2, __fmaf_rn(b[0], a0, __fmul_rn(b[1], a1)));
}

// The same with every operation rounded, as the CPU rasterizer computes it
// (rasterize_triangles_impl.cc:87-88).
__device__ __forceinline__ float dot3_rounded(const float b[3], float a0, float a1, float a2) {
  return __fadd_rn(__fadd_rn(__fmul_rn(b[0], a0), __fmul_rn(b[1], a1)), __fmul_rn(b[2], a2));
}

// NDC depth of a fragment (rasterize_triangles_impl.cc:87-89,
// rasterize_triangles_impl_cuda.cu.cc:300-303); `fused` selects the CUDA
// build's arithmetic.
__device__ __forceinline__ float fragment_z(const float b[3], float3 vz, float3 vw, bool fused) {
  const float cz = fused ? dot3_fused(b, vz.x, vz.y, vz.z) : dot3_rounded(b, vz.x, vz.y, vz.z);
  const float cw = fused ? dot3_fused(b, vw.x, vw.y, vw.z) : dot3_rounded(b, vw.x, vw.y, vw.z);
  return __fdiv_rn(cz, cw);
}

// DiscretizeZ / UndiscretizeZ (rasterize_triangles_impl_cuda.cu.cc:143-159):
// scale S = uint32 max / 2 as an integer (2^31 - 1), arithmetic in double.
// These are the reference formulas; the rasterizer uses the integer
// emulations below (GB300's FP64 rate made them its bottleneck), and
// dr_selftest_depth_codec checks the two against each other on every input.
__device__ __forceinline__ uint32_t discretize_z_fp64(float z) {
  return __double2uint_rz(__dmul_rn(__dadd_rn((double)z, 1.0), 2147483647.0));
}
__device__ __forceinline__ float undiscretize_z_fp64(uint32_t d) {
  return __double2float_rn(__dsub_rn(__ddiv_rn((double)d, 2147483647.0), 1.0));
}

typedef unsigned __int128 u128;

__device__ __forceinline__ int bitlen128(u128 x) {
  const uint64_t hi = uint64_t(x >> 64), lo = uint64_t(x);
  return hi ? 128 - __clzll(hi) : (lo ? 64 - __clzll(lo) : 0);
}

// Rounds x to a multiple of 2^g, ties to even (g >= 1).
__device__ __forceinline__ u128 round_bits_even(u128 x, int g) {
  const u128 one = 1;
  const u128 rem = x & ((one << g) - 1), half = one << (g - 1);
  u128 q = x >> g;
  if (rem > half || (rem == half && (q & 1))) q += 1;
  return q << g;
}

// x / 2^s rounded to nearest, ties to even (s >= 0), for x < 2^24.
__device__ __forceinline__ uint64_t shift_round_even(uint64_t x, int s) {
  if (s == 0) return x;
  if (s >= 64) return 0;  // x < 2^24 < half
  const uint64_t q = x >> s, rem = x & ((1ull << s) - 1), half = 1ull << (s - 1);
  return q + ((rem > half || (rem == half && (q & 1))) ? 1 : 0);
}

// Exact integer form of discretize_z_fp64 for z in [-1, 1] or NaN:
// a = RN_double(z + 1) as N * 2^-sh, then floor(RN_double(a * S)).
__device__ __forceinline__ uint32_t discretize_z(float z) {
  const uint32_t bits = __float_as_uint(z);
  const uint32_t mag = bits & 0x7fffffffu;
  // NaN: (NaN + 1) * S converts to 0x80000000 on the GPU (checked against
  // discretize_z_fp64 by dr_selftest_depth_codec). A constant keeps the
  // double-precision path out of the rasterizer entirely.
  if (mag > 0x7f800000u) return 0x80000000u;
  if (mag == 0) return 2147483647u;  // (0 + 1) * S
  const bool neg = bits >> 31;
  const int bexp = int(mag >> 23);
  if (bexp >= 120 && bexp <= 126) {
    // 2^-7 <= |z| < 1 (every visible depth but those near 0): the same
    // computation as below with sh = 24..30, where N < 2^31 and P < 2^62
    // fit 32- and 64-bit integers.
    const int sh = 150 - bexp;
    const uint32_t m = (mag & 0x7fffffu) | 0x800000u;
    const uint32_t n = neg ? (1u << sh) - m : (1u << sh) + m;
    const uint64_t P = uint64_t(n) * 2147483647u;
    const uint64_t frac_mask = (1ull << sh) - 1;
    if ((P & frac_mask) < frac_mask + 1 - (1ull << (sh - 22))) return uint32_t(P >> sh);
  }
  const uint64_t M = bexp ? ((mag & 0x7fffffu) | 0x800000u) : (mag & 0x7fffffu);
  const int E = bexp ? bexp - 150 : -149;  // |z| = M * 2^E
  uint64_t N;
  int sh;
  if (E >= -52) {  // 1 + z has at most 53 significant bits: exact
    sh = -E;
    N = neg ? (1ull << sh) - M : (1ull << sh) + M;
  } else if (!neg) {  // 1 + z in (1, 1 + 2^-29): ulp 2^-52
    sh = 52;
    N = (1ull << 52) + shift_round_even(M, -52 - E);
  } else {  // 1 + z in (1 - 2^-29, 1): ulp 2^-53
    sh = 53;
    N = (1ull << 53) - shift_round_even(M, -53 - E);
  }
  // a * S = P * 2^-sh exactly, P = N * S < 2^(sh + 32). Rounding P to 53
  // significant bits moves it by at most 2^(sh - 22) and never below
  // floor(P / 2^sh) * 2^sh (a multiple of the rounding unit), so the floor
  // only changes when P's fraction lies within 2^(sh - 22) of the next
  // integer: otherwise floor(P / 2^sh) is the answer.
  const uint64_t lo = N * 2147483647ull, hi = __umul64hi(N, 2147483647ull);
  if (sh < 64 && sh >= 23 &&
      (lo & ((1ull << sh) - 1)) < (1ull << sh) - (1ull << (sh - 22)))
    return uint32_t((lo >> sh) | (hi << (64 - sh)));
  u128 Q = u128(N) * 2147483647u;
  const int bl = bitlen128(Q);
  if (bl > 53) Q = round_bits_even(Q, bl - 53);
  return uint32_t(Q >> sh);
}

// Exact integer form of undiscretize_z_fp64: q = RN_double(d / S) from the
// repeating base-2^31 expansion of d / S, r = RN_double(q - 1), then
// RN_float(r). Fixed point in units of 2^-83 (q >= 1/S has ulp >= 2^-83).
__device__ __forceinline__ float undiscretize_z(uint32_t d) {
  const uint32_t S = 2147483647u;
  if (d >= S && d < 2 * S) {
    // q = d / S in [1, 2) (every depth in [0, 1)): with e = d - S and
    // T = e (2^31 + 1), floor(e / S * 2^93) / 2^41 = e 2^21 + T / 2^41, so
    // RN_double(q) - 1 = R 2^-52 with R = e 2^21 + T >> 41 + bit 40 of T
    // (the remainder is never zero, so there are no ties), exact in double;
    // then R rounds to 24 bits, ties to even.
    const uint64_t e = d - S;
    const uint64_t T = (e << 31) + e;
    const uint64_t R = (e << 21) + (T >> 41) + ((T >> 40) & 1u);
    if (R == 0) return 0.0f;
    const int bl = 64 - __clzll(R);
    if (bl <= 24) return float(uint32_t(R)) * 0x1p-52f;
    const int g = bl - 24;
    uint64_t mant = R >> g;
    const uint64_t rem = R & ((1ull << g) - 1), half = 1ull << (g - 1);
    if (rem > half || (rem == half && (mant & 1))) ++mant;
    return float(uint32_t(mant)) * __uint_as_float(uint32_t(127 + g - 52) << 23);
  }
  const u128 one = 1;
  const uint32_t I = (d >= S) + (d >= 2 * S);
  const uint64_t e = d - uint64_t(I) * S;  // d / S = I + e / S, e < S
  u128 Qf;  // q in units of 2^-83
  if (e == 0) {
    Qf = u128(I) << 83;
  } else {
    // floor(e / S * 2^93) = e * (2^62 + 2^31 + 1); the remainder is nonzero,
    // so rounding never ties.
    const u128 F = (u128(e) << 62) | (u128(e) << 31) | u128(e);
    if (I == 0) {
      const int n = 64 - __clzll(e);
      const int g = n + 9;  // keep 53 bits below F's leading bit n + 61
      const u128 q = (F >> g) + ((F >> (g - 1)) & 1);
      Qf = q << (n - 1);  // q * 2^(g - 93) in 2^-83 units
    } else if (I == 1) {
      const u128 q = (((one << 93) + F) >> 41) + ((F >> 40) & 1);
      Qf = q << 31;  // q * 2^-52
    } else {  // d = 2S + 1 only: q in (2, 3), ulp 2^-51
      const u128 q = (((one << 94) + F) >> 42) + ((F >> 41) & 1);
      Qf = q << 32;
    }
  }
  // r = q - 1: exact for q >= 1/2; otherwise |r| in (1/2, 1] rounds to a
  // multiple of 2^-53 (2^30 units).
  const u128 one83 = one << 83;
  bool rneg;
  u128 R;
  if (Qf >= one83) {
    rneg = false;
    R = Qf - one83;
  } else {
    rneg = true;
    R = one83 - Qf;
    if (Qf < (one << 82)) R = round_bits_even(R, 30);
  }
  if (R == 0) return 0.0f;
  const int bl = bitlen128(R);
  if (bl > 24) R = round_bits_even(R, bl - 24);
  const int bl2 = bitlen128(R);
  const int g = bl2 > 24 ? bl2 - 24 : 0;
  const float mant = float(uint32_t(R >> g));  // exact (< 2^24)
  const float v = ldexpf(mant, g - 83);
  return rneg ? -v : v;
}

// Order-preserving float -> uint32 map with -0 == +0 (float depth keys).
__device__ __forceinline__ uint32_t float_order_bits(float z) {
  if (z == 0.0f) z = 0.0f;
  const uint32_t u = __float_as_uint(z);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__device__ __forceinline__ unsigned long long empty_key(int depth_mode) {
  return depth_mode == DR_DEPTH_DISCRETIZED
             ? (unsigned long long)4294967294u << 32  // DiscretizeZ(1.0f)
             : (unsigned long long)float_order_bits(1.0f) << 32;
}

// ---------------------------------------------------------- fixed-point sums
// Deterministic accumulation: values are added as 64-bit integers in units of
// 2^-e, e chosen from a bound on what is added so that no sum can overflow;
// integer addition does not depend on order, so the sums are the same bits
// on every run.
constexpr int kFixedZero = -100000, kFixedFloat = -200000;

// e for sums of at most 2^log2_terms values of magnitude below 2 m, m given
// as its float bits: every sum stays below 2^62. kFixedZero when m is 0 (only
// zeros are added), kFixedFloat when m is not finite (callers fall back to
// float atomics, which carry the inf / NaN as the float path does).
__device__ __forceinline__ int fixed_exponent_of(unsigned m_bits, int log2_terms) {
  const float m = __uint_as_float(m_bits);
  if (!(m <= 3.402823466e38f)) return kFixedFloat;
  if (m == 0.0f) return kFixedZero;
  return 61 - ilogbf(m) - log2_terms;
}

// round(v 2^e) in integer arithmetic: v = m 2^x with a 24-bit integer m, so
// v 2^e = m 2^(x + e), shifted left exactly or right with rounding to
// nearest, ties to even (|v 2^e| < 2^62 by the choice of e).
__device__ __forceinline__ long long fixed_of(float v, int e) {
  const unsigned u = __float_as_uint(v);
  const int bexp = int((u >> 23) & 0xffu);
  const unsigned m = bexp ? ((u & 0x7fffffu) | 0x800000u) : (u & 0x7fffffu);
  const int sh = (bexp ? bexp - 150 : -149) + e;
  long long r;
  if (sh >= 0) {
    r = (long long)m << sh;
  } else if (sh < -24) {
    r = 0;  // m 2^sh < 1/2
  } else {
    const int s = -sh;
    const unsigned q = m >> s, rem = m & ((1u << s) - 1u), half = 1u << (s - 1);
    r = (long long)(q + ((rem > half || (rem == half && (q & 1u))) ? 1u : 0u));
  }
  return (u >> 31) ? -r : r;
}

__device__ __forceinline__ void add_fixed(unsigned long long* p, float v, int e) {
  atomicAdd(p, (unsigned long long)fixed_of(v, e));
}

// |v| for the fixed-point scale, +inf for a non-finite v.
__device__ __forceinline__ float fixed_mag(float v) {
  return isfinite(v) ? fabsf(v) : __int_as_float(0x7f800000);
}

// float(q 2^-e): the integer sum rounded to float once, then scaled (exact
// unless the result is subnormal).
__device__ __forceinline__ float fixed_back(unsigned long long q, int e) {
  return ldexpf(__ll2float_rn((long long)q), -e);
}

// ---------------------------------------------------------- reductions
template <typename T>
__device__ __forceinline__ T warp_inclusive_scan(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const T o = __shfl_up_sync(0xffffffffu, v, d);
    if (lane >= d) v += o;
  }
  return v;
}

// Exclusive scan over a block of NT threads; returns the block total.
template <int NT>
__device__ __forceinline__ int block_exclusive_scan(int v, int* smem_warp, int& excl) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int inc = warp_inclusive_scan(v);
  if (lane == 31) smem_warp[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int w = lane < NT / 32 ? smem_warp[lane] : 0;
    w = warp_inclusive_scan(w);
    if (lane < NT / 32) smem_warp[lane] = w;
  }
  __syncthreads();
  const int warp_base = warp ? smem_warp[warp - 1] : 0;
  const int total = smem_warp[NT / 32 - 1];
  excl = warp_base + inc - v;
  __syncthreads();
  return total;
}

}  // namespace dr
