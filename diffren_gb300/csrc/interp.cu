// Per-pixel kernels around the rasterizer: the clip-space vertex transform,
// barycentric attribute interpolation and differentiable barycentrics, each
// with its VJP. All run over the packed layers of a ragged batch in one
// launch; each thread owns one (layer, pixel) of one image.
#include <algorithm>
#include <string>

#include "common.cuh"
#include "internal.h"

namespace dr {
namespace {

constexpr int kBlock = 256;

__device__ __forceinline__ int3 load_tri(const int32_t* tris, const Batch& B, int img,
                                         int id) {
  const int32_t* t = tris + 3 * (B.triangle_offset[img] + id);
  return make_int3(__ldg(t), __ldg(t + 1), __ldg(t + 2));
}

// -------------------------------------------------------------- transform
// Each thread takes kVertsPerThread consecutive vertices: one image lookup,
// and for xyz vertices of one image starting on a 16-byte boundary three
// 16-byte loads (or stores, backward) cover the four rows.
constexpr int kVertsPerThread = 4;

// Row r of M times (x, y, z, w), products rounded and summed in order.
__device__ __forceinline__ float4 transform_one(const float (&m)[16], float x, float y, float z,
                                                float w) {
  float r[4];
#pragma unroll
  for (int k = 0; k < 4; ++k)
    r[k] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[4 * k], x), __fmul_rn(m[4 * k + 1], y)),
                               __fmul_rn(m[4 * k + 2], z)),
                     __fmul_rn(m[4 * k + 3], w));
  return make_float4(r[0], r[1], r[2], r[3]);
}

// d_v[c] = sum_r d_clip[r] M[r][c], in the order r = 0..3, fused.
__device__ __forceinline__ float transform_vjp(const float (&m)[16], float4 g, int c) {
  return __fmaf_rn(g.w, m[12 + c], __fmaf_rn(g.z, m[8 + c], __fmaf_rn(g.y, m[4 + c],
                                                                     __fmul_rn(g.x, m[c]))));
}

__device__ __forceinline__ void load_matrix(const float* M, int img, float (&m)[16]) {
#pragma unroll
  for (int k = 0; k < 16; ++k) m[k] = __ldg(M + 16 * img + k);
}

// The image holding dense vertex i (at or after `img`) and its packed index.
__device__ __forceinline__ int64_t packed_vertex(const Batch& B, int64_t i, int& img) {
  while (img + 1 < B.n && i >= B.pix_prefix[img + 1]) ++img;
  return B.vertex_offset[img] + (i - B.pix_prefix[img]);
}

// `vec`: v (dim 3) and out are 16-byte aligned.
__global__ void transform_kernel(const float* __restrict__ M, const float* __restrict__ v,
                                 int dim, Batch B, float4* __restrict__ out, bool vec) {
  const int64_t total = B.pix_prefix[B.n];  // total vertices (reused field)
  const int64_t i0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) * kVertsPerThread;
  if (i0 >= total) return;
  int img = find_segment(B.pix_prefix, B.n, i0);
  float m[16];
  load_matrix(M, img, m);
  const int64_t vi0 = B.vertex_offset[img] + (i0 - B.pix_prefix[img]);
  if (vec && dim == 3 && i0 + kVertsPerThread <= B.pix_prefix[img + 1] && (vi0 & 3) == 0) {
    const float4* src = reinterpret_cast<const float4*>(v + 3 * vi0);
    const float4 a = __ldg(src), b = __ldg(src + 1), c = __ldg(src + 2);
    out[vi0] = transform_one(m, a.x, a.y, a.z, 1.0f);
    out[vi0 + 1] = transform_one(m, a.w, b.x, b.y, 1.0f);
    out[vi0 + 2] = transform_one(m, b.z, b.w, c.x, 1.0f);
    out[vi0 + 3] = transform_one(m, c.y, c.z, c.w, 1.0f);
    return;
  }
  const int img0 = img;
  for (int u = 0; u < kVertsPerThread; ++u) {
    const int64_t i = i0 + u;
    if (i >= total) break;
    const int64_t vi = packed_vertex(B, i, img);
    if (img != img0) load_matrix(M, img, m);
    const float* p = v + dim * vi;
    const float w = dim == 4 ? __ldg(p + 3) : 1.0f;
    out[vi] = transform_one(m, __ldg(p), __ldg(p + 1), __ldg(p + 2), w);
  }
}

// VJP of transform_kernel w.r.t. the vertices: d_v[c] = sum_r d_clip[r] M[r][c]
// for c < dim. `vec`: d_v (dim 3) is 16-byte aligned.
__global__ void transform_bwd_kernel(const float* __restrict__ M,
                                     const float4* __restrict__ d_clip, int dim, Batch B,
                                     float* __restrict__ d_v, bool vec) {
  const int64_t total = B.pix_prefix[B.n];
  const int64_t i0 = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) * kVertsPerThread;
  if (i0 >= total) return;
  int img = find_segment(B.pix_prefix, B.n, i0);
  float m[16];
  load_matrix(M, img, m);
  const int64_t vi0 = B.vertex_offset[img] + (i0 - B.pix_prefix[img]);
  if (vec && dim == 3 && i0 + kVertsPerThread <= B.pix_prefix[img + 1] && (vi0 & 3) == 0) {
    float r[12];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const float4 g = __ldg(d_clip + vi0 + u);
#pragma unroll
      for (int c = 0; c < 3; ++c) r[3 * u + c] = transform_vjp(m, g, c);
    }
    float4* dst = reinterpret_cast<float4*>(d_v + 3 * vi0);
    dst[0] = make_float4(r[0], r[1], r[2], r[3]);
    dst[1] = make_float4(r[4], r[5], r[6], r[7]);
    dst[2] = make_float4(r[8], r[9], r[10], r[11]);
    return;
  }
  const int img0 = img;
  for (int u = 0; u < kVertsPerThread; ++u) {
    const int64_t i = i0 + u;
    if (i >= total) break;
    const int64_t vi = packed_vertex(B, i, img);
    if (img != img0) load_matrix(M, img, m);
    const float4 g = __ldg(d_clip + vi);
    for (int c = 0; c < dim; ++c) d_v[dim * vi + c] = transform_vjp(m, g, c);
  }
}

// ---------------------------------------------------------- interpolation
// out = fg ? (a0*b0 + a1*b1) + a2*b2 : background   (interpolate.py:24-63)
__global__ void __launch_bounds__(kBlock) interp_fwd_kernel(
    const float* __restrict__ attr, int K, const int32_t* __restrict__ tris,
    const int32_t* __restrict__ ids, const float* __restrict__ zb,
    const float* __restrict__ bary, const float* __restrict__ bg, Batch B, int L,
    float* __restrict__ out) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= int64_t(L) * B.pix_prefix[B.n]) return;
  const PixelRef r = decode(B, L, q);
  float* o = out + r.e * K;
  if (__ldg(zb + r.e) == 1.0f) {
    for (int k = 0; k < K; ++k) o[k] = bg ? __ldg(bg + k) : 0.0f;
    return;
  }
  const int3 t = load_tri(tris, B, r.img, __ldg(ids + r.e));
  const float b0 = __ldg(bary + 3 * r.e), b1 = __ldg(bary + 3 * r.e + 1),
              b2 = __ldg(bary + 3 * r.e + 2);
  const float* a = attr + B.vertex_offset[r.img] * K;
  const float* a0 = a + int64_t(t.x) * K;
  const float* a1 = a + int64_t(t.y) * K;
  const float* a2 = a + int64_t(t.z) * K;
  for (int k = 0; k < K; ++k)
    o[k] = __fadd_rn(__fadd_rn(__fmul_rn(__ldg(a0 + k), b0), __fmul_rn(__ldg(a1 + k), b1)),
                     __fmul_rn(__ldg(a2 + k), b2));
}

__device__ __forceinline__ void add_rows(float* dst, const float* src, float s, int K) {
  if ((K & 3) == 0 && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
    for (int k = 0; k < K; k += 4)
      atomicAdd(reinterpret_cast<float4*>(dst + k),
                make_float4(s * src[k], s * src[k + 1], s * src[k + 2], s * src[k + 3]));
  } else {
    for (int k = 0; k < K; ++k) atomicAdd(dst + k, s * src[k]);
  }
}

// VJP of interp_fwd: d_attr[v_i] += b_i * d_out on foreground,
// d_bary_i = <attr[v_i], d_out> on foreground (0 elsewhere),
// d_bg += d_out on background.
__global__ void __launch_bounds__(kBlock) interp_bwd_kernel(
    const float* __restrict__ d_out, const float* __restrict__ attr, int K,
    const int32_t* __restrict__ tris, const int32_t* __restrict__ ids,
    const float* __restrict__ zb, const float* __restrict__ bary, Batch B, int L,
    float* __restrict__ d_attr, float* __restrict__ d_bary, float* __restrict__ d_bg) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= int64_t(L) * B.pix_prefix[B.n]) return;
  const PixelRef r = decode(B, L, q);
  const float* g = d_out + r.e * K;
  float gl[DR_MAX_CHANNELS];
  for (int k = 0; k < K; ++k) gl[k] = __ldg(g + k);
  if (__ldg(zb + r.e) == 1.0f) {
    if (d_bg)
      for (int k = 0; k < K; ++k)
        if (gl[k] != 0.0f) atomicAdd(d_bg + k, gl[k]);
    if (d_bary) {
      d_bary[3 * r.e] = 0.0f;
      d_bary[3 * r.e + 1] = 0.0f;
      d_bary[3 * r.e + 2] = 0.0f;
    }
    return;
  }
  const int3 t = load_tri(tris, B, r.img, __ldg(ids + r.e));
  const int vid[3] = {t.x, t.y, t.z};
  const int64_t voff = B.vertex_offset[r.img];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float b = __ldg(bary + 3 * r.e + i);
    add_rows(d_attr + (voff + vid[i]) * K, gl, b, K);
    if (d_bary) {
      const float* a = attr + (voff + vid[i]) * K;
      float s = 0.0f;
      for (int k = 0; k < K; ++k) s = __fadd_rn(s, __fmul_rn(__ldg(a + k), gl[k]));
      d_bary[3 * r.e + i] = s;
    }
  }
}

// -------------------------------------------- differentiable barycentrics
// compute_triangle_matrix (rasterize.py:192-228): signed cofactors of the
// matrix with columns (x_i, y_i, w_i). Row i of D gives barycentric i.
struct TriMatrix {
  float d[3][3];
  float sign;
};

__device__ __forceinline__ float dif(float a, float b, float c, float d) {
  return __fsub_rn(__fmul_rn(a, b), __fmul_rn(c, d));
}

__device__ __forceinline__ TriMatrix tri_matrix(float4 p0, float4 p1, float4 p2) {
  TriMatrix m;
  // xyw[r][c]: coordinate r (x, y, w) of vertex c.
  const float x0 = p0.x, x1 = p1.x, x2 = p2.x;
  const float y0 = p0.y, y1 = p1.y, y2 = p2.y;
  const float w0 = p0.w, w1 = p1.w, w2 = p2.w;
  m.d[0][0] = dif(y1, w2, y2, w1);  // d11
  m.d[1][0] = dif(y2, w0, y0, w2);  // d21
  m.d[2][0] = dif(y0, w1, y1, w0);  // d31
  m.d[0][1] = dif(w1, x2, w2, x1);  // d12
  m.d[1][1] = dif(w2, x0, w0, x2);  // d22
  m.d[2][1] = dif(w0, x1, w1, x0);  // d32
  m.d[0][2] = dif(x1, y2, x2, y1);  // d13
  m.d[1][2] = dif(x2, y0, x0, y2);  // d23
  m.d[2][2] = dif(x0, y1, x1, y0);  // d33
  const float det = __fadd_rn(__fadd_rn(__fmul_rn(x0, m.d[0][0]), __fmul_rn(y0, m.d[0][1])),
                              __fmul_rn(w0, m.d[0][2]));
  m.sign = det > 0.0f ? 1.0f : (det < 0.0f ? -1.0f : (det == 0.0f ? 1.0f : det));
  return m;
}

// normalized_pixel_coordinates (rasterize.py:168-189): (2i + 1) / n - 1.
__device__ __forceinline__ float npc(int i, int n) {
  return __fsub_rn(__fdiv_rn(__int2float_rn(2 * i + 1), __int2float_rn(n)), 1.0f);
}

__device__ __forceinline__ float nan_to_num(float v) {
  if (v != v) return 0.0f;
  if (isinf(v)) return v > 0 ? 3.402823466e38f : -3.402823466e38f;
  return v;
}

__global__ void __launch_bounds__(kBlock) diffbary_fwd_kernel(
    const float4* __restrict__ clip, const int32_t* __restrict__ tris,
    const int32_t* __restrict__ ids, const float* __restrict__ zb, Batch B, int L,
    float* __restrict__ bary) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= int64_t(L) * B.pix_prefix[B.n]) return;
  const PixelRef r = decode(B, L, q);
  float* o = bary + 3 * r.e;
  if (__ldg(zb + r.e) == 1.0f) {
    o[0] = o[1] = o[2] = 0.0f;
    return;
  }
  const int3 t = load_tri(tris, B, r.img, __ldg(ids + r.e));
  const float4* vb = clip + B.vertex_offset[r.img];
  const TriMatrix m = tri_matrix(__ldg(vb + t.x), __ldg(vb + t.y), __ldg(vb + t.z));
  const float px = npc(r.x, B.width[r.img]), py = npc(r.y, B.height[r.img]);
  float u[3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    const float a = __fmul_rn(m.sign, m.d[i][0]), b = __fmul_rn(m.sign, m.d[i][1]),
                c = __fmul_rn(m.sign, m.d[i][2]);
    u[i] = __fadd_rn(__fadd_rn(__fmul_rn(a, px), __fmul_rn(b, py)), c);
  }
  const float s = __fadd_rn(__fadd_rn(u[0], u[1]), u[2]);
#pragma unroll
  for (int i = 0; i < 3; ++i) o[i] = nan_to_num(__fdiv_rn(u[i], s));
}

// VJP of diffbary_fwd w.r.t. the x, y, w clip coordinates of the three
// vertices (z is not an input of the barycentrics).
__global__ void __launch_bounds__(kBlock) diffbary_bwd_kernel(
    const float* __restrict__ d_bary, const float4* __restrict__ clip,
    const int32_t* __restrict__ tris, const int32_t* __restrict__ ids,
    const float* __restrict__ zb, Batch B, int L, float4* __restrict__ d_clip) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= int64_t(L) * B.pix_prefix[B.n]) return;
  const PixelRef r = decode(B, L, q);
  if (__ldg(zb + r.e) == 1.0f) return;
  const float g[3] = {__ldg(d_bary + 3 * r.e), __ldg(d_bary + 3 * r.e + 1),
                      __ldg(d_bary + 3 * r.e + 2)};
  if (g[0] == 0.0f && g[1] == 0.0f && g[2] == 0.0f) return;
  const int3 t = load_tri(tris, B, r.img, __ldg(ids + r.e));
  const float4* vb = clip + B.vertex_offset[r.img];
  const float4 p[3] = {__ldg(vb + t.x), __ldg(vb + t.y), __ldg(vb + t.z)};
  const TriMatrix m = tri_matrix(p[0], p[1], p[2]);
  const float px = npc(r.x, B.width[r.img]), py = npc(r.y, B.height[r.img]);
  float u[3];
#pragma unroll
  for (int i = 0; i < 3; ++i)
    u[i] = m.sign * m.d[i][0] * px + m.sign * m.d[i][1] * py + m.sign * m.d[i][2];
  const float s = u[0] + u[1] + u[2];
  float du[3];
  {
    float gb = 0.0f;
    bool finite[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
      const float b = u[i] / s;
      finite[i] = isfinite(b);
      gb += finite[i] ? g[i] * b : 0.0f;
    }
#pragma unroll
    for (int i = 0; i < 3; ++i) du[i] = ((finite[i] ? g[i] : 0.0f) - gb) / s;
  }
  // u_i = sign * (D_i0 px + D_i1 py + D_i2): dD_ij = sign * du_i * p_j.
  float dD[3][3];
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    dD[i][0] = m.sign * du[i] * px;
    dD[i][1] = m.sign * du[i] * py;
    dD[i][2] = m.sign * du[i];
  }
  // Cofactor derivatives (see tri_matrix for the entries).
  float dx[3] = {0, 0, 0}, dy[3] = {0, 0, 0}, dw[3] = {0, 0, 0};
  // d11 = y1 w2 - y2 w1
  dy[1] += dD[0][0] * p[2].w; dw[2] += dD[0][0] * p[1].y;
  dy[2] -= dD[0][0] * p[1].w; dw[1] -= dD[0][0] * p[2].y;
  // d21 = y2 w0 - y0 w2
  dy[2] += dD[1][0] * p[0].w; dw[0] += dD[1][0] * p[2].y;
  dy[0] -= dD[1][0] * p[2].w; dw[2] -= dD[1][0] * p[0].y;
  // d31 = y0 w1 - y1 w0
  dy[0] += dD[2][0] * p[1].w; dw[1] += dD[2][0] * p[0].y;
  dy[1] -= dD[2][0] * p[0].w; dw[0] -= dD[2][0] * p[1].y;
  // d12 = w1 x2 - w2 x1
  dw[1] += dD[0][1] * p[2].x; dx[2] += dD[0][1] * p[1].w;
  dw[2] -= dD[0][1] * p[1].x; dx[1] -= dD[0][1] * p[2].w;
  // d22 = w2 x0 - w0 x2
  dw[2] += dD[1][1] * p[0].x; dx[0] += dD[1][1] * p[2].w;
  dw[0] -= dD[1][1] * p[2].x; dx[2] -= dD[1][1] * p[0].w;
  // d32 = w0 x1 - w1 x0
  dw[0] += dD[2][1] * p[1].x; dx[1] += dD[2][1] * p[0].w;
  dw[1] -= dD[2][1] * p[0].x; dx[0] -= dD[2][1] * p[1].w;
  // d13 = x1 y2 - x2 y1
  dx[1] += dD[0][2] * p[2].y; dy[2] += dD[0][2] * p[1].x;
  dx[2] -= dD[0][2] * p[1].y; dy[1] -= dD[0][2] * p[2].x;
  // d23 = x2 y0 - x0 y2
  dx[2] += dD[1][2] * p[0].y; dy[0] += dD[1][2] * p[2].x;
  dx[0] -= dD[1][2] * p[2].y; dy[2] -= dD[1][2] * p[0].x;
  // d33 = x0 y1 - x1 y0
  dx[0] += dD[2][2] * p[1].y; dy[1] += dD[2][2] * p[0].x;
  dx[1] -= dD[2][2] * p[0].y; dy[0] -= dD[2][2] * p[1].x;
  float4* dv = d_clip + B.vertex_offset[r.img];
  const int vid[3] = {t.x, t.y, t.z};
#pragma unroll
  for (int i = 0; i < 3; ++i) atomicAdd(dv + vid[i], make_float4(dx[i], dy[i], 0.0f, dw[i]));
}

bool batch_for(const dr_image_desc* images, int n, int L, Batch& b, std::string& err) {
  return make_batch(images, n, L, 16, 16, b, err);
}

template <typename F>
int for_groups(const dr_image_desc* images, int n, int L, std::string& err, F&& f) {
  if (n < 0 || (n > 0 && !images)) { err = "invalid image table"; return DR_ERR_INVALID_ARGUMENT; }
  if (L < 1 || L > DR_MAX_LAYERS) { err = "num_layers must be in [1, 16]"; return DR_ERR_INVALID_ARGUMENT; }
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    if (!batch_for(images + g0, cnt, L, b, err)) return DR_ERR_INVALID_ARGUMENT;
    const int64_t total = int64_t(L) * b.pix_prefix[cnt];
    if (total > 0) f(b, unsigned((total + kBlock - 1) / kBlock));
  }
  return DR_OK;
}

}  // namespace

int transform_launch(const float* M, const float* v, int dim, const dr_image_desc* images,
                     int n, float* clip, cudaStream_t stream, std::string& err) {
  if (dim != 3 && dim != 4) { err = "vertex dim must be 3 or 4"; return DR_ERR_INVALID_ARGUMENT; }
  if ((reinterpret_cast<uintptr_t>(clip) & 15) != 0) {
    err = "clip_vertices must be 16-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    std::memset(&b, 0, sizeof(b));
    b.n = cnt;
    int64_t acc = 0;
    for (int i = 0; i < cnt; ++i) {
      b.pix_prefix[i] = acc;  // vertex prefix
      b.vertex_offset[i] = images[g0 + i].vertex_offset;
      acc += images[g0 + i].num_vertices;
    }
    b.pix_prefix[cnt] = acc;
    const int64_t per_block = 256 * kVertsPerThread;
    const bool vec = ((reinterpret_cast<uintptr_t>(v) | reinterpret_cast<uintptr_t>(clip)) & 15) == 0;
    if (acc > 0)
      transform_kernel<<<unsigned((acc + per_block - 1) / per_block), 256, 0, stream>>>(
          M + 16 * g0, v, dim, b, reinterpret_cast<float4*>(clip), vec);
  }
  return launch_status("transform", err);
}

int transform_bwd_launch(const float* M, const float* d_clip, int dim,
                         const dr_image_desc* images, int n, float* d_vertices,
                         cudaStream_t stream, std::string& err) {
  if (dim != 3 && dim != 4) { err = "vertex dim must be 3 or 4"; return DR_ERR_INVALID_ARGUMENT; }
  if ((reinterpret_cast<uintptr_t>(d_clip) & 15) != 0) {
    err = "d_clip_vertices must be 16-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    std::memset(&b, 0, sizeof(b));
    b.n = cnt;
    int64_t acc = 0;
    for (int i = 0; i < cnt; ++i) {
      b.pix_prefix[i] = acc;
      b.vertex_offset[i] = images[g0 + i].vertex_offset;
      acc += images[g0 + i].num_vertices;
    }
    b.pix_prefix[cnt] = acc;
    const int64_t per_block = 256 * kVertsPerThread;
    const bool vec = (reinterpret_cast<uintptr_t>(d_vertices) & 15) == 0;
    if (acc > 0)
      transform_bwd_kernel<<<unsigned((acc + per_block - 1) / per_block), 256, 0, stream>>>(
          M + 16 * g0, reinterpret_cast<const float4*>(d_clip), dim, b, d_vertices, vec);
  }
  return launch_status("transform backward", err);
}

int interp_fwd_launch(const float* attr, int K, const int32_t* tris, const int32_t* ids,
                      const float* z, const float* bary, const float* bg,
                      const dr_image_desc* images, int n, int L, float* out,
                      cudaStream_t stream, std::string& err) {
  if (K < 1 || K > DR_MAX_CHANNELS) { err = "channels must be in [1, 16]"; return DR_ERR_INVALID_ARGUMENT; }
  const int rc = for_groups(images, n, L, err, [&](const Batch& b, unsigned grid) {
    interp_fwd_kernel<<<grid, kBlock, 0, stream>>>(attr, K, tris, ids, z, bary, bg, b, L, out);
  });
  return rc != DR_OK ? rc : launch_status("interpolate", err);
}

int interp_bwd_launch(const float* d_out, const float* attr, int K, const int32_t* tris,
                      const int32_t* ids, const float* z, const float* bary,
                      const dr_image_desc* images, int n, int L, float* d_attr,
                      float* d_bary, float* d_bg, cudaStream_t stream, std::string& err) {
  if (K < 1 || K > DR_MAX_CHANNELS) { err = "channels must be in [1, 16]"; return DR_ERR_INVALID_ARGUMENT; }
  const int rc = for_groups(images, n, L, err, [&](const Batch& b, unsigned grid) {
    interp_bwd_kernel<<<grid, kBlock, 0, stream>>>(d_out, attr, K, tris, ids, z, bary, b, L,
                                                    d_attr, d_bary, d_bg);
  });
  return rc != DR_OK ? rc : launch_status("interpolate backward", err);
}

int diffbary_fwd_launch(const float* clip, const int32_t* tris, const int32_t* ids,
                        const float* z, const dr_image_desc* images, int n, int L,
                        float* bary, cudaStream_t stream, std::string& err) {
  const int rc = for_groups(images, n, L, err, [&](const Batch& b, unsigned grid) {
    diffbary_fwd_kernel<<<grid, kBlock, 0, stream>>>(reinterpret_cast<const float4*>(clip),
                                                      tris, ids, z, b, L, bary);
  });
  return rc != DR_OK ? rc : launch_status("differentiable barycentrics", err);
}

int diffbary_bwd_launch(const float* d_bary, const float* clip, const int32_t* tris,
                        const int32_t* ids, const float* z, const dr_image_desc* images,
                        int n, int L, float* d_clip, cudaStream_t stream, std::string& err) {
  if ((reinterpret_cast<uintptr_t>(d_clip) & 15) != 0) {
    err = "d_clip_vertices must be 16-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  const int rc = for_groups(images, n, L, err, [&](const Batch& b, unsigned grid) {
    diffbary_bwd_kernel<<<grid, kBlock, 0, stream>>>(
        d_bary, reinterpret_cast<const float4*>(clip), tris, ids, z, b, L,
        reinterpret_cast<float4*>(d_clip));
  });
  return rc != DR_OK ? rc : launch_status("differentiable barycentrics backward", err);
}

}  // namespace dr
