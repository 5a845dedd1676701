// Area-weighted vertex normals (diffren/jax/utils/mesh.py:22-52) and their
// VJP, over a ragged batch of meshes (one per image descriptor):
//
//   face_kernel    1 thread / triangle: n = cross(v1 - v0, v2 - v0),
//                  float4 atomics into its three vertices' sums.
//   normalize      1 thread / vertex: x * rsqrt(|x|^2 + 1e-12)
//                  (transforms.l2_normalize, transforms.py:26-37).
//   VJP            per vertex d x = r g - r^3 x (x . g); per triangle
//                  g_n = sum of its vertices' d x, d v1 += v_e2 x ... (cross
//                  product VJP) scattered with float4 atomics.
// Sums of float atomics vary in order between runs (as XLA's scatter-add).
#include <algorithm>
#include <cstring>
#include <string>

#include "common.cuh"
#include "internal.h"

namespace dr {
namespace {

struct NormalArgs {
  const float* v;        // [V, 3]
  const int32_t* tris;   // [T, 3] per mesh
  float4* acc;           // [V] sums (w unused)
  float* out;            // [V, 3]
  const float* d_out;    // [V, 3]
  float4* d_acc;         // [V] d sums
  float* d_v;            // [V, 3] accumulated
};

__device__ __forceinline__ float3 vload(const float* v, int64_t i) {
  return make_float3(__ldg(v + 3 * i), __ldg(v + 3 * i + 1), __ldg(v + 3 * i + 2));
}

__device__ __forceinline__ float3 cross3(float3 a, float3 b) {
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

__global__ void __launch_bounds__(256) face_kernel(NormalArgs a, Batch B) {
  const int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (g >= B.tri_start[B.n]) return;
  const int img = find_segment(B.tri_start, B.n, g);
  const int32_t* t = a.tris + 3 * (B.triangle_offset[img] + (g - B.tri_start[img]));
  const unsigned nv = unsigned(B.num_vertices[img]);
  const unsigned i0 = unsigned(t[0]), i1 = unsigned(t[1]), i2 = unsigned(t[2]);
  if (i0 >= nv || i1 >= nv || i2 >= nv) return;  // the rasterizer flags these
  const int64_t vo = B.vertex_offset[img];
  const float3 v0 = vload(a.v, vo + i0), v1 = vload(a.v, vo + i1), v2 = vload(a.v, vo + i2);
  const float3 eu = make_float3(v1.x - v0.x, v1.y - v0.y, v1.z - v0.z);
  const float3 ev = make_float3(v2.x - v0.x, v2.y - v0.y, v2.z - v0.z);
  const float3 n = cross3(eu, ev);
  const float4 n4 = make_float4(n.x, n.y, n.z, 0.0f);
  atomicAdd(a.acc + vo + i0, n4);
  atomicAdd(a.acc + vo + i1, n4);
  atomicAdd(a.acc + vo + i2, n4);
}

__global__ void __launch_bounds__(256) normalize_kernel(NormalArgs a, int64_t V) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= V) return;
  const float4 x = a.acc[i];
  const float r = rsqrtf(x.x * x.x + x.y * x.y + x.z * x.z + 1e-12f);
  a.out[3 * i] = x.x * r;
  a.out[3 * i + 1] = x.y * r;
  a.out[3 * i + 2] = x.z * r;
}

__global__ void __launch_bounds__(256) normalize_bwd_kernel(NormalArgs a, int64_t V) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= V) return;
  const float4 x = a.acc[i];
  const float3 g = vload(a.d_out, i);
  const float r = rsqrtf(x.x * x.x + x.y * x.y + x.z * x.z + 1e-12f);
  const float k = r * r * r * (x.x * g.x + x.y * g.y + x.z * g.z);
  a.d_acc[i] = make_float4(r * g.x - k * x.x, r * g.y - k * x.y, r * g.z - k * x.z, 0.0f);
}

__global__ void __launch_bounds__(256) face_bwd_kernel(NormalArgs a, Batch B) {
  const int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (g >= B.tri_start[B.n]) return;
  const int img = find_segment(B.tri_start, B.n, g);
  const int32_t* t = a.tris + 3 * (B.triangle_offset[img] + (g - B.tri_start[img]));
  const unsigned nv = unsigned(B.num_vertices[img]);
  const unsigned i0 = unsigned(t[0]), i1 = unsigned(t[1]), i2 = unsigned(t[2]);
  if (i0 >= nv || i1 >= nv || i2 >= nv) return;
  const int64_t vo = B.vertex_offset[img];
  const float4 a0 = a.d_acc[vo + i0], a1 = a.d_acc[vo + i1], a2 = a.d_acc[vo + i2];
  const float3 gn = make_float3(a0.x + a1.x + a2.x, a0.y + a1.y + a2.y, a0.z + a1.z + a2.z);
  const float3 v0 = vload(a.v, vo + i0), v1 = vload(a.v, vo + i1), v2 = vload(a.v, vo + i2);
  const float3 eu = make_float3(v1.x - v0.x, v1.y - v0.y, v1.z - v0.z);
  const float3 ev = make_float3(v2.x - v0.x, v2.y - v0.y, v2.z - v0.z);
  // n = eu x ev: d eu = ev x g, d ev = g x eu.
  const float3 du = cross3(ev, gn), dv = cross3(gn, eu);
  float* d = a.d_v;
  atomicAdd(d + 3 * (vo + i1), du.x);
  atomicAdd(d + 3 * (vo + i1) + 1, du.y);
  atomicAdd(d + 3 * (vo + i1) + 2, du.z);
  atomicAdd(d + 3 * (vo + i2), dv.x);
  atomicAdd(d + 3 * (vo + i2) + 1, dv.y);
  atomicAdd(d + 3 * (vo + i2) + 2, dv.z);
  atomicAdd(d + 3 * (vo + i0), -(du.x + dv.x));
  atomicAdd(d + 3 * (vo + i0) + 1, -(du.y + dv.y));
  atomicAdd(d + 3 * (vo + i0) + 2, -(du.z + dv.z));
}

// ---- Deterministic form: a vertex -> corner adjacency (CSR; corner 3 g + s
// is slot s of global triangle g, and each vertex lists its corners slot by
// slot, triangles in order) replaces the atomics: per triangle the face
// normal (forward) or the three corners' gradients (VJP) go to a buffer, and
// each vertex sums its own corners in that fixed order: slot 0, slot 1 and
// slot 2 sums in triangle order, then (s0 + s1) + s2, as three scatter-adds
// into zeros would.
__device__ __forceinline__ float3 cross3_rn(float3 a, float3 b) {
  return make_float3(__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)),
                     __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
                     __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x)));
}

struct CsrArgs {
  const float* v;
  const int32_t* tris;
  const int64_t* off;     // [V + 1]
  const int32_t* corner;  // [off[V]]
  float4* face;           // [T] face normals (forward)
  float4* acc;            // [V] sums
  float* out;             // [V, 3]
  const float* d_out;
  float4* d_acc;
  float4* cg;             // [3 T] corner gradients (VJP)
  float* d_v;             // [V, 3] accumulated
};

__global__ void __launch_bounds__(256) face_csr_kernel(CsrArgs a, Batch B) {
  const int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (g >= B.tri_start[B.n]) return;
  const int img = find_segment(B.tri_start, B.n, g);
  const int32_t* t = a.tris + 3 * (B.triangle_offset[img] + (g - B.tri_start[img]));
  const unsigned nv = unsigned(B.num_vertices[img]);
  const unsigned i0 = unsigned(t[0]), i1 = unsigned(t[1]), i2 = unsigned(t[2]);
  float3 n = make_float3(0.0f, 0.0f, 0.0f);
  if (i0 < nv && i1 < nv && i2 < nv) {  // the adjacency lists no corner of others
    const int64_t vo = B.vertex_offset[img];
    const float3 v0 = vload(a.v, vo + i0), v1 = vload(a.v, vo + i1), v2 = vload(a.v, vo + i2);
    n = cross3_rn(make_float3(__fsub_rn(v1.x, v0.x), __fsub_rn(v1.y, v0.y), __fsub_rn(v1.z, v0.z)),
                  make_float3(__fsub_rn(v2.x, v0.x), __fsub_rn(v2.y, v0.y), __fsub_rn(v2.z, v0.z)));
  }
  a.face[g] = make_float4(n.x, n.y, n.z, 0.0f);
}

__global__ void __launch_bounds__(256) vertex_csr_kernel(CsrArgs a, int64_t V) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= V) return;
  float3 s[3] = {make_float3(0.0f, 0.0f, 0.0f), make_float3(0.0f, 0.0f, 0.0f),
                 make_float3(0.0f, 0.0f, 0.0f)};
  for (int64_t k = a.off[i]; k < a.off[i + 1]; ++k) {
    const int c = __ldg(a.corner + k);
    const float4 n = __ldg(a.face + c / 3);
    float3& t = s[c % 3];
    t = make_float3(__fadd_rn(t.x, n.x), __fadd_rn(t.y, n.y), __fadd_rn(t.z, n.z));
  }
  const float3 x = make_float3(__fadd_rn(__fadd_rn(s[0].x, s[1].x), s[2].x),
                               __fadd_rn(__fadd_rn(s[0].y, s[1].y), s[2].y),
                               __fadd_rn(__fadd_rn(s[0].z, s[1].z), s[2].z));
  a.acc[i] = make_float4(x.x, x.y, x.z, 0.0f);
  const float r = rsqrtf(x.x * x.x + x.y * x.y + x.z * x.z + 1e-12f);
  a.out[3 * i] = x.x * r;
  a.out[3 * i + 1] = x.y * r;
  a.out[3 * i + 2] = x.z * r;
}

__global__ void __launch_bounds__(256) normalize_bwd_csr_kernel(CsrArgs a, int64_t V) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= V) return;
  const float4 x = a.acc[i];
  const float3 g = vload(a.d_out, i);
  const float r = rsqrtf(x.x * x.x + x.y * x.y + x.z * x.z + 1e-12f);
  const float k = r * r * r * (x.x * g.x + x.y * g.y + x.z * g.z);
  a.d_acc[i] = make_float4(r * g.x - k * x.x, r * g.y - k * x.y, r * g.z - k * x.z, 0.0f);
}

__global__ void __launch_bounds__(256) face_bwd_csr_kernel(CsrArgs a, Batch B) {
  const int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (g >= B.tri_start[B.n]) return;
  const int img = find_segment(B.tri_start, B.n, g);
  const int32_t* t = a.tris + 3 * (B.triangle_offset[img] + (g - B.tri_start[img]));
  const unsigned nv = unsigned(B.num_vertices[img]);
  const unsigned i0 = unsigned(t[0]), i1 = unsigned(t[1]), i2 = unsigned(t[2]);
  if (!(i0 < nv && i1 < nv && i2 < nv)) return;  // never listed in the adjacency
  const int64_t vo = B.vertex_offset[img];
  const float4 a0 = a.d_acc[vo + i0], a1 = a.d_acc[vo + i1], a2 = a.d_acc[vo + i2];
  const float3 gn = make_float3(a0.x + a1.x + a2.x, a0.y + a1.y + a2.y, a0.z + a1.z + a2.z);
  const float3 v0 = vload(a.v, vo + i0), v1 = vload(a.v, vo + i1), v2 = vload(a.v, vo + i2);
  const float3 eu = make_float3(v1.x - v0.x, v1.y - v0.y, v1.z - v0.z);
  const float3 ev = make_float3(v2.x - v0.x, v2.y - v0.y, v2.z - v0.z);
  // n = eu x ev: d eu = ev x g, d ev = g x eu.
  const float3 du = cross3(ev, gn), dv = cross3(gn, eu);
  a.cg[3 * g] = make_float4(-(du.x + dv.x), -(du.y + dv.y), -(du.z + dv.z), 0.0f);
  a.cg[3 * g + 1] = make_float4(du.x, du.y, du.z, 0.0f);
  a.cg[3 * g + 2] = make_float4(dv.x, dv.y, dv.z, 0.0f);
}

__global__ void __launch_bounds__(256) vertex_bwd_csr_kernel(CsrArgs a, int64_t V) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= V) return;
  float3 d = make_float3(0.0f, 0.0f, 0.0f);
  for (int64_t k = a.off[i]; k < a.off[i + 1]; ++k) {
    const float4 c = __ldg(a.cg + __ldg(a.corner + k));
    d = make_float3(d.x + c.x, d.y + c.y, d.z + c.z);
  }
  a.d_v[3 * i] += d.x;
  a.d_v[3 * i + 1] += d.y;
  a.d_v[3 * i + 2] += d.z;
}

int64_t vertex_extent(const dr_image_desc* images, int n) {
  int64_t V = 0;
  for (int i = 0; i < n; ++i)
    V = std::max(V, images[i].vertex_offset + int64_t(images[i].num_vertices));
  return V;
}

bool check_mesh(const float* v, const int32_t* tris, const dr_image_desc* images, int n,
                std::string& err) {
  if (n < 0 || (n > 0 && !images)) { err = "invalid image table"; return false; }
  bool any_vertices = false, any_triangles = false;
  for (int i = 0; i < n; ++i) {
    any_vertices |= images[i].num_vertices > 0;
    any_triangles |= images[i].num_triangles > 0;
  }
  if ((any_vertices && !v) || (any_triangles && !tris)) {
    err = "vertices and triangles must be non-null";
    return false;
  }
  return true;
}

// The mesh part of the batch table for images[0, n): the image sizes play
// no part in the normals.
bool mesh_batch(const dr_image_desc* images, int n, Batch& b, std::string& err) {
  std::memset(&b, 0, sizeof(b));
  b.n = n;
  int64_t tris = 0;
  for (int i = 0; i < n; ++i) {
    const dr_image_desc& d = images[i];
    if (d.num_triangles < 0 || d.num_vertices < 0 || d.vertex_offset < 0 ||
        d.triangle_offset < 0) {
      err = "mesh " + std::to_string(i) + ": negative count or offset";
      return false;
    }
    b.tri_start[i] = tris;
    b.num_vertices[i] = d.num_vertices;
    b.vertex_offset[i] = d.vertex_offset;
    b.triangle_offset[i] = d.triangle_offset;
    tris += d.num_triangles;
  }
  b.tri_start[n] = tris;
  if (tris >= (int64_t(1) << 31)) {
    err = "batch too large: triangles must be < 2^31";
    return false;
  }
  return true;
}

// Every group of the batch passes mesh_batch, checked before any launch.
bool check_tables(const dr_image_desc* images, int n, std::string& err) {
  Batch b;
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE)
    if (!mesh_batch(images + g0, std::min(n - g0, DR_MAX_BATCH_INLINE), b, err)) return false;
  return true;
}

}  // namespace

int normals_fwd_launch(const float* vertices, const int32_t* tris, const dr_image_desc* images,
                       int n, float* accum, float* normals, cudaStream_t stream,
                       std::string& err) {
  if (!check_mesh(vertices, tris, images, n, err)) return DR_ERR_INVALID_ARGUMENT;
  if (!check_tables(images, n, err)) return DR_ERR_INVALID_ARGUMENT;
  const int64_t V = vertex_extent(images, n);
  if (V == 0) return DR_OK;
  if (!accum || !normals) { err = "accum and normals must be non-null"; return DR_ERR_INVALID_ARGUMENT; }
  if ((reinterpret_cast<uintptr_t>(accum) & 15) != 0) {
    err = "accum must be 16-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  if (cudaMemsetAsync(accum, 0, size_t(V) * 16, stream) != cudaSuccess) {
    err = std::string("cudaMemsetAsync: ") + cudaGetErrorString(cudaGetLastError());
    return DR_ERR_CUDA;
  }
  NormalArgs a{vertices, tris, reinterpret_cast<float4*>(accum), normals, nullptr, nullptr,
               nullptr};
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    if (!mesh_batch(images + g0, cnt, b, err)) return DR_ERR_INVALID_ARGUMENT;
    const int64_t T = b.tri_start[cnt];
    if (T > 0) face_kernel<<<unsigned((T + 255) / 256), 256, 0, stream>>>(a, b);
  }
  normalize_kernel<<<unsigned((V + 255) / 256), 256, 0, stream>>>(a, V);
  return launch_status("vertex normals", err);
}

int normals_bwd_launch(const float* d_normals, const float* vertices, const int32_t* tris,
                       const dr_image_desc* images, int n, const float* accum,
                       float* d_accum, float* d_vertices, cudaStream_t stream,
                       std::string& err) {
  if (!check_mesh(vertices, tris, images, n, err)) return DR_ERR_INVALID_ARGUMENT;
  if (!check_tables(images, n, err)) return DR_ERR_INVALID_ARGUMENT;
  const int64_t V = vertex_extent(images, n);
  if (V == 0) return DR_OK;
  if (!d_normals || !accum || !d_accum || !d_vertices) {
    err = "d_normals, accum, d_accum and d_vertices must be non-null";
    return DR_ERR_INVALID_ARGUMENT;
  }
  if (((reinterpret_cast<uintptr_t>(accum) | reinterpret_cast<uintptr_t>(d_accum)) & 15) != 0) {
    err = "accum and d_accum must be 16-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  NormalArgs a{vertices, tris, const_cast<float4*>(reinterpret_cast<const float4*>(accum)),
               nullptr, d_normals, reinterpret_cast<float4*>(d_accum), d_vertices};
  normalize_bwd_kernel<<<unsigned((V + 255) / 256), 256, 0, stream>>>(a, V);
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    if (!mesh_batch(images + g0, cnt, b, err)) return DR_ERR_INVALID_ARGUMENT;
    const int64_t T = b.tri_start[cnt];
    if (T > 0) face_bwd_kernel<<<unsigned((T + 255) / 256), 256, 0, stream>>>(a, b);
  }
  return launch_status("vertex normals backward", err);
}


static bool check_csr(const int64_t* off, const int32_t* corner, const void* buf, const void* acc,
               std::string& err) {
  if (!off || !corner || !buf || !acc) {
    err = "vertex_offsets, corners and the scratch buffers must be non-null";
    return false;
  }
  if (((reinterpret_cast<uintptr_t>(buf) | reinterpret_cast<uintptr_t>(acc)) & 15) != 0) {
    err = "the scratch buffers must be 16-byte aligned";
    return false;
  }
  return true;
}

int normals_csr_fwd_launch(const float* vertices, const int32_t* tris,
                           const dr_image_desc* images, int n, const int64_t* off,
                           const int32_t* corner, float* face, float* accum, float* normals,
                           cudaStream_t stream, std::string& err) {
  if (!check_mesh(vertices, tris, images, n, err)) return DR_ERR_INVALID_ARGUMENT;
  if (!check_tables(images, n, err)) return DR_ERR_INVALID_ARGUMENT;
  const int64_t V = vertex_extent(images, n);
  if (V == 0) return DR_OK;
  if (!normals || !check_csr(off, corner, face, accum, err)) return DR_ERR_INVALID_ARGUMENT;
  CsrArgs a{};
  a.v = vertices; a.tris = tris; a.off = off; a.corner = corner;
  a.face = reinterpret_cast<float4*>(face);
  a.acc = reinterpret_cast<float4*>(accum);
  a.out = normals;
  int64_t T0 = 0;
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    if (!mesh_batch(images + g0, cnt, b, err)) return DR_ERR_INVALID_ARGUMENT;
    const int64_t T = b.tri_start[cnt];
    CsrArgs ag = a;
    ag.face = a.face + T0;  // global triangle index = group start + in-group index
    if (T > 0) face_csr_kernel<<<unsigned((T + 255) / 256), 256, 0, stream>>>(ag, b);
    T0 += T;
  }
  vertex_csr_kernel<<<unsigned((V + 255) / 256), 256, 0, stream>>>(a, V);
  return launch_status("vertex normals", err);
}

int normals_csr_bwd_launch(const float* d_normals, const float* vertices, const int32_t* tris,
                           const dr_image_desc* images, int n, const int64_t* off,
                           const int32_t* corner, const float* accum, float* d_accum,
                           float* corner_grad, float* d_vertices, cudaStream_t stream,
                           std::string& err) {
  if (!check_mesh(vertices, tris, images, n, err)) return DR_ERR_INVALID_ARGUMENT;
  if (!check_tables(images, n, err)) return DR_ERR_INVALID_ARGUMENT;
  const int64_t V = vertex_extent(images, n);
  if (V == 0) return DR_OK;
  if (!d_normals || !d_vertices || !check_csr(off, corner, corner_grad, d_accum, err) ||
      !accum || (reinterpret_cast<uintptr_t>(accum) & 15) != 0) {
    if (err.empty()) err = "d_normals, accum and d_vertices must be non-null (accum 16-byte aligned)";
    return DR_ERR_INVALID_ARGUMENT;
  }
  CsrArgs a{};
  a.v = vertices; a.tris = tris; a.off = off; a.corner = corner;
  a.acc = const_cast<float4*>(reinterpret_cast<const float4*>(accum));
  a.d_out = d_normals;
  a.d_acc = reinterpret_cast<float4*>(d_accum);
  a.cg = reinterpret_cast<float4*>(corner_grad);
  a.d_v = d_vertices;
  normalize_bwd_csr_kernel<<<unsigned((V + 255) / 256), 256, 0, stream>>>(a, V);
  int64_t T0 = 0;
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    if (!mesh_batch(images + g0, cnt, b, err)) return DR_ERR_INVALID_ARGUMENT;
    const int64_t T = b.tri_start[cnt];
    CsrArgs ag = a;
    ag.cg = a.cg + 3 * T0;
    if (T > 0) face_bwd_csr_kernel<<<unsigned((T + 255) / 256), 256, 0, stream>>>(ag, b);
    T0 += T;
  }
  vertex_bwd_csr_kernel<<<unsigned((V + 255) / 256), 256, 0, stream>>>(a, V);
  return launch_status("vertex normals backward", err);
}

}  // namespace dr
