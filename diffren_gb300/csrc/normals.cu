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

}  // namespace dr
