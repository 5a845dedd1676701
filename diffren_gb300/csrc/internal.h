// Host-side declarations shared by the diffren_gb300 translation units.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "common.cuh"

namespace dr {

// Fills the by-value batch table for images[0, n) (n <= DR_MAX_BATCH_INLINE)
// with screen tiles of TW x TH pixels.
inline bool make_batch(const dr_image_desc* images, int n, int L, int TW, int TH,
                       Batch& b, std::string& err) {
  std::memset(&b, 0, sizeof(b));
  b.n = n;
  b.num_layers = L;
  int64_t tris = 0, tiles = 0, pix = 0;
  for (int i = 0; i < n; ++i) {
    const dr_image_desc& d = images[i];
    if (d.width <= 0 || d.height <= 0 || d.width > DR_MAX_IMAGE_DIM ||
        d.height > DR_MAX_IMAGE_DIM) {
      err = "image " + std::to_string(i) + ": width and height must be in [1, " +
            std::to_string(DR_MAX_IMAGE_DIM) + "]";
      return false;
    }
    if (d.num_triangles < 0 || d.num_vertices < 0 || d.vertex_offset < 0 ||
        d.triangle_offset < 0 || d.pixel_offset < 0) {
      err = "image " + std::to_string(i) + ": negative count or offset";
      return false;
    }
    b.tri_start[i] = tris;
    b.tile_start[i] = int32_t(tiles);
    b.pix_prefix[i] = pix;
    b.pix_off[i] = d.pixel_offset;
    b.width[i] = d.width;
    b.height[i] = d.height;
    b.num_vertices[i] = d.num_vertices;
    b.vertex_offset[i] = d.vertex_offset;
    b.triangle_offset[i] = d.triangle_offset;
    b.tiles_x[i] = (d.width + TW - 1) / TW;
    tris += d.num_triangles;
    tiles += int64_t(b.tiles_x[i]) * ((d.height + TH - 1) / TH);
    pix += int64_t(d.width) * d.height;
  }
  b.tri_start[n] = tris;
  b.tile_start[n] = int32_t(tiles);
  b.pix_prefix[n] = pix;
  if (tris >= (int64_t(1) << 31) || tiles >= (int64_t(1) << 31)) {
    err = "batch too large: triangles and tiles must each be < 2^31";
    return false;
  }
  return true;
}

constexpr int kMaxDevices = 64;

// Host-side cache of one kernel's launch attributes on each device: the
// dynamic shared-memory limit raised so far, and SMs x resident blocks per
// SM for one shared-memory size. Host threads may launch concurrently, so
// every use holds the lock; the limit only grows.
struct LaunchCache {
  std::mutex mu;
  size_t raised[kMaxDevices] = {};
  size_t occ_smem[kMaxDevices] = {};
  int sms[kMaxDevices] = {};
  int per_sm[kMaxDevices] = {};
};

// Raises kern's dynamic shared-memory limit on the current device to smem
// when needed (`too_big` is the error when the device cannot), and returns
// the SM count and the resident blocks per SM of `threads`-thread blocks
// with smem bytes (at least 1).
template <typename K>
bool prepare_launch(LaunchCache& c, K kern, int threads, size_t smem, int& sms, int& per_sm,
                    const char* too_big, std::string& err) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    err = "no usable CUDA device";
    return false;
  }
  std::lock_guard<std::mutex> lock(c.mu);
  if (smem > 48 * 1024 && smem > c.raised[dev]) {
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)) !=
        cudaSuccess) {
      err = too_big;
      return false;
    }
    c.raised[dev] = smem;
  }
  if (c.per_sm[dev] == 0 || c.occ_smem[dev] != smem) {
    int n = 0, p = 0;
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p, kern, threads, smem);
    c.sms[dev] = std::max(1, n);
    c.per_sm[dev] = std::max(1, p);
    c.occ_smem[dev] = smem;
  }
  sms = c.sms[dev];
  per_sm = c.per_sm[dev];
  return true;
}

inline int launch_status(const char* what, std::string& err) {
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return DR_OK;
  err = std::string(what) + ": " + cudaGetErrorString(e);
  return DR_ERR_CUDA;
}

// abi.cu: message returned by dr_last_error() on this thread.
void set_last_error(const std::string& msg);

// raster.cu
size_t raster_workspace_bytes(const dr_image_desc* images, int n,
                              const dr_raster_config* cfg, std::string& err);
int raster_launch(const float* vertices, const int32_t* triangles,
                  const dr_image_desc* images, int n, const dr_raster_config* cfg,
                  int32_t* ids, float* z, float* bary, void* workspace,
                  size_t ws_bytes, cudaStream_t stream, std::string& err,
                  const SampleOutputs* samples = nullptr);
int depth_codec_selftest(unsigned long long* out, cudaStream_t stream, std::string& err);
// Byte offset of the device error word inside a raster workspace.
constexpr size_t kErrorFlagsOffset = 4;

// interp.cu
int transform_launch(const float* matrices, const float* vertices, int dim,
                     const dr_image_desc* images, int n, float* clip,
                     cudaStream_t stream, std::string& err);
int transform_bwd_launch(const float* matrices, const float* d_clip, int dim,
                         const dr_image_desc* images, int n, float* d_vertices,
                         cudaStream_t stream, std::string& err);
int interp_fwd_launch(const float* attr, int K, const int32_t* tris,
                      const int32_t* ids, const float* z, const float* bary,
                      const float* background, const dr_image_desc* images, int n,
                      int L, float* out, cudaStream_t stream, std::string& err);
int interp_bwd_launch(const float* d_out, const float* attr, int K,
                      const int32_t* tris, const int32_t* ids, const float* z,
                      const float* bary, const dr_image_desc* images, int n, int L,
                      float* d_attr, float* d_bary, float* d_bg,
                      cudaStream_t stream, std::string& err);
int diffbary_fwd_launch(const float* clip, const int32_t* tris, const int32_t* ids,
                        const float* z, const dr_image_desc* images, int n, int L,
                        float* bary, cudaStream_t stream, std::string& err);
int diffbary_bwd_launch(const float* d_bary, const float* clip, const int32_t* tris,
                        const int32_t* ids, const float* z,
                        const dr_image_desc* images, int n, int L, float* d_clip,
                        cudaStream_t stream, std::string& err);

// texture.cu
int texture_fwd_launch(const float* uv, int64_t n, const float* tex, int H, int W, int C,
                       int flags, float* out, cudaStream_t stream, std::string& err);
int texture_bwd_launch(const float* d_out, const float* uv, int64_t n, const float* tex,
                       int H, int W, int C, int flags, float* d_uv, float* d_tex,
                       void* scratch, size_t scratch_bytes, cudaStream_t stream,
                       std::string& err);
size_t texture_fixed_bytes(int H, int W, int C);

// light.cu
int point_light_fwd_launch(const float* dif, const float* nrm, const float* pos, int64_t n,
                           int sd, int sn, int sp, const dr_point_light* q, float* out, int oc,
                           cudaStream_t stream, std::string& err);
int point_light_bwd_launch(const float* d_out, int oc, const float* dif, const float* nrm,
                           const float* pos, int64_t n, int sd, int sn, int sp,
                           const dr_point_light* q, float* d_dif, float* d_nrm, float* d_pos,
                           int sg, cudaStream_t stream, std::string& err);

// composite.cu
int over_fwd_launch(const float* shaded, const float* z, int C, const dr_image_desc* images,
                    int n, int L, float* out, cudaStream_t stream, std::string& err);
int over_bwd_launch(const float* d_out, const float* shaded, const float* z, int C,
                    const dr_image_desc* images, int n, int L, float* d_shaded,
                    cudaStream_t stream, std::string& err);

// loss.cu
int squared_error_launch(const float* image, const float* target, int64_t n, float weight,
                         float* seed, double* partials, float* loss, cudaStream_t stream,
                         std::string& err);

// normals.cu
int normals_fwd_launch(const float* vertices, const int32_t* tris, const dr_image_desc* images,
                       int n, float* accum, float* normals, cudaStream_t stream,
                       std::string& err);
int normals_bwd_launch(const float* d_normals, const float* vertices, const int32_t* tris,
                       const dr_image_desc* images, int n, const float* accum,
                       float* d_accum, float* d_vertices, cudaStream_t stream,
                       std::string& err);
int normals_csr_fwd_launch(const float* vertices, const int32_t* tris,
                           const dr_image_desc* images, int n, const int64_t* off,
                           const int32_t* corner, float* face, float* accum, float* normals,
                           cudaStream_t stream, std::string& err);
int normals_csr_bwd_launch(const float* d_normals, const float* vertices, const int32_t* tris,
                           const dr_image_desc* images, int n, const int64_t* off,
                           const int32_t* corner, const float* accum, float* d_accum,
                           float* corner_grad, float* d_vertices, cudaStream_t stream,
                           std::string& err);

// splat.cu
int samples_fwd_launch(const float* attributes, int K, const float* clip,
                       const int32_t* tris, const int32_t* ids, const float* z,
                       const float* bary, const dr_image_desc* images, int n, int L,
                       float* attr_out, float* positions, cudaStream_t stream,
                       std::string& err);
int samples_bwd_launch(const float* d_attr_out, const float* d_positions,
                       const float* attributes, int K, const float* clip,
                       const int32_t* tris, const int32_t* ids, const float* z,
                       const float* bary, const float* positions,
                       const int32_t* vertex_ids, const dr_image_desc* images, int n,
                       int L, float* d_attributes, float* d_clip, float* d_bary,
                       uint32_t flags, void* scratch, size_t scratch_bytes,
                       cudaStream_t stream, std::string& err);
size_t samples_fixed_bytes(const dr_image_desc* images, int n, int K);
int positions_fwd_launch(const float* clip, const int32_t* tris, const int32_t* ids,
                         const float* z, const float* bary, const dr_image_desc* images,
                         int n, int L, float* positions, cudaStream_t stream,
                         std::string& err);
int positions_bwd_launch(const float* d_positions, const float* clip, const int32_t* tris,
                         const int32_t* ids, const float* z, const float* bary,
                         const dr_image_desc* images, int n, int L, float* d_clip,
                         float* d_bary, cudaStream_t stream, std::string& err);
int splat_fwd_launch(const float* positions, const float* z_buffer, const float* colors, int C,
                     const dr_image_desc* images, int n, int L, float* out, float* saved,
                     float* accum, float* normalized, cudaStream_t stream, std::string& err);
int splat_jvp_launch(const float* positions, const float* z_buffer, const float* colors,
                     const float* d_positions, const float* d_colors, int C,
                     const dr_image_desc* images, int n, int L, float* d_image,
                     cudaStream_t stream, std::string& err);
int splat_bwd_launch(const float* d_out, const float* positions, const float* z_buffer,
                     const float* colors, const float* saved, int C,
                     const dr_image_desc* images, int n, int L, uint32_t flags,
                     float* d_colors, float* d_positions, cudaStream_t stream,
                     std::string& err);

}  // namespace dr
