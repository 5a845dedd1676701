// extern "C" entry points of libdiffren_gb300.so (declared in
// include/diffren_gb300.h). Each validates its arguments, enqueues kernels on
// the caller's stream and returns a status; messages go to a thread-local
// string read by dr_last_error().
#include <string>

#include "diffren_gb300.h"
#include "internal.h"

namespace {

thread_local std::string g_error;

int finish(int rc, std::string& err) {
  if (rc != DR_OK) g_error = err.empty() ? "unknown error" : err;
  return rc;
}

cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

dr_image_desc single_image(int32_t nv, int32_t nt, int32_t w, int32_t h) {
  dr_image_desc d;
  d.width = w;
  d.height = h;
  d.num_vertices = nv;
  d.num_triangles = nt;
  d.vertex_offset = 0;
  d.triangle_offset = 0;
  d.pixel_offset = 0;
  return d;
}

dr_raster_config default_config(int32_t L, int32_t cull, int32_t depth_mode) {
  dr_raster_config c;
  c.num_layers = L;
  c.face_culling_mode = cull;
  c.depth_mode = depth_mode;
  c.tile_width = 0;
  c.tile_height = 0;
  c.large_tiles = 0;
  c.flags = 0;
  return c;
}

}  // namespace

namespace dr {
void set_last_error(const std::string& msg) { g_error = msg; }
}  // namespace dr

extern "C" {

const char* dr_last_error(void) { return g_error.c_str(); }

int32_t dr_abi_version(void) { return 3; }

size_t dr_rasterize_batch_workspace_bytes(const dr_image_desc* images,
                                          int32_t num_images,
                                          const dr_raster_config* config) {
  std::string err;
  const size_t n = dr::raster_workspace_bytes(images, num_images, config, err);
  if (n == 0) g_error = err;
  return n;
}

int dr_rasterize_batch(const float* vertices, const int32_t* triangles,
                       const dr_image_desc* images, int32_t num_images,
                       const dr_raster_config* config, int32_t* triangle_ids,
                       float* z_buffer, float* barycentrics, void* workspace,
                       size_t workspace_bytes, void* stream) {
  std::string err;
  return finish(dr::raster_launch(vertices, triangles, images, num_images, config,
                                  triangle_ids, z_buffer, barycentrics, workspace,
                                  workspace_bytes, as_stream(stream), err),
                err);
}

int dr_rasterize_batch_interpolate(const float* vertices, const int32_t* triangles,
                                   const dr_image_desc* images, int32_t num_images,
                                   const dr_raster_config* config, int32_t* triangle_ids,
                                   float* z_buffer, float* barycentrics,
                                   const float* attributes, int32_t num_channels,
                                   float* attributes_out, float* positions,
                                   int32_t* vertex_ids, void* workspace,
                                   size_t workspace_bytes, void* stream) {
  std::string err;
  dr::SampleOutputs so{attributes, num_channels, attributes_out,
                       reinterpret_cast<float4*>(positions), vertex_ids};
  return finish(dr::raster_launch(vertices, triangles, images, num_images, config,
                                  triangle_ids, z_buffer, barycentrics, workspace,
                                  workspace_bytes, as_stream(stream), err, &so),
                err);
}

size_t dr_rasterize_triangles_workspace_bytes(int32_t num_triangles,
                                              int32_t image_width,
                                              int32_t image_height,
                                              int32_t num_layers) {
  const dr_image_desc d = single_image(0, num_triangles, image_width, image_height);
  const dr_raster_config c = default_config(num_layers, DR_CULL_NONE, DR_DEPTH_DISCRETIZED);
  return dr_rasterize_batch_workspace_bytes(&d, 1, &c);
}

int dr_rasterize_triangles(const float* vertices, int32_t num_vertices,
                           const int32_t* triangles, int32_t num_triangles,
                           int32_t image_width, int32_t image_height,
                           int32_t num_layers, int32_t face_culling_mode,
                           int32_t depth_mode, int32_t* triangle_ids,
                           float* z_buffer, float* barycentrics,
                           void* workspace, size_t workspace_bytes,
                           void* stream) {
  const dr_image_desc d = single_image(num_vertices, num_triangles, image_width, image_height);
  const dr_raster_config c = default_config(num_layers, face_culling_mode, depth_mode);
  return dr_rasterize_batch(vertices, triangles, &d, 1, &c, triangle_ids, z_buffer,
                            barycentrics, workspace, workspace_bytes, stream);
}

int dr_read_error_flags(const void* workspace, uint32_t* flags, void* stream) {
  std::string err;
  if (!workspace || !flags) {
    err = "workspace and flags must be non-null";
    return finish(DR_ERR_INVALID_ARGUMENT, err);
  }
  const char* p = static_cast<const char*>(workspace) + dr::kErrorFlagsOffset;
  if (cudaMemcpyAsync(flags, p, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                      as_stream(stream)) != cudaSuccess ||
      cudaStreamSynchronize(as_stream(stream)) != cudaSuccess) {
    err = std::string("reading error flags: ") + cudaGetErrorString(cudaGetLastError());
    return finish(DR_ERR_CUDA, err);
  }
  return DR_OK;
}

int dr_selftest_depth_codec(unsigned long long* results, void* stream) {
  std::string err;
  return finish(dr::depth_codec_selftest(results, as_stream(stream), err), err);
}

int dr_transform_vertices(const float* matrices, const float* vertices, int32_t dim,
                          const dr_image_desc* images, int32_t num_images,
                          float* clip_vertices, void* stream) {
  std::string err;
  return finish(dr::transform_launch(matrices, vertices, dim, images, num_images,
                                     clip_vertices, as_stream(stream), err),
                err);
}

int dr_transform_vertices_bwd(const float* matrices, const float* d_clip_vertices,
                              int32_t dim, const dr_image_desc* images,
                              int32_t num_images, float* d_vertices, void* stream) {
  std::string err;
  return finish(dr::transform_bwd_launch(matrices, d_clip_vertices, dim, images,
                                         num_images, d_vertices, as_stream(stream), err),
                err);
}

int dr_interpolate_fwd(const float* attributes, int32_t num_channels,
                       const int32_t* triangles, const int32_t* triangle_ids,
                       const float* z_buffer, const float* barycentrics,
                       const float* background, const dr_image_desc* images,
                       int32_t num_images, int32_t num_layers, float* out,
                       void* stream) {
  std::string err;
  return finish(dr::interp_fwd_launch(attributes, num_channels, triangles, triangle_ids,
                                      z_buffer, barycentrics, background, images,
                                      num_images, num_layers, out, as_stream(stream), err),
                err);
}

int dr_interpolate_bwd(const float* d_out, const float* attributes,
                       int32_t num_channels, const int32_t* triangles,
                       const int32_t* triangle_ids, const float* z_buffer,
                       const float* barycentrics, const dr_image_desc* images,
                       int32_t num_images, int32_t num_layers,
                       float* d_attributes, float* d_barycentrics,
                       float* d_background, void* stream) {
  std::string err;
  return finish(dr::interp_bwd_launch(d_out, attributes, num_channels, triangles,
                                      triangle_ids, z_buffer, barycentrics, images,
                                      num_images, num_layers, d_attributes,
                                      d_barycentrics, d_background, as_stream(stream), err),
                err);
}

int dr_diff_barycentrics_fwd(const float* clip_vertices, const int32_t* triangles,
                             const int32_t* triangle_ids, const float* z_buffer,
                             const dr_image_desc* images, int32_t num_images,
                             int32_t num_layers, float* barycentrics, void* stream) {
  std::string err;
  return finish(dr::diffbary_fwd_launch(clip_vertices, triangles, triangle_ids, z_buffer,
                                        images, num_images, num_layers, barycentrics,
                                        as_stream(stream), err),
                err);
}

int dr_diff_barycentrics_bwd(const float* d_barycentrics, const float* clip_vertices,
                             const int32_t* triangles, const int32_t* triangle_ids,
                             const float* z_buffer, const dr_image_desc* images,
                             int32_t num_images, int32_t num_layers,
                             float* d_clip_vertices, void* stream) {
  std::string err;
  return finish(dr::diffbary_bwd_launch(d_barycentrics, clip_vertices, triangles,
                                        triangle_ids, z_buffer, images, num_images,
                                        num_layers, d_clip_vertices, as_stream(stream),
                                        err),
                err);
}

int dr_interpolate_with_positions_fwd(const float* attributes, int32_t num_channels,
                                      const float* clip_vertices, const int32_t* triangles,
                                      const int32_t* triangle_ids, const float* z_buffer,
                                      const float* barycentrics, const dr_image_desc* images,
                                      int32_t num_images, int32_t num_layers,
                                      float* attributes_out, float* positions, void* stream) {
  std::string err;
  return finish(dr::samples_fwd_launch(attributes, num_channels, clip_vertices, triangles,
                                       triangle_ids, z_buffer, barycentrics, images,
                                       num_images, num_layers, attributes_out, positions,
                                       as_stream(stream), err),
                err);
}

int dr_interpolate_with_positions_bwd_ex(
    const float* d_attributes_out, const float* d_positions, const float* attributes,
    int32_t num_channels, const float* clip_vertices, const int32_t* triangles,
    const int32_t* triangle_ids, const float* z_buffer, const float* barycentrics,
    const float* positions, const int32_t* vertex_ids, const dr_image_desc* images,
    int32_t num_images, int32_t num_layers, uint32_t flags, float* d_attributes,
    float* d_clip_vertices, float* d_barycentrics, void* scratch, size_t scratch_bytes,
    void* stream) {
  std::string err;
  return finish(dr::samples_bwd_launch(d_attributes_out, d_positions, attributes,
                                       num_channels, clip_vertices, triangles,
                                       triangle_ids, z_buffer, barycentrics, positions,
                                       vertex_ids, images, num_images, num_layers,
                                       d_attributes, d_clip_vertices, d_barycentrics, flags,
                                       scratch, scratch_bytes, as_stream(stream), err),
                err);
}

int dr_interpolate_with_positions_bwd(const float* d_attributes_out,
                                      const float* d_positions, const float* attributes,
                                      int32_t num_channels, const float* clip_vertices,
                                      const int32_t* triangles, const int32_t* triangle_ids,
                                      const float* z_buffer, const float* barycentrics,
                                      const float* positions, const int32_t* vertex_ids,
                                      const dr_image_desc* images, int32_t num_images,
                                      int32_t num_layers, float* d_attributes,
                                      float* d_clip_vertices, float* d_barycentrics,
                                      void* stream) {
  return dr_interpolate_with_positions_bwd_ex(
      d_attributes_out, d_positions, attributes, num_channels, clip_vertices, triangles,
      triangle_ids, z_buffer, barycentrics, positions, vertex_ids, images, num_images,
      num_layers, 0u, d_attributes, d_clip_vertices, d_barycentrics, nullptr, 0, stream);
}

size_t dr_interpolate_with_positions_bwd_scratch_bytes(const dr_image_desc* images,
                                                       int32_t num_images,
                                                       int32_t num_channels) {
  if (num_images < 0 || (num_images > 0 && !images) || num_channels < 1 ||
      num_channels > DR_MAX_CHANNELS)
    return 0;
  return dr::samples_fixed_bytes(images, num_images, num_channels);
}

int dr_texture_map_fwd(const float* uv, int64_t num_points, const float* texture,
                       int32_t height, int32_t width, int32_t channels, int32_t flags,
                       float* out, void* stream) {
  std::string err;
  return finish(dr::texture_fwd_launch(uv, num_points, texture, height, width, channels,
                                       flags, out, as_stream(stream), err),
                err);
}

int dr_texture_map_bwd(const float* d_out, const float* uv, int64_t num_points,
                       const float* texture, int32_t height, int32_t width,
                       int32_t channels, int32_t flags, float* d_uv, float* d_texture,
                       void* stream) {
  std::string err;
  if (flags & DR_TEXTURE_DETERMINISTIC) {
    err = "DR_TEXTURE_DETERMINISTIC needs dr_texture_map_bwd_ex and its scratch";
    return finish(DR_ERR_INVALID_ARGUMENT, err);
  }
  return finish(dr::texture_bwd_launch(d_out, uv, num_points, texture, height, width,
                                       channels, flags, d_uv, d_texture, nullptr, 0,
                                       as_stream(stream), err),
                err);
}

int dr_texture_map_bwd_ex(const float* d_out, const float* uv, int64_t num_points,
                          const float* texture, int32_t height, int32_t width,
                          int32_t channels, int32_t flags, float* d_uv, float* d_texture,
                          void* scratch, size_t scratch_bytes, void* stream) {
  std::string err;
  return finish(dr::texture_bwd_launch(d_out, uv, num_points, texture, height, width,
                                       channels, flags, d_uv, d_texture, scratch,
                                       scratch_bytes, as_stream(stream), err),
                err);
}

size_t dr_texture_map_bwd_scratch_bytes(int32_t height, int32_t width, int32_t channels) {
  if (height < 1 || width < 1 || channels < 1 || channels > DR_MAX_CHANNELS) return 0;
  return dr::texture_fixed_bytes(height, width, channels);
}

int dr_point_light_fwd(const float* diffuse, const float* normals, const float* positions,
                       int64_t num_samples, int32_t diffuse_stride, int32_t normals_stride,
                       int32_t positions_stride, const dr_point_light* params, float* out,
                       int32_t out_channels, void* stream) {
  std::string err;
  return finish(dr::point_light_fwd_launch(diffuse, normals, positions, num_samples,
                                           diffuse_stride, normals_stride, positions_stride,
                                           params, out, out_channels, as_stream(stream), err),
                err);
}

int dr_point_light_bwd(const float* d_out, int32_t out_channels, const float* diffuse,
                       const float* normals, const float* positions, int64_t num_samples,
                       int32_t diffuse_stride, int32_t normals_stride,
                       int32_t positions_stride, const dr_point_light* params,
                       float* d_diffuse, float* d_normals, float* d_positions,
                       int32_t grad_stride, void* stream) {
  std::string err;
  return finish(dr::point_light_bwd_launch(d_out, out_channels, diffuse, normals, positions,
                                           num_samples, diffuse_stride, normals_stride,
                                           positions_stride, params, d_diffuse, d_normals,
                                           d_positions, grad_stride, as_stream(stream), err),
                err);
}

int dr_composite_over_fwd(const float* shaded, const float* z_buffer, int32_t channels,
                          const dr_image_desc* images, int32_t num_images, int32_t num_layers,
                          float* out, void* stream) {
  std::string err;
  return finish(dr::over_fwd_launch(shaded, z_buffer, channels, images, num_images, num_layers,
                                    out, as_stream(stream), err),
                err);
}

int dr_composite_over_bwd(const float* d_out, const float* shaded, const float* z_buffer,
                          int32_t channels, const dr_image_desc* images, int32_t num_images,
                          int32_t num_layers, float* d_shaded, void* stream) {
  std::string err;
  return finish(dr::over_bwd_launch(d_out, shaded, z_buffer, channels, images, num_images,
                                    num_layers, d_shaded, as_stream(stream), err),
                err);
}

int dr_squared_error(const float* image, const float* target, int64_t count, float weight,
                     float* seed, double* partials, float* loss, void* stream) {
  std::string err;
  return finish(dr::squared_error_launch(image, target, count, weight, seed, partials, loss,
                                         as_stream(stream), err),
                err);
}

int dr_vertex_normals_fwd(const float* vertices, const int32_t* triangles,
                          const dr_image_desc* meshes, int32_t num_meshes, float* accum,
                          float* normals, void* stream) {
  std::string err;
  return finish(dr::normals_fwd_launch(vertices, triangles, meshes, num_meshes, accum, normals,
                                       as_stream(stream), err),
                err);
}

int dr_vertex_normals_bwd(const float* d_normals, const float* vertices,
                          const int32_t* triangles, const dr_image_desc* meshes,
                          int32_t num_meshes, const float* accum, float* d_accum,
                          float* d_vertices, void* stream) {
  std::string err;
  return finish(dr::normals_bwd_launch(d_normals, vertices, triangles, meshes, num_meshes,
                                       accum, d_accum, d_vertices, as_stream(stream), err),
                err);
}

int dr_vertex_normals_csr_fwd(const float* vertices, const int32_t* triangles,
                              const dr_image_desc* meshes, int32_t num_meshes,
                              const int64_t* vertex_offsets, const int32_t* corners,
                              float* face_scratch, float* accum, float* normals, void* stream) {
  std::string err;
  return finish(dr::normals_csr_fwd_launch(vertices, triangles, meshes, num_meshes,
                                           vertex_offsets, corners, face_scratch, accum,
                                           normals, as_stream(stream), err),
                err);
}

int dr_vertex_normals_csr_bwd(const float* d_normals, const float* vertices,
                              const int32_t* triangles, const dr_image_desc* meshes,
                              int32_t num_meshes, const int64_t* vertex_offsets,
                              const int32_t* corners, const float* accum, float* d_accum,
                              float* corner_scratch, float* d_vertices, void* stream) {
  std::string err;
  return finish(dr::normals_csr_bwd_launch(d_normals, vertices, triangles, meshes, num_meshes,
                                           vertex_offsets, corners, accum, d_accum,
                                           corner_scratch, d_vertices, as_stream(stream), err),
                err);
}

int dr_splat_positions_fwd(const float* clip_vertices, const int32_t* triangles,
                           const int32_t* triangle_ids, const float* z_buffer,
                           const float* barycentrics, const dr_image_desc* images,
                           int32_t num_images, int32_t num_layers, float* positions,
                           void* stream) {
  std::string err;
  return finish(dr::positions_fwd_launch(clip_vertices, triangles, triangle_ids, z_buffer,
                                         barycentrics, images, num_images, num_layers,
                                         positions, as_stream(stream), err),
                err);
}

int dr_splat_positions_bwd(const float* d_positions, const float* clip_vertices,
                           const int32_t* triangles, const int32_t* triangle_ids,
                           const float* z_buffer, const float* barycentrics,
                           const dr_image_desc* images, int32_t num_images,
                           int32_t num_layers, float* d_clip_vertices,
                           float* d_barycentrics, void* stream) {
  std::string err;
  return finish(dr::positions_bwd_launch(d_positions, clip_vertices, triangles,
                                         triangle_ids, z_buffer, barycentrics, images,
                                         num_images, num_layers, d_clip_vertices,
                                         d_barycentrics, as_stream(stream), err),
                err);
}

int dr_splat_fwd(const float* positions, const float* z_buffer, const float* colors,
                 int32_t num_channels, const dr_image_desc* images, int32_t num_images,
                 int32_t num_layers, float* out, float* saved, float* accum,
                 float* normalized, void* stream) {
  std::string err;
  return finish(dr::splat_fwd_launch(positions, z_buffer, colors, num_channels, images,
                                     num_images, num_layers, out, saved, accum, normalized,
                                     as_stream(stream), err),
                err);
}

int dr_splat_bwd_ex(const float* d_out, const float* positions, const float* z_buffer,
                    const float* colors, const float* saved, int32_t num_channels,
                    const dr_image_desc* images, int32_t num_images, int32_t num_layers,
                    uint32_t flags, float* d_colors, float* d_positions, void* stream) {
  std::string err;
  return finish(dr::splat_bwd_launch(d_out, positions, z_buffer, colors, saved, num_channels,
                                     images, num_images, num_layers, flags, d_colors,
                                     d_positions, as_stream(stream), err),
                err);
}

int dr_splat_bwd(const float* d_out, const float* positions, const float* z_buffer,
                 const float* colors, const float* saved, int32_t num_channels,
                 const dr_image_desc* images, int32_t num_images, int32_t num_layers,
                 float* d_colors, float* d_positions, void* stream) {
  return dr_splat_bwd_ex(d_out, positions, z_buffer, colors, saved, num_channels, images,
                         num_images, num_layers, 0u, d_colors, d_positions, stream);
}

int dr_splat_jvp(const float* positions, const float* z_buffer, const float* colors,
                 const float* d_positions, const float* d_colors, int32_t num_channels,
                 const dr_image_desc* images, int32_t num_images, int32_t num_layers,
                 float* d_image, void* stream) {
  std::string err;
  return finish(dr::splat_jvp_launch(positions, z_buffer, colors, d_positions, d_colors,
                                     num_channels, images, num_images, num_layers, d_image,
                                     as_stream(stream), err),
                err);
}

}  // extern "C"
