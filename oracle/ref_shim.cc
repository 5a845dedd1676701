// Test infrastructure only: a C entry point over the reference's own CPU
// rasterizer, diffren::RasterizeTrianglesImpl
// (diffren/common/kernels/rasterize_triangles_impl.h:53-58), compiled in place
// from the reference tree by oracle/Makefile into oracle/_ref/. The output
// clearing (ids -1, barycentrics 0, z 1) is what the reference's XLA CPU
// handler does before the call (rasterize_triangles_cpu.cc:55-60).
#include <algorithm>
#include <cstdint>

#include "diffren/common/kernels/rasterize_triangles_impl.h"

extern "C" int ref_rasterize_cpu(const float* vertices, const int32_t* triangles,
                                 int32_t triangle_count, int32_t image_width,
                                 int32_t image_height, int32_t num_layers,
                                 int32_t face_culling_mode, int32_t* triangle_ids,
                                 float* z_buffer, float* barycentrics) {
  const int64_t n = int64_t(num_layers) * image_width * image_height;
  std::fill_n(triangle_ids, n, -1);
  std::fill_n(barycentrics, 3 * n, 0.0f);
  std::fill_n(z_buffer, n, 1.0f);
  diffren::RasterizeTrianglesImpl(
      vertices, triangles, triangle_count, image_width, image_height, num_layers,
      static_cast<diffren::FaceCullingMode>(face_culling_mode), triangle_ids,
      z_buffer, barycentrics);
  return 0;
}
