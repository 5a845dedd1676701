// Test infrastructure only: a C entry point over the reference's own CUDA
// rasterizer, diffren::cuda::RasterizeTrianglesImpl
// (diffren/common/kernels/rasterize_triangles_impl_cuda.cu.h:35-42), which
// oracle/Makefile compiles with nvcc's default flags (floating-point
// contraction on, as the reference ships) into oracle/_ref/. All pointers
// are device pointers; the call is asynchronous on `stream`, like the
// reference function. Returns 0, or 1 with the reference's status message
// copied into `message` (when given).
#include <cstdint>
#include <cstring>

#include "diffren/common/kernels/rasterize_triangles_impl_cuda.cu.h"

extern "C" int ref_rasterize_cuda(const float* vertices, const int32_t* triangles,
                                  int32_t triangle_count, int32_t image_width,
                                  int32_t image_height, int32_t num_layers,
                                  int32_t face_culling_mode, int32_t* triangle_ids,
                                  float* z_buffer, float* barycentrics, void* stream,
                                  char* message, int32_t message_size) {
  const absl::Status s = diffren::cuda::RasterizeTrianglesImpl(
      vertices, triangles, triangle_count, image_width, image_height, num_layers,
      static_cast<diffren::FaceCullingMode>(face_culling_mode), triangle_ids, z_buffer,
      barycentrics, static_cast<cudaStream_t>(stream));
  if (s.ok()) return 0;
  if (message != nullptr && message_size > 0) {
    std::strncpy(message, s.message().c_str(), size_t(message_size) - 1);
    message[message_size - 1] = '\0';
  }
  return 1;
}
