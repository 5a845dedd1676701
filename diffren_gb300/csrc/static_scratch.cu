// Allocation-free rasterizer entry point.
//
// Some callers of this library cannot allocate device memory for the
// rasterizer's scratch space. The clearest case is an XLA custom call:
// diffren's own FFI handler receives only its input and result buffers from
// XLA, and memory obtained behind XLA's back (cudaMalloc inside the handler)
// bypasses XLA's allocator and its memory accounting. The reference solves
// this by reusing the barycentrics output as scratch; other hosts with a
// fixed device-memory arena (render plugins, embedded loops) are in the same
// position. For them, dr_rasterize_triangles_static_scratch keeps the
// scratch in a device array that is part of this library's module image.
//
// The array has a fixed size, DR_STATIC_SCRATCH_BYTES. A device takes it
// when this library's module is loaded in that device's context: under
// CUDA's default lazy loading that is the first static-scratch call on the
// device (the address lookup below loads the module), with
// CUDA_MODULE_LOADING=EAGER it is context creation. It is held until the
// context ends (process exit). Every call shares it and it keeps the
// previous call's contents; the rasterizer clears the part that must start
// at zero on each call. Calls whose work overlaps on the GPU (on different
// streams, or from different threads) race on the array: the caller must
// order them, e.g. by issuing them on one stream.
//
// The device address of the array belongs to a CUDA context. It is looked
// up once per (device, context) pair, with that device current, and cached;
// a new context on the device (after cudaDeviceReset, or a driver-API
// context made current by the caller) gets its own lookup.
#include <cuda.h>

#include <mutex>
#include <string>

#include "diffren_gb300.h"
#include "internal.h"

namespace {

static_assert(DR_STATIC_SCRATCH_BYTES % 256 == 0, "scratch size is 256-aligned");

__device__ __align__(256) unsigned char g_static_scratch[DR_STATIC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
struct CachedAddress {
  CUcontext context;
  void* address;
};
CachedAddress g_scratch_address[kMaxDevices] = {};
typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
CtxGetCurrentFn g_ctx_get_current = nullptr;

// The current CUDA context (null if none is bound yet), through the driver
// entry point the runtime hands out (no link against libcuda).
int current_context(CUcontext* ctx, std::string& err) {
  if (g_ctx_get_current == nullptr) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    const cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000,
                                                           cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || fn == nullptr) {
      err = "cuCtxGetCurrent is not available from the CUDA runtime";
      return DR_ERR_CUDA;
    }
    g_ctx_get_current = reinterpret_cast<CtxGetCurrentFn>(fn);
  }
  *ctx = nullptr;
  if (g_ctx_get_current(ctx) != CUDA_SUCCESS) {
    err = "cuCtxGetCurrent failed";
    return DR_ERR_CUDA;
  }
  return DR_OK;
}

// Device address of g_static_scratch in the current context. The host-side
// name of the array is only a stand-in; its device address is queried with
// the device current, once per (device, context).
int scratch_address(void** out, std::string& err) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    err = std::string("cudaGetDevice: ") + cudaGetErrorString(e);
    return DR_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    err = "device index out of range for the static scratch table";
    return DR_ERR_INVALID_ARGUMENT;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  CUcontext ctx = nullptr;
  int rc = current_context(&ctx, err);
  if (rc != DR_OK) return rc;
  CachedAddress& c = g_scratch_address[dev];
  if (ctx == nullptr || c.address == nullptr || c.context != ctx) {
    // The lookup binds the device's primary context when none is current
    // yet, and loads this library's module in it (which takes the array).
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || p == nullptr) {
      err = std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e);
      return DR_ERR_CUDA;
    }
    rc = current_context(&ctx, err);
    if (rc != DR_OK) return rc;
    c.context = ctx;
    c.address = p;
  }
  *out = c.address;
  return DR_OK;
}

}  // namespace

extern "C" int dr_rasterize_triangles_static_scratch(
    const float* vertices, int32_t num_vertices, const int32_t* triangles,
    int32_t num_triangles, int32_t image_width, int32_t image_height,
    int32_t num_layers, int32_t face_culling_mode, int32_t depth_mode,
    int32_t* triangle_ids, float* z_buffer, float* barycentrics, void* stream) {
  std::string err;
  dr_image_desc d;
  d.width = image_width;
  d.height = image_height;
  d.num_vertices = num_vertices;
  d.num_triangles = num_triangles;
  d.vertex_offset = 0;
  d.triangle_offset = 0;
  d.pixel_offset = 0;
  dr_raster_config c;
  c.num_layers = num_layers;
  c.face_culling_mode = face_culling_mode;
  c.depth_mode = depth_mode;
  c.tile_width = 0;
  c.tile_height = 0;
  c.large_tiles = 0;
  c.flags = 0;
  // Size check first: nothing runs on the GPU for an oversized request.
  const size_t need = dr::raster_workspace_bytes(&d, 1, &c, err);
  int rc = DR_OK;
  if (need == 0) {
    rc = DR_ERR_INVALID_ARGUMENT;
  } else if (need > DR_STATIC_SCRATCH_BYTES) {
    err = "dr_rasterize_triangles_static_scratch: this image and triangle count need " +
          std::to_string(need) + " bytes of scratch, more than the " +
          std::to_string(size_t(DR_STATIC_SCRATCH_BYTES)) +
          " bytes of the static array; use dr_rasterize_triangles with a workspace";
    rc = DR_ERR_WORKSPACE_TOO_SMALL;
  }
  void* scratch = nullptr;
  if (rc == DR_OK) rc = scratch_address(&scratch, err);
  if (rc == DR_OK)
    rc = dr::raster_launch(vertices, triangles, &d, 1, &c, triangle_ids, z_buffer,
                           barycentrics, scratch, DR_STATIC_SCRATCH_BYTES,
                           reinterpret_cast<cudaStream_t>(stream), err);
  if (rc != DR_OK) dr::set_last_error(err);
  return rc;
}

extern "C" int dr_read_static_scratch_error_flags(uint32_t* flags, void* stream) {
  std::string err;
  int rc = DR_OK;
  if (flags == nullptr) {
    err = "flags must be non-null";
    rc = DR_ERR_INVALID_ARGUMENT;
  }
  void* scratch = nullptr;
  if (rc == DR_OK) rc = scratch_address(&scratch, err);
  if (rc != DR_OK) {
    dr::set_last_error(err);
    return rc;
  }
  // Same word and same read as dr_read_error_flags on a caller workspace.
  return dr_read_error_flags(scratch, flags, stream);
}
