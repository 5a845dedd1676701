/*
 * diffren_gb300: C ABI of the GB300 (sm_103a) rasterize-then-splat path.
 *
 * Every entry point takes device pointers, plain sizes and a cudaStream_t
 * passed as `void* stream`, enqueues its kernels on that stream and returns
 * a status code (DR_OK = 0) without synchronizing. No entry point allocates
 * device memory: scratch space is a caller-owned workspace sized by the
 * matching *_workspace_bytes function, so every call can be captured in a
 * CUDA graph. On failure dr_last_error() returns a message (thread-local).
 *
 * Layouts (all row-major, float32 / int32):
 *   vertices      [V, 4]  clip-space xyzw, 16-byte aligned
 *   triangles     [T, 3]  vertex indices local to their mesh
 *   triangle_ids  [L, H, W], z_buffer [L, H, W], barycentrics [L, H, W, 3]
 *   layered images (interpolated attributes, shaded colors) [L, H, W, C]
 *   composited images [H, W, C]
 * Batches are packed: image i's layered buffers start at element
 * L * pixel_offset * (channels) and its composited buffer at
 * pixel_offset * C, where pixel_offset = sum of H*W of the images before it.
 *
 * Reference interfaces replaced (paths inside google-research/diffren):
 *   dr_rasterize_triangles  -> diffren::cuda::RasterizeTrianglesImpl
 *       (diffren/common/kernels/rasterize_triangles_impl_cuda.cu.h:35-42),
 *       reached from the XLA FFI handler rasterize_triangles
 *       (diffren/jax/internal/kernels/rasterize_triangles_gpu.cc:44-77);
 *       with DR_DEPTH_FLOAT it reproduces diffren::RasterizeTrianglesImpl
 *       (rasterize_triangles_impl.h:53-58, the CPU handler of
 *       rasterize_triangles_cpu.cc:43-79).
 *   dr_rasterize_batch      -> jax.vmap over rasterize_triangles, which the
 *       reference lowers to sequential per-image FFI calls
 *       (rasterize_triangles_xla.py:68-75, vmap_method='sequential_unrolled').
 *   dr_transform_vertices   -> transforms.transform_homogeneous
 *       (diffren/jax/utils/transforms.py:41-79) as used by
 *       rasterize.py:90-96 and splat.py:209-212.
 *   dr_interpolate_fwd/bwd  -> interpolate.interpolate_vertex_attribute
 *       (diffren/jax/internal/interpolate.py:24-63, 118-145) and its VJP.
 *   dr_diff_barycentrics_fwd/bwd -> rasterize.differentiable_barycentrics
 *       (diffren/jax/internal/rasterize.py:127-255) and its VJP.
 *   dr_splat_positions_fwd/bwd -> the clip-space interpolation and viewport
 *       transform of splat.splat_shaded_pixels (splat.py:207-221) and its VJP.
 *   dr_texture_map_fwd/bwd  -> utils.shaders.texture_map
 *       (diffren/jax/utils/shaders.py:40-65, utils/image.py:21-118).
 *   dr_composite_over_fwd/bwd -> the OVER mode of render.render_triangles
 *       (diffren/jax/render.py:134-140: foreground mask, composite.over of
 *       composite.py:20-37) and its VJP.
 *   dr_vertex_normals_fwd/bwd -> utils.mesh.compute_vertex_normals
 *       (diffren/jax/utils/mesh.py:22-52) and its VJP.
 *   dr_splat_fwd/bwd/jvp    -> splat.splat_at_pixel_centers + composite.over
 *       (diffren/jax/internal/splat.py:26-175, diffren/jax/composite.py:20-37)
 *       and their VJP and JVP.
 */
#ifndef DIFFREN_GB300_H_
#define DIFFREN_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DR_OK 0
#define DR_ERR_INVALID_ARGUMENT 1
#define DR_ERR_CUDA 2
#define DR_ERR_WORKSPACE_TOO_SMALL 3
#define DR_ERR_MISALIGNED 4

/* Values of diffren.jax.constants.FaceCullingMode (constants.py:20-24). */
#define DR_CULL_NONE 0
#define DR_CULL_BACK 1
#define DR_CULL_FRONT 2

/* Depth semantics of the rasterizer.
 * DISCRETIZED: the reference CUDA rasterizer. Depth enters a packed 64-bit
 *   key (32-bit discretized depth << 32 | triangle id); each pixel keeps the
 *   L smallest keys. Empty layers: id 0, z 1, barycentrics 0.
 * FLOAT: the reference CPU rasterizer. Fragments are ordered by float depth,
 *   ties to the lower triangle id. Empty layers: id -1, z 1, barycentrics 0. */
#define DR_DEPTH_DISCRETIZED 0
#define DR_DEPTH_FLOAT 1

/* Bits of the device error word (dr_read_error_flags). */
#define DR_FLAG_INDEX_OUT_OF_RANGE 1u /* a triangle named a vertex >= V or < 0;
                                         that triangle was skipped */
#define DR_FLAG_NONFINITE_VERTEX 2u   /* a triangle's clip vertex held a NaN or
                                         infinity; it is rasterized as the
                                         reference would (report only) */

/* One image of a batch: its mesh and its resolution. */
typedef struct dr_image_desc {
  int32_t width, height;
  int32_t num_vertices, num_triangles;
  int64_t vertex_offset;   /* first vertex of the mesh in `vertices` */
  int64_t triangle_offset; /* first triangle of the mesh in `triangles` */
  int64_t pixel_offset;    /* sum of width*height of the images before it */
} dr_image_desc;

typedef struct dr_raster_config {
  int32_t num_layers;        /* L >= 1, at most DR_MAX_LAYERS */
  int32_t face_culling_mode; /* DR_CULL_* */
  int32_t depth_mode;        /* DR_DEPTH_* */
  int32_t tile_width;        /* fine-raster tile, 0 = default (16) */
  int32_t tile_height;       /* 0 = default (16); tile_width*tile_height <= 1024 */
  int32_t large_tiles;       /* triangles spanning more tiles than this go to a
                                per-image list every tile scans; 0 = default */
  uint32_t flags;            /* DR_RASTER_* bits, 0 = none */
} dr_raster_config;

/* dr_raster_config.flags: background samples (z = 1) get their depth (and,
 * in dr_rasterize_batch_interpolate, zero attributes) but their triangle id
 * and barycentrics are left unwritten. For callers that tell background
 * samples by the depth buffer, as the splat path does; saves 16 bytes per
 * background layer sample. */
#define DR_RASTER_FOREGROUND_ONLY 1u
/* dr_raster_config.flags, dr_rasterize_batch_interpolate only: background
 * samples' interpolated attributes are left unwritten too. For callers whose
 * only reader of the attributes is the splat given the depth buffer (it
 * reads colors of foreground samples only); saves 4 K bytes per background
 * layer sample. */
#define DR_RASTER_FOREGROUND_ATTRIBUTES 2u

#define DR_MAX_LAYERS 16
#define DR_MAX_CHANNELS 16
#define DR_MAX_BATCH_INLINE 128 /* larger batches are split into launches */
#define DR_MAX_IMAGE_DIM 32768  /* largest image width or height */

/* Message of the last failing call on this thread ("" if none). */
const char* dr_last_error(void);
int32_t dr_abi_version(void);

/* ---------------------------------------------------------------- raster */

size_t dr_rasterize_batch_workspace_bytes(const dr_image_desc* images,
                                          int32_t num_images,
                                          const dr_raster_config* config);

/* Rasterizes every image of the batch (setup, tile binning and the
 * shared-memory fine rasterizer run once for the whole batch). `images` is a
 * host array. Outputs are packed [L, H_i, W_i] per image. */
int dr_rasterize_batch(const float* vertices, const int32_t* triangles,
                       const dr_image_desc* images, int32_t num_images,
                       const dr_raster_config* config, int32_t* triangle_ids,
                       float* z_buffer, float* barycentrics, void* workspace,
                       size_t workspace_bytes, void* stream);

/* dr_rasterize_batch fused with dr_interpolate_with_positions_fwd: the
 * rasterizer's epilogue, which already holds each layer sample's triangle
 * and barycentrics, also writes the splat position `positions`
 * [L, H_i, W_i, 4] of every foreground sample as (viewport xyz, clip w)
 * (background entries are left unwritten: pass z_buffer to the splat,
 * which then takes the foreground from it), when `vertex_ids` is non-null
 * the foreground samples' three vertex indices [L, H_i, W_i, 3] (the
 * Framebuffer's vertex_ids, rasterize.py:111-113) and, when
 * `attributes` [V, K] is non-null,
 * the interpolated attributes `attributes_out` [L, H_i, W_i, K] (background
 * 0) (interpolate.py:24-63, splat.py:207-221). Same bits as the separate
 * calls; saves their re-read of ids/z/barycentrics and vertex gathers. No
 * reference counterpart: the reference runs these as separate JAX ops. */
int dr_rasterize_batch_interpolate(const float* vertices, const int32_t* triangles,
                                   const dr_image_desc* images, int32_t num_images,
                                   const dr_raster_config* config, int32_t* triangle_ids,
                                   float* z_buffer, float* barycentrics,
                                   const float* attributes, int32_t num_channels,
                                   float* attributes_out, float* positions,
                                   int32_t* vertex_ids, void* workspace,
                                   size_t workspace_bytes, void* stream);

size_t dr_rasterize_triangles_workspace_bytes(int32_t num_triangles,
                                              int32_t image_width,
                                              int32_t image_height,
                                              int32_t num_layers);

/* Single image with default tiles: the drop-in for
 * diffren::cuda::RasterizeTrianglesImpl. Unlike the reference, the
 * barycentrics buffer is not used as scratch and indices are range-checked. */
int dr_rasterize_triangles(const float* vertices, int32_t num_vertices,
                           const int32_t* triangles, int32_t num_triangles,
                           int32_t image_width, int32_t image_height,
                           int32_t num_layers, int32_t face_culling_mode,
                           int32_t depth_mode, int32_t* triangle_ids,
                           float* z_buffer, float* barycentrics,
                           void* workspace, size_t workspace_bytes,
                           void* stream);

/* Allocation-free variant of dr_rasterize_triangles (no counterpart in the
 * reference). It is for callers that cannot allocate device memory for
 * scratch space, such as an XLA custom-call handler, which gets only its
 * input and result buffers from XLA. The scratch lives in a static device
 * array of DR_STATIC_SCRATCH_BYTES inside this library; requests that need
 * more return DR_ERR_WORKSPACE_TOO_SMALL without running anything. A device
 * takes the array's memory when the library's module loads in its context:
 * under CUDA's default lazy loading at the first static-scratch call on that
 * device, with CUDA_MODULE_LOADING=EAGER at context creation; it is held
 * until the process exits. The first call on a device (and in each new
 * context on it) looks up the array's device address with that device
 * current; make that first call before any stream capture. All calls share
 * the array, so calls that overlap on the GPU race: order them (e.g. one
 * stream). The call itself allocates nothing. */
#define DR_STATIC_SCRATCH_BYTES (64u << 20)
int dr_rasterize_triangles_static_scratch(
    const float* vertices, int32_t num_vertices, const int32_t* triangles,
    int32_t num_triangles, int32_t image_width, int32_t image_height,
    int32_t num_layers, int32_t face_culling_mode, int32_t depth_mode,
    int32_t* triangle_ids, float* z_buffer, float* barycentrics, void* stream);

/* dr_read_error_flags for dr_rasterize_triangles_static_scratch, whose
 * caller never sees the scratch array: synchronizes `stream` and reads the
 * DR_FLAG_* bits of the last static-scratch call on the current device. No
 * counterpart in the reference (it does not check indices). */
int dr_read_static_scratch_error_flags(uint32_t* flags, void* stream);

/* Synchronizes `stream` and reads the device error word of the last raster
 * call that used `workspace` (DR_FLAG_* bits). */
int dr_read_error_flags(const void* workspace, uint32_t* flags, void* stream);

/* Self-test of the rasterizer's depth codec: the integer emulation of the
 * reference's double-precision DiscretizeZ / UndiscretizeZ
 * (rasterize_triangles_impl_cuda.cu.cc:143-159) against those formulas on
 * every input. `results` is 7 device uint64s the caller initializes to
 * {0, UINT64_MAX, 0, UINT64_MAX, 0, 0, 0}; on completion they hold the
 * discretize mismatch count, the first bad float bit pattern, the
 * undiscretize mismatch count, the first bad discretized value, the
 * discretized value of a NaN depth, and the float-to-int32 and
 * float-to-int64 conversions of NaN on this GPU. */
int dr_selftest_depth_codec(unsigned long long* results, void* stream);

/* ------------------------------------------------------------- transform */

/* clip[v] = M_i @ (x, y, z, w or 1) for every vertex of image i, with the
 * float32 order ((m0 x + m1 y) + m2 z) + m3 w. `matrices` is [N, 4, 4] on the
 * device; `dim` is 3 or 4. */
int dr_transform_vertices(const float* matrices, const float* vertices,
                          int32_t dim, const dr_image_desc* images,
                          int32_t num_images, float* clip_vertices,
                          void* stream);

/* VJP w.r.t. the vertices: d_vertices [V, dim] = d_clip @ M_i (written). */
int dr_transform_vertices_bwd(const float* matrices, const float* d_clip_vertices,
                              int32_t dim, const dr_image_desc* images,
                              int32_t num_images, float* d_vertices, void* stream);

/* --------------------------------------------------------- interpolation */

/* out[l,y,x,:] = fg ? sum_i b_i * attr[tri[id][i], :] : background, where
 * fg = (z != 1). attributes [V, K]; background [K] (nullable = zeros). */
int dr_interpolate_fwd(const float* attributes, int32_t num_channels,
                       const int32_t* triangles, const int32_t* triangle_ids,
                       const float* z_buffer, const float* barycentrics,
                       const float* background, const dr_image_desc* images,
                       int32_t num_images, int32_t num_layers, float* out,
                       void* stream);

/* VJP. d_attributes [V, K] and d_background [K] are accumulated into (the
 * caller zeroes them); d_barycentrics [L,H,W,3] is written when non-null. */
int dr_interpolate_bwd(const float* d_out, const float* attributes,
                       int32_t num_channels, const int32_t* triangles,
                       const int32_t* triangle_ids, const float* z_buffer,
                       const float* barycentrics, const dr_image_desc* images,
                       int32_t num_images, int32_t num_layers,
                       float* d_attributes, float* d_barycentrics,
                       float* d_background, void* stream);

/* ------------------------------------------- differentiable barycentrics */

/* Float barycentrics from per-triangle adjugates (rasterize.py:127-255);
 * zero where fg = 0. Output [L, H, W, 3]. */
int dr_diff_barycentrics_fwd(const float* clip_vertices, const int32_t* triangles,
                             const int32_t* triangle_ids, const float* z_buffer,
                             const dr_image_desc* images, int32_t num_images,
                             int32_t num_layers, float* barycentrics,
                             void* stream);

/* VJP: accumulates d_clip_vertices [V, 4] (caller zeroes it). */
int dr_diff_barycentrics_bwd(const float* d_barycentrics,
                             const float* clip_vertices, const int32_t* triangles,
                             const int32_t* triangle_ids, const float* z_buffer,
                             const dr_image_desc* images, int32_t num_images,
                             int32_t num_layers, float* d_clip_vertices,
                             void* stream);

/* ----------------------------------------------------------------- splat */

#define DR_MAX_SPLAT_CHANNELS 8

/* Viewport positions of every layer sample for splatting (splat.py:207-221):
 * clip xyzw interpolated with the barycentrics (background (0, 0, 1, 1)),
 * viewport = ((xyz / w + 1) * (W, H, 1)) * 0.5, with fg = (z != 1) in the
 * fourth component. positions [L, H, W, 4], 16-byte aligned. */
int dr_splat_positions_fwd(const float* clip_vertices, const int32_t* triangles,
                           const int32_t* triangle_ids, const float* z_buffer,
                           const float* barycentrics, const dr_image_desc* images,
                           int32_t num_images, int32_t num_layers, float* positions,
                           void* stream);

/* VJP of dr_splat_positions_fwd w.r.t. the viewport x, y (viewport z only
 * enters comparisons): accumulates d_clip_vertices [V, 4] (caller zeroes
 * it) and writes d_barycentrics [L, H, W, 3] when non-null. */
int dr_splat_positions_bwd(const float* d_positions, const float* clip_vertices,
                           const int32_t* triangles, const int32_t* triangle_ids,
                           const float* z_buffer, const float* barycentrics,
                           const dr_image_desc* images, int32_t num_images,
                           int32_t num_layers, float* d_clip_vertices,
                           float* d_barycentrics, void* stream);

/* Fused dr_interpolate_fwd (background 0) and dr_splat_positions_fwd: one
 * pass over the layer samples writes attributes_out [L, H, W, K] and
 * positions [L, H, W, 4] with the same bits as the two separate calls. */
int dr_interpolate_with_positions_fwd(const float* attributes, int32_t num_channels,
                                      const float* clip_vertices, const int32_t* triangles,
                                      const int32_t* triangle_ids, const float* z_buffer,
                                      const float* barycentrics, const dr_image_desc* images,
                                      int32_t num_images, int32_t num_layers,
                                      float* attributes_out, float* positions, void* stream);

/* Its VJP: from d_attributes_out (nullable) and d_positions, accumulates
 * d_attributes [V, K] and d_clip_vertices [V, 4] (caller zeroes both) and
 * writes d_barycentrics when non-null. `positions` and `vertex_ids`
 * (nullable) are dr_rasterize_batch_interpolate's: with them the VJP reads
 * each foreground sample's vertex indices and clip w instead of gathering
 * its triangle and clip vertices. */
int dr_interpolate_with_positions_bwd(const float* d_attributes_out,
                                      const float* d_positions, const float* attributes,
                                      int32_t num_channels, const float* clip_vertices,
                                      const int32_t* triangles, const int32_t* triangle_ids,
                                      const float* z_buffer, const float* barycentrics,
                                      const float* positions, const int32_t* vertex_ids,
                                      const dr_image_desc* images, int32_t num_images,
                                      int32_t num_layers, float* d_attributes,
                                      float* d_clip_vertices, float* d_barycentrics,
                                      void* stream);

/* dr_interpolate_with_positions_bwd with flags. DR_SAMPLES_DETERMINISTIC:
 * d_attributes and d_clip_vertices are summed in 64-bit fixed point (a
 * power-of-two scale chosen from the largest value added, so that no sum
 * can overflow) instead of with float atomics: integer sums do not depend
 * on the order of the additions, so the gradients are the same bits on
 * every run (and within 2^-30 of the largest addend of the exact sum). Two
 * passes over the samples plus one over the vertices; `scratch` (256-byte
 * aligned) holds the sums. flags = 0 is dr_interpolate_with_positions_bwd
 * (scratch unused). */
#define DR_SAMPLES_DETERMINISTIC 1u
size_t dr_interpolate_with_positions_bwd_scratch_bytes(const dr_image_desc* images,
                                                       int32_t num_images,
                                                       int32_t num_channels);
int dr_interpolate_with_positions_bwd_ex(
    const float* d_attributes_out, const float* d_positions, const float* attributes,
    int32_t num_channels, const float* clip_vertices, const int32_t* triangles,
    const int32_t* triangle_ids, const float* z_buffer, const float* barycentrics,
    const float* positions, const int32_t* vertex_ids, const dr_image_desc* images,
    int32_t num_images, int32_t num_layers, uint32_t flags, float* d_attributes,
    float* d_clip_vertices, float* d_barycentrics, void* scratch, size_t scratch_bytes,
    void* stream);

/* ---------------------------------------------------------- shaders */

/* shaders.texture_map (diffren/jax/utils/shaders.py:40-65): bilinear
 * resampling (image.py:21-118) of a float [height, width, channels] texture
 * at uv [num_points, 2] (u along the width), out [num_points, channels],
 * with the reference's expression order. flags: DR_TEXTURE_PAD_ZERO pads
 * with zeros instead of the edge texels (pad_mode='constant'),
 * DR_TEXTURE_TEXEL_UNITS takes the points in texel units instead of uv
 * (image.bilinear_resample's locations). */
#define DR_TEXTURE_PAD_ZERO 1
#define DR_TEXTURE_TEXEL_UNITS 2
/* dr_texture_map_bwd_ex only: d_texture summed in 64-bit fixed point (the
 * scale from the largest |d_out|) instead of with float atomics, the same
 * bits on every run. */
#define DR_TEXTURE_DETERMINISTIC 4
int dr_texture_map_fwd(const float* uv, int64_t num_points, const float* texture,
                       int32_t height, int32_t width, int32_t channels, int32_t flags,
                       float* out, void* stream);

/* Its VJP: d_uv [num_points, 2] is written (nullable), d_texture
 * [height, width, channels] accumulated (nullable; caller zeroes it). */
int dr_texture_map_bwd(const float* d_out, const float* uv, int64_t num_points,
                       const float* texture, int32_t height, int32_t width,
                       int32_t channels, int32_t flags, float* d_uv, float* d_texture,
                       void* stream);

/* dr_texture_map_bwd with a scratch buffer (256-byte aligned, of
 * dr_texture_map_bwd_scratch_bytes bytes), which DR_TEXTURE_DETERMINISTIC
 * needs for its fixed-point sums. */
size_t dr_texture_map_bwd_scratch_bytes(int32_t height, int32_t width, int32_t channels);
int dr_texture_map_bwd_ex(const float* d_out, const float* uv, int64_t num_points,
                          const float* texture, int32_t height, int32_t width,
                          int32_t channels, int32_t flags, float* d_uv, float* d_texture,
                          void* scratch, size_t scratch_bytes, void* stream);

/* shaders.point_light (shaders.py:100-173): ambient + diffuse + Blinn-Phong
 * specular lighting with quadratic distance attenuation, per sample. */
typedef struct {
  float light[3];  /* point light location */
  float eye[3];    /* eye location */
  float ka, kd, ks, ns;
  float attenuation_constant, attenuation_linear, attenuation_quadratic;
} dr_point_light;

/* diffuse, normals and positions are rows of 3 floats, `*_stride` floats
 * apart (>= 3; columns of one packed attribute buffer can be passed in
 * place); out [num_samples, out_channels], out_channels 3, or 4 with the
 * last channel (alpha) set to 1. */
int dr_point_light_fwd(const float* diffuse, const float* normals, const float* positions,
                       int64_t num_samples, int32_t diffuse_stride, int32_t normals_stride,
                       int32_t positions_stride, const dr_point_light* params, float* out,
                       int32_t out_channels, void* stream);

/* Its VJP for d_out [num_samples, out_channels] (the alpha gradient is
 * ignored): d_diffuse, d_normals and d_positions (each nullable) are
 * written as rows `grad_stride` floats apart. */
int dr_point_light_bwd(const float* d_out, int32_t out_channels, const float* diffuse,
                       const float* normals, const float* positions, int64_t num_samples,
                       int32_t diffuse_stride, int32_t normals_stride,
                       int32_t positions_stride, const dr_point_light* params,
                       float* d_diffuse, float* d_normals, float* d_positions,
                       int32_t grad_stride, void* stream);

/* ------------------------------------------------------ compositing */

/* CompositingMode.OVER of render_triangles (render.py:134-140): shaded
 * [L, H, W, C] per image (alpha in the last channel, premultiplied) times
 * the foreground mask (z_buffer [L, H, W] != 1), composited back to front,
 * o = s[L-1]; o = s[l] + (1 - alpha[l]) * o (composite.py:20-37), into out
 * [H, W, C] per image. Channels >= 1, 1 <= num_layers <= DR_MAX_LAYERS. */
int dr_composite_over_fwd(const float* shaded, const float* z_buffer, int32_t channels,
                          const dr_image_desc* images, int32_t num_images, int32_t num_layers,
                          float* out, void* stream);

/* Its VJP: d_shaded [L, H, W, C] per image is written (background samples
 * get 0). */
int dr_composite_over_bwd(const float* d_out, const float* shaded, const float* z_buffer,
                          int32_t channels, const dr_image_desc* images, int32_t num_images,
                          int32_t num_layers, float* d_shaded, void* stream);

/* ------------------------------------------------------------- meshes */

/* mesh.compute_vertex_normals (diffren/jax/utils/mesh.py:22-52) over a
 * ragged batch of meshes, one per descriptor (only num_vertices,
 * num_triangles, vertex_offset and triangle_offset are read): face normals
 * cross(v1 - v0, v2 - v0) summed into each corner vertex, then
 * x * rsqrt(|x|^2 + 1e-12) (transforms.l2_normalize, transforms.py:26-37).
 * vertices [V, 3], normals [V, 3], accum [V, 4] scratch (16-byte aligned)
 * that the VJP reads back; V = max(vertex_offset + num_vertices).
 * Triangles with an out-of-range index add nothing. Meshes are disjoint
 * vertex ranges: a vertex covered by two descriptors sums both. The sums
 * use float atomics, so their order (and the last bits) varies by run. */
int dr_vertex_normals_fwd(const float* vertices, const int32_t* triangles,
                          const dr_image_desc* meshes, int32_t num_meshes, float* accum,
                          float* normals, void* stream);

/* Its VJP: d_accum [V, 4] scratch (16-byte aligned), d_vertices [V, 3]
 * accumulated (caller zeroes it). */
int dr_vertex_normals_bwd(const float* d_normals, const float* vertices,
                          const int32_t* triangles, const dr_image_desc* meshes,
                          int32_t num_meshes, const float* accum, float* d_accum,
                          float* d_vertices, void* stream);

/* The same normals without atomics, the same bits on every run, from a
 * vertex -> corner adjacency: corner 3 g + s is slot s of global triangle g
 * (triangles numbered in mesh order); vertex i's corners are
 * corners[vertex_offsets[i] .. vertex_offsets[i + 1]), slot 0 ones first
 * then slot 1 then slot 2, each in triangle order, listing no corner of a
 * triangle with an out-of-range index (diffren_gb300.mesh builds it once
 * per topology). Sums run in that order: the three per-slot sums in
 * triangle order, then (s0 + s1) + s2, as three scatter-adds into zeros
 * give. face_scratch [T, 4] and accum [V, 4] 16-byte aligned. */
int dr_vertex_normals_csr_fwd(const float* vertices, const int32_t* triangles,
                              const dr_image_desc* meshes, int32_t num_meshes,
                              const int64_t* vertex_offsets, const int32_t* corners,
                              float* face_scratch, float* accum, float* normals, void* stream);

/* Its VJP: d_accum [V, 4] and corner_scratch [3 T, 4] (16-byte aligned)
 * are scratch; d_vertices [V, 3] is accumulated into. */
int dr_vertex_normals_csr_bwd(const float* d_normals, const float* vertices,
                              const int32_t* triangles, const dr_image_desc* meshes,
                              int32_t num_meshes, const int64_t* vertex_offsets,
                              const int32_t* corners, const float* accum, float* d_accum,
                              float* corner_scratch, float* d_vertices, void* stream);

/* splat_at_pixel_centers + composite.over (splat.py:26-175,
 * composite.py:20-37): 3x3 Gaussian splats of every layer sample with the
 * per-tap surface test, normalization and back-to-front over compositing.
 * positions [L, H, W, 4] (viewport xyz, fg); z_buffer [L, H, W] (nullable)
 * is the rasterizer's depth: samples where it is 1 are background (viewport
 * z 1, no splat) and their positions are not read, so producers may leave
 * them unwritten; without it every position is read and its w is the
 * foreground flag. colors [L, H, W, C]
 * (1 <= C <= DR_MAX_SPLAT_CHANNELS, last channel alpha); out [H, W, C].
 * saved [3 (C + 1) + 2, P] receives the fg/surface/bg accumulators and
 * weights the VJP needs, one plane of P pixels per value, P = the largest
 * pixel_offset + width * height of the images, then (for three layers) each
 * pixel's surface classes of its 9 taps as 32-bit codes, then the list of
 * the screen tiles that hold foreground (nullable; the planes are written
 * only near foreground samples, where dr_splat_bwd reads them); accum and
 * normalized [3, H, W, C] are
 * the reference's debugging buffers (nullable). With C % 4 == 0 the color
 * and output buffers must be 16-byte aligned. */
int dr_splat_fwd(const float* positions, const float* z_buffer, const float* colors,
                 int32_t num_channels, const dr_image_desc* images, int32_t num_images,
                 int32_t num_layers, float* out, float* saved, float* accum,
                 float* normalized, void* stream);

/* VJP in gather form: each sample reads the adjoints of the 9 pixels it
 * reached (no atomics). Writes d_colors [L, H, W, C] and d_positions
 * [L, H, W, 4] as (d x, d y, 0, 0); with a z_buffer, d_positions of
 * background samples are left unwritten. `saved` is the forward's; with a
 * z_buffer the call resets a work counter kept in its last plane, so
 * backward calls on one saved buffer must not overlap on the GPU. */
int dr_splat_bwd(const float* d_out, const float* positions, const float* z_buffer,
                 const float* colors, const float* saved, int32_t num_channels,
                 const dr_image_desc* images, int32_t num_images, int32_t num_layers,
                 float* d_colors, float* d_positions, void* stream);

/* dr_splat_bwd with flags. DR_SPLAT_FOREGROUND_GRADIENTS (needs z_buffer):
 * d_colors of background samples are left unwritten as well, for callers
 * that read the color gradient at foreground samples only (the rasterizer's
 * fused interpolation VJP does); saves 4 C bytes per background layer
 * sample. flags = 0 is dr_splat_bwd. */
#define DR_SPLAT_FOREGROUND_GRADIENTS 1u
int dr_splat_bwd_ex(const float* d_out, const float* positions, const float* z_buffer,
                    const float* colors, const float* saved, int32_t num_channels,
                    const dr_image_desc* images, int32_t num_images, int32_t num_layers,
                    uint32_t flags, float* d_colors, float* d_positions, void* stream);

/* Forward-mode derivative of dr_splat_fwd's image for tangents of the
 * positions (d_positions [L, H, W, 4], x and y read) and, when non-null, of
 * the colors (d_colors [L, H, W, C]), with the discrete state (pixel floors,
 * surface classes, foreground) held fixed: the jax.jvp of
 * splat_at_pixel_centers + composite.over (splat.py:26-175,
 * composite.py:20-37). Writes d_image [H, W, C]. */
int dr_splat_jvp(const float* positions, const float* z_buffer, const float* colors,
                 const float* d_positions, const float* d_colors, int32_t num_channels,
                 const dr_image_desc* images, int32_t num_images, int32_t num_layers,
                 float* d_image, void* stream);

/* ------------------------------------------------------------- losses */

/* Beyond the reference interface: the squared-error objective its
 * optimization tests fit renders with (jnp.mean((image - target)**2),
 * diffren/jax/internal/splat_test.py:137-167) and its gradient, in one pass:
 * *loss = weight * sum_i (image_i - target_i)^2 and seed_i = (2 * weight) *
 * (image_i - target_i), the d_out to seed the renderer's VJP with (weight 1
 * gives the sum, 1 / count the mean). `partials` is scratch of
 * DR_SQUARED_ERROR_PARTIALS doubles; `loss` is one float on the device. The
 * sum order is fixed (deterministic). */
#define DR_SQUARED_ERROR_PARTIALS 1216
int dr_squared_error(const float* image, const float* target, int64_t count, float weight,
                     float* seed, double* partials, float* loss, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* DIFFREN_GB300_H_ */
