/*
 * Test infrastructure only: a CPU restatement of diffren's multi-layer
 * z-buffer triangle rasterizer, used as the checker for the CUDA kernels in
 * diffren_gb300/csrc. Nothing in the product links or calls this file.
 *
 * It restates, in plain C, the arithmetic of
 *   diffren/common/kernels/rasterize_utils.h:51-248          (fixed point,
 *       bounding box, unnormalized inverse, edge functions, inside test)
 *   diffren/common/kernels/rasterize_triangles_impl.cc:27-118 (CPU raster)
 *   diffren/common/kernels/rasterize_triangles_impl_cuda.cu.cc:143-188,
 *       244-395 (CUDA raster: discretized depth keys, L-smallest layers,
 *       unpack, barycentric recompute)
 * with every float operation written out so that no compiler contraction or
 * platform conversion rule changes a bit (build with -ffp-contract=off).
 * The reference's CUDA build is compiled by nvcc with its default
 * contraction, which fuses three multiply-adds of that path: the pixel
 * centre (2/n)(i + 0.5) - 1, the depth interpolation b0 z0 + b1 z1 + b2 z2
 * (and w) as fma(b2, z2, fma(b0, z0, b1 z1)), and the near-plane point
 * p0 + s (p1 - p0). The discretized semantics restate those as explicit
 * fmaf() calls; outputs of the compiled reference CUDA rasterizer agree bit
 * for bit with this form and not with the separately rounded one.
 *
 * Two depth semantics, selected by `depth_mode`:
 *   0 (DISCRETIZED): the reference CUDA rasterizer. Per fragment the key is
 *     (uint32 discretized depth << 32) | triangle id; each pixel keeps the L
 *     smallest keys. Empty layers: id 0, z 1, barycentrics 0.
 *   1 (FLOAT): the reference CPU rasterizer. Fragments are ordered by float
 *     depth with ties to the lower triangle id (the CPU loop visits triangles
 *     in id order and inserts on strict '<'). Empty layers: id -1, z 1,
 *     barycentrics 0.
 *
 * Float-to-integer conversions saturate out-of-range values and map NaN as
 * the GPU's cvt.rzi does (float to int32: 0; float to int64: INT64_MIN;
 * double to uint32, the depth conversion: 0x80000000), so that this file
 * gives the same bits on
 * x86-64 and aarch64 and matches the CUDA rasterizer.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t fx_t;

enum { kFractionalBits = 16 };
enum { kCullNone = 0, kCullBack = 1, kCullFront = 2 };
enum { kDepthDiscretized = 0, kDepthFloat = 1 };

static int f2i_sat(float f) {
  if (f != f) return 0;
  if (f >= 2147483648.0f) return INT32_MAX;
  if (f < -2147483648.0f) return INT32_MIN;
  return (int)f;
}

static fx_t f2l_sat(float f) {
  if (f != f) return INT64_MIN;
  if (f >= 9223372036854775808.0f) return INT64_MAX;
  if (f < -9223372036854775808.0f) return INT64_MIN;
  return (fx_t)f;
}

static uint32_t d2u_sat(double d) {
  if (d != d) return 0x80000000u;
  if (d >= 4294967296.0) return UINT32_MAX;
  if (d <= 0.0) return 0;
  return (uint32_t)d;
}

/* Wrapping int64 arithmetic (the reference relies on two's complement). */
static fx_t wmul(fx_t a, fx_t b) { return (fx_t)((uint64_t)a * (uint64_t)b); }
static fx_t wadd(fx_t a, fx_t b) { return (fx_t)((uint64_t)a + (uint64_t)b); }
static fx_t wsub(fx_t a, fx_t b) { return (fx_t)((uint64_t)a - (uint64_t)b); }
static fx_t wshl16(fx_t a) { return (fx_t)((uint64_t)a << kFractionalBits); }

/* rasterize_utils.h:57-59 */
static fx_t to_fixed(float f) { return f2l_sat(f * 65536.0f); }

/* rasterize_utils.h:63-84 */
static void add_point(float x, float y, float w, int W, int H, int* l, int* r,
                      int* b, int* t) {
  const float px = (0.5f * (x / w + 1.0f)) * (float)W;
  const float py = (0.5f * (y / w + 1.0f)) * (float)H;
  int v;
  v = f2i_sat(floorf(fminf((float)*l, px)));
  *l = v < 0 ? 0 : (v > W ? W : v);
  v = f2i_sat(ceilf(fmaxf((float)*r, px)));
  *r = v < 0 ? 0 : (v > W ? W : v);
  v = f2i_sat(floorf(fminf((float)*b, py)));
  *b = v < 0 ? 0 : (v > H ? H : v);
  v = f2i_sat(ceilf(fmaxf((float)*t, py)));
  *t = v < 0 ? 0 : (v > H ? H : v);
}

/* rasterize_utils.h:86-99: intersect edge (p0,p1) with the near plane;
 * `fused`: the CUDA build's p0 + s (p1 - p0) as one fma. */
static void add_near_point(const float* p0, const float* p1, int W, int H,
                           int* l, int* r, int* b, int* t, int fused) {
  const float denom = ((p0[2] - p1[2]) + p0[3]) - p1[3];
  if (denom != 0.0f) {
    const float s = (p0[2] + p0[3]) / denom;
    const float dx = p1[0] - p0[0], dy = p1[1] - p0[1], dw = p1[3] - p0[3];
    const float x = fused ? fmaf(s, dx, p0[0]) : p0[0] + s * dx;
    const float y = fused ? fmaf(s, dy, p0[1]) : p0[1] + s * dy;
    const float w = fused ? fmaf(s, dw, p0[3]) : p0[3] + s * dw;
    add_point(x, y, w, W, H, l, r, b, t);
  }
}

static int clip_visible(const float* p) { return p[3] > 0.0f && p[2] >= -p[3]; }

/* rasterize_utils.h:111-161 */
static int bounding_box(const float* v[3], int W, int H, int box[4], int fused) {
  int l = W, r = 0, b = H, t = 0;
  for (int i = 0; i < 3; ++i) {
    if (!clip_visible(v[i])) continue;
    add_point(v[i][0], v[i][1], v[i][3], W, H, &l, &r, &b, &t);
    const int n1 = (i + 1) % 3, n2 = (i + 2) % 3;
    if (!clip_visible(v[n1])) add_near_point(v[i], v[n1], W, H, &l, &r, &b, &t, fused);
    if (!clip_visible(v[n2])) add_near_point(v[i], v[n2], W, H, &l, &r, &b, &t, fused);
  }
  box[0] = l;
  box[1] = r;
  box[2] = b;
  box[3] = t;
  return (r > l) && (t > b);
}

/* rasterize_utils.h:176-206. Rows of m are the edge-function coefficients.
 * For NONE/FRONT the reference multiplies each int64 entry by a float sign,
 * which rounds it to float precision: that rounding is reproduced. */
static void edge_matrix(const float* v[3], int culling, fx_t m[9]) {
  const fx_t x0 = to_fixed(v[0][0]), x1 = to_fixed(v[1][0]), x2 = to_fixed(v[2][0]);
  const fx_t y0 = to_fixed(v[0][1]), y1 = to_fixed(v[1][1]), y2 = to_fixed(v[2][1]);
  const fx_t w0 = to_fixed(v[0][3]), w1 = to_fixed(v[1][3]), w2 = to_fixed(v[2][3]);
  /* Matrix rows are (x0 x1 x2; y0 y1 y2; w0 w1 w2). */
  m[0] = wsub(wmul(y1, w2), wmul(w1, y2));
  m[1] = wsub(wmul(x2, w1), wmul(w2, x1));
  m[2] = wsub(wmul(x1, y2), wmul(y1, x2));
  m[3] = wsub(wmul(y2, w0), wmul(w2, y0));
  m[4] = wsub(wmul(x0, w2), wmul(w0, x2));
  m[5] = wsub(wmul(x2, y0), wmul(y2, x0));
  m[6] = wsub(wmul(y0, w1), wmul(w0, y1));
  m[7] = wsub(wmul(x1, w0), wmul(w1, x0));
  m[8] = wsub(wmul(x0, y1), wmul(y0, x1));
  if (culling == kCullNone || culling == kCullFront) {
    const fx_t det_i = wadd(wadd(wmul(x0, m[0]), wmul(x1, m[3])), wmul(x2, m[6]));
    const float det = (float)det_i;
    const float sign = (culling == kCullNone) ? copysignf(1.0f, det) : -1.0f;
    for (int i = 0; i < 9; ++i) m[i] = f2l_sat((float)m[i] * sign);
  }
}

/* rasterize_utils.h:225-228: fixed-point NDC coordinate of pixel center;
 * `fused`: the CUDA build's single fma. */
static fx_t pixel_center_fixed(int i, int n, int fused) {
  const float scale = 2.0f / (float)n;
  const float c = (float)i + 0.5f;
  const float p = fused ? fmaf(scale, c, -1.0f) : scale * c - 1.0f;
  return to_fixed(p);
}

/* b0 a0 + b1 a1 + b2 a2: rasterize_triangles_impl.cc:87-88 (rounded), or
 * rasterize_triangles_impl_cuda.cu.cc:300-301 as the CUDA build fuses it. */
static float dot3(const float b[3], float a0, float a1, float a2, int fused) {
  if (fused) return fmaf(b[2], a2, fmaf(b[0], a0, b[1] * a1));
  return (b[0] * a0 + b[1] * a1) + b[2] * a2;
}

typedef struct {
  float b[3];
  float z;
  int inside;
} fragment_t;

/* rasterize_utils.h:220-248 and rasterize_triangles_impl.cc:79-89 */
static void shade_fragment(const fx_t m[9], fx_t px, fx_t py, const float* v[3],
                           int fused, fragment_t* f) {
  fx_t e[3];
  for (int i = 0; i < 3; ++i)
    e[i] = wadd(wadd(wmul(m[3 * i], px), wmul(m[3 * i + 1], py)), wshl16(m[3 * i + 2]));
  f->inside = (e[0] >= 0 && e[1] >= 0 && e[2] >= 0) && (e[0] > 0 || e[1] > 0 || e[2] > 0);
  if (!f->inside) return;
  const float sum = (float)wadd(wadd(e[0], e[1]), e[2]);
  for (int i = 0; i < 3; ++i) f->b[i] = (float)e[i] / sum;
  const float cz = dot3(f->b, v[0][2], v[1][2], v[2][2], fused);
  const float cw = dot3(f->b, v[0][3], v[1][3], v[2][3], fused);
  f->z = cz / cw;
}

/* rasterize_triangles_impl_cuda.cu.cc:143-148 */
static uint32_t discretize_z(float z) { return d2u_sat(((double)z + 1.0) * 2147483647.0); }
/* rasterize_triangles_impl_cuda.cu.cc:154-159 */
static float undiscretize_z(uint32_t d) { return (float)((double)d / 2147483647.0 - 1.0); }

/* Order-preserving map of float depth to uint32, with -0 == +0. */
static uint32_t float_order_bits(float z) {
  uint32_t u;
  if (z == 0.0f) z = 0.0f;
  memcpy(&u, &z, 4);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

static const float* vertex_ptr(const float* verts, const int32_t* tris, int64_t t, int i) {
  return verts + 4 * (int64_t)tris[3 * t + i];
}

/*
 * Rasterizes T triangles into L layers of a W x H image. Outputs are
 * [L, H, W] ids, [L, H, W] depth and [L, H, W, 3] barycentrics; every output
 * element is written. Returns 0, or -1 on invalid sizes / allocation failure.
 */
int oracle_rasterize(const float* verts, const int32_t* tris, int32_t T,
                     int32_t W, int32_t H, int32_t L, int32_t culling,
                     int32_t depth_mode, int32_t* ids, float* zbuf, float* bary) {
  if (W <= 0 || H <= 0 || L <= 0 || T < 0) return -1;
  const int64_t npix = (int64_t)W * H;
  uint64_t* keys = (uint64_t*)malloc(sizeof(uint64_t) * npix * L);
  if (!keys) return -1;
  const int fused = depth_mode == kDepthDiscretized;
  const uint64_t empty = (depth_mode == kDepthDiscretized)
                             ? ((uint64_t)discretize_z(1.0f) << 32)
                             : ((uint64_t)float_order_bits(1.0f) << 32);
  for (int64_t i = 0; i < npix * L; ++i) keys[i] = empty;

  for (int32_t t = 0; t < T; ++t) {
    const float* v[3] = {vertex_ptr(verts, tris, t, 0), vertex_ptr(verts, tris, t, 1),
                         vertex_ptr(verts, tris, t, 2)};
    int box[4];
    if (!bounding_box(v, W, H, box, fused)) continue;
    fx_t m[9];
    edge_matrix(v, culling, m);
    for (int iy = box[2]; iy < box[3]; ++iy) {
      const fx_t py = pixel_center_fixed(iy, H, fused);
      for (int ix = box[0]; ix < box[1]; ++ix) {
        fragment_t f;
        shade_fragment(m, pixel_center_fixed(ix, W, fused), py, v, fused, &f);
        if (!f.inside) continue;
        if (f.z < -1.0f || f.z > 1.0f) continue;
        uint64_t key;
        if (depth_mode == kDepthDiscretized) {
          key = ((uint64_t)discretize_z(f.z) << 32) | (uint32_t)t;
        } else {
          if (!(f.z < 1.0f)) continue; /* NaN and z == 1 never enter */
          key = ((uint64_t)float_order_bits(f.z) << 32) | (uint32_t)t;
        }
        /* Keep the L smallest keys, ascending. */
        uint64_t* k = keys + (int64_t)iy * W + ix;
        for (int l = 0; l < L && key < empty; ++l) {
          uint64_t* slot = k + npix * l;
          if (key < *slot) {
            const uint64_t tmp = *slot;
            *slot = key;
            key = tmp;
          }
        }
      }
    }
  }

  for (int32_t l = 0; l < L; ++l) {
    for (int32_t iy = 0; iy < H; ++iy) {
      for (int32_t ix = 0; ix < W; ++ix) {
        const int64_t p = npix * l + (int64_t)iy * W + ix;
        const uint64_t key = keys[p];
        float* b = bary + 3 * p;
        b[0] = b[1] = b[2] = 0.0f;
        if (key == empty) {
          ids[p] = (depth_mode == kDepthDiscretized) ? 0 : -1;
          zbuf[p] = 1.0f;
          continue;
        }
        const int32_t t = (int32_t)(uint32_t)(key & 0xffffffffu);
        ids[p] = t;
        const float* v[3] = {vertex_ptr(verts, tris, t, 0), vertex_ptr(verts, tris, t, 1),
                             vertex_ptr(verts, tris, t, 2)};
        fx_t m[9];
        edge_matrix(v, culling, m);
        fragment_t f;
        shade_fragment(m, pixel_center_fixed(ix, W, fused), pixel_center_fixed(iy, H, fused), v,
                       fused, &f);
        if (depth_mode == kDepthDiscretized) {
          /* Unpack (cu.cc:178-183), then barycentrics only where z != 1
           * (cu.cc:381-394); the recompute skips the inside test. */
          const float z = undiscretize_z((uint32_t)(key >> 32));
          zbuf[p] = z;
          if (z == 1.0f) continue;
        } else {
          zbuf[p] = f.z;
        }
        b[0] = f.b[0];
        b[1] = f.b[1];
        b[2] = f.b[2];
      }
    }
  }
  free(keys);
  return 0;
}

/* Clip-space transform with a fixed left-to-right float order:
 * out[r] = ((M[r][0]*x + M[r][1]*y) + M[r][2]*z) + M[r][3]*w. Vertices with
 * dim 3 get w = 1 (diffren/jax/utils/transforms.py:41-79). */
void oracle_transform(const float* M, const float* v, int64_t n, int32_t dim, float* out) {
  for (int64_t i = 0; i < n; ++i) {
    const float x = v[dim * i], y = v[dim * i + 1], z = v[dim * i + 2];
    const float w = dim == 4 ? v[dim * i + 3] : 1.0f;
    for (int r = 0; r < 4; ++r) {
      const float a = M[4 * r] * x;
      const float b = M[4 * r + 1] * y;
      const float c = M[4 * r + 2] * z;
      const float d = M[4 * r + 3] * w;
      out[4 * i + r] = ((a + b) + c) + d;
    }
  }
}
