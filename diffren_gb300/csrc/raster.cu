// Multi-layer z-buffer rasterizer for GB300: triangle setup, screen-tile
// binning and a persistent shared-memory fine rasterizer over an
// (image, tile) work queue. One launch sequence covers a whole ragged batch.
//
// Results are bit-identical to diffren's rasterizers
// (diffren/common/kernels/rasterize_triangles_impl_cuda.cu.cc:244-395 for
// DR_DEPTH_DISCRETIZED, rasterize_triangles_impl.cc:27-118 for
// DR_DEPTH_FLOAT): the per-fragment arithmetic is the reference's, and each
// pixel keeps the L smallest packed (depth | triangle id) keys, which is
// independent of the order fragments arrive in.
#include <algorithm>
#include <cstddef>
#include <cstring>
#include <string>

#include "common.cuh"
#include "internal.h"

static_assert(dr::kErrorFlagsOffset == 4, "error word is counters[1]");

namespace dr {
namespace {

// Fine-raster block = triangle chunk size. 128-thread blocks keep eight
// tiles in flight per SM (each tile's setup, scan and epilogue are serial
// latency chains), which measured faster than four 256-thread tiles and
// than sixteen 64-thread ones.
constexpr int kThreads = 128;
constexpr int kDefaultTile = 16;
constexpr int kDefaultLargeTiles = 16;

struct __align__(16) TriSetup {
  long long m[9];  // edge-function coefficients (unnormalized inverse)
  float vz[3];     // clip z of the three vertices
  float vw[3];     // clip w of the three vertices
  // The rest serves the fused epilogue only (the fine loop stages the first
  // 96 bytes): vertex indices and clip x, y, so that a sample's
  // interpolation reads one record instead of gathering its triangle and
  // vertices.
  int32_t vid[3];
  float vx[3];
  float vy[3];
  int32_t pad[3];
};
static_assert(sizeof(TriSetup) == 144, "TriSetup layout");
static_assert(offsetof(TriSetup, vz) == 72 && offsetof(TriSetup, vw) == 84 &&
                  offsetof(TriSetup, vid) == 96 && offsetof(TriSetup, vx) == 108 &&
                  offsetof(TriSetup, vy) == 120,
              "write_sample reads the record by these offsets");

struct RasterArgs {
  const float4* verts;
  const int32_t* tris;
  int culling, depth_mode, L, TW, TH, large_tiles;
  bool fg_only;  // DR_RASTER_FOREGROUND_ONLY: background ids / barycentrics unwritten
  bool fg_attr;  // DR_RASTER_FOREGROUND_ATTRIBUTES: background attributes unwritten
  int64_t total_tris;
  int32_t total_tiles;
  TriSetup* setup;
  int4* bbox;  // {left, right, bottom, top}; empty when culled
  int32_t* tile_count;  // triangles inside one tile (their slots come from here)
  int32_t* tile_multi;  // triangles spanning 2..large_tiles tiles
  int32_t* tile_fill;   // bin slots taken by the multi-tile triangles; after
                        // binning, the tiles in the fine rasterizer's order
  int32_t* tile_first;  // exclusive scan of tile_count + tile_multi, total_tiles + 1
  int32_t* bins;        // global triangle indices grouped by tile
  int32_t* large_count;  // per image
  int32_t* large_list;   // per image, at tri_start[image]
  uint32_t* counters;    // [0] work queue head, [1] error flags, [2, 8) tiles
                         // per cost class, [8, 14) their fill counts
  int32_t* ids;
  float* z;
  float* bary;
  SampleOutputs so;
};

// Workspace: the zeroed block first, then the rest; 256-byte aligned parts.
struct Layout {
  size_t counters, tile_count, tile_multi, tile_fill, large_count, zero_end;
  size_t tile_first, setup, bbox, bins, large_list, total;
};

size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

Layout make_layout(int64_t tris, int64_t tiles, int images, int large_tiles) {
  Layout l;
  size_t o = 0;
  l.counters = o; o = align_up(o + 64);  // queue head, error flags, tile order counts
  l.tile_count = o; o = align_up(o + 4 * tiles);
  l.tile_multi = o; o = align_up(o + 4 * tiles);
  l.tile_fill = o; o = align_up(o + 4 * tiles);
  l.large_count = o; o = align_up(o + 4 * size_t(images));
  l.zero_end = o;
  l.tile_first = o; o = align_up(o + 4 * (tiles + 1));
  l.setup = o; o = align_up(o + sizeof(TriSetup) * tris);
  l.bbox = o; o = align_up(o + 16 * tris);
  l.bins = o; o = align_up(o + 4 * size_t(large_tiles) * tris);
  l.large_list = o; o = align_up(o + 4 * tris);
  l.total = o;
  return l;
}

// True when no pixel center of `box` can pass the inside test: the sum of
// the three edge functions is linear in the fixed-point pixel coordinates
// (which are monotone in the pixel index), so it is <= 0 over the whole box
// iff it is <= 0 at the four corners. Only used when no int64 term can
// overflow (|m| < 2^43), so the test is exact.
__device__ bool cannot_cover(const long long m[9], int4 box, int W, int H, bool fused) {
  const long long lim = 1LL << 43;
#pragma unroll
  for (int i = 0; i < 9; ++i)
    if (m[i] >= lim || m[i] <= -lim) return false;
  const long long A = m[0] + m[3] + m[6];
  const long long B = m[1] + m[4] + m[7];
  const long long C = (m[2] + m[5] + m[8]) * 65536;
  const long long x0 = pixel_center_fixed(box.x, W, fused);
  const long long x1 = pixel_center_fixed(box.y - 1, W, fused);
  const long long y0 = pixel_center_fixed(box.z, H, fused);
  const long long y1 = pixel_center_fixed(box.w - 1, H, fused);
  const long long s00 = A * x0 + B * y0 + C, s10 = A * x1 + B * y0 + C;
  const long long s01 = A * x0 + B * y1 + C, s11 = A * x1 + B * y1 + C;
  return s00 <= 0 && s10 <= 0 && s01 <= 0 && s11 <= 0;
}

__device__ __forceinline__ void tile_rect(int4 box, int TW, int TH, int& tx0,
                                          int& tx1, int& ty0, int& ty1) {
  tx0 = box.x / TW;
  tx1 = (box.y - 1) / TW;
  ty0 = box.z / TH;
  ty1 = (box.w - 1) / TH;
}

// One thread per triangle of the batch: bounding box, edge matrix, exact
// coverage cull, per-tile counts (small triangles) or the large list.
// Bounded to 64 registers so that four blocks share an SM: the kernel waits
// on its index and vertex loads, and the extra warps hide more of that than
// the few bytes of spills cost (measured against three blocks and five).
__global__ void __launch_bounds__(256, 4) setup_kernel(RasterArgs a, Batch B) {
  const int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int lane = threadIdx.x & 31;
  // Lanes past the end still take part in the warp-wide tile match below.
  const bool live = g < a.total_tris;
  const int img = live ? find_segment(B.tri_start, B.n, g) : 0;
  const int64_t t = g - B.tri_start[img];
  const int W = B.width[img], H = B.height[img];
  const int32_t* tri = a.tris + 3 * (B.triangle_offset[img] + t);
  const int i0 = live ? tri[0] : 0, i1 = live ? tri[1] : 0, i2 = live ? tri[2] : 0;
  const unsigned nv = unsigned(B.num_vertices[img]);
  int4 box = make_int4(0, 0, 0, 0);
  bool valid = false;
  if (!live) {
  } else if (unsigned(i0) >= nv || unsigned(i1) >= nv || unsigned(i2) >= nv) {
    atomicOr(&a.counters[1], DR_FLAG_INDEX_OUT_OF_RANGE);
  } else {
    const float4* vb = a.verts + B.vertex_offset[img];
    const float4 v0 = vb[i0], v1 = vb[i1], v2 = vb[i2];
    // x - x == 0 exactly for finite x, NaN for NaN and infinities.
    const float probe = (v0.x - v0.x) + (v0.y - v0.y) + (v0.z - v0.z) + (v0.w - v0.w) +
                        (v1.x - v1.x) + (v1.y - v1.y) + (v1.z - v1.z) + (v1.w - v1.w) +
                        (v2.x - v2.x) + (v2.y - v2.y) + (v2.z - v2.z) + (v2.w - v2.w);
    if (probe != 0.0f) atomicOr(&a.counters[1], DR_FLAG_NONFINITE_VERTEX);
    const bool disc = a.depth_mode == DR_DEPTH_DISCRETIZED;
    valid = triangle_box(v0, v1, v2, W, H, box, disc);
    if (valid) {
      TriSetup s;
      edge_matrix(v0, v1, v2, a.culling, s.m);
      valid = !cannot_cover(s.m, box, W, H, disc);
      if (valid) {
        s.vz[0] = v0.z; s.vz[1] = v1.z; s.vz[2] = v2.z;
        s.vw[0] = v0.w; s.vw[1] = v1.w; s.vw[2] = v2.w;
        s.vid[0] = i0; s.vid[1] = i1; s.vid[2] = i2;
        s.vx[0] = v0.x; s.vx[1] = v1.x; s.vx[2] = v2.x;
        s.vy[0] = v0.y; s.vy[1] = v1.y; s.vy[2] = v2.y;
        s.pad[0] = s.pad[1] = s.pad[2] = 0;
        const int4* src = reinterpret_cast<const int4*>(&s);
        int4* dst = reinterpret_cast<int4*>(a.setup + g);
#pragma unroll
        for (int k = 0; k < 9; ++k) dst[k] = src[k];
      }
    }
  }
  if (!valid) box = make_int4(0, 0, 0, 0);
  if (live) a.bbox[g] = box;
  int tx0 = 0, tx1 = -1, ty0 = 0, ty1 = -1;
  if (valid) tile_rect(box, a.TW, a.TH, tx0, tx1, ty0, ty1);
  const int n = (tx1 - tx0 + 1) * (ty1 - ty0 + 1);
  const int base = B.tile_start[img], tx = B.tiles_x[img];
  // Triangles inside one tile count with one atomic per tile per warp.
  const bool single = valid && n == 1 && n <= a.large_tiles;
  const int tile0 = base + ty0 * tx + tx0;
  const unsigned group = __match_any_sync(0xffffffffu, single ? tile0 : -1 - lane);
  if (single) {
    // The warp's triangles in this tile take consecutive slots; the slot is
    // kept in the setup record, so the binning pass needs no atomic.
    const int leader = __ffs(group) - 1;
    int first = 0;
    if (lane == leader) first = atomicAdd(&a.tile_count[tile0], __popc(group));
    first = __shfl_sync(group, first, leader);
    a.setup[g].pad[0] = first + __popc(group & ((1u << lane) - 1u));
    return;
  }
  if (!valid) return;
  if (n <= a.large_tiles) {
    for (int y = ty0; y <= ty1; ++y)
      for (int x = tx0; x <= tx1; ++x) atomicAdd(&a.tile_multi[base + y * tx + x], 1);
  } else {
    const int slot = atomicAdd(&a.large_count[img], 1);
    a.large_list[B.tri_start[img] + slot] = int(g);
  }
}

// Exclusive scan of the per-tile counts (one block; tiles are few). A pass
// covers 16 Ki counts: warp w owns 512 consecutive counts, read 32 at a time
// with coalesced loads and scanned with warp shuffles, then the 32 warp
// totals are scanned once; the next pass's counts load meanwhile.
__global__ void __launch_bounds__(1024) tile_scan_kernel(const int32_t* count,
                                                         const int32_t* multi,
                                                         int32_t* first, int n) {
  __shared__ int warp_sums[32];
  constexpr int kRounds = 16, kChunk = 1024 * kRounds;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int carry = 0;
  int v[kRounds], next[kRounds];
  const auto load = [&](int base, int (&dst)[kRounds]) {
#pragma unroll
    for (int j = 0; j < kRounds; ++j) {
      const int i = base + warp * (32 * kRounds) + j * 32 + lane;
      dst[j] = i < n ? __ldg(count + i) + __ldg(multi + i) : 0;
    }
  };
  load(0, v);
  for (int base = 0; base < n; base += kChunk) {
    if (base + kChunk < n) load(base + kChunk, next);
    int run = 0;
#pragma unroll
    for (int j = 0; j < kRounds; ++j) {
      const int inc = warp_inclusive_scan(v[j]);
      const int excl = run + inc - v[j];
      run += __shfl_sync(0xffffffffu, inc, 31);
      v[j] = excl;  // exclusive prefix inside the warp's 512 counts
    }
    if (lane == 0) warp_sums[warp] = run;
    __syncthreads();
    if (warp == 0) warp_sums[lane] = warp_inclusive_scan(warp_sums[lane]);
    __syncthreads();
    const int offset = carry + (warp ? warp_sums[warp - 1] : 0);
#pragma unroll
    for (int j = 0; j < kRounds; ++j) {
      const int i = base + warp * (32 * kRounds) + j * 32 + lane;
      if (i < n) first[i] = offset + v[j];
    }
    carry += warp_sums[31];  // the same in every thread
    __syncthreads();          // warp_sums is rewritten by the next pass
#pragma unroll
    for (int j = 0; j < kRounds; ++j) v[j] = next[j];
  }
  if (threadIdx.x == 0) first[n] = carry;
}

// One thread per triangle: writes its index into the bin of every tile its
// box touches. Order inside a bin is irrelevant to the result.
__global__ void __launch_bounds__(256) bin_scatter_kernel(RasterArgs a, Batch B) {
  const int64_t g = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  bool binned = false;
  int tx0 = 0, tx1 = -1, ty0 = 0, ty1 = -1, base = 0, tx = 0;
  if (g < a.total_tris) {
    const int4 box = a.bbox[g];
    if (box.y > box.x) {
      tile_rect(box, a.TW, a.TH, tx0, tx1, ty0, ty1);
      if ((tx1 - tx0 + 1) * (ty1 - ty0 + 1) <= a.large_tiles) {
        binned = true;
        const int img = find_segment(B.tri_start, B.n, g);
        base = B.tile_start[img];
        tx = B.tiles_x[img];
      }
    }
  }
  // Triangles inside one tile (most of them) took their slot in setup;
  // the multi-tile ones take theirs after the tile's single-tile triangles.
  if (!binned) return;
  if (tx0 == tx1 && ty0 == ty1) {
    const int tile0 = base + ty0 * tx + tx0;
    a.bins[a.tile_first[tile0] + a.setup[g].pad[0]] = int(g);
    return;
  }
  for (int y = ty0; y <= ty1; ++y)
    for (int x = tx0; x <= tx1; ++x) {
      const int tile = base + y * tx + x;
      const int pos = a.tile_first[tile] + a.tile_count[tile] + atomicAdd(&a.tile_fill[tile], 1);
      a.bins[pos] = int(g);
    }
}

// Tile order of the fine rasterizer: the most expensive tiles first, so that
// no block is left with a heavy tile while the others have run out of work
// (the per-tile cost spans three orders of magnitude in ragged batches). The
// cost of a tile is its triangle count (binned plus the image's large ones),
// in six classes, heaviest first; inside a class tiles keep roughly their
// index order (block by block), which keeps an image's tiles together in L2.
// The order does not change any output: tiles are independent.
constexpr int kCostClasses = 6;

__device__ __forceinline__ int cost_class(const RasterArgs& a, int tile, int img) {
  const int c = a.tile_first[tile + 1] - a.tile_first[tile] + a.large_count[img];
  return c >= 512 ? 0 : c >= 128 ? 1 : c >= 32 ? 2 : c >= 8 ? 3 : c >= 2 ? 4 : 5;
}

// Tiles per cost class (counters[2 + class]), one shared-memory histogram
// per block.
__global__ void __launch_bounds__(256) tile_cost_kernel(RasterArgs a, Batch B) {
  __shared__ int h[kCostClasses];
  if (threadIdx.x < kCostClasses) h[threadIdx.x] = 0;
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < a.total_tiles) atomicAdd(&h[cost_class(a, i, find_segment(B.tile_start, B.n, i))], 1);
  __syncthreads();
  if (threadIdx.x < kCostClasses && h[threadIdx.x])
    atomicAdd(&a.counters[2 + threadIdx.x], unsigned(h[threadIdx.x]));
}

// Writes every tile index to its place in the order (tile_fill, free once
// the bins are filled): class c starts after the tiles of classes < c, and
// each block takes a run of its classes' slots (counters[8 + class]).
__global__ void __launch_bounds__(256) tile_order_kernel(RasterArgs a, Batch B) {
  __shared__ int h[kCostClasses], base[kCostClasses];
  if (threadIdx.x < kCostClasses) h[threadIdx.x] = 0;
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int c = 0, rank = 0;
  if (i < a.total_tiles) {
    c = cost_class(a, i, find_segment(B.tile_start, B.n, i));
    rank = atomicAdd(&h[c], 1);
  }
  __syncthreads();
  if (threadIdx.x < kCostClasses) {
    int start = 0;
    for (int k = 0; k < int(threadIdx.x); ++k) start += int(a.counters[2 + k]);
    const int n = h[threadIdx.x];
    base[threadIdx.x] = start + (n ? int(atomicAdd(&a.counters[8 + threadIdx.x], unsigned(n))) : 0);
  }
  __syncthreads();
  if (i < a.total_tiles) a.tile_fill[base[c] + rank] = i;
}

// Per chunk of up to kThreads triangles overlapping the tile, compacted to
// those with at least one candidate pixel (slot = rank among them).
struct FineSmem {
  long long* m;          // [9][kThreads]
  float* vz;             // [3][kThreads]
  float* vw;             // [3][kThreads]
  int* tid;              // [kThreads] local triangle id
  int* geom;             // [kThreads] x0 | y0 << 8 | width << 16 (tile-local)
  int* inv;              // [kThreads] ceil(2^20 / width)
  int* off;              // [kThreads + 1] exclusive candidate offsets
  long long* pxf;        // [TW] fixed-point pixel-center x
  long long* pyf;        // [TH]
  unsigned long long* keys;  // [L][TW*TH]
  unsigned char* first;  // [kThreads / 32 * TW*TH] slot holding candidate 32 g, per g
};

// The chunk's edge coefficients; the epilogue reuses the space for its list
// of occupied (layer, pixel) slots (16 bits each).
__host__ __device__ inline size_t chunk_m_bytes(int L, int TW, int TH) {
  const size_t m = size_t(9) * kThreads * 8, list = size_t(L) * TW * TH * 2;
  return ((m > list ? m : list) + 7) & ~size_t(7);
}

__host__ __device__ inline size_t fine_smem_bytes(int L, int TW, int TH) {
  return chunk_m_bytes(L, TW, TH) + size_t(TW + TH) * 8 +
         size_t(L) * TW * TH * 8 + size_t(6) * kThreads * 4 +
         size_t(4) * kThreads * 4 + 16 + size_t(kThreads / 32) * TW * TH + 64;
}

// Persistent fine rasterizer. Each block takes (image, tile) items from a
// global queue (heaviest tiles first, in tile_order_kernel's order), keeps
// the tile's L x TW x TH packed keys in shared memory, and spreads the
// (triangle, pixel) candidates of each chunk of the tile's triangles evenly
// over its threads (block prefix scan + binary search), so large and small
// triangles cost the same per pixel.
// Fused interpolation of one layer sample o with triangle `id` and the
// barycentrics just written: the splat position of a foreground sample
// (splat.py:207-221) with its clip w, its three vertex indices when
// requested (the Framebuffer's vertex_ids, rasterize.py:111-113), and the
// attributes (interpolate.py:24-63, background 0). The same operations, in
// the same order, as samples_fwd_kernel on the stored buffers.
__device__ __forceinline__ void write_sample(const RasterArgs& a, const Batch& B, int img,
                                          const TriSetup* t, float zz, const float b[3],
                                          int64_t o) {
  const SampleOutputs& so = a.so;
  const int K = so.K;
  const bool vec_rows = (K & 3) == 0;
  float4 c;
  float* ao = so.attr ? so.attr_out + o * K : nullptr;
  const bool fg = zz != 1.0f;
  if (fg) {
    // One record holds the vertex indices and clip coordinates (the sample
    // is foreground, so its key and record exist).
    const float2 z01 = __ldg(reinterpret_cast<const float2*>(t->vz));
    const int4 r5 = __ldg(reinterpret_cast<const int4*>(t) + 5);  // vz2, vw0..2
    const int4 r6 = __ldg(reinterpret_cast<const int4*>(t) + 6);  // vid0..2, vx0
    const int4 r7 = __ldg(reinterpret_cast<const int4*>(t) + 7);  // vx1, vx2, vy0, vy1
    const int4 r8 = __ldg(reinterpret_cast<const int4*>(t) + 8);  // vy2
    const int v0 = r6.x, v1 = r6.y, v2 = r6.z;
    c = lerp_clip(make_float4(__int_as_float(r6.w), __int_as_float(r7.z), z01.x,
                              __int_as_float(r5.y)),
                  make_float4(__int_as_float(r7.x), __int_as_float(r7.w), z01.y,
                              __int_as_float(r5.z)),
                  make_float4(__int_as_float(r7.y), __int_as_float(r8.x),
                              __int_as_float(r5.x), __int_as_float(r5.w)), b);
    if (ao) {
      const float* ab = so.attr + B.vertex_offset[img] * K;
      const float* a0 = ab + int64_t(v0) * K;
      const float* a1 = ab + int64_t(v1) * K;
      const float* a2 = ab + int64_t(v2) * K;
      for (int k = 0; k < K; k += 4) {
        const int n = min(4, K - k);
        const float4 x = load_chunk(a0 + k, n, vec_rows), y = load_chunk(a1 + k, n, vec_rows),
                     w = load_chunk(a2 + k, n, vec_rows);
        store_chunk(ao + k,
                    make_float4(lerp3(x.x, y.x, w.x, b), lerp3(x.y, y.y, w.y, b),
                                lerp3(x.z, y.z, w.z, b), lerp3(x.w, y.w, w.w, b)),
                    n, vec_rows);
      }
    }
    // w carries the interpolated clip w, which the VJP needs (background
    // and foreground are told apart by the depth buffer).
    so.positions[o] = viewport_of(c, __int2float_rn(B.width[img]),
                                  __int2float_rn(B.height[img]), c.w);
    if (so.vertex_ids) {
      int32_t* vo = so.vertex_ids + 3 * o;
      vo[0] = v0;
      vo[1] = v1;
      vo[2] = v2;
    }
  } else if (ao && !a.fg_attr) {
    // Background: attributes 0; the position is left unwritten (consumers
    // take background samples from the depth buffer).
    for (int k = 0; k < K; k += 4)
      store_chunk(ao + k, make_float4(0.0f, 0.0f, 0.0f, 0.0f), min(4, K - k), vec_rows);
  }
}

// kFused adds the sample outputs to the epilogue. LT > 0 fixes the layer
// count at compile time (the common L = 3), LT = 0 reads it.
template <bool kFused, int LT>
__global__ void __launch_bounds__(kThreads, 8) fine_raster_kernel(RasterArgs a,
                                                                             Batch B) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int s_warp[kThreads / 32];
  __shared__ int s_item;
  __shared__ int s_nfg;
  const int TW = a.TW, TH = a.TH, TP = TW * TH, L = LT > 0 ? LT : a.L;
  FineSmem s;
  {
    unsigned char* p = smem_raw;
    s.keys = reinterpret_cast<unsigned long long*>(p); p += size_t(L) * TP * 8;
    s.m = reinterpret_cast<long long*>(p); p += chunk_m_bytes(L, TW, TH);
    s.pxf = reinterpret_cast<long long*>(p); p += size_t(TW) * 8;
    s.pyf = reinterpret_cast<long long*>(p); p += size_t(TH) * 8;
    s.vz = reinterpret_cast<float*>(p); p += size_t(3) * kThreads * 4;
    s.vw = reinterpret_cast<float*>(p); p += size_t(3) * kThreads * 4;
    s.tid = reinterpret_cast<int*>(p); p += kThreads * 4;
    s.geom = reinterpret_cast<int*>(p); p += kThreads * 4;
    s.inv = reinterpret_cast<int*>(p); p += kThreads * 4;
    s.off = reinterpret_cast<int*>(p); p += (kThreads + 4) * 4;
    s.first = p;
  }
  const unsigned long long kEmpty = empty_key(a.depth_mode);
  const bool disc = a.depth_mode == DR_DEPTH_DISCRETIZED;

  for (;;) {
    if (threadIdx.x == 0) s_item = int(atomicAdd(&a.counters[0], 1u));
    __syncthreads();
    if (s_item >= a.total_tiles) break;
    const int item = a.tile_fill[s_item];  // heaviest tiles first
    const int img = find_segment(B.tile_start, B.n, item);
    const int local = item - B.tile_start[img];
    const int W = B.width[img], H = B.height[img];
    const int ntx = B.tiles_x[img];
    const int x0 = (local % ntx) * TW, y0 = (local / ntx) * TH;
    const int tw = min(TW, W - x0), th = min(TH, H - y0);
    const int64_t tri0 = B.tri_start[img];

    for (int p = threadIdx.x; p < L * TP; p += kThreads) s.keys[p] = kEmpty;
    for (int i = threadIdx.x; i < TW + TH; i += kThreads) {
      if (i < TW) s.pxf[i] = pixel_center_fixed(x0 + i, W, disc);
      else s.pyf[i - TW] = pixel_center_fixed(y0 + i - TW, H, disc);
    }
    const int bin0 = a.tile_first[item];
    const int nbin = a.tile_first[item + 1] - bin0;
    const int nlarge = a.large_count[img];
    const int nsrc = nbin + nlarge;
    __syncthreads();

    for (int c0 = 0; c0 < nsrc; c0 += kThreads) {
      const int i = c0 + threadIdx.x;
      int cnt = 0, g = 0, cx0 = 0, cy0 = 0, cw = 1;
      if (i < nsrc) {
        g = i < nbin ? a.bins[bin0 + i] : a.large_list[tri0 + (i - nbin)];
        const int4 box = a.bbox[g];
        cx0 = max(box.x, x0) - x0;
        cy0 = max(box.z, y0) - y0;
        const int cx1 = min(box.y, x0 + tw) - x0, cy1 = min(box.w, y0 + th) - y0;
        if (cx1 > cx0 && cy1 > cy0) {
          cw = cx1 - cx0;
          cnt = cw * (cy1 - cy0);
        }
      }
      // One scan gives each triangle with candidates its compacted slot
      // (bits 20+) and its first candidate (bits 0-19): at most
      // kThreads * 1024 candidates per chunk.
      int excl;
      const int tot = block_exclusive_scan<kThreads>(cnt | (cnt > 0 ? 1 << 20 : 0), s_warp, excl);
      const int total = tot & 0xfffff, ntri = tot >> 20;
      if (cnt > 0) {
        const int slot = excl >> 20, off = excl & 0xfffff;
        int4 r[6];
        const int4* src = reinterpret_cast<const int4*>(a.setup + g);
#pragma unroll
        for (int k = 0; k < 6; ++k) r[k] = __ldg(src + k);
        const long long* mm = reinterpret_cast<const long long*>(r);
        const float* ff = reinterpret_cast<const float*>(r) + 18;
#pragma unroll
        for (int k = 0; k < 9; ++k) s.m[k * kThreads + slot] = mm[k];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          s.vz[k * kThreads + slot] = ff[k];
          s.vw[k * kThreads + slot] = ff[3 + k];
        }
        s.tid[slot] = int(g - tri0);
        s.geom[slot] = cx0 | (cy0 << 8) | (cw << 16);
        s.inv[slot] = ((1 << 20) + cw - 1) / cw;
        s.off[slot] = off;
        // This triangle holds candidate 32 q for every q with 32 q in
        // [off, off + cnt).
        for (int q = (off + 31) >> 5; (q << 5) < off + cnt; ++q) s.first[q] = (unsigned char)slot;
      }
      if (threadIdx.x == 0) s.off[ntri] = total;
      __syncthreads();

      // Warp-wide groups of 32 consecutive candidates. The group's first
      // candidate lies in triangle j0 = first[q]; the triangles that start
      // inside the group mark their start positions in one 32-bit mask, and
      // lane t's triangle is j0 plus the marks at positions 1..t.
      const int lane = threadIdx.x & 31;
      for (int q = threadIdx.x >> 5; (q << 5) < total; q += kThreads / 32) {
        const int base = q << 5;
        const int j0 = s.first[q];
        const int jn = j0 + 1 + lane;
        const int d = jn <= ntri ? s.off[jn] - base : 32;
        const unsigned starts = __reduce_or_sync(0xffffffffu, d > 0 && d < 32 ? 1u << d : 0u);
        const int k = base + lane;
        if (k >= total) continue;
        const int j = j0 + __popc(starts & ((2u << lane) - 1u));
        const int geom = s.geom[j];
        const int rr = k - s.off[j];
        const int ry = int((unsigned(rr) * unsigned(s.inv[j])) >> 20);  // rr / width
        const int lx = (geom & 255) + (rr - ry * (geom >> 16));
        const int ly = ((geom >> 8) & 255) + ry;
        long long m[9];
#pragma unroll
        for (int t = 0; t < 9; ++t) m[t] = s.m[t * kThreads + j];
        long long e[3];
        edge_values(m, s.pxf[lx], s.pyf[ly], e);
        if (!inside(e)) continue;
        float b[3];
        barycentrics_of(e, b);
        const float3 vz = make_float3(s.vz[j], s.vz[kThreads + j], s.vz[2 * kThreads + j]);
        const float3 vw = make_float3(s.vw[j], s.vw[kThreads + j], s.vw[2 * kThreads + j]);
        const float z = fragment_z(b, vz, vw, disc);
        unsigned long long key;
        if (disc) {
          if (z < -1.0f || z > 1.0f) continue;  // NaN passes, as in the reference
          key = ((unsigned long long)discretize_z(z) << 32) | uint32_t(s.tid[j]);
        } else {
          if (!(z >= -1.0f && z < 1.0f)) continue;
          key = ((unsigned long long)float_order_bits(z) << 32) | uint32_t(s.tid[j]);
        }
        if (key >= kEmpty) continue;
        unsigned long long* kp = s.keys + ly * TW + lx;
        // Slot values only decrease, so a key above the current last layer
        // can never be among the pixel's L smallest.
        if (key > *reinterpret_cast<volatile unsigned long long*>(kp + (L - 1) * TP)) continue;
        for (int l = 0; l < L; ++l) {
          const unsigned long long old = atomicMin(kp + l * TP, key);
          if (old == kEmpty) break;
          key = max(key, old);
        }
      }
      __syncthreads();
    }

    // Epilogue: unpack, recompute barycentrics (and float depth) of the
    // winning triangle at each pixel, write all L layers; optionally also
    // each layer sample's splat position and interpolated attributes.
    const int64_t HW = int64_t(H) * W;
    const int64_t base = int64_t(L) * B.pix_off[img];
    if constexpr (LT > 0) {
      // Pass 1 writes background samples and lists the occupied slots
      // (layer * TP + pixel, in the chunk arrays' space, dead by now); pass
      // 2 runs the occupied slots with full warps.
      unsigned short* list = reinterpret_cast<unsigned short*>(s.m);
      if (threadIdx.x == 0) s_nfg = 0;
      __syncthreads();
      const int lane = threadIdx.x & 31;
      for (int p0 = 0; p0 < TP; p0 += kThreads) {
        const int p = p0 + threadIdx.x;
        const int lx = p % TW, ly = p / TW;
        const bool valid = p < TP && lx < tw && ly < th;
        const int64_t pix = int64_t(y0 + ly) * W + (x0 + lx);
#pragma unroll
        for (int l = 0; l < LT; ++l) {
          const unsigned long long key = valid ? s.keys[l * TP + p] : kEmpty;
          const bool full = valid && key != kEmpty;
          const unsigned ball = __ballot_sync(0xffffffffu, full);
          int slot0 = 0;
          if (lane == 0 && ball) slot0 = atomicAdd(&s_nfg, __popc(ball));
          slot0 = __shfl_sync(0xffffffffu, slot0, 0);
          if (full) {
            list[slot0 + __popc(ball & ((1u << lane) - 1u))] = (unsigned short)(l * TP + p);
          } else if (valid) {
            const int64_t o = base + l * HW + pix;
            const float b0[3] = {0.0f, 0.0f, 0.0f};
            a.z[o] = 1.0f;
            if (!a.fg_only) {
              a.ids[o] = disc ? 0 : -1;
              float* bo = a.bary + 3 * o;
              bo[0] = 0.0f;
              bo[1] = 0.0f;
              bo[2] = 0.0f;
            }
            if (kFused) write_sample(a, B, img, nullptr, 1.0f, b0, o);
          }
        }
      }
      __syncthreads();
      const int nfg = s_nfg;
      for (int f = threadIdx.x; f < nfg; f += kThreads) {
        const int q = list[f];
        const int l = q / TP, p = q - l * TP;
        const int lx = p % TW, ly = p / TW;
        const int64_t pix = int64_t(y0 + ly) * W + (x0 + lx);
        const unsigned long long key = s.keys[q];
        const int64_t o = base + l * HW + pix;
        float b[3] = {0.0f, 0.0f, 0.0f};
        const int id = int(uint32_t(key));
        const TriSetup* st = a.setup + tri0 + id;
        long long m[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) m[k] = __ldg(&st->m[k]);
        long long e[3];
        edge_values(m, s.pxf[lx], s.pyf[ly], e);
        float bb[3];
        barycentrics_of(e, bb);
        float zz;
        if (disc) {
          zz = undiscretize_z(uint32_t(key >> 32));
        } else {
          const float3 vz = make_float3(__ldg(&st->vz[0]), __ldg(&st->vz[1]), __ldg(&st->vz[2]));
          const float3 vw = make_float3(__ldg(&st->vw[0]), __ldg(&st->vw[1]), __ldg(&st->vw[2]));
          zz = fragment_z(bb, vz, vw, false);
        }
        if (!disc || zz != 1.0f) { b[0] = bb[0]; b[1] = bb[1]; b[2] = bb[2]; }
        a.ids[o] = id;
        a.z[o] = zz;
        float* bo = a.bary + 3 * o;
        bo[0] = b[0];
        bo[1] = b[1];
        bo[2] = b[2];
        if (kFused) write_sample(a, B, img, st, zz, b, o);
      }
      __syncthreads();
    } else {
      // Any layer count: one pass, pixel by pixel.
      for (int p = threadIdx.x; p < TP; p += kThreads) {
        const int lx = p % TW, ly = p / TW;
        if (lx >= tw || ly >= th) continue;
        const int64_t pix = int64_t(y0 + ly) * W + (x0 + lx);
        for (int l = 0; l < L; ++l) {
          const unsigned long long key = s.keys[l * TP + p];
          const int64_t o = base + l * HW + pix;
          float b[3] = {0.0f, 0.0f, 0.0f};
          int id;
          float zz;
          const TriSetup* st = nullptr;
          if (key == kEmpty) {
            id = disc ? 0 : -1;
            zz = 1.0f;
          } else {
            id = int(uint32_t(key));
            st = a.setup + tri0 + id;
            long long m[9];
  #pragma unroll
            for (int q = 0; q < 9; ++q) m[q] = __ldg(&st->m[q]);
            long long e[3];
            edge_values(m, s.pxf[lx], s.pyf[ly], e);
            float bb[3];
            barycentrics_of(e, bb);
            if (disc) {
              zz = undiscretize_z(uint32_t(key >> 32));
            } else {
              const float3 vz =
                  make_float3(__ldg(&st->vz[0]), __ldg(&st->vz[1]), __ldg(&st->vz[2]));
              const float3 vw =
                  make_float3(__ldg(&st->vw[0]), __ldg(&st->vw[1]), __ldg(&st->vw[2]));
              zz = fragment_z(bb, vz, vw, false);
            }
            if (!disc || zz != 1.0f) { b[0] = bb[0]; b[1] = bb[1]; b[2] = bb[2]; }
          }
          a.z[o] = zz;
          if (!a.fg_only || key != kEmpty) {
            a.ids[o] = id;
            float* bo = a.bary + 3 * o;
            bo[0] = b[0];
            bo[1] = b[1];
            bo[2] = b[2];
          }
          if (kFused) write_sample(a, B, img, st, zz, b, o);
        }
      }
      __syncthreads();
    }
  }
}

// Compares the integer depth codec with the reference's double formulas on
// every input: all 2^32 discretized values, and every float in [-1, 1]
// plus NaNs. out: [0] discretize mismatches, [1] first bad float bits,
// [2] undiscretize mismatches, [3] first bad discretized value, [4] the
// discretized value of a NaN depth, [5] / [6] the int32 / int64 conversion
// of a NaN float (toward zero).
__global__ void depth_codec_selftest_kernel(unsigned long long* out) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    const float nan = __uint_as_float(0x7fc00000u);
    out[4] = discretize_z_fp64(nan);
    out[5] = (unsigned long long)(unsigned)__float2int_rz(nan);
    out[6] = (unsigned long long)__float2ll_rz(nan);
  }
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < (1ull << 32);
       i += stride) {
    const uint32_t u = uint32_t(i);
    if (__float_as_uint(undiscretize_z(u)) != __float_as_uint(undiscretize_z_fp64(u))) {
      atomicAdd(&out[2], 1ull);
      atomicMin(&out[3], (unsigned long long)u);
    }
    const float z = __uint_as_float(u);
    const bool in_domain = (z != z) || (z >= -1.0f && z <= 1.0f);
    if (in_domain && discretize_z(z) != discretize_z_fp64(z)) {
      atomicAdd(&out[0], 1ull);
      atomicMin(&out[1], (unsigned long long)u);
    }
  }
}

// Raises the fine rasterizer's dynamic shared-memory limit and computes its
// persistent grid (resident blocks per SM x SMs) on the current device.
template <bool kFused, int LT>
bool prepare_fine(size_t smem, int& sms, int& per_sm, std::string& err) {
  static LaunchCache cache;
  return prepare_launch(cache, fine_raster_kernel<kFused, LT>, kThreads, smem, sms, per_sm,
                        "tile and layer count need more shared memory than the device has",
                        err);
}

int resolve_tile(int v) { return v > 0 ? v : kDefaultTile; }

bool check_config(const dr_raster_config* cfg, int& L, int& TW, int& TH, int& large,
                  std::string& err) {
  if (!cfg) { err = "config is null"; return false; }
  L = cfg->num_layers;
  TW = resolve_tile(cfg->tile_width);
  TH = resolve_tile(cfg->tile_height);
  large = cfg->large_tiles > 0 ? cfg->large_tiles : kDefaultLargeTiles;
  if (L < 1 || L > DR_MAX_LAYERS) { err = "num_layers must be in [1, 16]"; return false; }
  if (cfg->face_culling_mode < 0 || cfg->face_culling_mode > 2) {
    err = "face_culling_mode must be 0, 1 or 2";
    return false;
  }
  if (cfg->depth_mode != DR_DEPTH_DISCRETIZED && cfg->depth_mode != DR_DEPTH_FLOAT) {
    err = "depth_mode must be 0 (discretized) or 1 (float)";
    return false;
  }
  if (TW > 128 || TH > 128 || TW * TH > 1024) {
    err = "tile must satisfy width, height <= 128 and width*height <= 1024";
    return false;
  }
  if ((cfg->flags & ~(DR_RASTER_FOREGROUND_ONLY | DR_RASTER_FOREGROUND_ATTRIBUTES)) != 0) {
    err = "unknown raster config flags";
    return false;
  }
  return true;
}

}  // namespace

int depth_codec_selftest(unsigned long long* out, cudaStream_t stream, std::string& err) {
  if (!out) { err = "results buffer is null"; return DR_ERR_INVALID_ARGUMENT; }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  depth_codec_selftest_kernel<<<sms * 8, 256, 0, stream>>>(out);
  return launch_status("depth codec self-test", err);
}

size_t raster_workspace_bytes(const dr_image_desc* images, int n,
                              const dr_raster_config* cfg, std::string& err) {
  int L, TW, TH, large;
  if (!check_config(cfg, L, TW, TH, large, err)) return 0;
  if (n < 0 || (n > 0 && !images)) { err = "invalid image table"; return 0; }
  size_t best = 256;
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    if (!make_batch(images + g0, cnt, L, TW, TH, b, err)) return 0;
    const Layout lay = make_layout(b.tri_start[cnt], b.tile_start[cnt], cnt, large);
    best = std::max(best, lay.total);
  }
  return best;
}

int raster_launch(const float* vertices, const int32_t* triangles,
                  const dr_image_desc* images, int n, const dr_raster_config* cfg,
                  int32_t* ids, float* z, float* bary, void* workspace,
                  size_t ws_bytes, cudaStream_t stream, std::string& err,
                  const SampleOutputs* samples) {
  int L, TW, TH, large;
  if (!check_config(cfg, L, TW, TH, large, err)) return DR_ERR_INVALID_ARGUMENT;
  if (n < 0 || (n > 0 && !images)) { err = "invalid image table"; return DR_ERR_INVALID_ARGUMENT; }
  if (n == 0) return DR_OK;
  if (!ids || !z || !bary || !workspace) {
    err = "outputs and workspace must be non-null";
    return DR_ERR_INVALID_ARGUMENT;
  }
  if ((reinterpret_cast<uintptr_t>(vertices) & 15) != 0 ||
      (reinterpret_cast<uintptr_t>(workspace) & 255) != 0) {
    err = "vertices must be 16-byte aligned and the workspace 256-byte aligned";
    return DR_ERR_MISALIGNED;
  }
  SampleOutputs so{};
  if (samples) {
    so = *samples;
    if (!so.positions || (so.attr && (!so.attr_out || so.K < 1 || so.K > DR_MAX_CHANNELS))) {
      err = "positions must be non-null, and attributes need attributes_out and 1 to 16 "
            "channels";
      return DR_ERR_INVALID_ARGUMENT;
    }
    if (!so.attr) so.K = 0;
    const bool vec = so.attr && so.K % 4 == 0;
    if ((reinterpret_cast<uintptr_t>(so.positions) & 15) != 0 ||
        (vec && ((reinterpret_cast<uintptr_t>(so.attr) & 15) != 0 ||
                 (reinterpret_cast<uintptr_t>(so.attr_out) & 15) != 0))) {
      err = "positions (and, with a multiple of 4 channels, the attribute buffers) must be "
            "16-byte aligned";
      return DR_ERR_MISALIGNED;
    }
  }
  const size_t smem = fine_smem_bytes(L, TW, TH);
  const bool fused = so.positions != nullptr;
  // Instantiations: fused or not, three layers or any.
  using Fine = void (*)(RasterArgs, Batch);
  using Prep = bool (*)(size_t, int&, int&, std::string&);
  const int variant = (fused ? 2 : 0) + (L == 3 ? 1 : 0);
  const Fine fine[4] = {fine_raster_kernel<false, 0>, fine_raster_kernel<false, 3>,
                        fine_raster_kernel<true, 0>, fine_raster_kernel<true, 3>};
  const Prep prep[4] = {prepare_fine<false, 0>, prepare_fine<false, 3>,
                        prepare_fine<true, 0>, prepare_fine<true, 3>};
  int sms = 0, per_sm = 0;
  if (!prep[variant](smem, sms, per_sm, err)) return DR_ERR_INVALID_ARGUMENT;

  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    const int cnt = std::min(n - g0, DR_MAX_BATCH_INLINE);
    Batch b;
    if (!make_batch(images + g0, cnt, L, TW, TH, b, err)) return DR_ERR_INVALID_ARGUMENT;
    const int64_t tris = b.tri_start[cnt];
    const int tiles = b.tile_start[cnt];
    const Layout lay = make_layout(tris, tiles, cnt, large);
    if (lay.total > ws_bytes) {
      err = "workspace too small: need " + std::to_string(lay.total) + " bytes";
      return DR_ERR_WORKSPACE_TOO_SMALL;
    }
    char* ws = static_cast<char*>(workspace);
    RasterArgs a;
    a.verts = reinterpret_cast<const float4*>(vertices);
    a.tris = triangles;
    a.culling = cfg->face_culling_mode;
    a.depth_mode = cfg->depth_mode;
    a.fg_only = (cfg->flags & DR_RASTER_FOREGROUND_ONLY) != 0;
    a.fg_attr = (cfg->flags & DR_RASTER_FOREGROUND_ATTRIBUTES) != 0;
    a.L = L; a.TW = TW; a.TH = TH; a.large_tiles = large;
    a.total_tris = tris;
    a.total_tiles = tiles;
    a.setup = reinterpret_cast<TriSetup*>(ws + lay.setup);
    a.bbox = reinterpret_cast<int4*>(ws + lay.bbox);
    a.tile_count = reinterpret_cast<int32_t*>(ws + lay.tile_count);
    a.tile_multi = reinterpret_cast<int32_t*>(ws + lay.tile_multi);
    a.tile_fill = reinterpret_cast<int32_t*>(ws + lay.tile_fill);
    a.tile_first = reinterpret_cast<int32_t*>(ws + lay.tile_first);
    a.bins = reinterpret_cast<int32_t*>(ws + lay.bins);
    a.large_count = reinterpret_cast<int32_t*>(ws + lay.large_count);
    a.large_list = reinterpret_cast<int32_t*>(ws + lay.large_list);
    a.counters = reinterpret_cast<uint32_t*>(ws + lay.counters);
    a.ids = ids;
    a.z = z;
    a.bary = bary;
    a.so = so;

    if (cudaMemsetAsync(ws, 0, lay.zero_end, stream) != cudaSuccess) {
      err = std::string("cudaMemsetAsync: ") + cudaGetErrorString(cudaGetLastError());
      return DR_ERR_CUDA;
    }
    if (tris > 0) {
      const unsigned grid = unsigned((tris + 255) / 256);
      setup_kernel<<<grid, 256, 0, stream>>>(a, b);
    }
    tile_scan_kernel<<<1, 1024, 0, stream>>>(a.tile_count, a.tile_multi, a.tile_first, tiles);
    if (tris > 0) {
      const unsigned grid = unsigned((tris + 255) / 256);
      bin_scatter_kernel<<<grid, 256, 0, stream>>>(a, b);
    }
    if (tiles > 0) {
      const unsigned grid = unsigned((tiles + 255) / 256);
      tile_cost_kernel<<<grid, 256, 0, stream>>>(a, b);
      tile_order_kernel<<<grid, 256, 0, stream>>>(a, b);
    }
    const int blocks = std::max(1, std::min(tiles, sms * per_sm));
    fine[variant]<<<blocks, kThreads, smem, stream>>>(a, b);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
      err = std::string("raster launch failed: ") + cudaGetErrorString(e);
      return DR_ERR_CUDA;
    }
  }
  return DR_OK;
}

}  // namespace dr
