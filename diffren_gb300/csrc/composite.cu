// OVER compositing of shaded layers for the non-splat render mode
// (diffren/jax/render.py:134-140 with composite.over, composite.py:20-37):
// each layer sample is multiplied by its foreground mask (z != 1), then the
// layers are composited back to front, o = s[L-1]; o = s[l] + (1 - a[l]) o,
// in the reference's float order. One thread per composited pixel; the
// channels are independent given the layers' alphas (the last channel).
//
// The VJP recomputes each channel's partial composites o[l] and runs the
// chain front to back: d s[l] = g, d a[l] -= g . o[l+1], g *= (1 - a[l]);
// the mask multiply passes d s[l] * fg[l] on to the shaded input.
#include <algorithm>
#include <string>

#include "common.cuh"
#include "internal.h"

namespace dr {
namespace {

struct OverArgs {
  const float* shaded;  // [L, H, W, C] per image, packed
  const float* z;       // [L, H, W] per image, packed
  const float* d_out;   // [H, W, C] per image, packed
  float* out;
  float* d_shaded;
  int C;
  int L;
};

struct OverPixel {
  int64_t e0;   // element index of layer 0 in the layered buffers
  int64_t hw;   // layer stride in elements
  int64_t o;    // pixel index in the composited buffers
};

__device__ __forceinline__ OverPixel over_pixel(const Batch& B, int L, int64_t q) {
  int64_t p;
  const int img = locate(B, 1, q, p);
  OverPixel r;
  r.hw = int64_t(B.width[img]) * B.height[img];
  r.e0 = int64_t(L) * B.pix_off[img] + p;
  r.o = B.pix_off[img] + p;
  return r;
}

// LT: compile-time layer bound (the loops run to a.L <= LT).
template <int LT>
__global__ void __launch_bounds__(256) over_fwd_kernel(OverArgs a, Batch B) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= B.pix_prefix[B.n]) return;
  const OverPixel px = over_pixel(B, a.L, q);
  const int C = a.C, L = a.L;
  float fg[LT], keep[LT];
#pragma unroll
  for (int l = 0; l < LT; ++l) {
    if (l < L) {
      const int64_t e = px.e0 + l * px.hw;
      fg[l] = __ldg(a.z + e) != 1.0f ? 1.0f : 0.0f;
      keep[l] = __fsub_rn(1.0f, __fmul_rn(__ldg(a.shaded + e * C + C - 1), fg[l]));
    }
  }
  for (int c = 0; c < C; ++c) {
    float o = 0.0f;
#pragma unroll
    for (int l = LT - 1; l >= 0; --l) {
      if (l < L) {
        const float s = __fmul_rn(__ldg(a.shaded + (px.e0 + l * px.hw) * C + c), fg[l]);
        o = l == L - 1 ? s : __fadd_rn(s, __fmul_rn(keep[l], o));
      }
    }
    a.out[px.o * C + c] = o;
  }
}

template <int LT>
__global__ void __launch_bounds__(256) over_bwd_kernel(OverArgs a, Batch B) {
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= B.pix_prefix[B.n]) return;
  const OverPixel px = over_pixel(B, a.L, q);
  const int C = a.C, L = a.L;
  float fg[LT], keep[LT], d_alpha[LT];
#pragma unroll
  for (int l = 0; l < LT; ++l) {
    d_alpha[l] = 0.0f;
    if (l < L) {
      const int64_t e = px.e0 + l * px.hw;
      fg[l] = __ldg(a.z + e) != 1.0f ? 1.0f : 0.0f;
      keep[l] = __fsub_rn(1.0f, __fmul_rn(__ldg(a.shaded + e * C + C - 1), fg[l]));
    }
  }
  // The alpha channel goes last: its adjoint collects every channel's d a.
  for (int c = 0; c < C; ++c) {
    float s[LT], o[LT];
#pragma unroll
    for (int l = LT - 1; l >= 0; --l) {
      if (l < L) {
        s[l] = __fmul_rn(__ldg(a.shaded + (px.e0 + l * px.hw) * C + c), fg[l]);
        o[l] = l == L - 1 ? s[l] : __fadd_rn(s[l], __fmul_rn(keep[l], o[l + 1 < LT ? l + 1 : l]));
      }
    }
    float g = __ldg(a.d_out + px.o * C + c);
#pragma unroll
    for (int l = 0; l < LT; ++l) {
      if (l < L) {
        float ds = g;
        if (l + 1 < L) d_alpha[l] -= g * o[l + 1 < LT ? l + 1 : l];
        if (c == C - 1) ds += d_alpha[l];
        a.d_shaded[(px.e0 + l * px.hw) * C + c] = ds * fg[l];
        g = keep[l] * g;
      }
    }
  }
}

template <int LT>
void launch(const OverArgs& a, const Batch& b, bool backward, cudaStream_t stream) {
  const int64_t P = b.pix_prefix[b.n];
  if (P == 0) return;
  const unsigned blocks = unsigned((P + 255) / 256);
  if (backward)
    over_bwd_kernel<LT><<<blocks, 256, 0, stream>>>(a, b);
  else
    over_fwd_kernel<LT><<<blocks, 256, 0, stream>>>(a, b);
}

int over_launch(OverArgs a, const dr_image_desc* images, int n, bool backward,
                cudaStream_t stream, std::string& err) {
  if (n < 0 || (n > 0 && !images)) { err = "invalid image table"; return DR_ERR_INVALID_ARGUMENT; }
  if (a.L < 1 || a.L > DR_MAX_LAYERS) {
    err = "num_layers must be in [1, " + std::to_string(DR_MAX_LAYERS) + "]";
    return DR_ERR_INVALID_ARGUMENT;
  }
  if (a.C < 1) { err = "channels must be >= 1"; return DR_ERR_INVALID_ARGUMENT; }
  // Every group is checked before the first launch.
  Batch b;
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE)
    if (!make_batch(images + g0, std::min(n - g0, DR_MAX_BATCH_INLINE), a.L, 16, 16, b, err))
      return DR_ERR_INVALID_ARGUMENT;
  if (n > 0 && (!a.shaded || !a.z || (backward ? (!a.d_out || !a.d_shaded) : !a.out))) {
    err = "shaded, z_buffer and the outputs must be non-null";
    return DR_ERR_INVALID_ARGUMENT;
  }
  for (int g0 = 0; g0 < n; g0 += DR_MAX_BATCH_INLINE) {
    make_batch(images + g0, std::min(n - g0, DR_MAX_BATCH_INLINE), a.L, 16, 16, b, err);
    if (a.L <= 3)
      launch<3>(a, b, backward, stream);
    else
      launch<DR_MAX_LAYERS>(a, b, backward, stream);
  }
  return launch_status(backward ? "composite over backward" : "composite over", err);
}

}  // namespace

int over_fwd_launch(const float* shaded, const float* z, int C, const dr_image_desc* images,
                    int n, int L, float* out, cudaStream_t stream, std::string& err) {
  return over_launch(OverArgs{shaded, z, nullptr, out, nullptr, C, L}, images, n, false, stream,
                     err);
}

int over_bwd_launch(const float* d_out, const float* shaded, const float* z, int C,
                    const dr_image_desc* images, int n, int L, float* d_shaded,
                    cudaStream_t stream, std::string& err) {
  return over_launch(OverArgs{shaded, z, d_out, nullptr, d_shaded, C, L}, images, n, true,
                     stream, err);
}

}  // namespace dr
