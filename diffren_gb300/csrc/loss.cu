// Squared-error objective of a rendered image against a target, the loss the
// reference's optimization tests fit meshes with (jnp.mean((image -
// target)**2), diffren/jax/internal/splat_test.py:137-167), with its
// gradient, in one pass over the images:
//   loss = weight * sum_i (image_i - target_i)^2
//   seed_i = (2 * weight) * (image_i - target_i)   (d loss / d image)
// The seed goes straight into the renderer's VJP, so no second pass over the
// images forms the gradient. With weight = 1 the seed is 2 (image - target)
// exactly (a power-of-two multiply), the value autograd of the sum forms.
//
// The sum is deterministic: a fixed grid of kBlocks blocks (8 per SM of a
// GB300's 152) strides over the elements in a fixed order, each thread keeps
// a compensated (Kahan) float sum, each block reduces its threads' sums in
// double, and a one-block kernel adds the kBlocks partials in a fixed tree
// in double.
#include <string>

#include "diffren_gb300.h"
#include "internal.h"

namespace dr {
namespace {

constexpr int kThreads = 256;
constexpr int kBlocks = DR_SQUARED_ERROR_PARTIALS;

struct Kahan {
  float s = 0.0f, c = 0.0f;
  __device__ __forceinline__ void add(float x) {
    const float y = __fsub_rn(x, c);
    const float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
  }
};

// Sum of the block's per-thread values in double, in a fixed tree.
__device__ __forceinline__ double block_sum(double v, double* s_part) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) s_part[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < int(blockDim.x >> 5) ? s_part[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  }
  return v;
}

// VEC: both images and the seed are 16-byte aligned and n is a multiple of 4.
template <bool VEC>
__global__ void __launch_bounds__(kThreads) squared_error_kernel(const float* image,
                                                                  const float* target,
                                                                  int64_t n, float two_w,
                                                                  float* seed,
                                                                  double* partials) {
  __shared__ double s_part[kThreads / 32];
  Kahan k;
  const int64_t stride = int64_t(kBlocks) * kThreads;
  const int64_t t0 = int64_t(blockIdx.x) * kThreads + threadIdx.x;
  if constexpr (VEC) {
    const float4* a4 = reinterpret_cast<const float4*>(image);
    const float4* b4 = reinterpret_cast<const float4*>(target);
    float4* s4 = reinterpret_cast<float4*>(seed);
    for (int64_t i = t0; i < n / 4; i += stride) {
      const float4 a = __ldcs(a4 + i), b = __ldcs(b4 + i);
      float4 d;
      d.x = __fsub_rn(a.x, b.x);
      d.y = __fsub_rn(a.y, b.y);
      d.z = __fsub_rn(a.z, b.z);
      d.w = __fsub_rn(a.w, b.w);
      k.add(__fmul_rn(d.x, d.x));
      k.add(__fmul_rn(d.y, d.y));
      k.add(__fmul_rn(d.z, d.z));
      k.add(__fmul_rn(d.w, d.w));
      s4[i] = make_float4(__fmul_rn(two_w, d.x), __fmul_rn(two_w, d.y),
                          __fmul_rn(two_w, d.z), __fmul_rn(two_w, d.w));
    }
  } else {
    for (int64_t i = t0; i < n; i += stride) {
      const float d = __fsub_rn(image[i], target[i]);
      k.add(__fmul_rn(d, d));
      seed[i] = __fmul_rn(two_w, d);
    }
  }
  const double v = block_sum(double(k.s) - double(k.c), s_part);
  if (threadIdx.x == 0) partials[blockIdx.x] = v;
}

// One block of kTotalThreads threads; thread t adds partials t, t + 1024, ...
constexpr int kTotalThreads = 1024;

__global__ void __launch_bounds__(kTotalThreads) squared_error_total_kernel(
    const double* partials, float weight, float* loss) {
  __shared__ double s_part[kTotalThreads / 32];
  double p = 0.0;
  for (int i = threadIdx.x; i < kBlocks; i += kTotalThreads) p += partials[i];
  const double v = block_sum(p, s_part);
  if (threadIdx.x == 0) *loss = float(v * double(weight));
}

}  // namespace

int squared_error_launch(const float* image, const float* target, int64_t n, float weight,
                         float* seed, double* partials, float* loss, cudaStream_t stream,
                         std::string& err) {
  if (n < 0) { err = "count must be >= 0"; return DR_ERR_INVALID_ARGUMENT; }
  if (!loss || !partials) {
    err = "loss and partials must be non-null";
    return DR_ERR_INVALID_ARGUMENT;
  }
  if (n > 0 && (!image || !target || !seed)) {
    err = "image, target and seed must be non-null";
    return DR_ERR_INVALID_ARGUMENT;
  }
  const bool vec = ((reinterpret_cast<uintptr_t>(image) | reinterpret_cast<uintptr_t>(target) |
                     reinterpret_cast<uintptr_t>(seed)) & 15) == 0 &&
                   (n & 3) == 0;
  const float two_w = 2.0f * weight;
  if (vec)
    squared_error_kernel<true><<<kBlocks, kThreads, 0, stream>>>(image, target, n, two_w, seed,
                                                                 partials);
  else
    squared_error_kernel<false><<<kBlocks, kThreads, 0, stream>>>(image, target, n, two_w, seed,
                                                                  partials);
  squared_error_total_kernel<<<1, kTotalThreads, 0, stream>>>(partials, weight, loss);
  return launch_status("squared error", err);
}

}  // namespace dr
