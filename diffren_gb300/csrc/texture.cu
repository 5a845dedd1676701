// Texture-map shader (diffren/jax/utils/shaders.py:40-65) and its VJP:
// bilinear resampling of an [H, W, C] texture at uv * (W, H) with the
// texture padded by one edge texel (image.py:21-118, pad_mode='edge'), or by
// zeros (pad_mode='constant') and at locations in texel units, as
// image.bilinear_resample.
//
// Per point: location (row, col) = (v H, u W) - 0.5 + 1 in padded texels,
// floor clipped to [0, size], ceil weight clip(location - floor, 0, 1),
// result ((ll + ul) + ur) + lr with each corner (texel * w_row) * w_col: the
// reference's expression order, so results are the reference's bits. The
// VJP scatters to the four texels (float atomics) and differentiates the
// weights, with jnp.clip's gradient (1 strictly inside its bounds).
#include <algorithm>
#include <string>

#include "common.cuh"
#include "internal.h"

namespace dr {
namespace {

struct TexArgs {
  const float* uv;
  const float* tex;
  int H, W, C, flags;
  int64_t n;
  float* out;
  const float* d_out;
  float* d_uv;
  float* d_tex;
  // DR_TEXTURE_DETERMINISTIC: d_tex summed in 64-bit fixed point (see
  // fixed_exponent_of): the largest |d_out| (each texel adds w d_out with a
  // weight w <= 1), the sums [H W C], and ceil(log2(points x 4)).
  unsigned* fx_max;
  unsigned long long* fx_tex;
  int fx_log2_terms;
};

struct Axis {
  int f;      // floor index in padded texels, in [0, size]
  float cw;   // ceil weight
  float fw;   // floor weight
  float dcw;  // d cw / d location (1 strictly inside (0, 1), else 0)
};

__device__ __forceinline__ Axis axis_of(float loc, int size) {
  Axis a;
  const float fl = fminf(fmaxf(floorf(loc), 0.0f), __int2float_rn(size));
  a.f = __float2int_rz(fl);
  const float t = __fsub_rn(loc, fl);
  a.cw = fminf(fmaxf(t, 0.0f), 1.0f);
  a.fw = __fsub_rn(1.0f, a.cw);
  a.dcw = (t > 0.0f && t < 1.0f) ? 1.0f : 0.0f;
  return a;
}

// Texel (r, c) of the padded texture: padded index minus one, clamped to
// the edge; -1 for the zero border of constant padding.
__device__ __forceinline__ int64_t texel(const TexArgs& a, int r, int c) {
  if ((a.flags & DR_TEXTURE_PAD_ZERO) && (r == 0 || c == 0 || r > a.H || c > a.W)) return -1;
  r = min(max(r - 1, 0), a.H - 1);
  c = min(max(c - 1, 0), a.W - 1);
  return (int64_t(r) * a.W + c) * a.C;
}

__device__ __forceinline__ float fetch(const TexArgs& a, int64_t t, int k) {
  return t < 0 ? 0.0f : __ldg(a.tex + t + k);
}

struct Footprint {
  Axis r, c;
  int64_t t00, t10, t11, t01;
};

__device__ __forceinline__ Footprint footprint(const TexArgs& a, int64_t i) {
  Footprint f;
  const float u = __ldg(a.uv + 2 * i), v = __ldg(a.uv + 2 * i + 1);
  // query = uv * (W, H) - 0.5 (or texel units - 0.5), then + 1 into the
  // padded texture
  const bool texels = a.flags & DR_TEXTURE_TEXEL_UNITS;
  const float qc = __fsub_rn(texels ? u : __fmul_rn(u, __int2float_rn(a.W)), 0.5f);
  const float qr = __fsub_rn(texels ? v : __fmul_rn(v, __int2float_rn(a.H)), 0.5f);
  f.r = axis_of(__fadd_rn(qr, 1.0f), a.H);
  f.c = axis_of(__fadd_rn(qc, 1.0f), a.W);
  f.t00 = texel(a, f.r.f, f.c.f);
  f.t10 = texel(a, f.r.f + 1, f.c.f);
  f.t11 = texel(a, f.r.f + 1, f.c.f + 1);
  f.t01 = texel(a, f.r.f, f.c.f + 1);
  return f;
}

__global__ void __launch_bounds__(256) texture_fwd_kernel(TexArgs a) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const Footprint f = footprint(a, i);
  float* o = a.out + i * a.C;
  if ((a.C & 3) == 0 &&
      ((reinterpret_cast<uintptr_t>(a.tex) | reinterpret_cast<uintptr_t>(a.out)) & 15) == 0) {
    // Four channels per load and store.
    const float4 zero = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const auto fetch4 = [&](int64_t t, int k) {
      return t < 0 ? zero : __ldg(reinterpret_cast<const float4*>(a.tex + t + k));
    };
    const auto term = [](float x, float w0, float w1) {
      return __fmul_rn(__fmul_rn(x, w0), w1);
    };
    for (int k = 0; k < a.C; k += 4) {
      const float4 t00 = fetch4(f.t00, k), t10 = fetch4(f.t10, k), t11 = fetch4(f.t11, k),
                   t01 = fetch4(f.t01, k);
      float4 r;
      r.x = __fadd_rn(__fadd_rn(__fadd_rn(term(t00.x, f.r.fw, f.c.fw),
                                          term(t10.x, f.r.cw, f.c.fw)),
                                term(t11.x, f.r.cw, f.c.cw)),
                      term(t01.x, f.r.fw, f.c.cw));
      r.y = __fadd_rn(__fadd_rn(__fadd_rn(term(t00.y, f.r.fw, f.c.fw),
                                          term(t10.y, f.r.cw, f.c.fw)),
                                term(t11.y, f.r.cw, f.c.cw)),
                      term(t01.y, f.r.fw, f.c.cw));
      r.z = __fadd_rn(__fadd_rn(__fadd_rn(term(t00.z, f.r.fw, f.c.fw),
                                          term(t10.z, f.r.cw, f.c.fw)),
                                term(t11.z, f.r.cw, f.c.cw)),
                      term(t01.z, f.r.fw, f.c.cw));
      r.w = __fadd_rn(__fadd_rn(__fadd_rn(term(t00.w, f.r.fw, f.c.fw),
                                          term(t10.w, f.r.cw, f.c.fw)),
                                term(t11.w, f.r.cw, f.c.cw)),
                      term(t01.w, f.r.fw, f.c.cw));
      *reinterpret_cast<float4*>(o + k) = r;
    }
    return;
  }
  for (int k = 0; k < a.C; ++k) {
    const float ll = __fmul_rn(__fmul_rn(fetch(a, f.t00, k), f.r.fw), f.c.fw);
    const float ul = __fmul_rn(__fmul_rn(fetch(a, f.t10, k), f.r.cw), f.c.fw);
    const float ur = __fmul_rn(__fmul_rn(fetch(a, f.t11, k), f.r.cw), f.c.cw);
    const float lr = __fmul_rn(__fmul_rn(fetch(a, f.t01, k), f.r.fw), f.c.cw);
    o[k] = __fadd_rn(__fadd_rn(__fadd_rn(ll, ul), ur), lr);
  }
}

// The common case on 32-bit texel indices: four channels, edge padding, a
// texture of fewer than 2^29 texels, 8-byte aligned uv and 16-byte aligned
// texture and output. Same operations and order as texture_fwd_kernel.
__global__ void __launch_bounds__(256) texture_fwd4_kernel(TexArgs a) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const float2 uv = __ldg(reinterpret_cast<const float2*>(a.uv) + i);
  const bool texels = a.flags & DR_TEXTURE_TEXEL_UNITS;
  const float qc = __fsub_rn(texels ? uv.x : __fmul_rn(uv.x, __int2float_rn(a.W)), 0.5f);
  const float qr = __fsub_rn(texels ? uv.y : __fmul_rn(uv.y, __int2float_rn(a.H)), 0.5f);
  const Axis r = axis_of(__fadd_rn(qr, 1.0f), a.H);
  const Axis c = axis_of(__fadd_rn(qc, 1.0f), a.W);
  // padded rows / columns f and f + 1 are texture rows f - 1 and f, clamped
  const unsigned r0 = unsigned(max(r.f - 1, 0)) * unsigned(a.W);
  const unsigned r1 = unsigned(min(r.f, a.H - 1)) * unsigned(a.W);
  const unsigned c0 = unsigned(max(c.f - 1, 0)), c1 = unsigned(min(c.f, a.W - 1));
  const float4* T = reinterpret_cast<const float4*>(a.tex);
  const float4 t00 = __ldg(T + r0 + c0), t10 = __ldg(T + r1 + c0), t11 = __ldg(T + r1 + c1),
               t01 = __ldg(T + r0 + c1);
  const auto mix = [&](float x00, float x10, float x11, float x01) {
    const float ll = __fmul_rn(__fmul_rn(x00, r.fw), c.fw);
    const float ul = __fmul_rn(__fmul_rn(x10, r.cw), c.fw);
    const float ur = __fmul_rn(__fmul_rn(x11, r.cw), c.cw);
    const float lr = __fmul_rn(__fmul_rn(x01, r.fw), c.cw);
    return __fadd_rn(__fadd_rn(__fadd_rn(ll, ul), ur), lr);
  };
  reinterpret_cast<float4*>(a.out)[i] =
      make_float4(mix(t00.x, t10.x, t11.x, t01.x), mix(t00.y, t10.y, t11.y, t01.y),
                  mix(t00.z, t10.z, t11.z, t01.z), mix(t00.w, t10.w, t11.w, t01.w));
}

// The VJP of texture_fwd4_kernel (same conditions; d_tex 16-byte aligned).
__global__ void __launch_bounds__(256) texture_bwd4_kernel(TexArgs a) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const float4 g = __ldg(reinterpret_cast<const float4*>(a.d_out) + i);
  if (g.x == 0.0f && g.y == 0.0f && g.z == 0.0f && g.w == 0.0f) {
    if (a.d_uv) reinterpret_cast<float2*>(a.d_uv)[i] = make_float2(0.0f, 0.0f);
    return;
  }
  const float2 uv = __ldg(reinterpret_cast<const float2*>(a.uv) + i);
  const bool texels = a.flags & DR_TEXTURE_TEXEL_UNITS;
  const float qc = __fsub_rn(texels ? uv.x : __fmul_rn(uv.x, __int2float_rn(a.W)), 0.5f);
  const float qr = __fsub_rn(texels ? uv.y : __fmul_rn(uv.y, __int2float_rn(a.H)), 0.5f);
  const Axis r = axis_of(__fadd_rn(qr, 1.0f), a.H);
  const Axis c = axis_of(__fadd_rn(qc, 1.0f), a.W);
  const unsigned r0 = unsigned(max(r.f - 1, 0)) * unsigned(a.W);
  const unsigned r1 = unsigned(min(r.f, a.H - 1)) * unsigned(a.W);
  const unsigned c0 = unsigned(max(c.f - 1, 0)), c1 = unsigned(min(c.f, a.W - 1));
  if (a.d_tex) {
    float4* D = reinterpret_cast<float4*>(a.d_tex);
    const auto add = [&](unsigned t, float w) {
      atomicAdd(D + t, make_float4(g.x * w, g.y * w, g.z * w, g.w * w));
    };
    add(r0 + c0, r.fw * c.fw);
    add(r1 + c0, r.cw * c.fw);
    add(r1 + c1, r.cw * c.cw);
    add(r0 + c1, r.fw * c.cw);
  }
  if (a.d_uv) {
    const float4* T = reinterpret_cast<const float4*>(a.tex);
    const float4 t00 = __ldg(T + r0 + c0), t10 = __ldg(T + r1 + c0), t11 = __ldg(T + r1 + c1),
                 t01 = __ldg(T + r0 + c1);
    float du = 0.0f, dv = 0.0f;
    const auto step = [&](float gk, float d00, float d10, float d11, float d01) {
      du += gk * (r.fw * (d01 - d00) + r.cw * (d11 - d10));
      dv += gk * (c.fw * (d10 - d00) + c.cw * (d11 - d01));
    };
    step(g.x, t00.x, t10.x, t11.x, t01.x);
    step(g.y, t00.y, t10.y, t11.y, t01.y);
    step(g.z, t00.z, t10.z, t11.z, t01.z);
    step(g.w, t00.w, t10.w, t11.w, t01.w);
    reinterpret_cast<float2*>(a.d_uv)[i] =
        make_float2(du * c.dcw * (texels ? 1.0f : __int2float_rn(a.W)),
                    dv * r.dcw * (texels ? 1.0f : __int2float_rn(a.H)));
  }
}

__global__ void __launch_bounds__(256) texture_bwd_kernel(TexArgs a) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const float* g = a.d_out + i * a.C;
  bool any = false;
  for (int k = 0; k < a.C; ++k) any |= __ldg(g + k) != 0.0f;
  if (!any) {
    if (a.d_uv) {
      a.d_uv[2 * i] = 0.0f;
      a.d_uv[2 * i + 1] = 0.0f;
    }
    return;
  }
  const Footprint f = footprint(a, i);
  float du = 0.0f, dv = 0.0f;
  if (a.d_tex && (a.C & 3) == 0 && (reinterpret_cast<uintptr_t>(a.d_tex) & 15) == 0) {
    // Four channels per vector atomic.
    const float w00 = f.r.fw * f.c.fw, w10 = f.r.cw * f.c.fw, w11 = f.r.cw * f.c.cw,
                w01 = f.r.fw * f.c.cw;
    for (int k = 0; k < a.C; k += 4) {
      const float4 gk = make_float4(__ldg(g + k), __ldg(g + k + 1), __ldg(g + k + 2),
                                    __ldg(g + k + 3));
      const auto add = [&](int64_t t, float w) {
        if (t >= 0)
          atomicAdd(reinterpret_cast<float4*>(a.d_tex + t + k),
                    make_float4(gk.x * w, gk.y * w, gk.z * w, gk.w * w));
      };
      add(f.t00, w00);
      add(f.t10, w10);
      add(f.t11, w11);
      add(f.t01, w01);
    }
  }
  const bool scalar_tex = a.d_tex && !((a.C & 3) == 0 &&
                                       (reinterpret_cast<uintptr_t>(a.d_tex) & 15) == 0);
  for (int k = 0; k < a.C; ++k) {
    const float gk = __ldg(g + k);
    if (scalar_tex && gk != 0.0f) {
      if (f.t00 >= 0) atomicAdd(a.d_tex + f.t00 + k, gk * f.r.fw * f.c.fw);
      if (f.t10 >= 0) atomicAdd(a.d_tex + f.t10 + k, gk * f.r.cw * f.c.fw);
      if (f.t11 >= 0) atomicAdd(a.d_tex + f.t11 + k, gk * f.r.cw * f.c.cw);
      if (f.t01 >= 0) atomicAdd(a.d_tex + f.t01 + k, gk * f.r.fw * f.c.cw);
    }
    if (a.d_uv) {
      const float d00 = fetch(a, f.t00, k), d10 = fetch(a, f.t10, k);
      const float d11 = fetch(a, f.t11, k), d01 = fetch(a, f.t01, k);
      du += gk * (f.r.fw * (d01 - d00) + f.r.cw * (d11 - d10));
      dv += gk * (f.c.fw * (d10 - d00) + f.c.cw * (d11 - d01));
    }
  }
  if (a.d_uv) {
    const bool texels = a.flags & DR_TEXTURE_TEXEL_UNITS;
    a.d_uv[2 * i] = du * f.c.dcw * (texels ? 1.0f : __int2float_rn(a.W));
    a.d_uv[2 * i + 1] = dv * f.r.dcw * (texels ? 1.0f : __int2float_rn(a.H));
  }
}

// Deterministic VJP. Pass 1: the largest |d_out| (the bound on every value a
// texel receives). Pass 2: d_uv as texture_bwd_kernel writes it, and each
// corner's w d_out added in fixed point. Pass 3: the sums back to float,
// added to d_tex.
__global__ void __launch_bounds__(256) texture_bwd_bound_kernel(TexArgs a) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  float m = 0.0f;
  if (i < a.n)
    for (int k = 0; k < a.C; ++k) m = fmaxf(m, fixed_mag(__ldg(a.d_out + i * a.C + k)));
  const unsigned wm = __reduce_max_sync(0xffffffffu, __float_as_uint(m));
  if ((threadIdx.x & 31) == 0 && wm != 0u) atomicMax(a.fx_max, wm);
}

__global__ void __launch_bounds__(256) texture_bwd_fixed_kernel(TexArgs a) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const int e = fixed_exponent_of(__ldg(a.fx_max), a.fx_log2_terms);
  const float* g = a.d_out + i * a.C;
  const Footprint f = footprint(a, i);
  float du = 0.0f, dv = 0.0f;
  for (int k = 0; k < a.C; ++k) {
    const float gk = __ldg(g + k);
    if (a.d_tex && gk != 0.0f && e != kFixedZero) {
      const int64_t t[4] = {f.t00, f.t10, f.t11, f.t01};
      const float w[4] = {f.r.fw * f.c.fw, f.r.cw * f.c.fw, f.r.cw * f.c.cw, f.r.fw * f.c.cw};
      for (int j = 0; j < 4; ++j) {
        if (t[j] < 0) continue;
        const float v = gk * w[j];
        if (e == kFixedFloat)
          atomicAdd(a.d_tex + t[j] + k, v);  // a non-finite gradient: as the float path
        else
          add_fixed(a.fx_tex + t[j] + k, v, e);
      }
    }
    if (a.d_uv) {
      const float d00 = fetch(a, f.t00, k), d10 = fetch(a, f.t10, k);
      const float d11 = fetch(a, f.t11, k), d01 = fetch(a, f.t01, k);
      du += gk * (f.r.fw * (d01 - d00) + f.r.cw * (d11 - d10));
      dv += gk * (f.c.fw * (d10 - d00) + f.c.cw * (d11 - d01));
    }
  }
  if (a.d_uv) {
    const bool texels = a.flags & DR_TEXTURE_TEXEL_UNITS;
    a.d_uv[2 * i] = du * f.c.dcw * (texels ? 1.0f : __int2float_rn(a.W));
    a.d_uv[2 * i + 1] = dv * f.r.dcw * (texels ? 1.0f : __int2float_rn(a.H));
  }
}

__global__ void __launch_bounds__(256) texture_fixed_finalize_kernel(TexArgs a, int64_t nt) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  const int e = fixed_exponent_of(__ldg(a.fx_max), a.fx_log2_terms);
  if (e == kFixedZero || e == kFixedFloat) return;
  a.d_tex[i] += fixed_back(a.fx_tex[i], e);
}

bool check_tex(const float* uv, int64_t n, const float* tex, int H, int W, int C,
               std::string& err) {
  if (n < 0 || H < 1 || W < 1 || C < 1 || C > DR_MAX_CHANNELS || H >= (1 << 28) ||
      W >= (1 << 28)) {
    err = "texture must be [H >= 1, W >= 1, 1 <= C <= 16] and the point count >= 0";
    return false;
  }
  if (n > 0 && (!uv || !tex)) {
    err = "uv and texture must be non-null";
    return false;
  }
  return true;
}

}  // namespace

int texture_fwd_launch(const float* uv, int64_t n, const float* tex, int H, int W, int C,
                       int flags, float* out, cudaStream_t stream, std::string& err) {
  if (!check_tex(uv, n, tex, H, W, C, err)) return DR_ERR_INVALID_ARGUMENT;
  if (n == 0) return DR_OK;
  if (!out) { err = "out must be non-null"; return DR_ERR_INVALID_ARGUMENT; }
  TexArgs a{uv, tex, H, W, C, flags, n, out, nullptr, nullptr, nullptr, nullptr, nullptr, 0};
  const bool fast = C == 4 && !(flags & DR_TEXTURE_PAD_ZERO) &&
                    int64_t(H) * W < (int64_t(1) << 29) &&
                    (reinterpret_cast<uintptr_t>(uv) & 7) == 0 &&
                    ((reinterpret_cast<uintptr_t>(tex) | reinterpret_cast<uintptr_t>(out)) & 15) == 0;
  if (fast)
    texture_fwd4_kernel<<<unsigned((n + 255) / 256), 256, 0, stream>>>(a);
  else
    texture_fwd_kernel<<<unsigned((n + 255) / 256), 256, 0, stream>>>(a);
  return launch_status("texture map", err);
}

size_t texture_fixed_bytes(int H, int W, int C) {
  return 256 + size_t(H) * size_t(W) * size_t(C) * 8;
}

int texture_bwd_launch(const float* d_out, const float* uv, int64_t n, const float* tex,
                       int H, int W, int C, int flags, float* d_uv, float* d_tex,
                       void* scratch, size_t scratch_bytes, cudaStream_t stream,
                       std::string& err) {
  if (!check_tex(uv, n, tex, H, W, C, err)) return DR_ERR_INVALID_ARGUMENT;
  if ((flags & ~(DR_TEXTURE_PAD_ZERO | DR_TEXTURE_TEXEL_UNITS | DR_TEXTURE_DETERMINISTIC)) != 0) {
    err = "unknown texture flags";
    return DR_ERR_INVALID_ARGUMENT;
  }
  const bool det = (flags & DR_TEXTURE_DETERMINISTIC) != 0 && d_tex;
  if (det && (!scratch || (reinterpret_cast<uintptr_t>(scratch) & 255) != 0 ||
              scratch_bytes < texture_fixed_bytes(H, W, C))) {
    err = "DR_TEXTURE_DETERMINISTIC needs a 256-byte aligned scratch of "
          "dr_texture_map_bwd_scratch_bytes bytes";
    return DR_ERR_INVALID_ARGUMENT;
  }
  if (n == 0) return DR_OK;
  if (!d_out) { err = "d_out must be non-null"; return DR_ERR_INVALID_ARGUMENT; }
  TexArgs a{uv, tex, H, W, C, flags, n, nullptr, d_out, d_uv, d_tex, nullptr, nullptr, 0};
  const unsigned grid = unsigned((n + 255) / 256);
  if (det) {
    unsigned char* base = static_cast<unsigned char*>(scratch);
    a.fx_max = reinterpret_cast<unsigned*>(base);
    a.fx_tex = reinterpret_cast<unsigned long long*>(base + 256);
    int lt = 0;
    while ((int64_t(1) << lt) < 4 * n) ++lt;
    a.fx_log2_terms = lt;
    if (cudaMemsetAsync(scratch, 0, texture_fixed_bytes(H, W, C), stream) != cudaSuccess) {
      err = std::string("cudaMemsetAsync: ") + cudaGetErrorString(cudaGetLastError());
      return DR_ERR_CUDA;
    }
    texture_bwd_bound_kernel<<<grid, 256, 0, stream>>>(a);
    texture_bwd_fixed_kernel<<<grid, 256, 0, stream>>>(a);
    const int64_t nt = int64_t(H) * W * C;
    texture_fixed_finalize_kernel<<<unsigned((nt + 255) / 256), 256, 0, stream>>>(a, nt);
    return launch_status("texture map backward", err);
  }
  const bool fast = C == 4 && !(flags & DR_TEXTURE_PAD_ZERO) &&
                    int64_t(H) * W < (int64_t(1) << 29) &&
                    ((reinterpret_cast<uintptr_t>(uv) | reinterpret_cast<uintptr_t>(d_uv)) & 7) == 0 &&
                    ((reinterpret_cast<uintptr_t>(tex) | reinterpret_cast<uintptr_t>(d_out) |
                      reinterpret_cast<uintptr_t>(d_tex)) & 15) == 0;
  if (fast)
    texture_bwd4_kernel<<<grid, 256, 0, stream>>>(a);
  else
    texture_bwd_kernel<<<grid, 256, 0, stream>>>(a);
  return launch_status("texture map backward", err);
}

}  // namespace dr
