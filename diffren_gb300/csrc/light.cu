// Point-light shader (diffren/jax/utils/shaders.py:100-173) and its VJP as
// one elementwise kernel each, one thread per sample:
//   ld = normalize(light - p), vd = normalize(eye - p), h = normalize(ld + vd)
//   nol = clip(n . ld, 0, 1), noh = clip(n . h, 0, 1)
//   dist = |light - p|, decay = 1 / (c + l dist + q dist dist)
//   out = diffuse (ka + kd nol + ks noh^ns) decay
// with normalize(x) = x rsqrt(|x|^2 + 1e-12) (transforms.py:26-37). The
// VJP recomputes the forward and differentiates it by hand: clip passes the
// gradient inside [0, 1] (bounds included), |x| has no gradient at 0, and
// noh^ns none when ks or ns is 0.
//
// The three inputs are rows of 3 floats `stride` floats apart (so columns
// of one packed attribute buffer are read in place); the output is 3 or 4
// channels per sample (the 4th, alpha, is 1 and carries no gradient).
#include <string>

#include "common.cuh"
#include "internal.h"

namespace dr {
namespace {

struct LightArgs {
  const float* dif;
  const float* nrm;
  const float* pos;
  int64_t n;
  int sd, sn, sp;  // row strides (floats)
  dr_point_light q;
  float* out;
  int oc;
  const float* d_out;
  float* d_dif;
  float* d_nrm;
  float* d_pos;
  int sg;  // row stride of the three gradients
};

struct V3 {
  float x, y, z;
};

__device__ __forceinline__ V3 load3(const float* p) { return {__ldg(p), __ldg(p + 1), __ldg(p + 2)}; }
__device__ __forceinline__ V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 scale(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
// (x0 y0 + x1 y1) + x2 y2, each product rounded (the reductions' order).
__device__ __forceinline__ float dot(V3 a, V3 b) {
  return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}

constexpr float kEps = 1e-12f;

// Forward intermediates of one sample.
struct Lit {
  V3 tl, te, hs;       // light - p, eye - p, ld + vd
  float rl, re, rh;    // their rsqrt(|x|^2 + eps)
  V3 ld, vd, h;
  float dl, dh;        // n . ld, n . h (before clipping)
  float nol, noh, dist, denom, decay, luma;
};

__device__ __forceinline__ Lit shade(const dr_point_light& q, V3 n, V3 p) {
  Lit s;
  const V3 L = {q.light[0], q.light[1], q.light[2]};
  const V3 E = {q.eye[0], q.eye[1], q.eye[2]};
  s.tl = sub(L, p);
  s.te = sub(E, p);
  const float sl = dot(s.tl, s.tl);
  s.rl = rsqrtf(sl + kEps);
  s.ld = scale(s.tl, s.rl);
  s.re = rsqrtf(dot(s.te, s.te) + kEps);
  s.vd = scale(s.te, s.re);
  s.hs = add(s.ld, s.vd);
  s.rh = rsqrtf(dot(s.hs, s.hs) + kEps);
  s.h = scale(s.hs, s.rh);
  s.dl = dot(n, s.ld);
  s.dh = dot(n, s.h);
  s.nol = fminf(fmaxf(s.dl, 0.0f), 1.0f);
  s.noh = fminf(fmaxf(s.dh, 0.0f), 1.0f);
  s.dist = sqrtf(sl);
  s.denom = q.attenuation_constant + q.attenuation_linear * s.dist +
            q.attenuation_quadratic * s.dist * s.dist;
  s.decay = 1.0f / s.denom;
  s.luma = q.ka + q.kd * s.nol + q.ks * powf(s.noh, q.ns);
  return s;
}

// Gradient of x -> x r, r = rsqrt(|x|^2 + eps), for the output gradient g:
// r g - r^3 x (x . g).
__device__ __forceinline__ V3 normalize_vjp(V3 x, float r, V3 g) {
  const float k = r * r * r * dot(x, g);
  return {r * g.x - k * x.x, r * g.y - k * x.y, r * g.z - k * x.z};
}

__global__ void __launch_bounds__(256) point_light_fwd_kernel(LightArgs a) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const V3 c = load3(a.dif + i * a.sd), n = load3(a.nrm + i * a.sn), p = load3(a.pos + i * a.sp);
  const Lit s = shade(a.q, n, p);
  float* o = a.out + i * a.oc;
  o[0] = c.x * s.luma * s.decay;
  o[1] = c.y * s.luma * s.decay;
  o[2] = c.z * s.luma * s.decay;
  if (a.oc == 4) o[3] = 1.0f;
}

__global__ void __launch_bounds__(256) point_light_bwd_kernel(LightArgs a) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.n) return;
  const V3 c = load3(a.dif + i * a.sd), n = load3(a.nrm + i * a.sn), p = load3(a.pos + i * a.sp);
  const V3 g = load3(a.d_out + i * a.oc);
  const dr_point_light& q = a.q;
  const Lit s = shade(q, n, p);
  // out_k = c_k luma decay
  const float ld_ = s.luma * s.decay;
  if (a.d_dif) {
    float* d = a.d_dif + i * a.sg;
    d[0] = g.x * ld_;
    d[1] = g.y * ld_;
    d[2] = g.z * ld_;
  }
  if (!a.d_nrm && !a.d_pos) return;
  const float sg = dot(g, c);
  const float d_luma = sg * s.decay, d_decay = sg * s.luma;
  // luma = ka + kd nol + ks noh^ns
  const float d_nol = (s.dl >= 0.0f && s.dl <= 1.0f) ? q.kd * d_luma : 0.0f;
  float d_noh = 0.0f;
  if (q.ks != 0.0f && q.ns != 0.0f && s.dh >= 0.0f && s.dh <= 1.0f)
    d_noh = q.ks * q.ns * powf(s.noh, q.ns - 1.0f) * d_luma;
  // decay = 1 / denom, denom = c + l dist + q dist^2
  const float d_dist =
      -d_decay * s.decay * s.decay * (q.attenuation_linear + 2.0f * q.attenuation_quadratic * s.dist);
  // nol = n . ld, noh = n . h
  const V3 d_n = add(scale(s.ld, d_nol), scale(s.h, d_noh));
  const V3 d_ld0 = scale(n, d_nol);
  const V3 d_h = scale(n, d_noh);
  const V3 d_hs = normalize_vjp(s.hs, s.rh, d_h);  // h = normalize(ld + vd)
  const V3 d_ld = add(d_ld0, d_hs);
  V3 d_tl = normalize_vjp(s.tl, s.rl, d_ld);       // ld = normalize(tl)
  if (s.dist > 0.0f) d_tl = add(d_tl, scale(s.tl, d_dist / s.dist));  // dist = |tl|
  const V3 d_te = normalize_vjp(s.te, s.re, d_hs);  // vd = normalize(te)
  if (a.d_nrm) {
    float* d = a.d_nrm + i * a.sg;
    d[0] = d_n.x;
    d[1] = d_n.y;
    d[2] = d_n.z;
  }
  if (a.d_pos) {  // tl = light - p, te = eye - p
    float* d = a.d_pos + i * a.sg;
    d[0] = -d_tl.x - d_te.x;
    d[1] = -d_tl.y - d_te.y;
    d[2] = -d_tl.z - d_te.z;
  }
}

bool check_light(const float* dif, const float* nrm, const float* pos, int64_t n, int sd, int sn,
                 int sp, const dr_point_light* q, int oc, std::string& err) {
  if (n < 0 || !q) {
    err = "num_samples must be >= 0 and params non-null";
    return false;
  }
  if (n > 0 && (!dif || !nrm || !pos)) {
    err = "diffuse, normals and positions must be non-null";
    return false;
  }
  if (sd < 3 || sn < 3 || sp < 3) {
    err = "row strides must be at least 3 floats";
    return false;
  }
  if (oc != 3 && oc != 4) {
    err = "out_channels must be 3 or 4";
    return false;
  }
  return true;
}

}  // namespace

int point_light_fwd_launch(const float* dif, const float* nrm, const float* pos, int64_t n,
                           int sd, int sn, int sp, const dr_point_light* q, float* out, int oc,
                           cudaStream_t stream, std::string& err) {
  if (!check_light(dif, nrm, pos, n, sd, sn, sp, q, oc, err)) return DR_ERR_INVALID_ARGUMENT;
  if (n == 0) return DR_OK;
  if (!out) {
    err = "out must be non-null";
    return DR_ERR_INVALID_ARGUMENT;
  }
  LightArgs a{dif, nrm, pos, n, sd, sn, sp, *q, out, oc, nullptr, nullptr, nullptr, nullptr, 3};
  point_light_fwd_kernel<<<unsigned((n + 255) / 256), 256, 0, stream>>>(a);
  return launch_status("point light", err);
}

int point_light_bwd_launch(const float* d_out, int oc, const float* dif, const float* nrm,
                           const float* pos, int64_t n, int sd, int sn, int sp,
                           const dr_point_light* q, float* d_dif, float* d_nrm, float* d_pos,
                           int sg, cudaStream_t stream, std::string& err) {
  if (!check_light(dif, nrm, pos, n, sd, sn, sp, q, oc, err)) return DR_ERR_INVALID_ARGUMENT;
  if (n == 0) return DR_OK;
  if (!d_out) {
    err = "d_out must be non-null";
    return DR_ERR_INVALID_ARGUMENT;
  }
  if (sg < 3) {
    err = "gradient row stride must be at least 3 floats";
    return DR_ERR_INVALID_ARGUMENT;
  }
  LightArgs a{dif, nrm, pos, n, sd, sn, sp, *q, nullptr, oc, d_out, d_dif, d_nrm, d_pos, sg};
  point_light_bwd_kernel<<<unsigned((n + 255) / 256), 256, 0, stream>>>(a);
  return launch_status("point light backward", err);
}

}  // namespace dr
