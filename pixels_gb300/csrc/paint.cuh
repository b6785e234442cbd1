// Device counterparts of the scene's paint closures, evaluated in float64 in
// every build mode (their floors, rounds and thresholds are discontinuous, so
// they are always computed exactly as the reference computes them).
#pragma once
#include "jsmath.cuh"
#include "px_internal.cuh"

namespace px {

__device__ __forceinline__ uint32_t vox_of(double mat, double shade) {  // materials.ts:108-110
  return ((uint32_t)(long long)mat & 0xffu) | (((uint32_t)(long long)shade & 0xffu) << 8);
}

__device__ __forceinline__ uint32_t noise_hash(uint32_t ix, uint32_t iy, uint32_t iz, uint32_t seed) {
  uint32_t h = seed ^ (ix * 0x8DA6B343u) ^ (iy * 0xD8163841u) ^ (iz * 0xCB1AB31Fu);
  h ^= h >> 16; h *= 0x7FEB352Du; h ^= h >> 15; h *= 0x846CA68Bu; h ^= h >> 16;
  return h;
}

// float32 triangle-wave sine of the synthetic noise paint; explicit
// round-to-nearest intrinsics keep every step a separate float32 operation.
__device__ __forceinline__ float sin_poly_f32(float t) {
  float u = __fsub_rn(t, floorf(t));
  float v = __fsub_rn(__fmul_rn(u, 4.0f), 2.0f);
  float w = __fsub_rn(fabsf(v), 1.0f);
  float w2 = __fmul_rn(w, w);
  float p = __fsub_rn(__fmul_rn(w2, 0.0751f), 0.6432f);
  p = __fadd_rn(__fmul_rn(p, w2), 1.5708f);
  float r = __fmul_rn(p, w);
  return v >= 0.0f ? r : -r;
}

__device__ __noinline__ double sin_cr(double x, uint32_t& st) {
  double r = px_sin(x);
  if (r != r && x == x) st |= ST_RANGE;
  return r;
}
__device__ __noinline__ double atan2_cr(double y, double x) { return px_atan2(y, x); }

// Fast-path transcendentals: CUDA's own double sin/atan2 (documented maximum
// error 2 ulp) decide a paint threshold when the result is farther than
// FAST_ULPS ulps (8x the documented bound) from it; otherwise the correctly
// rounded routines above decide.  Either way the decision equals the one the
// correctly rounded value gives.
constexpr double FAST_ULPS = 16.0;
__device__ __forceinline__ double ulp_of(double v) { return fabs(v) * 0x1p-52 + 0x1p-1074; }

// floor(((a + PI) / (2 PI)) * 8) for the chip-stack stripes, where a = atan2(y, x).
// The map a -> q is monotone, so q at a -/+ the error bound brackets the exact q.
__device__ __forceinline__ double stripe_index(double y, double x, uint32_t& st) {
  const double PI = 3.141592653589793;
  double a = atan2(y, x);
  double e = FAST_ULPS * ulp_of(a);
  double qlo = floor((((a - e) + PI) / (2 * PI)) * 8), qhi = floor((((a + e) + PI) / (2 * PI)) * 8);
  if (qlo == qhi) return qlo;
  double ac = atan2_cr(y, x);
  return floor(((ac + PI) / (2 * PI)) * 8);
}

// Math.hypot(a, b) < r and Math.hypot(a, b) > r, decided from s = a*a + b*b
// against r*r where that is certain, else from the engine's hypot itself.
// The engine's result H is within 2^-50 (relative) of the exact E = sqrt(a^2 +
// b^2), and s within 2^-52 of E^2 (plus underflow, absolute 2^-1073): s below
// r*r (1 - 2^-40) gives E < r (1 - 2^-42), so H < r; s above r*r (1 + 2^-40)
// gives E > r (1 + 2^-43), so H > r.  Inputs are finite (|a|, |b| <= 2^11 m)
// and r > 2^-100 (checked), so nothing overflows and the underflow is far
// below the margin.
__device__ __forceinline__ int hypot_vs(double a, double b, double r) {  // -1: H < r, 1: H > r, 0: H == r
  if (r > 0x1p-100 && r < 0x1p100 && fabs(a) < 0x1p11 && fabs(b) < 0x1p11) {
    const double s = a * a + b * b, r2 = r * r;
    if (s < r2 * (1.0 - 0x1p-40)) return -1;
    if (s > r2 * (1.0 + 0x1p-40)) return 1;
  }
  const double h = px_hypot2(a, b);
  return h < r ? -1 : (h > r ? 1 : 0);
}

// One paint call at a voxel centre (metres, after the optional frame).
__device__ __noinline__ uint32_t paint_eval(uint32_t kind, const double* __restrict__ p, double x, double y, double z,
                                            uint32_t& st) {
  const double PI = 3.141592653589793;
  switch (kind) {
    case PK_CHIP: {  // penthouse.ts:371-377 (stripe only matters on the edge of even layers)
      bool edge = hypot_vs(x - __ldg(p), z - __ldg(p + 2), __ldg(p + 3)) > 0;
      double layer = fmod(floor((y - __ldg(p + 1)) / 0.0045), 2.0);
      bool stripe = false;
      if (edge && layer == 0) stripe = fmod(stripe_index(z - __ldg(p + 2), x - __ldg(p), st), 2.0) == 0;
      return vox_of(__ldg(p + 4), edge && stripe && layer == 0 ? 255 : 0);
    }
    case PK_TUFTED: {  // penthouse.ts:495-501
      double u = (z - __ldg(p)) / 0.16, v = (y - __ldg(p + 1)) / 0.16;
      double ru = px_round(u), rv = px_round(v);
      double du = u - ru, dv = v - rv;
      bool odd = fmod(ru + rv, 2.0) == 0;
      return vox_of(__ldg(p + 2), odd && hypot_vs(du, dv, 0.12) < 0 ? 200 : 0);
    }
    case PK_CARD: {  // penthouse.ts:597-600
      bool edge = fabs(x - __ldg(p) - __ldg(p + 2)) > 0.022 || fabs(z - __ldg(p + 1)) > 0.034;
      return vox_of(__ldg(p + 3), edge ? 0 : 255);
    }
    case PK_WHITE: {  // penthouse.ts:744-748
      double k = floor((x - __ldg(p)) / 0.0254);
      double f = (x - __ldg(p)) / 0.0254 - k;
      return vox_of(__ldg(p + 1), f < 0.12 ? 120 : 0);
    }
    case PK_BLACK: {  // penthouse.ts:749-756
      double u = (x - __ldg(p)) / 0.0254;
      double k = floor(u + 0.5);
      double f = u + 0.5 - k;
      double n = fmod(fmod(k - 1, 7.0) + 7, 7.0);
      bool has = n == 0 || n == 1 || n == 3 || n == 4 || n == 5;
      return has && fabs(f - 0.5) < 0.3 ? vox_of(__ldg(p + 1), 0) : 0u;
    }
    case PK_VASE: {  // penthouse.ts:810-816 (the motif only matters off the bands)
      double h = (y - __ldg(p + 1)) / __ldg(p + 3);
      bool band = (h > 0.04 && h < 0.06) || (h > 0.36 && h < 0.38) || (h > 0.47 && h < 0.49);
      bool motif = false;
      if (!band && h > 0.08 && h < 0.33) {
        const double yy = z - __ldg(p + 2), xx = x - __ldg(p);
        double a = atan2(yy, xx);
        double inner = sin(h * 30);
        double arg = a * 5 + inner * 2;
        double s = sin(arg);
        // |arg - arg_ref| <= 5 |a - a_ref| + 2 |inner - inner_ref| + rounding; sin is 1-Lipschitz
        double e = 5 * FAST_ULPS * ulp_of(a) + 2 * FAST_ULPS * ulp_of(1.0) + 8 * ulp_of(arg) + FAST_ULPS * ulp_of(1.0);
        if (s - 0.55 > e) motif = true;
        else if (0.55 - s > e) motif = false;
        else {
          double ac = atan2_cr(yy, xx);
          motif = sin_cr(ac * 5 + sin_cr(h * 30, st) * 2, st) > 0.55;
        }
      }
      return vox_of(__ldg(p + 4), band || motif ? 255 : 0);
    }
    case PK_PAINTING: {  // penthouse.ts:840-845
      double shade = 0;
      for (int i = 0; i < 9; i++) {
        const double* b = p + 1 + 4 * i;
        if (hypot_vs(x - __ldg(b), (y - __ldg(b + 1)) * 1.3, __ldg(b + 2)) < 0) shade = __ldg(b + 3);
      }
      double arg = x * 9 + y * 3;
      double s = fabs(sin(arg));
      double e = FAST_ULPS * ulp_of(1.0);
      bool stripe;
      if (s < 0.06 - e) stripe = true;
      else if (s > 0.06 + e) stripe = false;
      else stripe = fabs(sin_cr(arg, st)) < 0.06;
      return vox_of(__ldg(p), stripe ? 255 : shade);
    }
    case PK_NOISE: {  // synthetic scenes: integer hash + float32 sine
      double sc = __ldg(p + 1);
      double ix = floor(x * sc), iy = floor(y * sc), iz = floor(z * sc);
      uint32_t h = noise_hash((uint32_t)(long long)ix, (uint32_t)(long long)iy, (uint32_t)(long long)iz,
                              (uint32_t)(long long)__ldg(p));
      float jitter = __fmul_rn((float)(h & 0xffffu), 1.0f / 65536.0f);
      float a = __fmul_rn(__double2float_rn(x), __double2float_rn(__ldg(p + 2)));
      float b = __fmul_rn(__double2float_rn(y), __double2float_rn(__ldg(p + 3)));
      float c = __fmul_rn(__double2float_rn(z), __double2float_rn(__ldg(p + 4)));
      float t = __fadd_rn(__fadd_rn(__fadd_rn(a, b), c), jitter);
      float s = sin_poly_f32(t);
      return s > __double2float_rn(__ldg(p + 5)) ? (uint32_t)__ldg(p + 6) : (uint32_t)__ldg(p + 7);
    }
  }
  return 0;
}

// The correctly rounded decisions of the same paints (validation mode compares).
__device__ __noinline__ uint32_t paint_eval_cr(uint32_t kind, const double* __restrict__ p, double x, double y, double z,
                                               uint32_t& st) {
  const double PI = 3.141592653589793;
  switch (kind) {
    case PK_CHIP: {
      double a = atan2_cr(z - __ldg(p + 2), x - __ldg(p));
      bool edge = px_hypot2(x - __ldg(p), z - __ldg(p + 2)) > __ldg(p + 3);
      bool stripe = fmod(floor(((a + PI) / (2 * PI)) * 8), 2.0) == 0;
      double layer = fmod(floor((y - __ldg(p + 1)) / 0.0045), 2.0);
      return vox_of(__ldg(p + 4), edge && stripe && layer == 0 ? 255 : 0);
    }
    case PK_TUFTED: {  // the engine's hypot itself
      double u = (z - __ldg(p)) / 0.16, v = (y - __ldg(p + 1)) / 0.16;
      double ru = px_round(u), rv = px_round(v);
      bool odd = fmod(ru + rv, 2.0) == 0;
      return vox_of(__ldg(p + 2), odd && px_hypot2(u - ru, v - rv) < 0.12 ? 200 : 0);
    }
    case PK_VASE: {
      double a = atan2_cr(z - __ldg(p + 2), x - __ldg(p));
      double h = (y - __ldg(p + 1)) / __ldg(p + 3);
      bool band = (h > 0.04 && h < 0.06) || (h > 0.36 && h < 0.38) || (h > 0.47 && h < 0.49);
      bool motif = h > 0.08 && h < 0.33 && sin_cr(a * 5 + sin_cr(h * 30, st) * 2, st) > 0.55;
      return vox_of(__ldg(p + 4), band || motif ? 255 : 0);
    }
    case PK_PAINTING: {
      double shade = 0;
      for (int i = 0; i < 9; i++) {
        const double* b = p + 1 + 4 * i;
        if (px_hypot2(x - __ldg(b), (y - __ldg(b + 1)) * 1.3) < __ldg(b + 2)) shade = __ldg(b + 3);
      }
      bool stripe = fabs(sin_cr(x * 9 + y * 3, st)) < 0.06;
      return vox_of(__ldg(p), stripe ? 255 : shade);
    }
  }
  return paint_eval(kind, p, x, y, z, st);
}

}  // namespace px
