// Mixed mode: certified float32 evaluation of the paints with the most calls
// in the penthouse, tufted leather (penthouse.ts:495-501), the painting
// (penthouse.ts:840-845) and the vases (penthouse.ts:810-816).  Every float64 value the reference forms is
// enclosed in a float32 interval with directed rounding; an interval is widened
// by 2^-23 of its magnitude for each float64 rounding the reference applies
// (at most 2^-53 relative).  A decision (Math.round, a parity, a threshold) is
// taken from the intervals only when it cannot differ from the reference's;
// otherwise the call returns false and the float64 evaluation decides.
//
// Math.hypot(a, b) is computed by the engine from m = max(|a|, |b|) as
// sqrt(1 + (min/m)^2) * m with one division, one square, one compensated sum,
// one square root and one product: at most 4 roundings of 2^-53, so within
// 2^-50 relative of sqrt(a^2 + b^2); the intervals use 2^-22.
// Math.sin(t) is enclosed from sinf at a point m of t's interval: CUDA's
// sinf has a documented maximum error of 2 ulp (at most 2^-22 for results in
// [-1, 1]) and sin is 1-Lipschitz, so |sin(t) - sinf(m)| <= |t - m| + 2^-22;
// the enclosure uses the interval's full width plus 2^-21.
#pragma once
#include "paint.cuh"
#include "px_internal.cuh"
#include "sdf32.cuh"

namespace px {

// one float64 rounding of a value in the interval (relative 2^-53 <= 2^-23)
__device__ __forceinline__ Iv r64(Iv v) {
  return {__fsub_rd(v.lo, __fmul_ru(fabsf(v.lo), 0x1p-23f)), __fadd_ru(v.hi, __fmul_ru(fabsf(v.hi), 0x1p-23f))};
}
__device__ __forceinline__ Iv ivf(float2 f) { return {f.x, f.y}; }

// Math.hypot(a, b) < thr, thr enclosed as [thr.x, thr.y]: 1 true, 0 false, 2 undecided
__device__ __forceinline__ int hypot_lt32(Iv a, Iv b, float2 thr) {
  const Iv t = ilen2(a, b);
  const float hi = __fmul_ru(t.hi, 1.0f + 0x1p-22f), lo = __fmul_rd(t.lo, 1.0f - 0x1p-22f);
  if (hi < thr.x) return 1;
  if (lo >= thr.y) return 0;
  return 2;
}

// Math.round of a value in u: the integer, or NAN when undecided
__device__ __forceinline__ float round32(Iv u) {
  const float a = floorf(__fadd_rd(u.lo, 0.5f)), b = floorf(__fadd_ru(u.hi, 0.5f));
  return a == b ? a : __int_as_float(0x7fc00000);
}

// Math.sin of a value in t: sinf at a point of t, padded by t's width and sinf's error
__device__ __forceinline__ Iv isin32(Iv t) {
  const float m = fminf(fmaxf(0.5f * (t.lo + t.hi), t.lo), t.hi);
  const float sm = sinf(m);
  const float r = __fadd_ru(__fsub_ru(t.hi, t.lo), 0x1p-21f);
  return {__fsub_rd(sm, r), __fadd_ru(sm, r)};
}

// Math.atan2(y, x) for y in Y, x in X.  atan2f at a point m of the box has a
// documented maximum error of 3 ulp (below 2^-20 for results within pi);
// |grad atan2| = 1/r, so over a box at distance r_lo > 0 from the origin that
// the negative x axis (the branch cut) does not cross, atan2 differs from its
// value at m by at most |p - m| / r_lo.  ok = false for any other box.
__device__ __forceinline__ Iv iatan2_32(Iv Y, Iv X, bool& ok) {
  ok = !(X.lo < 0.f && Y.lo <= 0.f && Y.hi >= 0.f);
  const float cx = X.lo > 0.f ? X.lo : (X.hi < 0.f ? -X.hi : 0.f), cy = Y.lo > 0.f ? Y.lo : (Y.hi < 0.f ? -Y.hi : 0.f);
  const float r_lo = sqrt_lo(__fadd_rd(__fmul_rd(cx, cx), __fmul_rd(cy, cy)));
  ok = ok && r_lo > 0x1p-60f;
  const float mx = fminf(fmaxf(0.5f * (X.lo + X.hi), X.lo), X.hi), my = fminf(fmaxf(0.5f * (Y.lo + Y.hi), Y.lo), Y.hi);
  const float d = __fadd_ru(fmaxf(__fsub_ru(mx, X.lo), __fsub_ru(X.hi, mx)), fmaxf(__fsub_ru(my, Y.lo), __fsub_ru(Y.hi, my)));
  const float pad = __fadd_ru(__fdiv_ru(d, ok ? r_lo : 1.f), 0x1p-20f);
  const float m = atan2f(my, mx);
  return {__fsub_rd(m, pad), __fadd_ru(m, pad)};
}

// three-valued comparisons of a value in h with a float64 constant enclosed as
// [c.x, c.y]: 1 true, 0 false, 2 undecided; and their conjunction/disjunction
__device__ __forceinline__ int gt32(Iv h, float2 c) { return h.lo > c.y ? 1 : (h.hi <= c.x ? 0 : 2); }
__device__ __forceinline__ int lt32(Iv h, float2 c) { return h.hi < c.x ? 1 : (h.lo >= c.y ? 0 : 2); }
__device__ __forceinline__ int and3(int a, int b) { return (a == 0 || b == 0) ? 0 : (a == 1 && b == 1 ? 1 : 2); }
__device__ __forceinline__ int or3(int a, int b) { return (a == 1 || b == 1) ? 1 : (a == 0 && b == 0 ? 0 : 2); }

__device__ __forceinline__ uint32_t vox32(float mat, float shade) {
  return ((uint32_t)(int)mat & 0xffu) | (((uint32_t)(int)shade & 0xffu) << 8);
}

// The synthetic scenes' noise paint (PK_NOISE, paint.cuh) from the voxel's
// indices, in float32 with the float64 path's results: the float32 roundings of
// the voxel centre's float64 coordinates come from the world's axis tables, and
// floor(x * scale) from a float32 enclosure of the float64 product when no
// integer lies inside it (false: the float64 path decides).  q: seed bits,
// [scale] enclosure, fx, fy, fz and the threshold as float32, the two values.
__device__ __forceinline__ bool noise32(const float2* __restrict__ q, float fx, float fy, float fz, uint32_t& out) {
  const float2 sc = __ldg(q + 1);
  // the float64 coordinate lies in [pred(f), succ(f)] of its rounding f > 0; the
  // product's float64 rounding lies in the directed float32 bounds of that box
  auto cell = [&](float f, uint32_t& c) {
    const float a = floorf(__fmul_rd(__int_as_float(__float_as_int(f) - 1), sc.x));
    const float b = floorf(__fmul_ru(__int_as_float(__float_as_int(f) + 1), sc.y));
    c = (uint32_t)(int)a;
    return a == b && a < 16777216.f;
  };
  uint32_t ix, iy, iz;
  const bool okx = cell(fx, ix), oky = cell(fy, iy), okz = cell(fz, iz);
  if (!(okx && oky && okz)) return false;
  const uint32_t h = noise_hash(ix, iy, iz, __float_as_uint(__ldg(q).x));
  const float jitter = __fmul_rn((float)(h & 0xffffu), 1.0f / 65536.0f);
  const float2 f01 = __ldg(q + 2), f23 = __ldg(q + 3);
  const float t = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(fx, f01.x), __fmul_rn(fy, f01.y)), __fmul_rn(fz, f23.x)), jitter);
  const float2 vals = __ldg(q + 4);
  out = sin_poly_f32(t) > f23.y ? __float_as_uint(vals.x) : __float_as_uint(vals.y);
  return true;
}

// Float32 parameter blocks (written by the host, paint_params32 in px_api.cu),
// positions relative to the op's anchor:
//   tufted:   [0] z0, [1] floor, [2] 1/0.16, [3] 0.12, [4] (material, 0)
//   painting: [0] (9 ax + 3 ay) mod 2 pi, [1] 1.3, [2] 0.06, [3] (material, 0),
//             [4 + 4i] blob x, [5 + 4i] blob y, [6 + 4i] blob r, [7 + 4i] (shade, 0)
//   vase:     [0] x0, [1] y0, [2] z0, [3] 1/height, [4..12] 0.04, 0.06, 0.36, 0.38,
//             0.47, 0.49, 0.08, 0.33, 0.55, [13] (material, 0)
// (rx, ry, rz): the voxel centre relative to the anchor.
__device__ __forceinline__ bool paint32(uint32_t kind, const float2* __restrict__ q, Iv rx, Iv ry, Iv rz,
                                        uint32_t& out) {
  if (kind == PK_TUFTED) {
    const Iv inv = ivf(__ldg(q + 2));
    const Iv u = r64(icmul(r64(isub(rz, ivf(__ldg(q + 0)))), inv));  // (z - z0) / 0.16
    const Iv v = r64(icmul(r64(isub(ry, ivf(__ldg(q + 1)))), inv));  // (y - floor) / 0.16
    const float nu = round32(u), nv = round32(v);
    if (nu != nu || nv != nv) return false;
    const float mat = __ldg(q + 4).x;
    if (((int)nu + (int)nv) & 1) { out = vox32(mat, 0.f); return true; }  // (ru + rv) % 2 != 0
    const Iv du = {__fsub_rd(u.lo, nu), __fsub_ru(u.hi, nu)}, dv = {__fsub_rd(v.lo, nv), __fsub_ru(v.hi, nv)};
    const int h = hypot_lt32(du, dv, __ldg(q + 3));
    if (h == 2) return false;
    out = vox32(mat, h ? 200.f : 0.f);
    return true;
  }
  if (kind == PK_PAINTING) {
    const Iv k13 = ivf(__ldg(q + 1));
    float shade = 0.f;
#pragma unroll 1
    for (int i = 0; i < 9; i++) {
      const float2* b = q + 4 + 4 * i;
      const Iv a = r64(isub(rx, ivf(__ldg(b))));                    // x - bx
      const Iv c = r64(icmul(r64(isub(ry, ivf(__ldg(b + 1)))), k13));  // (y - by) * 1.3
      const int h = hypot_lt32(a, c, __ldg(b + 2));
      if (h == 2) return false;
      if (h) shade = __ldg(b + 3).x;
    }
    // x * 9 + y * 3, reduced by a multiple of 2 pi (exact for the real value)
    Iv t = iadd(ivf(__ldg(q + 0)), iadd(icmul(rx, iv(9.f)), icmul(ry, iv(3.f))));
    t = {__fsub_rd(t.lo, 0x1p-40f), __fadd_ru(t.hi, 0x1p-40f)};  // the reference's roundings of x*9 + y*3
    const Iv s = iabs(isin32(t));
    const float2 thr = __ldg(q + 2);
    bool stripe;
    if (s.hi < thr.x) stripe = true;
    else if (s.lo >= thr.y) stripe = false;
    else return false;
    out = vox32(__ldg(q + 3).x, stripe ? 255.f : shade);
    return true;
  }
  if (kind == PK_VASE) {
    const Iv h = r64(icmul(r64(isub(ry, ivf(__ldg(q + 1)))), ivf(__ldg(q + 3))));  // (y - y0) / height
    const int band = or3(and3(gt32(h, __ldg(q + 4)), lt32(h, __ldg(q + 5))),
                         or3(and3(gt32(h, __ldg(q + 6)), lt32(h, __ldg(q + 7))),
                             and3(gt32(h, __ldg(q + 8)), lt32(h, __ldg(q + 9)))));
    if (band == 2) return false;
    const float mat = __ldg(q + 13).x;
    if (band == 1) { out = vox32(mat, 255.f); return true; }
    const int mid = and3(gt32(h, __ldg(q + 10)), lt32(h, __ldg(q + 11)));
    if (mid == 2) return false;
    if (mid == 0) { out = vox32(mat, 0.f); return true; }
    bool ok;
    const Iv a = iatan2_32(r64(isub(rz, ivf(__ldg(q + 2)))), r64(isub(rx, ivf(__ldg(q + 0)))), ok);
    if (!ok) return false;
    const Iv inner = isin32(r64(icmul(h, iv(30.f))));                       // sin(h * 30)
    const Iv arg = r64(iadd(r64(icmul(a, iv(5.f))), icmul(inner, iv(2.f))));  // a * 5 + inner * 2
    const int motif = gt32(isin32(arg), __ldg(q + 12));
    if (motif == 2) return false;
    out = vox32(mat, motif ? 255.f : 0.f);
    return true;
  }
  return false;
}

}  // namespace px
