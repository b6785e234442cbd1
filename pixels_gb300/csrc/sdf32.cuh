// Float32 interval evaluator of the SDF bytecode (the mixed build mode).
//
// Every quantity is an interval [lo, hi] of float32 computed with directed
// rounding (__f*_rd / __f*_ru), so it encloses the exact real value of the
// reference expression evaluated on the exact float64 inputs.  Coordinates
// are relative to a per-op anchor (the centre of the op's bounds), which
// keeps magnitudes at the op's extent instead of the world's.  The reference's
// float64 result differs from that exact value by far less than the margin M
// (2^-30 m for |coordinates| <= 2^10 m), so a decision whose threshold lies
// outside [lo - M, hi + M] is the reference's decision; anything else — and
// any polygon crossing test that the intervals cannot settle — is re-done in
// float64 (sdf64.cuh).  Only multiplications by constant intervals and squares
// occur, so no general interval product is needed.
#pragma once
#include "px_internal.cuh"

#ifndef PX_SDF32I_INLINE
#define PX_SDF32I_INLINE __forceinline__
#endif

namespace px {

struct Iv {
  float lo, hi;
};

__device__ __forceinline__ Iv iv(float a) { return {a, a}; }
__device__ __forceinline__ Iv iadd(Iv a, Iv b) { return {__fadd_rd(a.lo, b.lo), __fadd_ru(a.hi, b.hi)}; }
__device__ __forceinline__ Iv isub(Iv a, Iv b) { return {__fsub_rd(a.lo, b.hi), __fsub_ru(a.hi, b.lo)}; }
__device__ __forceinline__ Iv ineg(Iv a) { return {-a.hi, -a.lo}; }
// |a|: the least magnitude is max(lo, -hi, 0) and the largest max(-lo, hi), the
// same bounds as the case split, in three min/max operations and no selects
__device__ __forceinline__ Iv iabs(Iv a) { return {fmaxf(fmaxf(a.lo, -a.hi), 0.f), fmaxf(-a.lo, a.hi)}; }
__device__ __forceinline__ Iv imax0(Iv a) { return {fmaxf(a.lo, 0.f), fmaxf(a.hi, 0.f)}; }
__device__ __forceinline__ Iv imin0(Iv a) { return {fminf(a.lo, 0.f), fminf(a.hi, 0.f)}; }
__device__ __forceinline__ Iv imax(Iv a, Iv b) { return {fmaxf(a.lo, b.lo), fmaxf(a.hi, b.hi)}; }
__device__ __forceinline__ Iv imin(Iv a, Iv b) { return {fminf(a.lo, b.lo), fminf(a.hi, b.hi)}; }
__device__ __forceinline__ Iv iclamp01(Iv a) { return {fminf(fmaxf(a.lo, 0.f), 1.f), fminf(fmaxf(a.hi, 0.f), 1.f)}; }
__device__ __forceinline__ Iv isqr(Iv a) {
  const Iv m = iabs(a);  // the least and largest magnitude
  return {__fmul_rd(m.lo, m.lo), __fmul_ru(m.hi, m.hi)};
}
// Bounds of sqrt(v), v >= 0, from the hardware reciprocal square root.  CUDA
// documents rsqrtf's maximum error as 2 ulp: 1/sqrt(v) = r (1 + d) with
// |d| <= 2^-22, so sqrt(v) = v r (1 + d).  v r rounded down and shrunk by
// (1 - 2^-20), resp. rounded up and grown by (1 + 2^-20), lies below, resp.
// above sqrt(v), with a factor-4 margin on the documented bound.  This costs a
// few instructions where the IEEE directed square roots (__fsqrt_rd/_ru) run a
// long sequence, longer still at zero.  Outside [2^-100, 2^100]: 0 and 2^-50
// bound the square roots of smaller values; larger ones (and infinity) take
// the IEEE directed square roots.
__device__ __forceinline__ float sqrt_lo(float v) {
  if (v < 0x1p-100f) return 0.f;
  if (v > 0x1p100f) return __fsqrt_rd(v);
  return __fmul_rd(__fmul_rd(v, rsqrtf(v)), 1.f - 0x1p-20f);
}
__device__ __forceinline__ float sqrt_hi(float v) {
  if (v < 0x1p-100f) return v > 0.f ? 0x1p-50f : 0.f;
  if (v > 0x1p100f) return __fsqrt_ru(v);
  return __fmul_ru(__fmul_ru(v, rsqrtf(v)), 1.f + 0x1p-20f);
}
__device__ __forceinline__ Iv isqrt(Iv a) { return {sqrt_lo(fmaxf(a.lo, 0.f)), sqrt_hi(fmaxf(a.hi, 0.f))}; }
// x * c for a constant interval c that does not straddle zero (or is [0, 0]): the
// sign of x picks which end of c bounds each product, so the bound is the lesser
// (greater) of the two directed products -- two multiplies and a min/max in place
// of a compare and a select
__device__ __forceinline__ Iv icmul(Iv x, Iv c) {
  if (c.lo >= 0.f)
    return {fminf(__fmul_rd(x.lo, c.lo), __fmul_rd(x.lo, c.hi)), fmaxf(__fmul_ru(x.hi, c.hi), __fmul_ru(x.hi, c.lo))};
  return {fminf(__fmul_rd(x.hi, c.lo), __fmul_rd(x.hi, c.hi)), fmaxf(__fmul_ru(x.lo, c.hi), __fmul_ru(x.lo, c.lo))};
}
// x * c for any constant interval c (one that straddles zero is bounded by its magnitude)
__device__ __forceinline__ Iv icmul_any(Iv x, Iv c) {
  if (c.lo >= 0.f || c.hi <= 0.f) return icmul(x, c);
  const float m = __fmul_ru(fmaxf(-c.lo, c.hi), fmaxf(fabsf(x.lo), fabsf(x.hi)));
  return {-m, m};
}
__device__ __forceinline__ Iv ilen2(Iv a, Iv b) { return isqrt(iadd(isqr(a), isqr(b))); }
__device__ __forceinline__ Iv ilen3(Iv a, Iv b, Iv c) { return isqrt(iadd(iadd(isqr(a), isqr(b)), isqr(c))); }
__device__ __forceinline__ Iv ldp(const Iv* p, int k) {
  float2 v = __ldg(reinterpret_cast<const float2*>(p) + k);
  return {v.x, v.y};
}

// b + a0 u + a1 v for intervals b, u, v and (constant) intervals a0, a1, in
// centre-radius form with directed fused multiply-adds and no sign selects: with
// w in [w.lo, w.lo + dw] and a in [a.lo, a.lo + da], a w - a.lo w.lo lies within
// +-(|a.lo| dw + da (|w.lo| + dw)); the centre sum is bounded below and above by
// chains of __fmaf_rd / __fmaf_ru (each rounds an exact a b + c), and the result is
// [lower - R, upper + R + width(b)], every step rounded outward.  Cheaper on the
// ALU pipe than the products' min/max of interval arithmetic.
__device__ __forceinline__ Iv lin2(Iv b, Iv a0, Iv u, Iv a1, Iv v) {
  const float du = __fsub_ru(u.hi, u.lo), dv = __fsub_ru(v.hi, v.lo);
  const float lo = __fmaf_rd(a1.lo, v.lo, __fmaf_rd(a0.lo, u.lo, b.lo));
  const float hi = __fmaf_ru(a1.lo, v.lo, __fmaf_ru(a0.lo, u.lo, b.lo));
  float R = __fmaf_ru(fabsf(a0.lo), du, __fmul_ru(fabsf(a1.lo), dv));
  R = __fmaf_ru(__fsub_ru(a0.hi, a0.lo), __fadd_ru(fabsf(u.lo), du), R);
  R = __fmaf_ru(__fsub_ru(a1.hi, a1.lo), __fadd_ru(fabsf(v.lo), dv), R);
  return {__fsub_rd(lo, R), __fadd_ru(__fadd_ru(hi, R), __fsub_ru(b.hi, b.lo))};
}
// b + a u, the same way
__device__ __forceinline__ Iv lin1(Iv b, Iv a, Iv u) {
  const float du = __fsub_ru(u.hi, u.lo);
  const float lo = __fmaf_rd(a.lo, u.lo, b.lo), hi = __fmaf_ru(a.lo, u.lo, b.lo);
  const float R = __fmaf_ru(__fsub_ru(a.hi, a.lo), __fadd_ru(fabsf(u.lo), du), __fmul_ru(fabsf(a.lo), du));
  return {__fsub_rd(lo, R), __fadd_ru(__fadd_ru(hi, R), __fsub_ru(b.hi, b.lo))};
}

// shapes.ts:146-161 on intervals.  Records per vertex i: vix, viy, vjy, ex, ey, 1/den.
__device__ __forceinline__ Iv sd_polygon32(Iv px_, Iv py_, const Iv* __restrict__ r, int n, float M, bool& amb) {
  Iv d = iadd(isqr(isub(px_, ldp(r, 0))), isqr(isub(py_, ldp(r, 1))));
  bool flip_all = false;
  for (int i = 0; i < n; i++) {
    const Iv* e = r + 6 * i;
    Iv vix = ldp(e, 0), viy = ldp(e, 1), vjy = ldp(e, 2), ex = ldp(e, 3), ey = ldp(e, 4), inv = ldp(e, 5);
    Iv wx = isub(px_, vix), wy = isub(py_, viy);
    Iv t = iclamp01(icmul(lin2({0.f, 0.f}, ex, wx, ey, wy), inv));
    Iv bx = lin1(wx, ineg(ex), t), by = lin1(wy, ineg(ey), t);
    d = imin(d, iadd(isqr(bx), isqr(by)));
    // crossing test (c1 && c2 && c3) || (!c1 && !c2 && !c3), decided only when certain
    bool c1t = py_.lo >= __fadd_ru(viy.hi, M), c1f = py_.hi < __fsub_rd(viy.lo, M);
    bool c2t = py_.hi < __fsub_rd(vjy.lo, M), c2f = py_.lo >= __fadd_ru(vjy.hi, M);
    if (!(c1t || c1f) || !(c2t || c2f)) { amb = true; continue; }
    if (c1t != c2t) continue;  // no flip whatever c3 is
    Iv L = icmul(wy, ex), R = icmul(wx, ey);
    float m3 = __fadd_ru(__fmul_ru(__fadd_ru(fmaxf(fabsf(L.lo), fabsf(L.hi)), fmaxf(fabsf(R.lo), fabsf(R.hi))), 0x1p-40f), 0x1p-60f);
    bool c3t = L.lo > __fadd_ru(R.hi, m3), c3f = L.hi < __fsub_rd(R.lo, m3);
    if (!(c3t || c3f)) { amb = true; continue; }
    if (c1t ? c3t : !c3t) flip_all = !flip_all;
  }
  Iv s = isqrt(d);
  return flip_all ? ineg(s) : s;
}

// shapes.ts:164-173 on intervals.  Records per segment: ax, ay, ex, ey, 1/den.
__device__ __forceinline__ Iv sd_polyline32(Iv px_, Iv py_, const Iv* __restrict__ r, int nseg) {
  Iv d = {INFINITY, INFINITY};
  for (int i = 0; i < nseg; i++) {
    const Iv* e = r + 5 * i;
    Iv ex = ldp(e, 2), ey = ldp(e, 3), inv = ldp(e, 4);
    Iv wx = isub(px_, ldp(e, 0)), wy = isub(py_, ldp(e, 1));
    Iv t = iclamp01(icmul(lin2({0.f, 0.f}, ex, wx, ey, wy), inv));
    d = imin(d, iadd(isqr(lin1(wx, ineg(ex), t)), isqr(lin1(wy, ineg(ey), t))));
  }
  return isqrt(d);
}

__device__ __forceinline__ Iv prim32(uint32_t op, int cnt, const Iv* __restrict__ p, Iv x, Iv y, Iv z, float M, bool& amb) {
  switch (op) {
    case OP_BOX: case OP_ROUNDBOX: {
      Iv qx = isub(iabs(isub(x, ldp(p, 0))), ldp(p, 3)), qy = isub(iabs(isub(y, ldp(p, 1))), ldp(p, 4)),
         qz = isub(iabs(isub(z, ldp(p, 2))), ldp(p, 5));
      Iv r = iadd(ilen3(imax0(qx), imax0(qy), imax0(qz)), imin0(imax(imax(qx, qy), qz)));
      return op == OP_BOX ? r : isub(r, ldp(p, 6));
    }
    case OP_SPHERE:
      return isub(ilen3(isub(x, ldp(p, 0)), isub(y, ldp(p, 1)), isub(z, ldp(p, 2))), ldp(p, 3));
    case OP_ELLIPSOID: {  // params hold 1/rx, 1/ry, 1/rz
      Iv l = ilen3(icmul(isub(x, ldp(p, 0)), ldp(p, 3)), icmul(isub(y, ldp(p, 1)), ldp(p, 4)),
                   icmul(isub(z, ldp(p, 2)), ldp(p, 5)));
      return icmul(isub(l, iv(1.f)), ldp(p, 6));
    }
    case OP_CYL_X: case OP_CYL_Y: case OP_CYL_Z: {
      Iv a, b, h;
      if (op == OP_CYL_Y) { a = isub(x, ldp(p, 0)); b = isub(z, ldp(p, 2)); h = isub(y, ldp(p, 1)); }
      else if (op == OP_CYL_X) { a = isub(y, ldp(p, 1)); b = isub(z, ldp(p, 2)); h = isub(x, ldp(p, 0)); }
      else { a = isub(x, ldp(p, 0)); b = isub(y, ldp(p, 1)); h = isub(z, ldp(p, 2)); }
      Iv dr = isub(ilen2(a, b), ldp(p, 3)), dh = isub(iabs(h), ldp(p, 4));
      return iadd(imin0(imax(dr, dh)), ilen2(imax0(dr), imax0(dh)));
    }
    case OP_CAPSULE: {  // params: a, ba, 1/bb, r
      Iv px_ = isub(x, ldp(p, 0)), py_ = isub(y, ldp(p, 1)), pz_ = isub(z, ldp(p, 2));
      Iv bax = ldp(p, 3), bay = ldp(p, 4), baz = ldp(p, 5);
      Iv h = iclamp01(icmul(iadd(iadd(icmul(px_, bax), icmul(py_, bay)), icmul(pz_, baz)), ldp(p, 6)));
      return isub(ilen3(isub(px_, icmul(h, bax)), isub(py_, icmul(h, bay)), isub(pz_, icmul(h, baz))), ldp(p, 7));
    }
    case OP_TORUS_X: case OP_TORUS_Y: case OP_TORUS_Z: {
      Iv a, b, h;
      if (op == OP_TORUS_Y) { a = isub(x, ldp(p, 0)); b = isub(z, ldp(p, 2)); h = isub(y, ldp(p, 1)); }
      else if (op == OP_TORUS_X) { a = isub(y, ldp(p, 1)); b = isub(z, ldp(p, 2)); h = isub(x, ldp(p, 0)); }
      else { a = isub(x, ldp(p, 0)); b = isub(y, ldp(p, 1)); h = isub(z, ldp(p, 2)); }
      return isub(ilen2(isub(ilen2(a, b), ldp(p, 3)), h), ldp(p, 4));
    }
    case OP_LATHE_SOLID:
      return sd_polygon32(ilen2(isub(x, ldp(p, 0)), isub(z, ldp(p, 2))), isub(y, ldp(p, 1)), p + 3, cnt, M, amb);
    case OP_LATHE_SHELL:
      return isub(sd_polyline32(ilen2(isub(x, ldp(p, 0)), isub(z, ldp(p, 2))), isub(y, ldp(p, 1)), p + 4, cnt - 1),
                  ldp(p, 3));
    case OP_PRISM: {
      Iv d2 = sd_polygon32(isub(x, ldp(p, 0)), isub(z, ldp(p, 1)), p + 4, cnt, M, amb);
      Iv dy = isub(iabs(isub(y, ldp(p, 2))), ldp(p, 3));
      return iadd(imin0(imax(d2, dy)), ilen2(imax0(d2), imax0(dy)));
    }
    case OP_STADIUM: {  // Math.hypot encloses like len2
      Iv dx = imax0(isub(iabs(isub(x, ldp(p, 0))), ldp(p, 2)));
      Iv d2 = isub(ilen2(dx, isub(z, ldp(p, 1))), ldp(p, 3));
      Iv dy = isub(iabs(isub(y, ldp(p, 4))), ldp(p, 5));
      return iadd(imin0(imax(d2, dy)), ilen2(imax0(d2), imax0(dy)));
    }
  }
  return {-INFINITY, INFINITY};
}

// A run of rotations composed into x' = M x + t (code32 flag C32_AFFINE): p holds
// M row by row, then t, as constant intervals.  In centre-radius form, with
// directed fused multiply-adds and no sign selects: x_j lies in [c_j, c_j + d_j]
// (c_j its lower bound, d_j its width rounded up) and M_rj in [m, m + e], so
// M_rj x_j - m c_j = m (x_j - c_j) + (M_rj - m) x_j lies in [-R_rj, R_rj] with
// R_rj = |m| d_j + e (|c_j| + d_j); sum_j m c_j + t.lo is bounded below and above
// by chains of __fmaf_rd / __fmaf_ru (each rounds an exact a b + c), and the
// row's interval is [lower - R, upper + R + (t.hi - t.lo)], every step outward.
__device__ __forceinline__ void aff32(const Iv* __restrict__ p, Iv& x, Iv& y, Iv& z) {
  const float c[3] = {x.lo, y.lo, z.lo};
  const float d[3] = {__fsub_ru(x.hi, x.lo), __fsub_ru(y.hi, y.lo), __fsub_ru(z.hi, z.lo)};
  const float g[3] = {__fadd_ru(fabsf(c[0]), d[0]), __fadd_ru(fabsf(c[1]), d[1]), __fadd_ru(fabsf(c[2]), d[2])};
  Iv o[3];
#pragma unroll
  for (int r = 0; r < 3; r++) {
    const Iv t = ldp(p, 9 + r);
    float lo = t.lo, hi = t.lo, R = 0.f;
#pragma unroll
    for (int j = 0; j < 3; j++) {
      const Iv m = ldp(p, 3 * r + j);
      lo = __fmaf_rd(m.lo, c[j], lo);
      hi = __fmaf_ru(m.lo, c[j], hi);
      R = __fmaf_ru(fabsf(m.lo), d[j], R);
      R = __fmaf_ru(__fsub_ru(m.hi, m.lo), g[j], R);
    }
    o[r] = {__fsub_rd(lo, R), __fadd_ru(__fadd_ru(hi, R), __fsub_ru(t.hi, t.lo))};
  }
  x = o[0];
  y = o[1];
  z = o[2];
}

// code32[i] is the offset of instruction i's float32 parameters (C32_OFF bits),
// with the flags of a composed run of rotations (C32_AFFINE, C32_SKIP).
__device__ PX_SDF32I_INLINE Iv sdf32i(const uint2* __restrict__ code, const uint32_t* __restrict__ code32, int n,
                                  const Iv* __restrict__ P, Iv x, Iv y, Iv z, float M, bool& amb) {
  Iv s0 = {0.f, 0.f}, s1 = s0, s2 = s0, s3 = s0;
  Iv ax0 = s0, ay0 = s0, az0 = s0, ax1 = s0, ay1 = s0, az1 = s0, ax2 = s0, ay2 = s0, az2 = s0;
  for (int i = 0; i < n; i++) {
    const uint32_t w0 = __ldg(&code[i].x);
    const uint32_t op = w0 & 0xffu;
    const int cnt = (int)(w0 >> 8);
    const uint32_t c32 = __ldg(code32 + i);
    if (c32 & C32_SKIP) continue;
    const Iv* p = P + (c32 & C32_OFF);
    if (op < OP_ROT_X) {
      Iv v = prim32(op, cnt, p, x, y, z, M, amb);
      s3 = s2; s2 = s1; s1 = s0; s0 = v;
      continue;
    }
    switch (op) {
      case OP_ROT_X: case OP_ROT_Y: case OP_ROT_Z: {
        ax2 = ax1; ay2 = ay1; az2 = az1; ax1 = ax0; ay1 = ay0; az1 = az0; ax0 = x; ay0 = y; az0 = z;
        if (c32 & C32_AFFINE) {
          aff32(p, x, y, z);
          break;
        }
        Iv p0 = ldp(p, 0), p1 = ldp(p, 1), c = ldp(p, 2), sn = ldp(p, 3);
        if (op == OP_ROT_Y) {
          Iv dx = isub(x, p0), dz = isub(z, p1);
          x = iadd(iadd(p0, icmul(dx, c)), icmul(dz, sn));
          z = iadd(isub(p1, icmul(dx, sn)), icmul(dz, c));
        } else if (op == OP_ROT_X) {
          Iv dy = isub(y, p0), dz = isub(z, p1);
          y = iadd(iadd(p0, icmul(dy, c)), icmul(dz, sn));
          z = iadd(isub(p1, icmul(dy, sn)), icmul(dz, c));
        } else {
          Iv dx = isub(x, p0), dy = isub(y, p1);
          x = iadd(iadd(p0, icmul(dx, c)), icmul(dy, sn));
          y = iadd(isub(p1, icmul(dx, sn)), icmul(dy, c));
        }
        break;
      }
      case OP_ROT_END:
        x = ax0; y = ay0; z = az0; ax0 = ax1; ay0 = ay1; az0 = az1; ax1 = ax2; ay1 = ay2; az1 = az2;
        break;
      case OP_OFFSET: s0 = iadd(s0, ldp(p, 0)); break;
      case OP_NEGMAX: { Iv b = s0; s0 = s1; s1 = s2; s2 = s3; s0 = imax(s0, ineg(b)); break; }
      case OP_MAX: { Iv b = s0; s0 = s1; s1 = s2; s2 = s3; s0 = imax(s0, b); break; }
      case OP_MIN: { Iv b = s0; s0 = s1; s1 = s2; s2 = s3; s0 = imin(s0, b); break; }
    }
  }
  return s0;
}


// Shapes whose code uses only primitives extruded along y (box, rounded box,
// cylinder and torus about y, stadium, prism), rotations about y and the
// combinators: the x/z part of every primitive is the same for all voxels of a
// column, so two voxels of one column (same x, z; y0, y1) are evaluated in one
// pass, sharing that part (a prism's polygon distance, a cylinder's radius...).
// Each result encloses the same expression as sdf32i's, in the same order of
// operations on every value.
__host__ __device__ constexpr bool op_is_y_separable(uint32_t op) {
  return op == OP_BOX || op == OP_ROUNDBOX || op == OP_CYL_Y || op == OP_TORUS_Y || op == OP_STADIUM ||
         op == OP_PRISM || op == OP_ROT_Y || op == OP_ROT_END || op == OP_OFFSET || op == OP_NEGMAX ||
         op == OP_MAX || op == OP_MIN;
}

struct Iv2 {
  Iv a, b;  // the values at y0 and y1
};

__device__ __forceinline__ Iv2 prim32_y2(uint32_t op, int cnt, const Iv* __restrict__ p, Iv x, Iv y0, Iv y1, Iv z,
                                         float M, bool& amb) {
  switch (op) {
    case OP_BOX: case OP_ROUNDBOX: {
      const Iv qx = isub(iabs(isub(x, ldp(p, 0))), ldp(p, 3)), qz = isub(iabs(isub(z, ldp(p, 2))), ldp(p, 5));
      const Iv sx = isqr(imax0(qx)), sz = isqr(imax0(qz)), mxz = qx;
      const Iv cy = ldp(p, 1), hy = ldp(p, 4);
      Iv out[2];
#pragma unroll
      for (int k = 0; k < 2; k++) {
        const Iv qy = isub(iabs(isub(k ? y1 : y0, cy)), hy);
        out[k] = iadd(isqrt(iadd(iadd(sx, isqr(imax0(qy))), sz)), imin0(imax(imax(mxz, qy), qz)));
      }
      if (op == OP_ROUNDBOX) {
        const Iv r = ldp(p, 6);
        out[0] = isub(out[0], r);
        out[1] = isub(out[1], r);
      }
      return {out[0], out[1]};
    }
    case OP_CYL_Y: {
      const Iv dr = isub(ilen2(isub(x, ldp(p, 0)), isub(z, ldp(p, 2))), ldp(p, 3));
      const Iv cy = ldp(p, 1), hh = ldp(p, 4);
      Iv out[2];
#pragma unroll
      for (int k = 0; k < 2; k++) {
        const Iv dh = isub(iabs(isub(k ? y1 : y0, cy)), hh);
        out[k] = iadd(imin0(imax(dr, dh)), ilen2(imax0(dr), imax0(dh)));
      }
      return {out[0], out[1]};
    }
    case OP_TORUS_Y: {
      const Iv t = isub(ilen2(isub(x, ldp(p, 0)), isub(z, ldp(p, 2))), ldp(p, 3));
      const Iv cy = ldp(p, 1), r = ldp(p, 4);
      return {isub(ilen2(t, isub(y0, cy)), r), isub(ilen2(t, isub(y1, cy)), r)};
    }
    case OP_STADIUM: {
      const Iv dx = imax0(isub(iabs(isub(x, ldp(p, 0))), ldp(p, 2)));
      const Iv d2 = isub(ilen2(dx, isub(z, ldp(p, 1))), ldp(p, 3));
      const Iv cy = ldp(p, 4), hh = ldp(p, 5);
      Iv out[2];
#pragma unroll
      for (int k = 0; k < 2; k++) {
        const Iv dy = isub(iabs(isub(k ? y1 : y0, cy)), hh);
        out[k] = iadd(imin0(imax(d2, dy)), ilen2(imax0(d2), imax0(dy)));
      }
      return {out[0], out[1]};
    }
    case OP_PRISM: {
      const Iv d2 = sd_polygon32(isub(x, ldp(p, 0)), isub(z, ldp(p, 1)), p + 4, cnt, M, amb);
      const Iv cy = ldp(p, 2), hh = ldp(p, 3);
      Iv out[2];
#pragma unroll
      for (int k = 0; k < 2; k++) {
        const Iv dy = isub(iabs(isub(k ? y1 : y0, cy)), hh);
        out[k] = iadd(imin0(imax(d2, dy)), ilen2(imax0(d2), imax0(dy)));
      }
      return {out[0], out[1]};
    }
  }
  return {{-INFINITY, INFINITY}, {-INFINITY, INFINITY}};
}

// sdf32i for a y-separable shape at (x, y0, z) and (x, y1, z).
__device__ __forceinline__ Iv2 sdf32i_y2(const uint2* __restrict__ code, const uint32_t* __restrict__ code32, int n,
                                         const Iv* __restrict__ P, Iv x, Iv y0, Iv y1, Iv z, float M, bool& amb) {
  const Iv zero = {0.f, 0.f};
  Iv2 s0 = {zero, zero}, s1 = s0, s2 = s0, s3 = s0;
  Iv ax0 = zero, az0 = zero, ax1 = zero, az1 = zero, ax2 = zero, az2 = zero;
  for (int i = 0; i < n; i++) {
    const uint32_t w0 = __ldg(&code[i].x);
    const uint32_t op = w0 & 0xffu;
    const int cnt = (int)(w0 >> 8);
    const Iv* p = P + (__ldg(code32 + i) & C32_OFF);  // no composed runs in y-extruded programs
    switch (op) {
      case OP_ROT_Y: {  // rotations about y keep y: x and z only
        ax2 = ax1; az2 = az1; ax1 = ax0; az1 = az0; ax0 = x; az0 = z;
        const Iv p0 = ldp(p, 0), p1 = ldp(p, 1), c = ldp(p, 2), sn = ldp(p, 3);
        const Iv dx = isub(x, p0), dz = isub(z, p1);
        x = iadd(iadd(p0, icmul(dx, c)), icmul(dz, sn));
        z = iadd(isub(p1, icmul(dx, sn)), icmul(dz, c));
        break;
      }
      case OP_ROT_END:
        x = ax0; z = az0; ax0 = ax1; az0 = az1; ax1 = ax2; az1 = az2;
        break;
      case OP_OFFSET: {
        const Iv o = ldp(p, 0);
        s0 = {iadd(s0.a, o), iadd(s0.b, o)};
        break;
      }
      case OP_NEGMAX: case OP_MAX: case OP_MIN: {
        const Iv2 b = s0;
        s0 = s1; s1 = s2; s2 = s3;
        if (op == OP_NEGMAX) s0 = {imax(s0.a, ineg(b.a)), imax(s0.b, ineg(b.b))};
        else if (op == OP_MAX) s0 = {imax(s0.a, b.a), imax(s0.b, b.b)};
        else s0 = {imin(s0.a, b.a), imin(s0.b, b.b)};
        break;
      }
      default: {
        const Iv2 v = prim32_y2(op, cnt, p, x, y0, y1, z, M, amb);
        s3 = s2; s2 = s1; s1 = s0; s0 = v;
      }
    }
  }
  return s0;
}

}  // namespace px
