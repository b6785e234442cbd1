// JavaScript Math functions the voxeliser's paint and SDF code calls per voxel,
// written for host and device with identical operation sequences, so the GPU
// and any host build produce the same bits.
//
//   px_hypot2   Math.hypot(a, b): scale by the larger magnitude, sum the squares
//               with Kahan compensated summation, sqrt, rescale.  (Not
//               sqrt(a*a+b*b) and not C hypot: the engine method.)
//   px_round    Math.round: round half toward +infinity.
//   px_sin      Math.sin, correctly rounded in practice: Cody-Waite reduction by
//               pi/2 in three pieces (exact products through fma), then the
//               Taylor series of sin/cos in double-double arithmetic.
//   px_atan2    Math.atan2, correctly rounded in practice: quotient in
//               double-double, table reduction atan(t) = atan(k/32) +
//               atan((t - k/32) / (1 + t k/32)), Taylor series of atan in
//               double-double, quadrant fix-up in double-double.
// Double-double building blocks are Dekker/Knuth TwoSum, FastTwoSum and an
// fma-based TwoProduct (Bailey's double-double arithmetic).  A correctly
// rounded result matches any other correctly rounded implementation (and the C
// library wherever it rounds correctly).  px_sin's argument must satisfy
// |x| < 2^28; larger arguments return NaN (callers flag a range error).
#pragma once
#include <math.h>
#include "jsmath_tables.h"

#ifdef __CUDACC__
#define PX_HD __host__ __device__ __forceinline__
#else
#define PX_HD static inline
#endif

struct px_dd { double hi, lo; };

PX_HD px_dd px_two_sum(double a, double b) {
  double s = a + b;
  double bb = s - a;
  double e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
PX_HD px_dd px_fast_two_sum(double a, double b) {  // requires |a| >= |b| or a == 0
  double s = a + b;
  double e = b - (s - a);
  return {s, e};
}
PX_HD px_dd px_two_prod(double a, double b) {
  double p = a * b;
  double e = fma(a, b, -p);
  return {p, e};
}
PX_HD px_dd px_dd_add(px_dd a, px_dd b) {
  px_dd s = px_two_sum(a.hi, b.hi);
  px_dd t = px_two_sum(a.lo, b.lo);
  s.lo = s.lo + t.hi;
  s = px_fast_two_sum(s.hi, s.lo);
  s.lo = s.lo + t.lo;
  return px_fast_two_sum(s.hi, s.lo);
}
PX_HD px_dd px_dd_neg(px_dd a) { return {-a.hi, -a.lo}; }
PX_HD px_dd px_dd_sub(px_dd a, px_dd b) { return px_dd_add(a, px_dd_neg(b)); }
PX_HD px_dd px_dd_mul(px_dd a, px_dd b) {
  px_dd p = px_two_prod(a.hi, b.hi);
  double c = a.hi * b.lo;
  double d = a.lo * b.hi;
  p.lo = p.lo + (c + d);
  return px_fast_two_sum(p.hi, p.lo);
}
PX_HD px_dd px_dd_mul_d(px_dd a, double b) {
  px_dd p = px_two_prod(a.hi, b);
  double c = a.lo * b;
  p.lo = p.lo + c;
  return px_fast_two_sum(p.hi, p.lo);
}
PX_HD px_dd px_dd_div(px_dd a, px_dd b) {
  double q1 = a.hi / b.hi;
  px_dd r = px_dd_sub(a, px_dd_mul_d(b, q1));
  double q2 = r.hi / b.hi;
  r = px_dd_sub(r, px_dd_mul_d(b, q2));
  double q3 = r.hi / b.hi;
  px_dd q = px_fast_two_sum(q1, q2);
  return px_dd_add(q, px_dd{q3, 0.0});
}

PX_HD double px_round(double x) {
  if (!isfinite(x)) return x;
  double r = floor(x);
  if (x - r >= 0.5) r = r + 1.0;
  return r;
}

PX_HD double px_hypot2(double a, double b) {
  a = fabs(a);
  b = fabs(b);
  if (isinf(a) || isinf(b)) return INFINITY;
  if (a != a || b != b) return NAN;
  double m = a > b ? a : b;
  if (m == 0) return 0.0;
  double sum = 0.0, comp = 0.0;
  double n = a / m;
  double summand = n * n - comp;
  double prelim = sum + summand;
  comp = (prelim - sum) - summand;
  sum = prelim;
  n = b / m;
  summand = n * n - comp;
  prelim = sum + summand;
  comp = (prelim - sum) - summand;
  sum = prelim;
  return sqrt(sum) * m;
}

// sin or cos of a reduced double-double argument |r| <= pi/4 + tiny.
PX_HD px_dd px_sincos_dd(px_dd r, int want_cos) {
  px_dd r2 = px_dd_mul(r, r);
  // Horner over n = 14 .. 0 of (-1)^n r^(2n) / (2n + 1 + want_cos - 1)!
  int top = 14;
  int base = want_cos ? 0 : 1;
  px_dd s = {PX_TAB(PX_INVFACT)[2 * top + base][0], PX_TAB(PX_INVFACT)[2 * top + base][1]};
  if (top & 1) s = px_dd_neg(s);
  for (int n = top - 1; n >= 0; n--) {
    px_dd c = {PX_TAB(PX_INVFACT)[2 * n + base][0], PX_TAB(PX_INVFACT)[2 * n + base][1]};
    if (n & 1) c = px_dd_neg(c);
    s = px_dd_add(px_dd_mul(s, r2), c);
  }
  return want_cos ? s : px_dd_mul(s, r);
}

PX_HD double px_sin(double x) {
  if (x != x || isinf(x)) return NAN;
  double ax = fabs(x);
  if (ax < 0x1p-26) return x;
  if (!(ax < 0x1p28)) return NAN;
  double kd = rint(x * PX_2OPI);
  px_dd p1 = px_two_prod(kd, PX_PIO2_1);
  px_dd p2 = px_two_prod(kd, PX_PIO2_2);
  double p3 = kd * PX_PIO2_3;
  px_dd r = px_two_sum(x, -p1.hi);
  r = px_dd_add(r, px_dd{-p1.lo, 0.0});
  r = px_dd_add(r, px_dd{-p2.hi, 0.0});
  r = px_dd_add(r, px_dd{-p2.lo, 0.0});
  r = px_dd_add(r, px_dd{-p3, 0.0});
  long long k = (long long)kd;
  int q = (int)(k & 3);
  px_dd v = px_sincos_dd(r, q & 1);
  if (q & 2) v = px_dd_neg(v);
  return v.hi + v.lo;
}

PX_HD double px_atan2(double y, double x) {
  if (x != x || y != y) return NAN;
  const double pi = PX_PI_HI, pio2 = PX_PIO2_HI;
  if (y == 0) return signbit(x) ? copysign(pi, y) : y;
  if (isinf(x)) {
    if (isinf(y)) return copysign(x > 0 ? 0.7853981633974483 : 2.356194490192345, y);
    return x > 0 ? copysign(0.0, y) : copysign(pi, y);
  }
  if (isinf(y) || x == 0) return copysign(pio2, y);
  double a = fabs(y), b = fabs(x);
  int swap = a > b;
  px_dd t = swap ? px_dd_div(px_dd{b, 0.0}, px_dd{a, 0.0}) : px_dd_div(px_dd{a, 0.0}, px_dd{b, 0.0});
  int k = (int)rint(t.hi * 32.0);
  if (k > 32) k = 32;
  if (k < 0) k = 0;
  double c = (double)k * 0.03125;
  px_dd num = px_dd_add(t, px_dd{-c, 0.0});
  px_dd den = px_dd_add(px_dd{1.0, 0.0}, px_dd_mul_d(t, c));
  px_dd u = px_dd_div(num, den);
  px_dd u2 = px_dd_mul(u, u);
  const int top = 11;
  px_dd s = {PX_TAB(PX_INVODD)[top][0], PX_TAB(PX_INVODD)[top][1]};
  if (top & 1) s = px_dd_neg(s);
  for (int n = top - 1; n >= 0; n--) {
    px_dd cn = {PX_TAB(PX_INVODD)[n][0], PX_TAB(PX_INVODD)[n][1]};
    if (n & 1) cn = px_dd_neg(cn);
    s = px_dd_add(px_dd_mul(s, u2), cn);
  }
  px_dd at = px_dd_add(px_dd{PX_TAB(PX_ATAN_TAB)[k][0], PX_TAB(PX_ATAN_TAB)[k][1]}, px_dd_mul(u, s));
  if (swap) at = px_dd_sub(px_dd{PX_PIO2_HI, PX_PIO2_LO}, at);
  if (signbit(x)) at = px_dd_sub(px_dd{PX_PI_HI, PX_PI_LO}, at);
  double r = at.hi + at.lo;
  return signbit(y) ? -r : r;
}
