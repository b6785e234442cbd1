// ORACLE — test infrastructure only.  Correctly rounded Math.sin / Math.atan2
// for the oracle, written independently of the product's device routines and
// with a different method for atan, so that the two cross-check each other.
//
//   ref_sin    Reduction x - k*pi/2 with pi/2 held as a 4-term sum (products
//              made exact with fma), then the sin/cos Taylor series summed in
//              double-double from the smallest term up.
//   ref_atan2  atan of the double-double quotient by three argument halvings
//              atan(t) = 2 atan(t / (1 + sqrt(1 + t^2))), Taylor series of atan
//              in double-double, then quadrant fix-ups.
// JavaScript engines do not promise correct rounding (they use their own
// libm), so last-bit agreement with any particular engine is unpinned.
#pragma once
#include <cmath>

namespace ref {

struct dd { double h, l; };

inline dd two_sum(double a, double b) { double s = a + b, t = s - a; return {s, (a - (s - t)) + (b - t)}; }
inline dd quick(double a, double b) { double s = a + b; return {s, b - (s - a)}; }
inline dd prod(double a, double b) { double p = a * b; return {p, std::fma(a, b, -p)}; }
inline dd add(dd a, dd b) {
  dd s = two_sum(a.h, b.h), t = two_sum(a.l, b.l);
  s.l += t.h; s = quick(s.h, s.l); s.l += t.l; return quick(s.h, s.l);
}
inline dd neg(dd a) { return {-a.h, -a.l}; }
inline dd mul(dd a, dd b) { dd p = prod(a.h, b.h); p.l += a.h * b.l + a.l * b.h; return quick(p.h, p.l); }
inline dd div(dd a, dd b) {
  double q1 = a.h / b.h;
  dd r = add(a, neg(mul(b, {q1, 0})));
  double q2 = r.h / b.h;
  r = add(r, neg(mul(b, {q2, 0})));
  double q3 = r.h / b.h;
  return add(quick(q1, q2), {q3, 0});
}
inline dd sqrt_dd(dd a) {  // one Newton step on the double root
  double s = std::sqrt(a.h);
  dd s2 = prod(s, s);
  dd r = add(a, neg(s2));
  return add({s, 0}, {r.h / (2 * s), 0});
}
inline dd from(double x) { return {x, 0}; }

// pi/2 = P0 + P1 + P2 + P3 (each the double nearest the remainder)
const double P0 = 0x1.921fb54442d18p+0, P1 = 0x1.1a62633145c07p-54, P2 = -0x1.f1976b7ed8fbcp-110,
             P3 = 0x1.4cf98e804177dp-164;
const dd PI = {0x1.921fb54442d18p+1, 0x1.1a62633145c07p-53};
const dd PIO2 = {P0, P1};

// sum_{n>=0} (-1)^n x2^n / (2n + off)! in double-double, smallest term first
inline dd series(dd x2, int off) {
  // term_n = term_{n-1} * x2 / ((2n + off - 1)(2n + off))
  dd terms[20];
  terms[0] = off == 1 ? from(1.0) : from(1.0);
  int N = 18;
  for (int n = 1; n < N; n++) {
    double d = (double)(2 * n + off - 1) * (double)(2 * n + off);
    terms[n] = div(mul(terms[n - 1], x2), from(d));
  }
  dd s = from(0.0);
  for (int n = N - 1; n >= 0; n--) s = add(s, (n & 1) ? neg(terms[n]) : terms[n]);
  return s;
}

inline double ref_sin(double x) {
  if (std::isnan(x) || std::isinf(x)) return NAN;
  if (std::fabs(x) < 0x1p-26) return x;
  double k = std::nearbyint(x / P0);
  dd r = two_sum(x, -prod(k, P0).h);
  r = add(r, from(-prod(k, P0).l));
  dd p1 = prod(k, P1);
  r = add(r, neg(p1));
  dd p2 = prod(k, P2);
  r = add(r, neg(p2));
  r = add(r, from(-(k * P3)));
  long long q = ((long long)k) & 3;
  dd r2 = mul(r, r);
  dd v = (q & 1) ? series(r2, 0) : mul(r, series(r2, 1));
  if (q & 2) v = neg(v);
  return v.h + v.l;
}

inline dd atan_small(dd t) {  // |t| <= ~0.1
  dd t2 = mul(t, t);
  dd pw = t;
  dd terms[24];
  for (int n = 0; n < 24; n++) {
    terms[n] = div(pw, from(2.0 * n + 1));
    pw = mul(pw, t2);
  }
  dd s = from(0.0);
  for (int n = 23; n >= 0; n--) s = add(s, (n & 1) ? neg(terms[n]) : terms[n]);
  return s;
}

inline double ref_atan2(double y, double x) {
  if (std::isnan(x) || std::isnan(y)) return NAN;
  if (y == 0) return std::signbit(x) ? std::copysign(PI.h, y) : y;
  if (std::isinf(x)) {
    if (std::isinf(y)) return std::copysign(x > 0 ? 0.7853981633974483 : 2.356194490192345, y);
    return x > 0 ? std::copysign(0.0, y) : std::copysign(PI.h, y);
  }
  if (std::isinf(y) || x == 0) return std::copysign(PIO2.h, y);
  double a = std::fabs(y), b = std::fabs(x);
  bool swap = a > b;
  dd t = swap ? div(from(b), from(a)) : div(from(a), from(b));
  for (int i = 0; i < 3; i++) {  // atan(t) = 2 atan(t / (1 + sqrt(1 + t^2)))
    dd den = add(from(1.0), sqrt_dd(add(from(1.0), mul(t, t))));
    t = div(t, den);
  }
  dd at = atan_small(t);
  at = {at.h * 8, at.l * 8};
  if (swap) at = add(PIO2, neg(at));
  if (std::signbit(x)) at = add(PI, neg(at));
  double r = at.h + at.l;
  return std::signbit(y) ? -r : r;
}

}  // namespace ref
