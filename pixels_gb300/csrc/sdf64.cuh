// Float64 SDF bytecode evaluator: one thread evaluates one op's shape at one
// point.  Every primitive keeps the reference closure's operation order
// (shapes.ts:40-320, penthouse.ts:73-78,250); the translation unit is compiled
// with -fmad=false, so no multiply-add is fused and every step rounds like a
// JavaScript number.  Math.max/min are fmax/fmin: parameters are validated
// finite, so no NaN reaches them, and a signed zero never changes a comparison.
#pragma once
#include "jsmath.cuh"
#include "px_internal.cuh"

namespace px {

__device__ __forceinline__ double len2d(double x, double y) { return sqrt(x * x + y * y); }
__device__ __forceinline__ double len3d(double x, double y, double z) { return sqrt(x * x + y * y + z * z); }

// shapes.ts:146-161.  The host expands the polygon into per-vertex records
// (vix, viy, vjy, ex, ey, den) with ex = vjx - vix, ey = vjy - viy and
// den = ex*ex + ey*ey || 1e-12 computed once in float64 exactly as every call
// of the reference computes them, so the results are the same bits.
__device__ __forceinline__ double sd_polygon64(double px_, double py_, const double* __restrict__ r, int n) {
  double d0x = px_ - __ldg(r), d0y = py_ - __ldg(r + 1);
  double d = d0x * d0x + d0y * d0y;
  double s = 1.0;
  for (int i = 0; i < n; i++) {
    const double* e = r + 6 * i;
    double vix = __ldg(e), viy = __ldg(e + 1), vjy = __ldg(e + 2), ex = __ldg(e + 3), ey = __ldg(e + 4);
    double wx = px_ - vix, wy = py_ - viy;
    double t = fmin(1.0, fmax(0.0, (wx * ex + wy * ey) / __ldg(e + 5)));
    double bx = wx - ex * t, by = wy - ey * t;
    d = fmin(d, bx * bx + by * by);
    bool c1 = py_ >= viy, c2 = py_ < vjy, c3 = ex * wy > ey * wx;
    if ((c1 && c2 && c3) || (!c1 && !c2 && !c3)) s = -s;
  }
  return s * sqrt(d);
}

// shapes.ts:164-173, records per segment (ax, ay, ex, ey, den).
__device__ __forceinline__ double sd_polyline64(double px_, double py_, const double* __restrict__ r, int nseg) {
  double d = INFINITY;
  for (int i = 0; i < nseg; i++) {
    const double* e = r + 5 * i;
    double ex = __ldg(e + 2), ey = __ldg(e + 3);
    double wx = px_ - __ldg(e), wy = py_ - __ldg(e + 1);
    double t = fmin(1.0, fmax(0.0, (wx * ex + wy * ey) / __ldg(e + 4)));
    double qx = wx - ex * t, qy = wy - ey * t;
    d = fmin(d, qx * qx + qy * qy);
  }
  return sqrt(d);
}

__device__ __forceinline__ double prim64(uint32_t op, int cnt, const double* __restrict__ p, double x, double y, double z) {
  switch (op) {
    case OP_BOX: {  // shapes.ts:40-44
      double qx = fabs(x - __ldg(p)) - __ldg(p + 3), qy = fabs(y - __ldg(p + 1)) - __ldg(p + 4),
             qz = fabs(z - __ldg(p + 2)) - __ldg(p + 5);
      double out = len3d(fmax(qx, 0.0), fmax(qy, 0.0), fmax(qz, 0.0));
      return out + fmin(fmax(fmax(qx, qy), qz), 0.0);
    }
    case OP_ROUNDBOX: {  // shapes.ts:56-59
      double qx = fabs(x - __ldg(p)) - __ldg(p + 3), qy = fabs(y - __ldg(p + 1)) - __ldg(p + 4),
             qz = fabs(z - __ldg(p + 2)) - __ldg(p + 5);
      return len3d(fmax(qx, 0.0), fmax(qy, 0.0), fmax(qz, 0.0)) + fmin(fmax(fmax(qx, qy), qz), 0.0) - __ldg(p + 6);
    }
    case OP_SPHERE:  // shapes.ts:68
      return len3d(x - __ldg(p), y - __ldg(p + 1), z - __ldg(p + 2)) - __ldg(p + 3);
    case OP_ELLIPSOID:  // shapes.ts:79
      return (len3d((x - __ldg(p)) / __ldg(p + 3), (y - __ldg(p + 1)) / __ldg(p + 4), (z - __ldg(p + 2)) / __ldg(p + 5)) - 1.0) *
             __ldg(p + 6);
    case OP_CYL_X: case OP_CYL_Y: case OP_CYL_Z: {  // shapes.ts:93-100
      double a, b, h;
      if (op == OP_CYL_Y) { a = x - __ldg(p); b = z - __ldg(p + 2); h = y - __ldg(p + 1); }
      else if (op == OP_CYL_X) { a = y - __ldg(p + 1); b = z - __ldg(p + 2); h = x - __ldg(p); }
      else { a = x - __ldg(p); b = y - __ldg(p + 1); h = z - __ldg(p + 2); }
      double dr = len2d(a, b) - __ldg(p + 3), dh = fabs(h) - __ldg(p + 4);
      return fmin(fmax(dr, dh), 0.0) + len2d(fmax(dr, 0.0), fmax(dh, 0.0));
    }
    case OP_CAPSULE: {  // shapes.ts:120-124
      double px_ = x - __ldg(p), py_ = y - __ldg(p + 1), pz_ = z - __ldg(p + 2);
      double bax = __ldg(p + 3), bay = __ldg(p + 4), baz = __ldg(p + 5);
      double h = fmin(1.0, fmax(0.0, (px_ * bax + py_ * bay + pz_ * baz) / __ldg(p + 6)));
      return len3d(px_ - bax * h, py_ - bay * h, pz_ - baz * h) - __ldg(p + 7);
    }
    case OP_TORUS_X: case OP_TORUS_Y: case OP_TORUS_Z: {  // shapes.ts:133-139
      double a, b, h;
      if (op == OP_TORUS_Y) { a = x - __ldg(p); b = z - __ldg(p + 2); h = y - __ldg(p + 1); }
      else if (op == OP_TORUS_X) { a = y - __ldg(p + 1); b = z - __ldg(p + 2); h = x - __ldg(p); }
      else { a = x - __ldg(p); b = y - __ldg(p + 1); h = z - __ldg(p + 2); }
      return len2d(len2d(a, b) - __ldg(p + 3), h) - __ldg(p + 4);
    }
    case OP_LATHE_SOLID:  // shapes.ts:194-195
      return sd_polygon64(len2d(x - __ldg(p), z - __ldg(p + 2)), y - __ldg(p + 1), p + 3, cnt);
    case OP_LATHE_SHELL:  // shapes.ts:192
      return sd_polyline64(len2d(x - __ldg(p), z - __ldg(p + 2)), y - __ldg(p + 1), p + 4, cnt - 1) - __ldg(p + 3);
    case OP_PRISM: {  // shapes.ts:214-218
      double d2 = sd_polygon64(x - __ldg(p), z - __ldg(p + 1), p + 4, cnt);
      double dy = fabs(y - __ldg(p + 2)) - __ldg(p + 3);
      return fmin(fmax(d2, dy), 0.0) + len2d(fmax(d2, 0.0), fmax(dy, 0.0));
    }
    case OP_STADIUM: {  // penthouse.ts:73-78
      double dx = fmax(fabs(x - __ldg(p)) - __ldg(p + 2), 0.0);
      double d2 = px_hypot2(dx, z - __ldg(p + 1)) - __ldg(p + 3);
      double dy = fabs(y - __ldg(p + 4)) - __ldg(p + 5);
      return fmin(fmax(d2, dy), 0.0) + px_hypot2(fmax(d2, 0.0), fmax(dy, 0.0));
    }
  }
  return 0.0;
}

// Evaluate the postfix bytecode of one shape at (x, y, z).
__device__ __noinline__ double sdf64(const uint2* __restrict__ code, int n, const double* __restrict__ P,
                                     double x, double y, double z) {
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;                 // value stack, s0 = top
  double ax0 = 0, ay0 = 0, az0 = 0, ax1 = 0, ay1 = 0, az1 = 0, ax2 = 0, ay2 = 0, az2 = 0;  // saved points
  for (int i = 0; i < n; i++) {
    uint2 ins = __ldg(code + i);
    uint32_t op = ins.x & 0xffu;
    int cnt = (int)(ins.x >> 8);
    const double* p = P + ins.y;
    if (op < OP_ROT_X) {
      double v = prim64(op, cnt, p, x, y, z);
      s3 = s2; s2 = s1; s1 = s0; s0 = v;
      continue;
    }
    switch (op) {
      case OP_ROT_X: case OP_ROT_Y: case OP_ROT_Z: {
        ax2 = ax1; ay2 = ay1; az2 = az1; ax1 = ax0; ay1 = ay0; az1 = az0; ax0 = x; ay0 = y; az0 = z;
        double p0 = __ldg(p), p1 = __ldg(p + 1), c = __ldg(p + 2), sn = __ldg(p + 3);
        if (op == OP_ROT_Y) {  // shapes.ts:273-274
          double dx = x - p0, dz = z - p1;
          x = p0 + c * dx + sn * dz;
          z = p1 - sn * dx + c * dz;
        } else if (op == OP_ROT_X) {  // shapes.ts:293-294
          double dy = y - p0, dz = z - p1;
          y = p0 + c * dy + sn * dz;
          z = p1 - sn * dy + c * dz;
        } else {  // shapes.ts:313-314
          double dx = x - p0, dy = y - p1;
          x = p0 + c * dx + sn * dy;
          y = p1 - sn * dx + c * dy;
        }
        break;
      }
      case OP_ROT_END:
        x = ax0; y = ay0; z = az0; ax0 = ax1; ay0 = ay1; az0 = az1; ax1 = ax2; ay1 = ay2; az1 = az2;
        break;
      case OP_OFFSET: s0 = s0 + __ldg(p); break;                                       // penthouse.ts:250
      case OP_NEGMAX: { double b = s0; s0 = s1; s1 = s2; s2 = s3; s0 = fmax(s0, -b); break; }  // shapes.ts:244
      case OP_MAX: { double b = s0; s0 = s1; s1 = s2; s2 = s3; s0 = fmax(s0, b); break; }      // shapes.ts:255
      case OP_MIN: { double b = s0; s0 = s1; s1 = s2; s2 = s3; s0 = fmin(s0, b); break; }      // shapes.ts:231
    }
  }
  return s0;
}

// sdf64 for programs deeper than its registers hold (nested CSG and rotation
// trees): the value stack and the saved points live in local memory.  Same
// operations in the same order as sdf64.
__device__ __noinline__ double sdf64_deep(const uint2* __restrict__ code, int n, const double* __restrict__ P,
                                          double x, double y, double z) {
  double st[DEEP_MAX_STACK];
  double saved[DEEP_MAX_ROT][3];
  int sp = 0, rp = 0;  // the validator bounds both depths
  for (int i = 0; i < n; i++) {
    uint2 ins = __ldg(code + i);
    uint32_t op = ins.x & 0xffu;
    int cnt = (int)(ins.x >> 8);
    const double* p = P + ins.y;
    if (op < OP_ROT_X) {
      st[sp++] = prim64(op, cnt, p, x, y, z);
      continue;
    }
    switch (op) {
      case OP_ROT_X: case OP_ROT_Y: case OP_ROT_Z: {
        saved[rp][0] = x; saved[rp][1] = y; saved[rp][2] = z;
        rp++;
        double p0 = __ldg(p), p1 = __ldg(p + 1), c = __ldg(p + 2), sn = __ldg(p + 3);
        if (op == OP_ROT_Y) {  // shapes.ts:273-274
          double dx = x - p0, dz = z - p1;
          x = p0 + c * dx + sn * dz;
          z = p1 - sn * dx + c * dz;
        } else if (op == OP_ROT_X) {  // shapes.ts:293-294
          double dy = y - p0, dz = z - p1;
          y = p0 + c * dy + sn * dz;
          z = p1 - sn * dy + c * dz;
        } else {  // shapes.ts:313-314
          double dx = x - p0, dy = y - p1;
          x = p0 + c * dx + sn * dy;
          y = p1 - sn * dx + c * dy;
        }
        break;
      }
      case OP_ROT_END:
        rp--;
        x = saved[rp][0]; y = saved[rp][1]; z = saved[rp][2];
        break;
      case OP_OFFSET: st[sp - 1] = st[sp - 1] + __ldg(p); break;                          // penthouse.ts:250
      case OP_NEGMAX: sp--; st[sp - 1] = fmax(st[sp - 1], -st[sp]); break;                // shapes.ts:244
      case OP_MAX: sp--; st[sp - 1] = fmax(st[sp - 1], st[sp]); break;                    // shapes.ts:255
      case OP_MIN: sp--; st[sp - 1] = fmin(st[sp - 1], st[sp]); break;                    // shapes.ts:231
    }
  }
  return st[0];
}

}  // namespace px
