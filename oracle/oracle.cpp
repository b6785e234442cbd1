// ORACLE — test infrastructure only.  A CPU float64 restatement of the
// reference voxeliser, used by tests, smoke() and the CPU baseline of the
// benchmark to check and time the CUDA library.  Nothing in the product links
// or calls this file.
//
// Restates (paths relative to the reference project):
//   src/world/shapes.ts:24-414   SDF closures, CSG, rotations, apply()
//   src/world/VoxelWorld.ts      grid / pool / LIFO free list / compactCell / cellDensity
//   src/world/materials.ts       OPAQUE via the glass flag (tables passed in by the caller)
//   src/gpu/GpuWorld.ts:52-109   super-grid counts, density texture, free list
//   src/scene/penthouse.ts       the seven paint closures (P1-P7)
// Input is the PXIR op list (pixels_gb300/ir.py); each op carries the
// constants the reference's closures capture.  Compiled with
// -ffp-contract=off and no fast-math so every operation rounds like JS.
//
// Pinning: the only outputs of the reference available are its README's
// published figures (grid dims at 64/80/100/128 voxels per metre and live-brick
// counts rounded to thousands), which the tests check; the reference is
// TypeScript and no JavaScript runtime exists on either machine, so no output
// of the reference itself could be produced.  Beyond those figures parity with
// the reference is unpinned.
//
// Transcendentals: Math.sin/Math.atan2 are correctly rounded double-double
// routines (jsmath_ref.h); Math.hypot is the engine method (scale by the
// largest magnitude, Kahan-sum the squares, sqrt, rescale).  Last-ulp parity
// with a JavaScript engine is unpinned (no JavaScript runtime is available).

#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <thread>
#include <vector>
#include <algorithm>

#include "jsmath_ref.h"

namespace {

// ---------------------------------------------------------------------------
// JS number semantics

inline double js_max(double a, double b) { return (a != a || b != b) ? NAN : (a > b ? a : (b > a ? b : (a == 0 && !std::signbit(a) ? a : b))); }
inline double js_min(double a, double b) { return (a != a || b != b) ? NAN : (a < b ? a : (b < a ? b : (a == 0 && std::signbit(a) ? a : b))); }
inline double js_or_eps(double v) { return (v == 0 || v != v) ? 1e-12 : v; }

// Math.round: half toward +infinity (x - floor(x) is exact for finite x).
inline double js_round(double x) {
  if (!std::isfinite(x)) return x;
  double r = std::floor(x);
  if (x - r >= 0.5) r += 1;
  return r;
}

// Math.hypot of two operands, scaled compensated method.
inline double js_hypot2(double a, double b) {
  a = std::fabs(a); b = std::fabs(b);
  if (std::isinf(a) || std::isinf(b)) return INFINITY;
  if (a != a || b != b) return NAN;
  double m = a > b ? a : b;
  if (m == 0) return 0;
  double sum = 0, comp = 0;
  const double v[2] = {a, b};
  for (int i = 0; i < 2; i++) {
    double n = v[i] / m;
    double summand = n * n - comp;
    double prelim = sum + summand;
    comp = (prelim - sum) - summand;
    sum = prelim;
  }
  return std::sqrt(sum) * m;
}

inline double len2(double x, double y) { return std::sqrt(x * x + y * y); }                 // shapes.ts:24
inline double len3(double x, double y, double z) { return std::sqrt(x * x + y * y + z * z); }  // shapes.ts:25

// ---------------------------------------------------------------------------
// Evaluation ledger (the algorithmic work the reference's procedure prescribes)

struct Ledger {
  uint64_t flops = 0, divs = 0, sqrts = 0, trans = 0;
};
thread_local Ledger* g_ledger = nullptr;
inline void L(uint64_t f, uint64_t d = 0, uint64_t s = 0, uint64_t t = 0) {
  if (g_ledger) { g_ledger->flops += f; g_ledger->divs += d; g_ledger->sqrts += s; g_ledger->trans += t; }
}

// ---------------------------------------------------------------------------
// IR

struct IrOp {
  uint8_t kind, flags; uint16_t paint_kind;
  uint32_t paint_value, paint_param, code_begin, code_len, pad0;
  double mn[3], mx[3], slack;
  double frame[4];
  double pad1[2];
};
static_assert(sizeof(IrOp) == 128, "PXIR op is 128 bytes");

enum {
  OP_BOX = 1, OP_ROUNDBOX, OP_SPHERE, OP_ELLIPSOID, OP_CYL_X, OP_CYL_Y, OP_CYL_Z, OP_CAPSULE,
  OP_TORUS_X, OP_TORUS_Y, OP_TORUS_Z, OP_LATHE_SOLID, OP_LATHE_SHELL, OP_PRISM, OP_STADIUM,
  OP_ROT_X = 20, OP_ROT_Y, OP_ROT_Z, OP_ROT_END, OP_OFFSET, OP_NEGMAX, OP_MAX, OP_MIN
};
enum { PK_CONST = 0, PK_CHIP, PK_TUFTED, PK_CARD, PK_WHITE, PK_BLACK, PK_VASE, PK_PAINTING, PK_NOISE };
enum { OPF_CONTAINS = 1, OPF_HAS_SLACK = 2, OPF_PAINT_FRAME = 4 };

// ---------------------------------------------------------------------------
// Shapes: one object per closure of shapes.ts

struct Node {
  virtual ~Node() {}
  virtual double sdf(double x, double y, double z) const = 0;
};
using NodeP = std::unique_ptr<Node>;

struct Box : Node {  // shapes.ts:40-44
  double cx, cy, cz, hx, hy, hz;
  double sdf(double x, double y, double z) const override {
    L(18, 0, 1);
    double qx = std::fabs(x - cx) - hx, qy = std::fabs(y - cy) - hy, qz = std::fabs(z - cz) - hz;
    double out = len3(js_max(qx, 0), js_max(qy, 0), js_max(qz, 0));
    return out + js_min(js_max(js_max(qx, qy), qz), 0);
  }
};
struct RoundBox : Node {  // shapes.ts:56-59
  double cx, cy, cz, hx, hy, hz, r;
  double sdf(double x, double y, double z) const override {
    L(19, 0, 1);
    double qx = std::fabs(x - cx) - hx, qy = std::fabs(y - cy) - hy, qz = std::fabs(z - cz) - hz;
    return len3(js_max(qx, 0), js_max(qy, 0), js_max(qz, 0)) + js_min(js_max(js_max(qx, qy), qz), 0) - r;
  }
};
struct Sphere : Node {  // shapes.ts:68
  double cx, cy, cz, r;
  double sdf(double x, double y, double z) const override {
    L(9, 0, 1);
    return len3(x - cx, y - cy, z - cz) - r;
  }
};
struct Ellipsoid : Node {  // shapes.ts:79
  double cx, cy, cz, rx, ry, rz, rmin;
  double sdf(double x, double y, double z) const override {
    L(10, 3, 1);
    return (len3((x - cx) / rx, (y - cy) / ry, (z - cz) / rz) - 1) * rmin;
  }
};
struct Cylinder : Node {  // shapes.ts:93-100
  int axis;  // 0 x, 1 y, 2 z
  double cx, cy, cz, r, hh;
  double sdf(double x, double y, double z) const override {
    L(16, 0, 2);
    double a, b, h;
    if (axis == 1) { a = x - cx; b = z - cz; h = y - cy; }
    else if (axis == 0) { a = y - cy; b = z - cz; h = x - cx; }
    else { a = x - cx; b = y - cy; h = z - cz; }
    double dr = len2(a, b) - r, dh = std::fabs(h) - hh;
    return js_min(js_max(dr, dh), 0) + len2(js_max(dr, 0), js_max(dh, 0));
  }
};
struct Capsule : Node {  // shapes.ts:120-124
  double ax, ay, az, bax, bay, baz, bb, r;
  double sdf(double x, double y, double z) const override {
    L(22, 1, 1);
    double px = x - ax, py = y - ay, pz = z - az;
    double h = js_min(1, js_max(0, (px * bax + py * bay + pz * baz) / bb));
    return len3(px - bax * h, py - bay * h, pz - baz * h) - r;
  }
};
struct Torus : Node {  // shapes.ts:133-139
  int axis;
  double cx, cy, cz, R, r;
  double sdf(double x, double y, double z) const override {
    L(11, 0, 2);
    double a, b, h;
    if (axis == 1) { a = x - cx; b = z - cz; h = y - cy; }
    else if (axis == 0) { a = y - cy; b = z - cz; h = x - cx; }
    else { a = x - cx; b = y - cy; h = z - cz; }
    return len2(len2(a, b) - R, h) - r;
  }
};

// shapes.ts:146-161 (Inigo Quilez's polygon distance with crossing parity)
double sdPolygon(double px, double py, const double* pts, int n) {
  L(5 + 25 * (uint64_t)n + 1, (uint64_t)n, 1);
  double d = (px - pts[0]) * (px - pts[0]) + (py - pts[1]) * (py - pts[1]);
  double s = 1;
  for (int i = 0, j = n - 1; i < n; j = i, i++) {
    double vix = pts[i * 2], viy = pts[i * 2 + 1], vjx = pts[j * 2], vjy = pts[j * 2 + 1];
    double ex = vjx - vix, ey = vjy - viy;
    double wx = px - vix, wy = py - viy;
    double t = js_min(1, js_max(0, (wx * ex + wy * ey) / js_or_eps(ex * ex + ey * ey)));
    double bx = wx - ex * t, by = wy - ey * t;
    d = js_min(d, bx * bx + by * by);
    bool c1 = py >= viy, c2 = py < vjy, c3 = ex * wy > ey * wx;
    if ((c1 && c2 && c3) || (!c1 && !c2 && !c3)) s = -s;
  }
  return s * std::sqrt(d);
}
// shapes.ts:164-173
double sdPolyline(double px, double py, const double* pts, int n) {
  L(20 * (uint64_t)(n - 1), (uint64_t)(n - 1), 1);
  double d = INFINITY;
  for (int i = 0; i + 3 < 2 * n; i += 2) {
    double ax = pts[i], ay = pts[i + 1], ex = pts[i + 2] - ax, ey = pts[i + 3] - ay;
    double wx = px - ax, wy = py - ay;
    double t = js_min(1, js_max(0, (wx * ex + wy * ey) / js_or_eps(ex * ex + ey * ey)));
    double qx = wx - ex * t, qy = wy - ey * t;
    d = js_min(d, qx * qx + qy * qy);
  }
  return std::sqrt(d);
}
struct LatheSolid : Node {  // shapes.ts:194-195
  double cx, cy, cz; std::vector<double> poly;
  double sdf(double x, double y, double z) const override {
    L(6);
    return sdPolygon(len2(x - cx, z - cz), y - cy, poly.data(), (int)poly.size() / 2);
  }
};
struct LatheShell : Node {  // shapes.ts:192 (half = shell / 2)
  double cx, cy, cz, half; std::vector<double> prof;
  double sdf(double x, double y, double z) const override {
    L(7);
    return sdPolyline(len2(x - cx, z - cz), y - cy, prof.data(), (int)prof.size() / 2) - half;
  }
};
struct Prism : Node {  // shapes.ts:214-218
  double cx, cz, ym, hy; std::vector<double> pts;
  double sdf(double x, double y, double z) const override {
    L(11, 0, 1);
    double d2 = sdPolygon(x - cx, z - cz, pts.data(), (int)pts.size() / 2);
    double dy = std::fabs(y - ym) - hy;
    return js_min(js_max(d2, dy), 0) + len2(js_max(d2, 0), js_max(dy, 0));
  }
};
struct Stadium : Node {  // penthouse.ts:73-78
  double cx, cz, hl, r, ym, hy;
  double sdf(double x, double y, double z) const override {
    L(12 + 24, 4, 2);
    double dx = js_max(std::fabs(x - cx) - hl, 0);
    double d2 = js_hypot2(dx, z - cz) - r;
    double dy = std::fabs(y - ym) - hy;
    return js_min(js_max(d2, dy), 0) + js_hypot2(js_max(d2, 0), js_max(dy, 0));
  }
};
struct Offset : Node {  // penthouse.ts:250
  NodeP s; double k;
  double sdf(double x, double y, double z) const override { L(1); return s->sdf(x, y, z) + k; }
};
struct Subtract : Node {  // shapes.ts:242-246
  NodeP a; std::vector<NodeP> b;
  double sdf(double x, double y, double z) const override {
    double d = a->sdf(x, y, z);
    for (auto& s : b) { L(1); d = js_max(d, -s->sdf(x, y, z)); }
    return d;
  }
};
struct Intersect : Node {  // shapes.ts:255
  NodeP a, b;
  double sdf(double x, double y, double z) const override { L(1); return js_max(a->sdf(x, y, z), b->sdf(x, y, z)); }
};
struct Union : Node {  // shapes.ts:229-233
  std::vector<NodeP> c;
  double sdf(double x, double y, double z) const override {
    double d = INFINITY;
    for (auto& s : c) { L(1); d = js_min(d, s->sdf(x, y, z)); }
    return d;
  }
};
struct RotY : Node {  // shapes.ts:272-275
  NodeP s; double px, pz, c, sn;
  double sdf(double x, double y, double z) const override {
    L(10);
    double dx = x - px, dz = z - pz;
    return s->sdf(px + c * dx + sn * dz, y, pz - sn * dx + c * dz);
  }
};
struct RotX : Node {  // shapes.ts:292-295
  NodeP s; double py, pz, c, sn;
  double sdf(double x, double y, double z) const override {
    L(10);
    double dy = y - py, dz = z - pz;
    return s->sdf(x, py + c * dy + sn * dz, pz - sn * dy + c * dz);
  }
};
struct RotZ : Node {  // shapes.ts:312-315
  NodeP s; double px, py, c, sn;
  double sdf(double x, double y, double z) const override {
    L(10);
    double dx = x - px, dy = y - py;
    return s->sdf(px + c * dx + sn * dy, py - sn * dx + c * dy, z);
  }
};

// Rebuild the closure tree from postfix bytecode.
bool decode_shape(const uint32_t* code, uint32_t n, const double* P, size_t np, NodeP& out, std::string& err) {
  std::vector<NodeP> st;
  struct Pending { int op; uint32_t off; size_t depth; };
  std::vector<Pending> rots;
  auto need = [&](uint32_t off, size_t k) { return (size_t)off + k <= np; };
  for (uint32_t i = 0; i < n; i++) {
    uint32_t w0 = code[2 * i], off = code[2 * i + 1];
    int op = (int)(w0 & 0xff), cnt = (int)(w0 >> 8);
    switch (op) {
      case OP_BOX: { if (!need(off, 6)) goto bad; auto b = std::make_unique<Box>(); const double* p = P + off;
        b->cx = p[0]; b->cy = p[1]; b->cz = p[2]; b->hx = p[3]; b->hy = p[4]; b->hz = p[5]; st.push_back(std::move(b)); break; }
      case OP_ROUNDBOX: { if (!need(off, 7)) goto bad; auto b = std::make_unique<RoundBox>(); const double* p = P + off;
        b->cx = p[0]; b->cy = p[1]; b->cz = p[2]; b->hx = p[3]; b->hy = p[4]; b->hz = p[5]; b->r = p[6]; st.push_back(std::move(b)); break; }
      case OP_SPHERE: { if (!need(off, 4)) goto bad; auto b = std::make_unique<Sphere>(); const double* p = P + off;
        b->cx = p[0]; b->cy = p[1]; b->cz = p[2]; b->r = p[3]; st.push_back(std::move(b)); break; }
      case OP_ELLIPSOID: { if (!need(off, 7)) goto bad; auto b = std::make_unique<Ellipsoid>(); const double* p = P + off;
        b->cx = p[0]; b->cy = p[1]; b->cz = p[2]; b->rx = p[3]; b->ry = p[4]; b->rz = p[5]; b->rmin = p[6]; st.push_back(std::move(b)); break; }
      case OP_CYL_X: case OP_CYL_Y: case OP_CYL_Z: { if (!need(off, 5)) goto bad; auto b = std::make_unique<Cylinder>(); const double* p = P + off;
        b->axis = op - OP_CYL_X; b->cx = p[0]; b->cy = p[1]; b->cz = p[2]; b->r = p[3]; b->hh = p[4]; st.push_back(std::move(b)); break; }
      case OP_CAPSULE: { if (!need(off, 8)) goto bad; auto b = std::make_unique<Capsule>(); const double* p = P + off;
        b->ax = p[0]; b->ay = p[1]; b->az = p[2]; b->bax = p[3]; b->bay = p[4]; b->baz = p[5]; b->bb = p[6]; b->r = p[7]; st.push_back(std::move(b)); break; }
      case OP_TORUS_X: case OP_TORUS_Y: case OP_TORUS_Z: { if (!need(off, 5)) goto bad; auto b = std::make_unique<Torus>(); const double* p = P + off;
        b->axis = op - OP_TORUS_X; b->cx = p[0]; b->cy = p[1]; b->cz = p[2]; b->R = p[3]; b->r = p[4]; st.push_back(std::move(b)); break; }
      case OP_LATHE_SOLID: { if (cnt < 2 || !need(off, 3 + 2 * (size_t)cnt)) goto bad; auto b = std::make_unique<LatheSolid>(); const double* p = P + off;
        b->cx = p[0]; b->cy = p[1]; b->cz = p[2]; b->poly.assign(p + 3, p + 3 + 2 * cnt); st.push_back(std::move(b)); break; }
      case OP_LATHE_SHELL: { if (cnt < 2 || !need(off, 4 + 2 * (size_t)cnt)) goto bad; auto b = std::make_unique<LatheShell>(); const double* p = P + off;
        b->cx = p[0]; b->cy = p[1]; b->cz = p[2]; b->half = p[3]; b->prof.assign(p + 4, p + 4 + 2 * cnt); st.push_back(std::move(b)); break; }
      case OP_PRISM: { if (cnt < 3 || !need(off, 4 + 2 * (size_t)cnt)) goto bad; auto b = std::make_unique<Prism>(); const double* p = P + off;
        b->cx = p[0]; b->cz = p[1]; b->ym = p[2]; b->hy = p[3]; b->pts.assign(p + 4, p + 4 + 2 * cnt); st.push_back(std::move(b)); break; }
      case OP_STADIUM: { if (!need(off, 6)) goto bad; auto b = std::make_unique<Stadium>(); const double* p = P + off;
        b->cx = p[0]; b->cz = p[1]; b->hl = p[2]; b->r = p[3]; b->ym = p[4]; b->hy = p[5]; st.push_back(std::move(b)); break; }
      case OP_ROT_X: case OP_ROT_Y: case OP_ROT_Z:
        if (!need(off, 4)) goto bad;
        rots.push_back({op, off, st.size()});
        break;
      case OP_ROT_END: {
        if (rots.empty() || st.size() != rots.back().depth + 1) goto bad;
        Pending pr = rots.back(); rots.pop_back();
        const double* p = P + pr.off;
        NodeP child = std::move(st.back()); st.pop_back();
        if (pr.op == OP_ROT_Y) { auto r = std::make_unique<RotY>(); r->s = std::move(child); r->px = p[0]; r->pz = p[1]; r->c = p[2]; r->sn = p[3]; st.push_back(std::move(r)); }
        else if (pr.op == OP_ROT_X) { auto r = std::make_unique<RotX>(); r->s = std::move(child); r->py = p[0]; r->pz = p[1]; r->c = p[2]; r->sn = p[3]; st.push_back(std::move(r)); }
        else { auto r = std::make_unique<RotZ>(); r->s = std::move(child); r->px = p[0]; r->py = p[1]; r->c = p[2]; r->sn = p[3]; st.push_back(std::move(r)); }
        break;
      }
      case OP_OFFSET: {
        if (st.empty() || !need(off, 1)) goto bad;
        auto o = std::make_unique<Offset>(); o->s = std::move(st.back()); st.pop_back(); o->k = P[off]; st.push_back(std::move(o)); break;
      }
      case OP_NEGMAX: {
        if (st.size() < 2) goto bad;
        NodeP b = std::move(st.back()); st.pop_back();
        // consecutive subtract steps extend one Subtract node (variadic b)
        Subtract* cur = dynamic_cast<Subtract*>(st.back().get());
        if (!cur || cur->b.empty() || !cur->a) {
          auto s = std::make_unique<Subtract>(); s->a = std::move(st.back()); st.pop_back();
          s->b.push_back(std::move(b)); st.push_back(std::move(s));
        } else {
          cur->b.push_back(std::move(b));
        }
        break;
      }
      case OP_MAX: {
        if (st.size() < 2) goto bad;
        auto s = std::make_unique<Intersect>(); s->b = std::move(st.back()); st.pop_back(); s->a = std::move(st.back()); st.pop_back();
        st.push_back(std::move(s)); break;
      }
      case OP_MIN: {
        if (st.size() < 2) goto bad;
        NodeP b = std::move(st.back()); st.pop_back();
        Union* cur = dynamic_cast<Union*>(st.back().get());
        if (!cur) { auto u = std::make_unique<Union>(); u->c.push_back(std::move(st.back())); st.pop_back(); u->c.push_back(std::move(b)); st.push_back(std::move(u)); }
        else cur->c.push_back(std::move(b));
        break;
      }
      default: goto bad;
    }
  }
  if (st.size() != 1 || !rots.empty()) goto bad;
  out = std::move(st.back());
  return true;
bad:
  err = "malformed SDF bytecode";
  return false;
}

// ---------------------------------------------------------------------------
// Paint closures (penthouse.ts)

const double PI = 3.141592653589793;

inline uint32_t vox(double mat, double shade) {  // materials.ts:108-110
  return ((uint32_t)(int64_t)mat & 0xffu) | (((uint32_t)(int64_t)shade & 0xffu) << 8);
}

uint32_t noise_hash(uint32_t ix, uint32_t iy, uint32_t iz, uint32_t seed) {
  uint32_t h = seed ^ (ix * 0x8DA6B343u) ^ (iy * 0xD8163841u) ^ (iz * 0xCB1AB31Fu);
  h ^= h >> 16; h *= 0x7FEB352Du; h ^= h >> 15; h *= 0x846CA68Bu; h ^= h >> 16;
  return h;
}
float sin_poly_f32(float t) {
  volatile float u = t - std::floor(t);
  volatile float v = u * 4.0f; v = v - 2.0f;
  volatile float w = std::fabs((float)v) - 1.0f;
  volatile float w2 = w * w;
  volatile float p = w2 * 0.0751f; p = p - 0.6432f;
  p = p * w2; p = p + 1.5708f;
  volatile float r = p * w;
  return v >= 0 ? (float)r : -(float)r;
}

uint32_t paint_eval(int kind, const double* p, double x, double y, double z) {
  switch (kind) {
    case PK_CHIP: {  // penthouse.ts:371-377
      L(20, 2, 1, 1);
      double a = ref::ref_atan2(z - p[2], x - p[0]);
      bool edge = js_hypot2(x - p[0], z - p[2]) > p[3];
      bool stripe = std::fmod(std::floor(((a + PI) / (2 * PI)) * 8), 2) == 0;
      double layer = std::fmod(std::floor((y - p[1]) / 0.0045), 2);
      return vox(p[4], edge && stripe && layer == 0 ? 255 : 0);
    }
    case PK_TUFTED: {  // penthouse.ts:495-501
      L(14, 4, 1);
      double u = (z - p[0]) / 0.16, v = (y - p[1]) / 0.16;
      double du = u - js_round(u), dv = v - js_round(v);
      bool odd = std::fmod(js_round(u) + js_round(v), 2) == 0;
      return vox(p[2], odd && js_hypot2(du, dv) < 0.12 ? 200 : 0);
    }
    case PK_CARD: {  // penthouse.ts:597-600
      L(4);
      bool edge = std::fabs(x - p[0] - p[2]) > 0.022 || std::fabs(z - p[1]) > 0.034;
      return vox(p[3], edge ? 0 : 255);
    }
    case PK_WHITE: {  // penthouse.ts:744-748
      L(5, 2);
      double k = std::floor((x - p[0]) / 0.0254);
      double f = (x - p[0]) / 0.0254 - k;
      return vox(p[1], f < 0.12 ? 120 : 0);
    }
    case PK_BLACK: {  // penthouse.ts:749-756
      L(8, 1);
      double u = (x - p[0]) / 0.0254;
      double k = std::floor(u + 0.5);
      double f = u + 0.5 - k;
      double n = std::fmod(std::fmod(k - 1, 7) + 7, 7);
      bool has = n == 0 || n == 1 || n == 3 || n == 4 || n == 5;
      return has && std::fabs(f - 0.5) < 0.3 ? vox(p[1], 0) : 0;
    }
    case PK_VASE: {  // penthouse.ts:810-816
      L(16, 1, 0, 3);
      double a = ref::ref_atan2(z - p[2], x - p[0]);
      double h = (y - p[1]) / p[3];
      bool band = (h > 0.04 && h < 0.06) || (h > 0.36 && h < 0.38) || (h > 0.47 && h < 0.49);
      bool motif = h > 0.08 && h < 0.33 && ref::ref_sin(a * 5 + ref::ref_sin(h * 30) * 2) > 0.55;
      return vox(p[4], band || motif ? 255 : 0);
    }
    case PK_PAINTING: {  // penthouse.ts:840-845
      L(9 * 16 + 6, 18, 9, 1);
      double shade = 0;
      for (int i = 0; i < 9; i++) {
        const double* b = p + 1 + 4 * i;
        if (js_hypot2(x - b[0], (y - b[1]) * 1.3) < b[2]) shade = b[3];
      }
      bool stripe = std::fabs(ref::ref_sin(x * 9 + y * 3)) < 0.06;
      return vox(p[0], stripe ? 255 : shade);
    }
    case PK_NOISE: {  // synthetic scenes
      L(16);
      double ix = std::floor(x * p[1]), iy = std::floor(y * p[1]), iz = std::floor(z * p[1]);
      uint32_t h = noise_hash((uint32_t)(int64_t)ix, (uint32_t)(int64_t)iy, (uint32_t)(int64_t)iz, (uint32_t)(int64_t)p[0]);
      volatile float jitter = (float)(h & 0xffffu) * (1.0f / 65536.0f);
      volatile float a = (float)x * (float)p[2];
      volatile float b = (float)y * (float)p[3];
      volatile float c = (float)z * (float)p[4];
      volatile float t = a + b; t = t + c; t = t + jitter;
      float s = sin_poly_f32(t);
      return s > (float)p[5] ? (uint32_t)p[6] : (uint32_t)p[7];
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// VoxelWorld (VoxelWorld.ts)

const uint32_t UNIFORM = 0x80000000u;  // VoxelWorld.ts:13
const int BRICK = 8, BRICK_VOXELS = 512;

struct AllocEvent {
  uint32_t op, ci;
  uint8_t seq, free_;  // seq: 0 alloc / 1 free within one (op, cell); free_: 1 = free
  uint32_t local;      // pool index in the thread-local world
};

struct World {
  int dx, dy, dz, bx, by, bz;
  std::vector<AllocEvent>* log = nullptr;  // set when bricks are split across threads
  uint32_t cur_op = 0;
  size_t cur_ci = 0;
  std::vector<uint32_t> grid;
  std::vector<uint16_t> pool;
  uint32_t poolCapacity, poolUsed = 0;
  std::vector<uint32_t> freeList;
  uint64_t allocs = 0, frees = 0;

  World(int dx_, int dy_, int dz_, uint32_t initialPoolBricks)  // VoxelWorld.ts:35-45
      : dx(dx_), dy(dy_), dz(dz_), bx(dx_ / BRICK), by(dy_ / BRICK), bz(dz_ / BRICK) {
    grid.assign((size_t)bx * by * bz, 0);
    poolCapacity = initialPoolBricks ? initialPoolBricks : 1;
    pool.assign((size_t)poolCapacity * BRICK_VOXELS, 0);
  }
  size_t cellIndex(int x, int y, int z) const { return (size_t)x + (size_t)bx * ((size_t)y + (size_t)by * z); }  // :47-49
  void setBrickUniform(size_t ci, uint32_t v) {  // :89-97
    uint32_t g = grid[ci];
    if (g != 0 && !(g & UNIFORM)) freeBrick(g - 1);
    uint32_t next = v == 0 ? 0 : (UNIFORM | v);
    if (grid[ci] != next) grid[ci] = next;
  }
  uint32_t editableBrick(size_t ci) {  // :103-110
    uint32_t g = grid[ci];
    if (g != 0 && !(g & UNIFORM)) return g - 1;
    uint32_t p = allocBrick(g == 0 ? 0 : (g & 0xffff));
    grid[ci] = p + 1;
    return p;
  }
  uint32_t allocBrick(uint16_t fill) {  // :112-122
    uint32_t p;
    allocs++;
    if (!freeList.empty()) { p = freeList.back(); freeList.pop_back(); }
    else {
      if (poolUsed >= poolCapacity) growPool();
      p = poolUsed++;
    }
    std::fill(pool.begin() + (size_t)p * BRICK_VOXELS, pool.begin() + (size_t)(p + 1) * BRICK_VOXELS, fill);
    if (log) log->push_back({cur_op, (uint32_t)cur_ci, 0, 0, p});
    return p;
  }
  void freeBrick(uint32_t p) {  // :124-127
    frees++;
    freeList.push_back(p);
    if (log) log->push_back({cur_op, (uint32_t)cur_ci, 1, 1, p});
  }
  void growPool() {  // :129-136
    uint32_t cap = (uint32_t)std::ceil(poolCapacity * 1.5);
    pool.resize((size_t)cap * BRICK_VOXELS, 0);
    poolCapacity = cap;
  }
  void compactCell(size_t ci) {  // :147-156
    uint32_t g = grid[ci];
    if (g == 0 || (g & UNIFORM)) return;
    uint32_t p = g - 1;
    size_t base = (size_t)p * BRICK_VOXELS;
    uint16_t first = pool[base];
    for (int i = 1; i < BRICK_VOXELS; i++) if (pool[base + i] != first) return;
    freeBrick(p);
    grid[ci] = first == 0 ? 0 : (UNIFORM | first);
  }
};

// ---------------------------------------------------------------------------
// apply (shapes.ts:334-414)

struct Stats {
  uint64_t pairs = 0, contains_tests = 0, brick_evals = 0, sub_evals = 0, voxel_evals = 0, paint_evals = 0;
  uint64_t flops = 0, divs = 0, sqrts = 0, trans = 0;
  uint64_t allocs = 0, frees = 0;
};

struct OpCtx {
  const IrOp* op;
  const Node* shape;
  const double* paint_params;
};

void apply(World& world, const OpCtx& oc, double vs, Stats& st, int bz_mod, int bz_count) {
  const IrOp& op = *oc.op;
  const Node& shape = *oc.shape;
  const double slack = op.slack;
  const bool constPaint = op.paint_kind == PK_CONST;
  const uint32_t pv = constPaint ? op.paint_value : 0;
  const int kind = op.kind;  // 0 Add, 1 Carve, 2 Paint

  double fx0 = std::floor(op.mn[0] / vs - 0.5), fy0 = std::floor(op.mn[1] / vs - 0.5), fz0 = std::floor(op.mn[2] / vs - 0.5);
  double fx1 = std::ceil(op.mx[0] / vs + 0.5), fy1 = std::ceil(op.mx[1] / vs + 0.5), fz1 = std::ceil(op.mx[2] / vs + 0.5);
  double vx0 = js_max(0, fx0), vy0 = js_max(0, fy0), vz0 = js_max(0, fz0);
  double vx1 = js_min(world.dx - 1, fx1), vy1 = js_min(world.dy - 1, fy1), vz1 = js_min(world.dz - 1, fz1);
  if (!(vx0 <= vx1) || !(vy0 <= vy1) || !(vz0 <= vz1)) return;  // :347 (NaN bounds also skip)

  const double brickHalfDiag = 4 * std::sqrt(3.0) * vs * slack + vs * 0.01;  // :349
  const double subHalfDiag = 2 * std::sqrt(3.0) * vs * slack + vs * 0.01;    // :350
  uint16_t scratch[BRICK_VOXELS];

  int bz0 = (int)vz0 >> 3, bz1 = (int)vz1 >> 3;
  for (int bz = bz0; bz <= bz1; bz++) {
    if (bz_count > 1 && bz % bz_count != bz_mod) continue;  // this thread's slabs only
    for (int by = (int)vy0 >> 3; by <= ((int)vy1 >> 3); by++)
      for (int bx = (int)vx0 >> 3; bx <= ((int)vx1 >> 3); bx++) {
        st.pairs++;
        size_t ci = world.cellIndex(bx, by, bz);
        world.cur_ci = ci;
        int ox = bx * BRICK, oy = by * BRICK, oz = bz * BRICK;
        bool full = false;
        if (op.flags & OPF_CONTAINS) {  // :359-361 (box contains, shapes.ts:47-48)
          st.contains_tests++;
          double x0 = (ox + 0.5) * vs, y0 = (oy + 0.5) * vs, z0 = (oz + 0.5) * vs;
          double x1 = (ox + 7.5) * vs, y1 = (oy + 7.5) * vs, z1 = (oz + 7.5) * vs;
          full = x0 >= op.mn[0] && x1 <= op.mx[0] && y0 >= op.mn[1] && y1 <= op.mx[1] && z0 >= op.mn[2] && z1 <= op.mx[2];
        }
        if (!full) {  // :362-366
          st.brick_evals++;
          double d = shape.sdf((ox + 4) * vs, (oy + 4) * vs, (oz + 4) * vs);
          if (d > brickHalfDiag) continue;
          full = d < -brickHalfDiag;
        }
        uint32_t g = world.grid[ci];
        if (full) {  // :368-373
          if (kind == 0 && constPaint) { world.setBrickUniform(ci, pv); continue; }
          if (kind == 1) { world.setBrickUniform(ci, 0); continue; }
          if (kind == 2 && g == 0) continue;
          if (kind == 2 && constPaint && (g & UNIFORM)) { world.setBrickUniform(ci, pv); continue; }
        }
        if (kind == 2 && g == 0) continue;  // :374

        if (g == 0) std::fill(scratch, scratch + BRICK_VOXELS, (uint16_t)0);  // :377-379
        else if (g & UNIFORM) std::fill(scratch, scratch + BRICK_VOXELS, (uint16_t)(g & 0xffff));
        else std::memcpy(scratch, world.pool.data() + (size_t)(g - 1) * BRICK_VOXELS, sizeof scratch);

        bool changed = false;
        for (int s = 0; s < 8; s++) {  // :382-406
          int sx = ox + (s & 1) * 4, sy = oy + ((s >> 1) & 1) * 4, sz = oz + ((s >> 2) & 1) * 4;
          bool subFull = full;
          if (!full) {
            st.sub_evals++;
            double d = shape.sdf((sx + 2) * vs, (sy + 2) * vs, (sz + 2) * vs);
            if (d > subHalfDiag) continue;
            subFull = d < -subHalfDiag;
          }
          for (int z = sz; z < sz + 4; z++)
            for (int y = sy; y < sy + 4; y++)
              for (int x = sx; x < sx + 4; x++) {
                double px = (x + 0.5) * vs, py = (y + 0.5) * vs, pz = (z + 0.5) * vs;
                if (!subFull) {
                  st.voxel_evals++;
                  if (shape.sdf(px, py, pz) > 0) continue;
                }
                int li = (x & 7) | ((y & 7) << 3) | ((z & 7) << 6);
                uint16_t cur = scratch[li];
                uint32_t next;
                if (kind == 1) next = 0;
                else if (kind == 2 && cur == 0) continue;
                else if (!constPaint) {
                  st.paint_evals++;
                  double qx = px, qz = pz;
                  if (op.flags & OPF_PAINT_FRAME) {  // localPaint, penthouse.ts:88-91
                    L(10);
                    double fpx = op.frame[0], fpz = op.frame[1], c = op.frame[2], sn = op.frame[3];
                    double ddx = px - fpx, ddz = pz - fpz;
                    qx = fpx + c * ddx + sn * ddz;
                    qz = fpz - sn * ddx + c * ddz;
                  }
                  next = paint_eval(op.paint_kind, oc.paint_params, qx, py, qz);
                } else next = pv;
                uint16_t n16 = (uint16_t)next;  // Uint16Array store
                if (next != cur) {  // :401 compares the unstored value
                  scratch[li] = n16;
                  changed = true;
                }
              }
        }
        if (!changed) continue;  // :407-412
        uint32_t p = world.editableBrick(ci);
        std::memcpy(world.pool.data() + (size_t)p * BRICK_VOXELS, scratch, sizeof scratch);
        world.compactCell(ci);
      }
  }
}

struct Program {
  std::vector<IrOp> ops;
  std::vector<NodeP> shapes;
  const double* params = nullptr;
  size_t nparams = 0;
  std::vector<double> param_store;
};

bool load_program(const void* buf, size_t bytes, Program& prog, std::string& err) {
  if (bytes < 32) { err = "IR too short"; return false; }
  const uint32_t* h = (const uint32_t*)buf;
  if (h[0] != 0x52495850u || h[1] != 1) { err = "bad IR magic/version"; return false; }
  size_t n_ops = h[2], n_code = h[3], n_params = h[4];
  size_t need = 32 + n_ops * sizeof(IrOp) + n_code * 8 + n_params * 8;
  if (bytes < need) { err = "IR truncated"; return false; }
  const char* p = (const char*)buf + 32;
  prog.ops.resize(n_ops);
  std::memcpy(prog.ops.data(), p, n_ops * sizeof(IrOp));
  p += n_ops * sizeof(IrOp);
  std::vector<uint32_t> code(n_code * 2);
  std::memcpy(code.data(), p, n_code * 8);
  p += n_code * 8;
  prog.param_store.resize(n_params);
  std::memcpy(prog.param_store.data(), p, n_params * 8);
  prog.params = prog.param_store.data();
  prog.nparams = n_params;
  prog.shapes.resize(n_ops);
  for (size_t i = 0; i < n_ops; i++) {
    const IrOp& o = prog.ops[i];
    if ((size_t)o.code_begin + o.code_len > n_code || o.code_len == 0) { err = "op code range out of bounds"; return false; }
    if (!decode_shape(code.data() + 2 * (size_t)o.code_begin, o.code_len, prog.params, n_params, prog.shapes[i], err)) return false;
    if (o.kind > 2) { err = "bad op kind"; return false; }
    for (int k = 0; k < 3; k++)
      if (!std::isfinite(o.mn[k]) || !std::isfinite(o.mx[k])) { err = "non-finite shape bounds"; return false; }
    if (!std::isfinite(o.slack)) { err = "non-finite slack"; return false; }
    if (o.paint_kind == PK_CONST && o.paint_value > 0xffffu) { err = "constant paint is not a u16"; return false; }
    if (o.paint_kind > PK_NOISE) { err = "bad paint kind"; return false; }
  }
  return true;
}

}  // namespace

// ---------------------------------------------------------------------------
// C API

extern "C" {

struct oracle_result {
  int32_t dx, dy, dz, bx, by, bz;
  uint32_t pool_used, n_free;       // pool bricks used, holes in the LIFO free list
  uint32_t* grid;                   // bx*by*bz
  uint16_t* pool;                   // pool_used * 512
  uint32_t* free_list;              // n_free, push order
  uint64_t pairs, contains_tests, brick_evals, sub_evals, voxel_evals, paint_evals;
  uint64_t flops, divs, sqrts, trans, allocs, frees;
  char error[256];
};

// Build the world from an IR op list, one op after the other (shapes.ts:417-431).
int oracle_build(const void* ir, size_t bytes, double vpm, int dx, int dy, int dz,
                 uint32_t initial_pool_bricks, int count_flops, oracle_result* out) {
  std::memset(out, 0, sizeof *out);
  Program prog;
  std::string err;
  if (!load_program(ir, bytes, prog, err)) { std::snprintf(out->error, sizeof out->error, "%s", err.c_str()); return 1; }
  if (dx <= 0 || dy <= 0 || dz <= 0 || dx % 8 || dy % 8 || dz % 8) { std::snprintf(out->error, sizeof out->error, "dims must be positive multiples of 8"); return 1; }
  const double vs = 1 / vpm;
  World w(dx, dy, dz, initial_pool_bricks);
  Stats st;
  Ledger led;
  if (count_flops) g_ledger = &led;
  for (size_t i = 0; i < prog.ops.size(); i++) {
    OpCtx oc{&prog.ops[i], prog.shapes[i].get(), prog.params + prog.ops[i].paint_param};
    w.cur_op = (uint32_t)i;
    apply(w, oc, vs, st, 0, 1);
  }
  g_ledger = nullptr;
  out->dx = dx; out->dy = dy; out->dz = dz; out->bx = w.bx; out->by = w.by; out->bz = w.bz;
  out->pool_used = w.poolUsed;
  out->n_free = (uint32_t)w.freeList.size();
  out->grid = (uint32_t*)std::malloc(w.grid.size() * 4);
  std::memcpy(out->grid, w.grid.data(), w.grid.size() * 4);
  out->pool = (uint16_t*)std::malloc((size_t)w.poolUsed * BRICK_VOXELS * 2 + 2);
  std::memcpy(out->pool, w.pool.data(), (size_t)w.poolUsed * BRICK_VOXELS * 2);
  out->free_list = (uint32_t*)std::malloc(w.freeList.size() * 4 + 4);
  std::memcpy(out->free_list, w.freeList.data(), w.freeList.size() * 4);
  out->pairs = st.pairs; out->contains_tests = st.contains_tests; out->brick_evals = st.brick_evals;
  out->sub_evals = st.sub_evals; out->voxel_evals = st.voxel_evals; out->paint_evals = st.paint_evals;
  out->flops = led.flops; out->divs = led.divs; out->sqrts = led.sqrts; out->trans = led.trans;
  out->allocs = w.allocs; out->frees = w.frees;
  return 0;
}

// The same build with bricks split across host threads: thread t owns the
// brick slabs bz = t (mod threads) and runs every op on them in order (a
// brick's result depends only on the ops that touch it).  The threads' pool
// alloc/free events are then merged in (op, cell) order -- the order of the
// single-threaded loop (shapes.ts:353-355) -- and the LIFO allocator
// (VoxelWorld.ts:112-127) is replayed once to give the same pool indices.
int oracle_build_mt(const void* ir, size_t bytes, double vpm, int dx, int dy, int dz, int threads,
                    oracle_result* out) {
  std::memset(out, 0, sizeof *out);
  Program prog;
  std::string err;
  if (!load_program(ir, bytes, prog, err)) { std::snprintf(out->error, sizeof out->error, "%s", err.c_str()); return 1; }
  if (dx <= 0 || dy <= 0 || dz <= 0 || dx % 8 || dy % 8 || dz % 8) { std::snprintf(out->error, sizeof out->error, "dims must be positive multiples of 8"); return 1; }
  if (threads < 1) threads = 1;
  const double vs = 1 / vpm;
  std::vector<std::unique_ptr<World>> worlds;
  std::vector<std::vector<AllocEvent>> logs(threads);
  std::vector<Stats> stats(threads);
  for (int t = 0; t < threads; t++) {
    worlds.emplace_back(new World(dx, dy, dz, 1024));
    worlds.back()->log = &logs[t];
  }
  std::vector<std::thread> pool_threads;
  for (int t = 0; t < threads; t++)
    pool_threads.emplace_back([&, t] {
      World& w = *worlds[t];
      for (size_t i = 0; i < prog.ops.size(); i++) {
        OpCtx oc{&prog.ops[i], prog.shapes[i].get(), prog.params + prog.ops[i].paint_param};
        w.cur_op = (uint32_t)i;
        apply(w, oc, vs, stats[t], t, threads);
      }
    });
  for (auto& th : pool_threads) th.join();
  struct Tagged { AllocEvent e; int t; };
  std::vector<Tagged> all;
  for (int t = 0; t < threads; t++)
    for (auto& e : logs[t]) all.push_back({e, t});
  std::sort(all.begin(), all.end(), [](const Tagged& a, const Tagged& b) {
    if (a.e.op != b.e.op) return a.e.op < b.e.op;
    if (a.e.ci != b.e.ci) return a.e.ci < b.e.ci;
    return a.e.seq < b.e.seq;
  });
  std::vector<std::vector<uint32_t>> local_to_global(threads);
  for (int t = 0; t < threads; t++) local_to_global[t].assign(worlds[t]->poolUsed, 0xffffffffu);
  std::vector<uint32_t> stack;
  uint32_t used = 0;
  for (auto& x : all) {
    if (!x.e.free_) {
      uint32_t g;
      if (!stack.empty()) { g = stack.back(); stack.pop_back(); }
      else g = used++;
      local_to_global[x.t][x.e.local] = g;
    } else {
      stack.push_back(local_to_global[x.t][x.e.local]);
    }
  }
  World& w0 = *worlds[0];
  const size_t ncells = w0.grid.size();
  out->dx = dx; out->dy = dy; out->dz = dz; out->bx = w0.bx; out->by = w0.by; out->bz = w0.bz;
  out->pool_used = used;
  out->n_free = (uint32_t)stack.size();
  out->grid = (uint32_t*)std::malloc(ncells * 4);
  out->pool = (uint16_t*)std::calloc((size_t)used * BRICK_VOXELS + 1, 2);
  for (size_t ci = 0; ci < ncells; ci++) {
    int bz = (int)(ci / ((size_t)w0.bx * w0.by));
    const World& wt = *worlds[bz % threads];
    uint32_t g = wt.grid[ci];
    if (g != 0 && !(g & UNIFORM)) {
      uint32_t gl = local_to_global[bz % threads][g - 1];
      std::memcpy(out->pool + (size_t)gl * BRICK_VOXELS, wt.pool.data() + (size_t)(g - 1) * BRICK_VOXELS, BRICK_VOXELS * 2);
      g = gl + 1;
    }
    out->grid[ci] = g;
  }
  out->free_list = (uint32_t*)std::malloc(stack.size() * 4 + 4);
  std::memcpy(out->free_list, stack.data(), stack.size() * 4);
  for (int t = 0; t < threads; t++) {
    out->pairs += stats[t].pairs; out->contains_tests += stats[t].contains_tests;
    out->brick_evals += stats[t].brick_evals; out->sub_evals += stats[t].sub_evals;
    out->voxel_evals += stats[t].voxel_evals; out->paint_evals += stats[t].paint_evals;
    out->allocs += worlds[t]->allocs; out->frees += worlds[t]->frees;
  }
  return 0;
}

void oracle_free(oracle_result* r) {
  std::free(r->grid); std::free(r->pool); std::free(r->free_list);
  r->grid = nullptr; r->pool = nullptr; r->free_list = nullptr;
}

// GpuWorld.ts:90-101: super-grid counts and the density texture's red channel.
// opaque[256]: OPAQUE table (VoxelWorld.ts:190-196); udens[256]: uniform density per id.
void oracle_derive(const oracle_result* r, const uint8_t* opaque, const uint8_t* udens,
                   uint32_t* super_counts, uint8_t* density) {
  int sx = (r->bx + 3) / 4, sy = (r->by + 3) / 4, sz = (r->bz + 3) / 4;
  std::memset(super_counts, 0, (size_t)sx * sy * sz * 4);
  for (int z = 0; z < r->bz; z++)
    for (int y = 0; y < r->by; y++)
      for (int x = 0; x < r->bx; x++) {
        size_t ci = (size_t)x + (size_t)r->bx * ((size_t)y + (size_t)r->by * z);
        uint32_t g = r->grid[ci];
        if (g != 0) super_counts[(x >> 2) + sx * ((y >> 2) + sy * (z >> 2))]++;
        uint8_t d;
        if (g == 0) d = 0;
        else if (g & UNIFORM) d = udens[g & 0xff];
        else {  // VoxelWorld.ts:163-169
          const uint16_t* b = r->pool + (size_t)(g - 1) * BRICK_VOXELS;
          int n = 0;
          for (int i = 0; i < BRICK_VOXELS; i++) { uint16_t v = b[i]; if (v != 0 && opaque[v & 0xff]) n++; }
          d = (uint8_t)js_round(((double)n / BRICK_VOXELS) * 255);
        }
        density[ci] = d;
      }
}

}  // extern "C"
