// Host runtime of the C ABI (include/pixels_gb300.h): world state, PXIR
// validation, per-op derived data, device buffers and the launch sequence of
// one build.  Compiled with -ffp-contract=off: the per-op float64 constants
// (voxel ranges, classify thresholds) must round exactly as the reference's
// JavaScript does (shapes.ts:341-350).
#include <algorithm>
#include <new>
#include <chrono>
#include <cstdlib>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <limits>
#include <mutex>
#include <thread>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/pixels_gb300.h"
#include "px_internal.cuh"
#include "sdf32.cuh"

using namespace px;

namespace {

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  bool borrowed = false;  // another world's buffer (pipelined serving): never reallocated or freed here
};

// The world's host op tables are filled by several host threads at once: a
// resize must not first zero them on one thread, so their elements are
// default-initialised (left as they are) instead of value-initialised.
template <class T>
struct DefaultInitAlloc : std::allocator<T> {
  template <class U>
  struct rebind {
    using other = DefaultInitAlloc<U>;
  };
  DefaultInitAlloc() = default;
  template <class U>
  DefaultInitAlloc(const DefaultInitAlloc<U>&) noexcept {}
  template <class U>
  void construct(U* ptr) noexcept {
    ::new (static_cast<void*>(ptr)) U;
  }
  template <class U, class... Args>
  void construct(U* ptr, Args&&... args) {
    ::new (static_cast<void*>(ptr)) U(std::forward<Args>(args)...);
  }
};
template <class T>
using hvec = std::vector<T, DefaultInitAlloc<T>>;

// one host-to-device copy of a build's op tables
struct Upload {
  void* dst;
  const void* src;
  size_t bytes;
  uint8_t fill = 0;  // without a source: the byte value of the clear
};

}  // namespace

struct px_world {
  int dx, dy, dz, BX, BY, BZ, TX, TY, TZ;
  double vpm, vs;
  size_t ncells, ntiles;
  int n_sms = 0;

  // world state on the device
  uint32_t* d_grid = nullptr;
  uint32_t* d_pool32 = nullptr;   // pool as voxel pairs (capacity * 256 words)
  WorldState* d_state = nullptr;  // poolUsed and hole count as the builds commit them (device)
  bool shares_state = false;      // grid, pool, counts, holes and state belong to another world
  uint16_t* d_pcount = nullptr;   // per pool brick: opaque, non-air voxels (written as bricks are written)
  bool pcount_valid = true;       // d_pcount holds every referenced brick's count (tables unchanged since)
  bool pcount_refresh = false;    // the build in flight recounts them from the pool
  uint32_t pool_cap = 0;
  uint32_t pool_used = 0;
  uint32_t n_holes = 0;
  DevBuf holes_a, holes_b;        // current free list (holes), double-buffered across builds
  bool holes_in_a = true;

  // ops queued by px_submit_ops (and the ops of the last committed build)
  hvec<OpDev> ops, last_ops;
  hvec<uint2> last_boxes, last_code;
  hvec<double> last_params;
  bool ops_resident = false;   // the device op tables already hold `ops`
  hvec<uint2> boxes;
  std::vector<uint2> h_boxes;  // boxes + 32-op group boxes as uploaded
  hvec<uint2> code;
  hvec<double> params;
  hvec<uint32_t> code32, last_code32;   // per instruction: float32 parameter offset
  hvec<float2> p32, last_p32;           // float32 interval parameters
  hvec<float2> bases, last_bases;       // per-op brick-row offsets (mixed mode)
  int validate = 0;
  uint64_t ops_applied = 0;

  // per-build device scratch
  DevBuf d_ops, d_boxes, d_code, d_params, d_code32, d_p32, d_bases;
  std::vector<uint32_t> h_cull_order;  // the ops along a Morton curve of their boxes (cull_sorted_kernel)
  bool cull_sorted = false;
  DevBuf tile_cnt, tile_off, tile_ops, tile_boxes;
  DevBuf evt, fsrc, pos, etype, ew, depth, tree, replay_tmp;
  DevBuf staging, stage_cell, stage_src, touched;
  uint64_t stage_hint = 0;      // staging slots the next build reserves (grown on overflow)
  uint32_t rescue_cap = 1u << 16;  // voxels a build may leave to float64 (grown on overflow)
  DevBuf rescue;
  DevBuf chunk_op, pcode, psub, pmask, chunk_counter, vitems, pitems;
  std::vector<uint32_t> h_chunk_op;  // the chunks in classify order: (chunk, op of its first pair | single-op bit)
  std::vector<Upload> h_uploads;     // the op-table copies of the build being enqueued
  std::vector<uint32_t> h_painted;  // the build's painted ops, float64-only ones first
  // totals of the queued op list, summed as it is converted: (op, brick) pairs,
  // tile-list entries, painted ops (float64-only and certified float32 ones)
  struct QueueTotals {
    uint64_t pairs = 0, tile_pairs = 0;
    std::vector<uint32_t> painted64, painted32;
    void clear() { pairs = tile_pairs = 0; painted64.clear(); painted32.clear(); }
  } q, last_q;
  std::vector<uint8_t> h_op_bucket;  // per op: cost bucket (0..63) of one evaluation
  uint8_t class_order[VCLASSES] = {0};  // sub-block class order of the resident ops
  uint8_t vclass_order[VQ_CLASSES] = {0};  // voxel class order (each group on its own)
  uint32_t vq_nonempty = 0;                // bit g: voxel group g has ops
  DevBuf paint_items, pvals;    // sub-blocks to paint and the paint values
  DevBuf bmark, work;           // bricks the apply pass visits (bitmap, list)
  DevBuf work_counter;
  DevBuf res;
  DevBuf opaque, udens, super_counts, density;
  DevBuf axis32;  // float32 roundings of the voxel centres' coordinates: x, then y, then z
  // derive on build (px_set_derive_on_build): every build ends with the derived
  // upload buffers and the GPU free list for a device limit of derive_max bricks
  uint32_t derive_max = 0;
  DevBuf free_list;
  uint32_t free_len = 0;
  bool free_valid = false;      // free_list holds the current world's GPU free list
  bool free_over = false;       // ... or poolUsed exceeded the capacity (GpuWorld.ts:59)
  BuildResult* h_res = nullptr;   // pinned
  bool host_reads = false;        // the device reads pageable host memory (host page tables)
  bool uploads_pending = false;   // an upload kernel may still read the host op tables

  // in-flight build
  bool in_flight = false;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev_fold0 = nullptr, ev_fold1 = nullptr, ev_mid = nullptr;
  cudaEvent_t ev_eval = nullptr;   // evaluation passes done (the apply stream waits for it)
  cudaEvent_t ev_done = nullptr;   // the build's result block is on the host
  cudaStream_t apply_stream = nullptr;  // pipelined builds: the apply pass's stream (nullptr: the build's)
  bool no_retry = false;           // pipelined builds: a failed build is reported, not retried
  size_t last_P = 0;
  uint32_t last_stage_cap = 0, last_touched_cap = 0;
  int last_mode = 0;
  int retries = 0;
  uint32_t last_H = 0, last_U0 = 0;
  FinalizeArgs fin{};
  bool derived_valid = false;

  // batched builds (px_batch_*): the world's last build is captured in a graph
  bool capturing = false;        // enqueue records no timing events
  bool batch_locked = false;     // buffers are referenced by a graph: no rebuild, reset or destroy
  bool batch_holes_in_a = true;  // holes_in_a of the captured build
  uint32_t pairs_per_block = 0;  // launch shape: persistent grids sized to the build (0: whole GPU)

  px_stats stats{};
  std::string err;
};

namespace {

int fail(px_world* w, int code, const char* fmt, ...) {
  if (w) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    std::vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    w->err = buf;
  }
  return code;
}

#define CU(call)                                                                           \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess) return fail(w, PX_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

int ensure(px_world* w, DevBuf& b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (b.bytes >= bytes) return PX_OK;
  if (b.borrowed) return fail(w, PX_E_OOM, "a shared buffer of %zu bytes is too small (%zu needed)", b.bytes, bytes);
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
  size_t want = bytes + bytes / 4;
  if (cudaMalloc(&b.p, want) != cudaSuccess) {
    cudaGetLastError();
    return fail(w, PX_E_OOM, "cudaMalloc of %zu bytes failed", want);
  }
  b.bytes = want;
  return PX_OK;
}
void release(DevBuf& b) {
  if (b.borrowed) { b = DevBuf{}; return; }
  if (b.p) cudaFree(b.p);
  b.p = nullptr;
  b.bytes = 0;
}

inline double js_max(double a, double b) { return a > b ? a : b; }  // finite inputs (validated)
inline double js_min(double a, double b) { return a < b ? a : b; }

// float32 enclosures of float64 values (mixed mode)
// the neighbouring floats of a float (by its bit pattern; inlined, unlike nextafterf)
inline float float_below(float f) {
  if (f == 0.0f) return -std::numeric_limits<float>::denorm_min();
  uint32_t b;
  std::memcpy(&b, &f, 4);
  b = f > 0.0f ? b - 1 : b + 1;
  std::memcpy(&f, &b, 4);
  return f;
}
inline float float_above(float f) {
  if (f == 0.0f) return std::numeric_limits<float>::denorm_min();
  uint32_t b;
  std::memcpy(&b, &f, 4);
  b = f > 0.0f ? b + 1 : b - 1;
  std::memcpy(&f, &b, 4);
  return f;
}
// float32 bounds of a float64 value: the largest float <= v, the smallest float >= v
inline float rd32(double v) {
  float f = (float)v;
  if ((double)f > v) f = float_below(f);
  return f;
}
inline float ru32(double v) {
  float f = (float)v;
  if ((double)f < v) f = float_above(f);
  return f;
}
inline float2 enc(double v, double pad = 0.0) { return make_float2(rd32(v - pad), ru32(v + pad)); }

// Runs of k >= 2 rotations (not all about y: those stay y-extruded) whose k ends
// are consecutive instructions -- rotateZ(rotateY(rotateZ(shape))) and the like:
// flag[first rotation] = C32_AFFINE | k; the run's other rotations and its ends
// but the first, C32_SKIP.
void rotation_runs(const uint32_t* code, uint32_t n, std::vector<uint32_t>& flag) {
  auto is_rot = [](uint32_t op) { return op == OP_ROT_X || op == OP_ROT_Y || op == OP_ROT_Z; };
  std::vector<int> close(n, -1), stack;
  for (uint32_t i = 0; i < n; i++) {
    const uint32_t op = code[2 * i] & 0xffu;
    if (is_rot(op)) stack.push_back((int)i);
    else if (op == OP_ROT_END && !stack.empty()) { close[stack.back()] = (int)i; stack.pop_back(); }
  }
  for (uint32_t i = 0; i < n; i++) {
    if (!is_rot(code[2 * i] & 0xffu) || (i && is_rot(code[2 * (i - 1)] & 0xffu))) continue;
    uint32_t k = 0;
    bool all_y = true;
    while (i + k < n && is_rot(code[2 * (i + k)] & 0xffu)) { all_y = all_y && (code[2 * (i + k)] & 0xffu) == OP_ROT_Y; k++; }
    if (k < 2 || all_y || k > 255) continue;
    const int e0 = close[i + k - 1];
    bool consecutive = e0 >= 0;
    for (uint32_t j = 0; j < k && consecutive; j++) consecutive = close[i + k - 1 - j] == e0 + (int)j;
    if (!consecutive) continue;
    flag[i] = C32_AFFINE | k;
    for (uint32_t j = 1; j < k; j++) flag[i + j] = C32_SKIP;
    for (uint32_t j = 1; j < k; j++) flag[(uint32_t)e0 + j] = C32_SKIP;
  }
}

// The k rotations from instruction i composed into x' = M x + t (shapes.ts:263-320:
// each maps the point about its pivot with its float64 cos and sin), in the op's
// anchor coordinates, as float32 intervals: M row by row, then t.  The exact map
// is the composition of the exact rotations on those float64 constants; the
// float64 arithmetic here errs by far less than the padding.
bool compose_rotations(const uint32_t* code, uint32_t i, uint32_t k, const double* P, const double A[3],
                       std::vector<float2>& p32) {
  double M[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, t[3] = {0, 0, 0};
  double mag = 0;  // a bound of the magnitudes summed into t
  for (uint32_t j = 0; j < k; j++) {  // the outermost rotation acts first on the point
    const uint32_t op = code[2 * (i + j)] & 0xffu;
    const double* q = P + code[2 * (i + j) + 1];
    const double p0 = q[0], p1 = q[1], c = q[2], sn = q[3];
    double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, b[3] = {0, 0, 0};
    int u = 0, v = 2;  // the rotated axes: x' about (u, v) = (p0, p1)
    if (op == OP_ROT_X) { u = 1; v = 2; } else if (op == OP_ROT_Z) { u = 0; v = 1; }
    R[u][u] = c; R[u][v] = sn; R[v][u] = -sn; R[v][v] = c;
    b[u] = p0 - c * p0 - sn * p1;
    b[v] = p1 + sn * p0 - c * p1;
    mag += std::fabs(p0) + std::fabs(p1);
    double M2[3][3], t2[3];
    for (int r = 0; r < 3; r++) {
      t2[r] = b[r];
      for (int cc = 0; cc < 3; cc++) {
        M2[r][cc] = 0;
        for (int m = 0; m < 3; m++) M2[r][cc] += R[r][m] * M[m][cc];
        t2[r] += R[r][cc] * t[cc];
      }
    }
    std::memcpy(M, M2, sizeof M);
    std::memcpy(t, t2, sizeof t);
  }
  bool ok = true;
  const double padM = 0x1p-44 * (double)k, amag = std::fabs(A[0]) + std::fabs(A[1]) + std::fabs(A[2]);
  const double padT = (mag * 3 + amag * 3 + 1.0) * 0x1p-44 * (double)k;
  for (int r = 0; r < 3; r++)
    for (int cc = 0; cc < 3; cc++) {
      const float2 e = enc(M[r][cc], padM);
      if (!std::isfinite(e.x) || !std::isfinite(e.y)) ok = false;
      p32.push_back(e);
    }
  for (int r = 0; r < 3; r++) {  // x' - A = M (X + A) + t - A in anchor coordinates X = x - A
    double tr = t[r] - A[r];
    for (int cc = 0; cc < 3; cc++) tr += M[r][cc] * A[cc];
    const float2 e = enc(tr, padT);
    if (!std::isfinite(e.x) || !std::isfinite(e.y) || std::fabs(tr) > 4 * MIXED_MAX_COORD) ok = false;
    p32.push_back(e);
  }
  return ok;
}

// The lean voxel kernel's reading of a program (LP_* forms in px_internal.cuh), or
// lp[LP_FORM] = 0.  A stage is one rotation, or a run composed by rotation_runs.
void lean_program(const uint32_t* code, uint32_t n, uint8_t lp[8]) {
  if (n > 40) return;
  std::vector<uint32_t> flag(n, 0u);
  rotation_runs(code, n, flag);
  auto op_at = [&](uint32_t i) { return code[2 * i] & 0xffu; };
  auto is_prim = [&](uint32_t i) { return i < n && op_at(i) >= OP_BOX && op_at(i) < OP_ROT_X; };
  auto is_rot = [&](uint32_t i) { return i < n && (op_at(i) == OP_ROT_X || op_at(i) == OP_ROT_Y || op_at(i) == OP_ROT_Z); };
  // a stage at i: returns its kind and instruction count, and the ends it needs
  auto stage = [&](uint32_t i, uint32_t& kind, uint32_t& len) {
    kind = 0; len = 0;
    if (!is_rot(i)) return true;
    if (flag[i] & C32_AFFINE) { kind = LP_AFFINE; len = flag[i] & 0xffu; return true; }
    if (is_rot(i + 1)) return false;  // an uncomposed run (all about y): not a lean program
    kind = op_at(i) - OP_ROT_X + 1; len = 1;
    return true;
  };
  auto ends = [&](uint32_t i, uint32_t len) {
    for (uint32_t j = 0; j < len; j++) if (i + j >= n || op_at(i + j) != OP_ROT_END) return false;
    return true;
  };
  auto comb_of = [&](uint32_t i) -> uint32_t {
    if (i >= n) return 0;
    const uint32_t o = op_at(i);
    return o == OP_NEGMAX ? LP_NEGMAX : o == OP_MAX ? LP_MAX : o == OP_MIN ? LP_MIN : 0;
  };
  uint32_t k1, l1;
  if (!stage(0, k1, l1)) return;
  uint32_t i = l1;
  if (!is_prim(i)) return;
  const uint32_t p1 = i++;
  uint32_t form = 1, p2 = LP_NONE, s2 = LP_NONE, k2 = 0, comb = 0;
  if (is_prim(i) && comb_of(i + 1)) {  // form 2: both primitives in the one stage
    form = 2; p2 = i; comb = comb_of(i + 1); i += 2;
    if (!ends(i, l1)) return;
    i += l1;
  } else {
    if (!ends(i, l1)) return;
    i += l1;
    uint32_t l2;
    if (i < n && (is_rot(i) || is_prim(i))) {  // form 3: a second staged primitive, then comb
      if (!stage(i, k2, l2)) return;
      s2 = i; i += l2;
      if (!is_prim(i)) return;
      p2 = i++;
      if (!ends(i, l2)) return;
      i += l2;
      comb = comb_of(i);
      if (!comb) return;
      i++;
      form = 3;
    }
  }
  uint32_t off = LP_NONE;
  if (i < n && op_at(i) == OP_OFFSET) off = i++;
  if (i != n) return;
  lp[LP_FORM] = (uint8_t)form; lp[LP_COMB] = (uint8_t)comb;
  lp[LP_P1] = (uint8_t)p1; lp[LP_P2] = (uint8_t)p2;
  lp[LP_S1] = l1 ? 0 : LP_NONE; lp[LP_S2] = (uint8_t)(k2 ? s2 : LP_NONE);
  lp[LP_KINDS] = (uint8_t)(k1 | (k2 << 4)); lp[LP_OFF] = (uint8_t)off;
}

// Convert one op's SDF parameters to float32 intervals relative to the op's
// anchor.  Positions are shifted by the anchor; reciprocals (1/r, 1/|e|^2)
// replace the divisions; polygon edges are expanded to per-vertex records.
// Returns false when a value falls outside the range the float32 path
// certifies (the op then runs in float64 only).
bool convert32(const uint32_t* code, uint32_t n, const double* P, const double A[3], std::vector<uint32_t>& code32,
               std::vector<float2>& p32) {
  bool ok = true;
  auto put = [&](double v, double pad) {
    float2 e = enc(v, pad);
    if (!std::isfinite(e.x) || !std::isfinite(e.y) || std::fabs(v) > MIXED_MAX_COORD) ok = false;
    p32.push_back(e);
  };
  auto val = [&](double v) { put(v, 0.0); };
  auto pos = [&](double v, int axis) { double r = v - A[axis]; put(r, (std::fabs(v) + std::fabs(A[axis])) * 0x1p-52); };
  auto inv = [&](double v) {
    double r = 1.0 / v;
    float2 e = enc(r, std::fabs(r) * 0x1p-51);
    if (!std::isfinite(e.x) || !std::isfinite(e.y) || std::fabs(r) > 0x1p60 || v == 0.0) ok = false;
    p32.push_back(e);
  };
  auto edge = [&](double vjx, double vjy, double vix, double viy, bool with_vjy, bool polyline) {
    double ex = vjx - vix, ey = vjy - viy;  // polygon: from i to j = i - 1; polyline: from a to b
    if (polyline) { val(vix); val(viy); }
    else { val(vix); val(viy); if (with_vjy) val(vjy); }
    put(ex, (std::fabs(vjx) + std::fabs(vix)) * 0x1p-52);
    put(ey, (std::fabs(vjy) + std::fabs(viy)) * 0x1p-52);
    double den = ex * ex + ey * ey;
    if (den == 0.0) {  // the reference's `|| 1e-12`; e is exactly zero then
      p32.push_back(make_float2(rd32(1e12), ru32(1e12)));
    } else {
      double r = 1.0 / den;
      float2 e = enc(r, std::fabs(r) * 0x1p-46);
      if (!std::isfinite(e.x) || !std::isfinite(e.y) || std::fabs(r) > 0x1p60) ok = false;
      p32.push_back(e);
    }
  };
  // runs of rotations whose ends follow each other: composed into one affine map
  std::vector<uint32_t> flag(n, 0u);
  rotation_runs(code, n, flag);
  for (uint32_t i = 0; i < n; i++) {
    uint32_t op = code[2 * i] & 0xffu, cnt = code[2 * i] >> 8;
    const double* p = P + code[2 * i + 1];
    if (flag[i] & C32_SKIP) {
      code32.push_back(C32_SKIP);
      continue;
    }
    if (flag[i] & C32_AFFINE) {
      code32.push_back(C32_AFFINE | (uint32_t)p32.size());
      if (!compose_rotations(code, i, flag[i] & 0xffu, P, A, p32)) ok = false;
      continue;
    }
    code32.push_back((uint32_t)p32.size());
    switch (op) {
      case OP_BOX: pos(p[0], 0); pos(p[1], 1); pos(p[2], 2); val(p[3]); val(p[4]); val(p[5]); break;
      case OP_ROUNDBOX: pos(p[0], 0); pos(p[1], 1); pos(p[2], 2); val(p[3]); val(p[4]); val(p[5]); val(p[6]); break;
      case OP_SPHERE: pos(p[0], 0); pos(p[1], 1); pos(p[2], 2); val(p[3]); break;
      case OP_ELLIPSOID: pos(p[0], 0); pos(p[1], 1); pos(p[2], 2); inv(p[3]); inv(p[4]); inv(p[5]); val(p[6]); break;
      case OP_CYL_X: case OP_CYL_Y: case OP_CYL_Z:
      case OP_TORUS_X: case OP_TORUS_Y: case OP_TORUS_Z:
        pos(p[0], 0); pos(p[1], 1); pos(p[2], 2); val(p[3]); val(p[4]); break;
      case OP_CAPSULE: pos(p[0], 0); pos(p[1], 1); pos(p[2], 2); val(p[3]); val(p[4]); val(p[5]); inv(p[6]); val(p[7]); break;
      case OP_LATHE_SOLID: {
        pos(p[0], 0); pos(p[1], 1); pos(p[2], 2);
        const double* v = p + 3;
        for (uint32_t k = 0; k < cnt; k++) {
          uint32_t j = k ? k - 1 : cnt - 1;
          edge(v[2 * j], v[2 * j + 1], v[2 * k], v[2 * k + 1], true, false);
        }
        break;
      }
      case OP_LATHE_SHELL: {
        pos(p[0], 0); pos(p[1], 1); pos(p[2], 2); val(p[3]);
        const double* v = p + 4;
        for (uint32_t k = 0; k + 1 < cnt; k++) edge(v[2 * k + 2], v[2 * k + 3], v[2 * k], v[2 * k + 1], false, true);
        break;
      }
      case OP_PRISM: {
        pos(p[0], 0); pos(p[1], 2); pos(p[2], 1); val(p[3]);
        const double* v = p + 4;
        for (uint32_t k = 0; k < cnt; k++) {
          uint32_t j = k ? k - 1 : cnt - 1;
          edge(v[2 * j], v[2 * j + 1], v[2 * k], v[2 * k + 1], true, false);
        }
        break;
      }
      case OP_STADIUM: pos(p[0], 0); pos(p[1], 2); val(p[2]); val(p[3]); pos(p[4], 1); val(p[5]); break;
      case OP_ROT_X: pos(p[0], 1); pos(p[1], 2); val(p[2]); val(p[3]); break;
      case OP_ROT_Y: pos(p[0], 0); pos(p[1], 2); val(p[2]); val(p[3]); break;
      case OP_ROT_Z: pos(p[0], 0); pos(p[1], 1); val(p[2]); val(p[3]); break;
      case OP_OFFSET: val(p[0]); break;
      default: break;
    }
  }
  return ok;
}

// Validate one op's SDF bytecode: opcodes, parameter ranges, finite values,
// stack and rotation depths.  `deep` is set when the program needs more than
// the register evaluators hold (it then runs on the deep float64 evaluator).
bool check_code(const uint32_t* code, uint32_t n, const double* P, size_t np, std::string& why, bool& deep) {
  int depth = 0, rot = 0, max_depth = 0, max_rot = 0;
  for (uint32_t i = 0; i < n; i++) {
    uint32_t w0 = code[2 * i], off = code[2 * i + 1];
    uint32_t op = w0 & 0xffu, cnt = w0 >> 8;
    size_t need = 0;
    switch (op) {
      case OP_BOX: need = 6; break;
      case OP_ROUNDBOX: need = 7; break;
      case OP_SPHERE: need = 4; break;
      case OP_ELLIPSOID: need = 7; break;
      case OP_CYL_X: case OP_CYL_Y: case OP_CYL_Z: need = 5; break;
      case OP_CAPSULE: need = 8; break;
      case OP_TORUS_X: case OP_TORUS_Y: case OP_TORUS_Z: need = 5; break;
      case OP_STADIUM: need = 6; break;
      case OP_LATHE_SOLID:
        if (cnt < 2) { why = "lathe polygon needs 2+ points"; return false; }
        need = 3 + 2 * (size_t)cnt; break;
      case OP_LATHE_SHELL:
        if (cnt < 2) { why = "lathe profile needs 2+ points"; return false; }
        need = 4 + 2 * (size_t)cnt; break;
      case OP_PRISM:
        if (cnt < 3) { why = "prism needs 3+ points"; return false; }
        need = 4 + 2 * (size_t)cnt; break;
      case OP_ROT_X: case OP_ROT_Y: case OP_ROT_Z:
        need = 4;
        if (++rot > DEEP_MAX_ROT) { why = "rotations nested deeper than 16"; return false; }
        max_rot = std::max(max_rot, rot);
        break;
      case OP_ROT_END:
        if (--rot < 0) { why = "unmatched rotation end"; return false; }
        break;
      case OP_OFFSET: need = 1; if (depth < 1) { why = "offset of nothing"; return false; } break;
      case OP_NEGMAX: case OP_MAX: case OP_MIN:
        if (depth < 2) { why = "combinator needs two operands"; return false; }
        depth--; break;
      default: why = "unknown opcode"; return false;
    }
    if (need) {
      if ((size_t)off + need > np) { why = "parameters out of range"; return false; }
      for (size_t k = 0; k < need; k++)
        if (!std::isfinite(P[off + k])) { why = "non-finite parameter"; return false; }
    }
    if (op < OP_ROT_X) {
      if (++depth > DEEP_MAX_STACK) { why = "SDF stack deeper than 32"; return false; }
      max_depth = std::max(max_depth, depth);
    }
  }
  if (depth != 1 || rot != 0) { why = "bytecode does not leave exactly one distance"; return false; }
  deep = max_depth > MAX_STACK || max_rot > MAX_ROT;
  return true;
}

// Grow the device pool to at least `need` bricks, keeping the first `keep`
// bricks (growPool, VoxelWorld.ts:129-136, grows by 1.5x).
int grow_pool(px_world* w, uint64_t need, uint32_t keep, cudaStream_t s) {
  if (need <= w->pool_cap) return PX_OK;
  if (w->shares_state) return fail(w, PX_E_OOM, "the shared pool of %u bricks cannot grow here", w->pool_cap);
  uint64_t cap = w->pool_cap ? w->pool_cap : 1;
  while (cap < need) cap = (uint64_t)std::ceil(cap * 1.5) + 1;
  if (cap > 0x3fffffffull) return fail(w, PX_E_OOM, "pool of %llu bricks exceeds the index range", (unsigned long long)cap);
  uint32_t* np_ = nullptr;
  uint16_t* nc_ = nullptr;
  if (cudaMalloc((void**)&np_, (size_t)cap * 1024) != cudaSuccess) {
    cudaGetLastError();
    return fail(w, PX_E_OOM, "pool of %llu bricks", (unsigned long long)cap);
  }
  if (cudaMalloc((void**)&nc_, (size_t)cap * 2) != cudaSuccess) {
    cudaGetLastError();
    cudaFree(np_);
    return fail(w, PX_E_OOM, "pool of %llu bricks", (unsigned long long)cap);
  }
  if (keep) {
    CU(cudaMemcpyAsync(np_, w->d_pool32, (size_t)keep * 1024, cudaMemcpyDeviceToDevice, s));
    CU(cudaMemcpyAsync(nc_, w->d_pcount, (size_t)keep * 2, cudaMemcpyDeviceToDevice, s));
  }
  CU(cudaStreamSynchronize(s));
  cudaFree(w->d_pool32);
  cudaFree(w->d_pcount);
  w->d_pool32 = np_;
  w->d_pcount = nc_;
  w->pool_cap = (uint32_t)cap;
  return PX_OK;
}

}  // namespace

// Host exceptions never cross the C ABI: an entry point that allocates host
// memory (op tables, worlds) turns a failed allocation into PX_E_OOM.
template <class F>
int guarded(px_world* w, F&& f) {
  try {
    return f();
  } catch (const std::bad_alloc&) {
    if (w) try { w->err = "host allocation failed"; } catch (...) {}
    return PX_E_OOM;
  } catch (...) {
    if (w) try { w->err = "unexpected host exception"; } catch (...) {}
    return PX_E_CUDA;
  }
}

extern "C" {

static int world_create_impl(int dx, int dy, int dz, double vpm, uint32_t initial_pool_bricks, px_world** out) {
  if (!out) return PX_E_INVALID_ARG;
  *out = nullptr;
  if (dx <= 0 || dy <= 0 || dz <= 0 || dx % 8 || dy % 8 || dz % 8) return PX_E_INVALID_ARG;
  if (dx / 8 > MAX_AXIS_BRICKS || dy / 8 > MAX_AXIS_BRICKS || dz / 8 > MAX_AXIS_BRICKS) return PX_E_INVALID_ARG;
  if (!(vpm > 0) || !std::isfinite(vpm)) return PX_E_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return PX_E_NO_DEVICE;
  }
  px_world* w = new px_world();
  w->dx = dx; w->dy = dy; w->dz = dz;
  w->BX = dx / 8; w->BY = dy / 8; w->BZ = dz / 8;
  w->TX = (w->BX + 3) / 4; w->TY = (w->BY + 3) / 4; w->TZ = (w->BZ + 3) / 4;
  for (int k = 0; k < VCLASSES; k++) w->class_order[k] = (uint8_t)k;
  for (int k = 0; k < VQ_CLASSES; k++) w->vclass_order[k] = (uint8_t)k;
  w->vpm = vpm;
  w->vs = 1 / vpm;  // config.ts:13
  w->ncells = (size_t)w->BX * w->BY * w->BZ;
  w->ntiles = (size_t)w->TX * w->TY * w->TZ;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&w->n_sms, cudaDevAttrMultiProcessorCount, dev);
  {
    int pma = 0, hpt = 0;
    cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, dev);
    cudaDeviceGetAttribute(&hpt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
    w->host_reads = pma == 1 && hpt == 1 && getenv("PIXELS_GB300_NO_HOST_READS") == nullptr;
  }
  int rc;
  DevBuf g;
  if ((rc = ensure(w, g, w->ncells * 4)) != PX_OK) { delete w; return rc; }
  w->d_grid = (uint32_t*)g.p;
  if (cudaMemset(w->d_grid, 0, w->ncells * 4) != cudaSuccess) { delete w; return PX_E_CUDA; }
  uint32_t cap = initial_pool_bricks ? initial_pool_bricks : 1;
  if (cudaMalloc((void**)&w->d_pool32, (size_t)cap * 1024) != cudaSuccess) { cudaFree(w->d_grid); delete w; return PX_E_OOM; }
  if (cudaMalloc((void**)&w->d_pcount, (size_t)cap * 2) != cudaSuccess) {
    cudaFree(w->d_grid); cudaFree(w->d_pool32); delete w; return PX_E_OOM;
  }
  w->pool_cap = cap;
  if (cudaMallocHost((void**)&w->h_res, sizeof(BuildResult)) != cudaSuccess) { delete w; return PX_E_OOM; }
  if (cudaMalloc((void**)&w->d_state, sizeof(WorldState)) != cudaSuccess ||
      cudaMemset(w->d_state, 0, sizeof(WorldState)) != cudaSuccess) {
    cudaGetLastError();
    delete w;
    return PX_E_OOM;
  }
  cudaEventCreate(&w->ev0);
  cudaEventCreate(&w->ev1);
  cudaEventCreate(&w->ev_fold0);
  cudaEventCreate(&w->ev_fold1);
  cudaEventCreate(&w->ev_mid);
  cudaEventCreateWithFlags(&w->ev_eval, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&w->ev_done, cudaEventDisableTiming);
  // material tables (VoxelWorld.ts:159-170,190-196): filled by px_set_tables or the defaults
  uint8_t op_tab[256], ud_tab[256];
  for (int i = 0; i < 256; i++) { op_tab[i] = i ? 1 : 0; ud_tab[i] = 255; }
  ensure(w, w->opaque, 256);
  ensure(w, w->udens, 256);
  cudaMemcpy(w->opaque.p, op_tab, 256, cudaMemcpyHostToDevice);
  cudaMemcpy(w->udens.p, ud_tab, 256, cudaMemcpyHostToDevice);
  {  // the voxel centres' coordinates as the paint calls form them, (i + 0.5) * vs, rounded to float32
    std::vector<float> ax((size_t)dx + dy + dz);
    size_t at = 0;
    for (int n : {dx, dy, dz})
      for (int i = 0; i < n; i++) ax[at++] = (float)(((double)i + 0.5) * w->vs);
    if ((rc = ensure(w, w->axis32, ax.size() * 4)) != PX_OK ||
        cudaMemcpy(w->axis32.p, ax.data(), ax.size() * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
      cudaGetLastError();
      px_world_destroy(w);
      return rc ? rc : PX_E_CUDA;
    }
  }
  *out = w;
  return PX_OK;
}

// Opacity (OPAQUE, VoxelWorld.ts:190-196) and uniform-brick density per material id.
int px_set_material_tables(px_world* w, const uint8_t* opaque256, const uint8_t* uniform_density256) {
  if (!w || !opaque256 || !uniform_density256) return PX_E_INVALID_ARG;
  CU(cudaMemcpy(w->opaque.p, opaque256, 256, cudaMemcpyHostToDevice));
  CU(cudaMemcpy(w->udens.p, uniform_density256, 256, cudaMemcpyHostToDevice));
  w->derived_valid = false;
  w->pcount_valid = false;  // the pool bricks' opaque counts follow the old table
  return PX_OK;
}

void px_world_destroy(px_world* w) {
  if (!w || w->batch_locked) return;  // a batch's world outlives the batch
  if (w->in_flight || w->uploads_pending) cudaStreamSynchronize(w->stream);
  if (!w->shares_state) {
    cudaFree(w->d_grid);
    cudaFree(w->d_pool32);
    cudaFree(w->d_pcount);
    cudaFree(w->d_state);
  }
  DevBuf* bufs[] = {&w->holes_a, &w->holes_b, &w->d_ops, &w->d_boxes, &w->d_code, &w->d_params, &w->d_code32,
                    &w->d_p32, &w->d_bases, &w->tile_cnt,
                    &w->tile_off, &w->tile_ops, &w->evt, &w->fsrc, &w->pos, &w->etype,
                    &w->ew, &w->replay_tmp, &w->depth, &w->tree, &w->staging, &w->touched,
                    &w->stage_cell, &w->stage_src, &w->chunk_op, &w->pcode, &w->psub, &w->pmask,
                    &w->chunk_counter, &w->vitems, &w->work_counter, &w->res, &w->opaque,
                    &w->udens, &w->super_counts, &w->density, &w->paint_items, &w->pvals, &w->tile_boxes, &w->bmark, &w->work, &w->pitems,
                    &w->free_list, &w->rescue};
  for (DevBuf* b : bufs) release(*b);
  if (w->h_res) cudaFreeHost(w->h_res);
  if (w->ev0) cudaEventDestroy(w->ev0);
  if (w->ev1) cudaEventDestroy(w->ev1);
  if (w->ev_fold0) cudaEventDestroy(w->ev_fold0);
  if (w->ev_fold1) cudaEventDestroy(w->ev_fold1);
  if (w->ev_mid) cudaEventDestroy(w->ev_mid);
  if (w->ev_eval) cudaEventDestroy(w->ev_eval);
  if (w->ev_done) cudaEventDestroy(w->ev_done);
  delete w;
}

// Float32 parameters of the certified paint evaluation (paint32.cuh) for one
// op, relative to its anchor A.  Returns false (float64 only) for a paint
// frame or values outside the certified range.
bool paint_params32(uint32_t kind, bool framed, const double* p, const double A[3], std::vector<float2>& out) {
  if (kind == PK_NOISE && !framed) {  // noise32: the float32 values the float64 path converts to
    const double sc = p[1];
    const float sl = rd32(sc), sh = ru32(sc);
    if (!(sl > 0.f) || !std::isfinite(sh)) return false;
    for (int k : {6, 7})
      if (!(p[k] >= 0 && p[k] <= 65535.0 && p[k] == std::floor(p[k]))) return false;
    auto bits = [](uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; };
    out.push_back(make_float2(bits((uint32_t)(long long)p[0]), 0.f));
    out.push_back(make_float2(sl, sh));
    out.push_back(make_float2((float)p[2], (float)p[3]));
    out.push_back(make_float2((float)p[4], (float)p[5]));
    out.push_back(make_float2(bits((uint32_t)p[6]), bits((uint32_t)p[7])));
    return true;
  }
  if (framed || (kind != PK_TUFTED && kind != PK_PAINTING && kind != PK_VASE)) return false;
  if (kind == PK_VASE && !(p[3] > 0x1p-20 && p[3] < 0x1p20)) return false;
  bool ok = true;
  auto put = [&](float2 e, double v) {
    if (!std::isfinite(e.x) || !std::isfinite(e.y) || std::fabs(v) > MIXED_MAX_COORD) ok = false;
    out.push_back(e);
  };
  auto pos = [&](double v, int axis) {  // v - A[axis], enclosing the real difference
    const double r = v - A[axis];
    put(enc(r, (std::fabs(v) + std::fabs(A[axis])) * 0x1p-52), v);
  };
  auto thr = [&](double v) { put(make_float2(rd32(v), ru32(v)), v); };
  auto intv = [&](double v) {  // a value the reference converts with (x & 0xff) after truncation
    put(make_float2((float)((long long)v & 0xff), 0.f), 0.0);
  };
  if (kind == PK_TUFTED) {  // penthouse.ts:495-501
    pos(p[0], 2);
    pos(p[1], 1);
    const double r = 1.0 / 0.16;  // the real 1/0.16 (float64 0.16) lies within 2^-53 of r
    put(enc(r, r * 0x1p-52), r);
    thr(0.12);
    intv(p[2]);
  } else if (kind == PK_VASE) {  // penthouse.ts:810-816
    pos(p[0], 0);
    pos(p[1], 1);
    pos(p[2], 2);
    const double r = 1.0 / p[3];  // the real 1/height lies within 2^-53 (relative) of r
    put(enc(r, r * 0x1p-52), r);
    for (double c : {0.04, 0.06, 0.36, 0.38, 0.47, 0.49, 0.08, 0.33, 0.55}) thr(c);
    intv(p[4]);
  } else {  // penthouse.ts:840-845
    const long double K = 9.0L * (long double)A[0] + 3.0L * (long double)A[1];
    const long double k = std::floor(K / (2.0L * 3.14159265358979323846264338327950288L) + 0.5L);
    const long double Kr = K - k * (2.0L * 3.14159265358979323846264338327950288L);
    put(enc((double)Kr, 0x1p-40), 0.0);  // generous pad for the reduction's rounding
    const double k13 = 1.3;
    put(enc(k13, 0.0), k13);
    thr(0.06);
    intv(p[0]);
    for (int i = 0; i < 9; i++) {
      const double* b = p + 1 + 4 * i;
      pos(b[0], 0);
      pos(b[1], 1);
      thr(b[2]);
      intv(b[3]);
    }
  }
  return ok;
}

}  // extern "C"

namespace {

// Relative cost of one evaluation of an op's shape (ordering only: the
// costliest work is taken first so that no long item starts last); code: the
// op's instructions (opcode | count << 8, parameter offset).
float op_cost(const uint32_t* code, uint32_t code_len, uint32_t flags) {
  float c = 0.f;
  for (uint32_t i = 0; i < code_len; i++) {
    const uint32_t x = code[2 * (size_t)i], op = x & 0xffu, cnt = x >> 8;
    if (op == OP_LATHE_SOLID || op == OP_PRISM) c += 0.7f * (float)cnt;
    else if (op == OP_LATHE_SHELL) c += 0.6f * (float)cnt;
    else if (op == OP_ELLIPSOID || op == OP_CAPSULE || op == OP_STADIUM || (op >= OP_TORUS_X && op <= OP_TORUS_Z)) c += 1.5f;
    else if (op < OP_ROT_X) c += 1.f;
    else if (op <= OP_ROT_Z) c += 0.5f;
    else c += 0.1f;
  }
  if (flags & OPF_FP64_ONLY) c *= 8.f;
  if (flags & OPF_CONTAINS) c *= 0.5f;
  return c;
}

// One contiguous range of a submitted op list, converted by one host thread:
// offsets into its own arrays, rebased when the ranges are merged in order.
struct SubmitChunk {
  std::vector<OpDev> ops;
  std::vector<uint2> boxes, code;
  std::vector<double> xparams;     // expanded polygon records (device float64 layout)
  std::vector<uint32_t> code32;    // float32 parameter offset per instruction
  std::vector<float2> bases, p32;
  std::vector<uint32_t> xfix;      // instructions whose parameter offset is a polygon record
  uint64_t n_pairs = 0, n_tile_pairs = 0;        // the range's (op, brick) pairs and tile-list entries
  std::vector<uint32_t> painted64, painted32;    // its painted ops (range-local indices)
  int rc = PX_OK;
  std::string err;
};

int chunk_fail(SubmitChunk& out, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  out.rc = code;
  out.err = buf;
  return code;
}

int convert_ops(const px_world* w, const IrOp* iops, size_t i0, size_t i1, const uint32_t* code, size_t n_code,
                const double* P, size_t n_params, size_t param_base, SubmitChunk& out) {
  const double vs = w->vs;
  out.ops.reserve(i1 - i0);
  out.boxes.reserve(i1 - i0);
  out.code.reserve(4 * (i1 - i0));
  out.code32.reserve(4 * (i1 - i0));
  out.p32.reserve(32 * (i1 - i0));
  out.bases.reserve(16 * (i1 - i0));
  for (size_t i = i0; i < i1; i++) {
    const IrOp& o = iops[i];
    std::string why;
    if (o.kind > 2) return chunk_fail(out, PX_E_INVALID_IR, "op %zu: bad kind", i);
    if (o.paint_kind >= PK_COUNT) return chunk_fail(out, PX_E_INVALID_IR, "op %zu: unknown paint kind", i);
    if (o.paint_kind == PK_CONST && o.paint_value > 0xffffu) return chunk_fail(out, PX_E_INVALID_IR, "op %zu: paint is not a u16", i);
    if (o.paint_kind != PK_CONST) {
      size_t np = (size_t)PAINT_NPARAMS[o.paint_kind];
      if ((size_t)o.paint_param + np > n_params) return chunk_fail(out, PX_E_INVALID_IR, "op %zu: paint parameters out of range", i);
      for (size_t k = 0; k < np; k++)
        if (!std::isfinite(P[o.paint_param + k])) return chunk_fail(out, PX_E_INVALID_IR, "op %zu: non-finite paint parameter", i);
      if (o.paint_kind == PK_NOISE)  // its two results are voxel values (u16), like every other paint's
        for (int k = 6; k < 8; k++) {
          const double v = P[o.paint_param + k];
          if (!(v >= 0 && v <= 65535 && v == std::floor(v)))
            return chunk_fail(out, PX_E_INVALID_IR, "op %zu: noise paint values must be integers in [0, 65535]", i);
        }
    }
    for (int k = 0; k < 3; k++)
      if (!std::isfinite(o.mn[k]) || !std::isfinite(o.mx[k])) return chunk_fail(out, PX_E_INVALID_IR, "op %zu: non-finite bounds", i);
    if (!std::isfinite(o.slack)) return chunk_fail(out, PX_E_INVALID_IR, "op %zu: non-finite slack", i);
    for (int k = 0; k < 4; k++)
      if (!std::isfinite(o.frame[k])) return chunk_fail(out, PX_E_INVALID_IR, "op %zu: non-finite paint frame", i);
    if (o.code_len == 0 || (size_t)o.code_begin + o.code_len > n_code) return chunk_fail(out, PX_E_INVALID_IR, "op %zu: code range", i);
    bool deep = false;
    if (!check_code(code + 2 * (size_t)o.code_begin, o.code_len, P, n_params, why, deep))
      return chunk_fail(out, PX_E_INVALID_IR, "op %zu: %s", i, why.c_str());

    OpDev d{};
    d.kind = o.kind;
    d.flags = o.flags & OPF_FROM_IR;
    if (deep) d.flags |= OPF_DEEP | OPF_FP64_ONLY;  // beyond the register evaluators: float64, stack in local memory
    d.paint_kind = o.paint_kind;
    d.paint_value = o.paint_value;
    d.code_off = (uint32_t)out.code.size();  // + the chunk's code base (merge)
    for (uint32_t k = 0; k < o.code_len; k++) {
      const uint32_t* ins = code + 2 * ((size_t)o.code_begin + k);
      const uint32_t opc = ins[0] & 0xffu, cnt = ins[0] >> 8;
      if (opc == OP_LATHE_SOLID || opc == OP_LATHE_SHELL || opc == OP_PRISM) {
        // device polygon records with the per-edge constants (same float64 values
        // as every reference call computes), appended after the IR's parameters
        const double* pp = P + ins[1];
        const uint32_t off = (uint32_t)out.xparams.size();  // + the chunk's record base (merge)
        out.xfix.push_back((uint32_t)out.code.size());
        const int head = opc == OP_LATHE_SOLID ? 3 : 4;
        for (int h = 0; h < head; h++) out.xparams.push_back(pp[h]);
        const double* v = pp + head;
        auto den_of = [](double ex, double ey) { double dd = ex * ex + ey * ey; return dd == 0.0 ? 1e-12 : dd; };
        if (opc == OP_LATHE_SHELL) {
          for (uint32_t q = 0; q + 1 < cnt; q++) {
            double ax = v[2 * q], ay = v[2 * q + 1], ex = v[2 * q + 2] - ax, ey = v[2 * q + 3] - ay;
            out.xparams.insert(out.xparams.end(), {ax, ay, ex, ey, den_of(ex, ey)});
          }
        } else {
          for (uint32_t q = 0; q < cnt; q++) {
            uint32_t j = q ? q - 1 : cnt - 1;
            double vix = v[2 * q], viy = v[2 * q + 1], vjx = v[2 * j], vjy = v[2 * j + 1];
            double ex = vjx - vix, ey = vjy - viy;
            out.xparams.insert(out.xparams.end(), {vix, viy, vjy, ex, ey, den_of(ex, ey)});
          }
        }
        out.code.push_back(make_uint2(ins[0], off));
      } else {
        out.code.push_back(make_uint2(ins[0], ins[1] + (uint32_t)param_base));
      }
    }
    d.code_len = o.code_len;
    uint32_t first_prim = 0;  // work class: the shape's first primitive (+16 if y-extruded, below)
    for (uint32_t k = 0; k < o.code_len && !first_prim; k++) {
      const uint32_t opk = code[2 * ((size_t)o.code_begin + k)] & 0xffu;
      if (opk >= OP_BOX && opk < OP_ROT_X) first_prim = opk;
    }
    d.paint_off = (uint32_t)(param_base + o.paint_param);
    for (int k = 0; k < 3; k++) { d.mn[k] = o.mn[k]; d.mx[k] = o.mx[k]; }
    for (int k = 0; k < 4; k++) d.frame[k] = o.frame[k];
    // shapes.ts:341-347: voxel range of the op, clamped to the world
    double vx0 = js_max(0, std::floor(o.mn[0] / vs - 0.5)), vy0 = js_max(0, std::floor(o.mn[1] / vs - 0.5)),
           vz0 = js_max(0, std::floor(o.mn[2] / vs - 0.5));
    double vx1 = js_min(w->dx - 1, std::ceil(o.mx[0] / vs + 0.5)), vy1 = js_min(w->dy - 1, std::ceil(o.mx[1] / vs + 0.5)),
           vz1 = js_min(w->dz - 1, std::ceil(o.mx[2] / vs + 0.5));
    uint2 box;
    if (vx0 > vx1 || vy0 > vy1 || vz0 > vz1) {
      d.bx0 = d.by0 = d.bz0 = 1; d.bx1 = d.by1 = d.bz1 = 0; d.nx = d.ny = 0;
      d.inv_nx = d.inv_nxy = 0;
      box = make_uint2(3u << 30, 0u);
    } else {
      d.bx0 = (int)vx0 >> 3; d.by0 = (int)vy0 >> 3; d.bz0 = (int)vz0 >> 3;
      d.bx1 = (int)vx1 >> 3; d.by1 = (int)vy1 >> 3; d.bz1 = (int)vz1 >> 3;
      d.nx = d.bx1 - d.bx0 + 1; d.ny = d.by1 - d.by0 + 1;
      {  // n / d = the high 64 bits of n * ceil(2^64 / d), exactly, for n, d < 2^32
        auto magic = [](uint64_t dv) { return dv > 1 ? ~0ull / dv + 1 : 0ull; };
        d.inv_nx = magic((uint64_t)d.nx);
        d.inv_nxy = magic((uint64_t)d.nx * (uint64_t)d.ny);
      }
      box = make_uint2((uint32_t)d.bx0 | ((uint32_t)d.by0 << 10) | ((uint32_t)d.bz0 << 20),
                       (uint32_t)d.bx1 | ((uint32_t)d.by1 << 10) | ((uint32_t)d.bz1 << 20));
    }
    // contains() per axis (shapes.ts:47-48,360): monotone in the brick index, so a range
    d.cbx0 = d.cby0 = d.cbz0 = 1;
    d.cbx1 = d.cby1 = d.cbz1 = 0;
    if ((o.flags & OPF_CONTAINS) && d.bx0 <= d.bx1) {
      int32_t* lo[3] = {&d.cbx0, &d.cby0, &d.cbz0};
      int32_t* hi[3] = {&d.cbx1, &d.cby1, &d.cbz1};
      const int b0[3] = {d.bx0, d.by0, d.bz0}, b1[3] = {d.bx1, d.by1, d.bz1};
      for (int k = 0; k < 3; k++) {
        int first = -1, last = -2;
        for (int b = b0[k]; b <= b1[k]; b++) {
          int ob = b * 8;
          if ((ob + 0.5) * vs >= o.mn[k] && (ob + 7.5) * vs <= o.mx[k]) {
            if (first < 0) first = b;
            last = b;
          }
        }
        if (first < 0) { *lo[k] = 1; *hi[k] = 0; } else { *lo[k] = first; *hi[k] = last; }
      }
    }
    // A lone box (shapes.ts:40-44): d = |max(q, 0)| + min(max(qx, qy, qz), 0) with
    // q = |p - c| - h is > 0 exactly when some q_k > 0 (a positive q_k >= 2^-60
    // squares without underflow, so the length is positive; otherwise the length
    // is 0 and d = max q_k <= 0).  In float64, q_k <= 0 iff |fl(p_k - c_k)| <= h_k,
    // and fl(p_k - c_k) is monotone in the voxel index, so the voxels inside on
    // each axis form one run: evaluate the reference's expression once per voxel
    // row of the op's bricks and keep the run.  A voxel is inside iff it is in
    // all three runs (the same decision as evaluating the SDF at its centre).
    d.vr[0] = d.vr[2] = d.vr[4] = 1;
    d.vr[1] = d.vr[3] = d.vr[5] = 0;
    if (o.code_len == 1 && (code[2 * (size_t)o.code_begin] & 0xffu) == OP_BOX && d.bx0 <= d.bx1) {
      const double* bp = P + code[2 * (size_t)o.code_begin + 1];
      const int b0[3] = {d.bx0, d.by0, d.bz0}, b1[3] = {d.bx1, d.by1, d.bz1};
      bool runs = true;
      for (int k = 0; k < 3; k++) {
        int first = 1, last = 0, n_in = 0;
        for (int v = b0[k] * 8; v <= b1[k] * 8 + 7; v++) {
          const double t = ((double)v + 0.5) * vs;
          const double q = std::fabs(t - bp[k]) - bp[3 + k];
          if (q <= 0) {
            if (n_in == 0) first = v;
            last = v;
            n_in++;
          }
        }
        if (n_in && n_in != last - first + 1) runs = false;  // not one run: evaluate per voxel
        d.vr[2 * k] = n_in ? first : 1;
        d.vr[2 * k + 1] = n_in ? last : 0;
      }
      if (runs) d.flags |= OPF_BOX_RANGES;
    }
    // shapes.ts:349-350
    d.bhd = 4 * std::sqrt(3.0) * vs * o.slack + vs * 0.01;
    d.shd = 2 * std::sqrt(3.0) * vs * o.slack + vs * 0.01;
    // mixed mode: anchor, float32 parameters, certified thresholds
    for (int k = 0; k < 3; k++) d.anchor[k] = 0.5 * (o.mn[k] + o.mx[k]);
    {
      const double M = MIXED_MARGIN;
      d.thr[T_BSK_HI] = ru32(d.bhd + M); d.thr[T_BSK_LO] = rd32(d.bhd - M);
      d.thr[T_BFU_HI] = rd32(-d.bhd - M); d.thr[T_BFU_LO] = ru32(-d.bhd + M);
      d.thr[T_SSK_HI] = ru32(d.shd + M); d.thr[T_SSK_LO] = rd32(d.shd - M);
      d.thr[T_SFU_HI] = rd32(-d.shd - M); d.thr[T_SFU_LO] = ru32(-d.shd + M);
      d.thr[T_V_HI] = ru32(M); d.thr[T_V_LO] = rd32(-M);
      d.thr[T_M] = ru32(M);
      // Lipschitz decisions of voxels from their sub-block centre's value: a voxel
      // centre lies sqrt(n1 + 9 n3) / 2 voxels from the centre (n3 axes at offset
      // 1.5, the others at 0.5), plus the float64 rounding of both points
      {
        const double L = std::max(1.0, o.slack) * (1 + 0x1p-40);
        const double dist[4] = {std::sqrt(3.0) / 2, std::sqrt(11.0) / 2, std::sqrt(19.0) / 2, std::sqrt(27.0) / 2};
        for (int k = 0; k < 4; k++) d.lip[k] = ru32(L * (dist[k] * vs + 0x1p-40) + M);
      }
      // (b*8 + 0.5)*vs - anchor per brick row, padded for the float64 rounding of the
      // reference's voxel centres ((x + 0.5)*vs, |x*vs| <= 2^10 m)
      d.base_off = (uint32_t)out.bases.size();  // + the chunk's base offset (merge)
      if (d.bx0 <= d.bx1) {
        const int b0[3] = {d.bx0, d.by0, d.bz0}, b1[3] = {d.bx1, d.by1, d.bz1};
        for (int k = 0; k < 3; k++)
          for (int b = b0[k]; b <= b1[k]; b++) out.bases.push_back(enc((b * 8 + 0.5) * vs - d.anchor[k], 0x1p-38));
      }
      size_t c32_before = out.code32.size(), p32_before = out.p32.size();
      bool ok32 = convert32(code + 2 * (size_t)o.code_begin, o.code_len, P, d.anchor, out.code32, out.p32);
      double ext = (double)w->dx * vs;
      if ((double)w->dy * vs > ext) ext = (double)w->dy * vs;
      if ((double)w->dz * vs > ext) ext = (double)w->dz * vs;
      if (!ok32 || ext > MIXED_MAX_COORD) d.flags |= OPF_FP64_ONLY;
      {  // shapes extruded along y: two voxels of a column share the x/z work (sdf32i_y2)
        bool ysep = true;
        for (uint32_t k = 0; k < o.code_len; k++)
          ysep = ysep && op_is_y_separable(code[2 * ((size_t)o.code_begin + k)] & 0xffu);
        if (ysep) d.flags |= OPF_Y_SEPARABLE;
        d.vclass = (first_prim & 15u) | (ysep && !(d.flags & OPF_FP64_ONLY) ? 16u : 0u);
        // a program of the lean voxel kernel (LP_* forms)
        for (int k = 0; k < 8; k++) d.lp[k] = 0;
        if (!(d.flags & (OPF_FP64_ONLY | OPF_DEEP))) lean_program(code + 2 * (size_t)o.code_begin, o.code_len, d.lp);
        // the voxel queue's group and class: one primitive under at most one rotation
        // (by primitive and rotation), the other lean forms (by first primitive and
        // form), the interpreter's programs (by sub-block class)
        const uint32_t p1op = d.lp[LP_FORM] ? code[2 * ((size_t)o.code_begin + d.lp[LP_P1])] & 15u : 0u;
        const uint32_t k1 = d.lp[LP_KINDS] & 15u;
        if (d.lp[LP_FORM] == 1 && k1 != LP_AFFINE) d.vq_class = 32u * VQ_NARROW + (p1op | (k1 ? 16u : 0u));
        else if (d.lp[LP_FORM] == 1) d.vq_class = 32u * VQ_AFFINE + p1op;
        else if (d.lp[LP_FORM]) d.vq_class = 32u * VQ_WIDE + (p1op | (d.lp[LP_FORM] == 3 ? 16u : 0u));
        else d.vq_class = 32u * VQ_GENERIC + d.vclass;
      }
      d.paint_slot = NO_SLOT;
      d.paint32_off = NO_SLOT;
      if (!(d.flags & OPF_FP64_ONLY) && o.kind != KIND_CARVE &&
          (paint_is_heavy(o.paint_kind) || o.paint_kind == PK_NOISE)) {
        const size_t at = out.p32.size();
        if (paint_params32(o.paint_kind, (o.flags & OPF_PAINT_FRAME) != 0, P + o.paint_param, d.anchor, out.p32))
          d.paint32_off = (uint32_t)at;  // + the chunk's float32 base (merge)
        else
          out.p32.resize(at);
      }
      (void)c32_before;
      (void)p32_before;
    }
    d.cost = op_cost(code + 2 * (size_t)o.code_begin, o.code_len, d.flags);
    // the op's first (op, brick) pair (range-local; rebased when the ranges merge), its
    // tile-list entries, and whether its paint is called per voxel
    d.pair_base = out.n_pairs;
    d.paint_slot = NO_SLOT;
    if (d.bx0 <= d.bx1) {
      out.n_pairs += (uint64_t)d.nx * d.ny * (uint64_t)(d.bz1 - d.bz0 + 1);
      out.n_tile_pairs += (uint64_t)(d.bx1 / 4 - d.bx0 / 4 + 1) * (uint64_t)(d.by1 / 4 - d.by0 / 4 + 1) *
                          (uint64_t)(d.bz1 / 4 - d.bz0 / 4 + 1);
      if (d.kind != KIND_CARVE && d.paint_kind != PK_CONST)
        (d.paint32_off == NO_SLOT ? out.painted64 : out.painted32).push_back((uint32_t)out.ops.size());
    }
    out.ops.push_back(d);
    out.boxes.push_back(box);
  }
  return PX_OK;
}

// A small pool of host threads for op conversion (started on first use).
// Between jobs a worker spins briefly before it sleeps, so that the jobs of
// one submit (conversion, then the merge) start without a thread wake-up each.
class HostPool {
 public:
  static HostPool& get() {
    static HostPool* p = new HostPool();  // never destroyed: its threads live as long as the process
    return *p;
  }
  int size() const { return (int)workers_.size() + 1; }
  // run f(k) for k in [0, n) on the pool and the calling thread
  void run(int n, const std::function<void(int)>& f) {
    if (n <= 1 || workers_.empty()) {
      for (int k = 0; k < n; k++) f(k);
      return;
    }
    std::lock_guard<std::mutex> one_job(run_mu_);  // callers on other threads wait their turn
    job_ = &f;
    n_ = n;
    next_.store(0);
    done_.store(0);
    {
      std::lock_guard<std::mutex> g(mu_);
      gen_.fetch_add(1, std::memory_order_release);
    }
    cv_.notify_all();
    work();
    // the workers' part: spin briefly, then sleep until the last one reports
    const int want = (int)workers_.size();
    const auto t0 = std::chrono::steady_clock::now();
    while (done_.load(std::memory_order_acquire) != want) {
      if (std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(200)) {
        std::unique_lock<std::mutex> g(mu_);
        done_cv_.wait(g, [&] { return done_.load(std::memory_order_acquire) == want; });
        break;
      }
    }
    job_ = nullptr;
  }

 private:
  HostPool() {
    unsigned hc = std::thread::hardware_concurrency();
    int n = (int)std::min<unsigned>(hc > 1 ? hc - 1 : 0, 15);
    for (int i = 0; i < n; i++) workers_.emplace_back([this] { loop(); });
    for (auto& t : workers_) t.detach();
  }
  void work() {
    for (;;) {
      const int k = next_.fetch_add(1);
      if (k >= n_) break;
      (*job_)(k);
    }
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      // spin up to 50 us for the next job (the jobs of one submit follow each
      // other within microseconds), then sleep: longer spinning would take the
      // cores from the caller's other threads between submits
      const auto t0 = std::chrono::steady_clock::now();
      uint32_t i = 0;
      while (gen_.load(std::memory_order_acquire) == seen) {
        if ((++i & 255u) == 0 && std::chrono::steady_clock::now() - t0 > std::chrono::microseconds(50)) {
          std::unique_lock<std::mutex> g(mu_);
          cv_.wait(g, [&] { return gen_.load(std::memory_order_acquire) != seen; });
          break;
        }
      }
      seen = gen_.load(std::memory_order_acquire);
      work();
      if (done_.fetch_add(1, std::memory_order_acq_rel) + 1 == (int)workers_.size()) {
        std::lock_guard<std::mutex> g(mu_);
        done_cv_.notify_one();
      }
    }
  }
  std::vector<std::thread> workers_;
  std::mutex run_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)>* job_ = nullptr;
  int n_ = 0;
  std::atomic<int> next_{0}, done_{0};
  std::atomic<uint64_t> gen_{0};
};

// The build scratch that scales with the (op, brick) pairs P, the tile-list
// entries, the paint slots, the touched bricks, the allocator events E_max and
// the staging slots.
int ensure_pair_scratch(px_world* w, uint64_t P, uint64_t tile_pairs, uint64_t n_slots,
                               uint64_t touched_bound, size_t E_max, uint64_t stage_cap) {
  int rc;
  if ((rc = ensure(w, w->tile_cnt, 4 * w->ntiles)) || (rc = ensure(w, w->tile_off, 4 * w->ntiles)) ||
      (rc = ensure(w, w->tile_ops, 4 * tile_pairs)) || (rc = ensure(w, w->tile_boxes, 8 * tile_pairs)) ||
      (rc = ensure(w, w->evt, P)) || (rc = ensure(w, w->fsrc, 8 * P)) ||
      (rc = ensure(w, w->pos, 4 * P)) || (rc = ensure(w, w->etype, E_max)) || (rc = ensure(w, w->ew, 8 * E_max)) ||
      (rc = ensure(w, w->replay_tmp, replay_temp_bytes(P))) || (rc = ensure(w, w->depth, 4 * (E_max + 32))) ||
      (rc = ensure(w, w->tree, 4 * (E_max / 16 + 512))) || (rc = ensure(w, w->staging, 1024 * stage_cap)) ||
      (rc = ensure(w, w->stage_cell, 4 * stage_cap)) || (rc = ensure(w, w->stage_src, 8 * stage_cap)) ||
      (rc = ensure(w, w->touched, 8 * touched_bound)) ||
      (rc = ensure(w, w->work_counter, 16)) || (rc = ensure(w, w->res, sizeof(BuildResult))) ||
      (rc = ensure(w, w->chunk_op, 8 * ((P + 31) / 32))) || (rc = ensure(w, w->pcode, P)) ||
      (rc = ensure(w, w->psub, 2 * P)) || (rc = ensure(w, w->pmask, 64 * P)) || (rc = ensure(w, w->chunk_counter, 1024)) || (rc = ensure(w, w->pitems, 8 * P)) ||
      (rc = ensure(w, w->vitems, 16 * 8 * P)) || (rc = ensure(w, w->paint_items, 8 * 16 * n_slots + 8)) ||
      (rc = ensure(w, w->pvals, 2048 * n_slots + 4)) || (rc = ensure(w, w->bmark, 4 * ((w->ncells + 31) / 32))) ||
      (rc = ensure(w, w->work, 4 * touched_bound + 4)) || (rc = ensure(w, w->rescue, 16 * (size_t)w->rescue_cap)))
    return rc;
  return PX_OK;
}

// Staging slots a build with P pairs reserves (a guess: a build that needs more
// commits nothing and is retried with larger buffers).
uint64_t stage_slots(const px_world* w, uint64_t P) {
  const uint64_t touched_bound = P < w->ncells ? P : w->ncells;
  uint64_t stage_cap = std::max(std::max((uint64_t)4096, w->stage_hint), (uint64_t)(P / 4));
  if (stage_cap > touched_bound) stage_cap = touched_bound ? touched_bound : 1;
  return stage_cap;
}

}  // namespace

namespace px {
// Serving: the scratch of any build of at most P pairs and no paint slots,
// allocated ahead so that no serving step stops to allocate.  Also grows the
// pool so that such a build's staging guess fits.
int reserve_build_scratch(px_world* w, uint64_t P, uint32_t max_ops) {
  if (w->in_flight || w->batch_locked) return fail(w, PX_E_INVALID_ARG, "the world is busy");
  {  // op tables of up to max_ops one-instruction ops with up to 16 parameters and 64 bricks per axis
    const size_t n = max_ops ? max_ops : 1;
    const void* before[7] = {w->d_ops.p, w->d_boxes.p, w->d_code.p, w->d_params.p, w->d_code32.p, w->d_p32.p, w->d_bases.p};
    int rc0;
    if ((rc0 = ensure(w, w->d_ops, sizeof(OpDev) * n)) || (rc0 = ensure(w, w->d_boxes, sizeof(uint2) * (n + (n + 31) / 32 + (n + 1) / 2))) ||
        (rc0 = ensure(w, w->d_code, sizeof(uint2) * n)) || (rc0 = ensure(w, w->d_params, sizeof(double) * 16 * n)) ||
        (rc0 = ensure(w, w->d_code32, sizeof(uint32_t) * n)) || (rc0 = ensure(w, w->d_p32, sizeof(float2) * 16 * n)) ||
        (rc0 = ensure(w, w->d_bases, sizeof(float2) * 192 * n)))
      return rc0;
    const void* after[7] = {w->d_ops.p, w->d_boxes.p, w->d_code.p, w->d_params.p, w->d_code32.p, w->d_p32.p, w->d_bases.p};
    for (int k = 0; k < 7; k++)
      if (after[k] != before[k]) w->ops_resident = false;  // a reallocated table lost its resident copy
  }
  const uint64_t touched_bound = P < w->ncells ? P : w->ncells;
  const size_t E_max = (size_t)w->pool_cap + 2 * P;  // the holes are pool bricks
  const uint64_t stage_cap = stage_slots(w, P);
  int rc = grow_pool(w, (uint64_t)w->pool_used + stage_cap, w->pool_used, nullptr);
  if (rc) return rc;
  if ((rc = ensure_pair_scratch(w, P, P, 0, touched_bound, E_max, stage_cap))) return rc;
  if ((rc = ensure(w, w->holes_a, 4 * E_max + 4))) return rc;
  return ensure(w, w->holes_b, 4 * E_max + 4);
}
uint64_t build_stage_slots(const px_world* w, uint64_t P) { return stage_slots(w, P); }

#ifndef PIPELINE_PAIRS_PER_BLOCK
#define PIPELINE_PAIRS_PER_BLOCK 64
#endif

px_world* twin_create(px_world* w, uint64_t P, uint32_t max_ops, int* rc) {
  *rc = PX_OK;
  px_world* t = new px_world();
  t->dx = w->dx; t->dy = w->dy; t->dz = w->dz;
  t->BX = w->BX; t->BY = w->BY; t->BZ = w->BZ; t->TX = w->TX; t->TY = w->TY; t->TZ = w->TZ;
  t->vpm = w->vpm; t->vs = w->vs; t->ncells = w->ncells; t->ntiles = w->ntiles; t->n_sms = w->n_sms;
  for (int k = 0; k < VCLASSES; k++) t->class_order[k] = w->class_order[k];
  for (int k = 0; k < VQ_CLASSES; k++) t->vclass_order[k] = w->vclass_order[k];
  t->vq_nonempty = w->vq_nonempty;
  t->host_reads = w->host_reads;
  t->validate = w->validate;
  t->rescue_cap = w->rescue_cap;
  t->stage_hint = w->stage_hint;
  t->pairs_per_block = PIPELINE_PAIRS_PER_BLOCK;
  // the shared world: grid, pool, opaque counts, device state, free lists, material tables
  t->shares_state = true;
  t->d_grid = w->d_grid; t->d_pool32 = w->d_pool32; t->d_pcount = w->d_pcount; t->d_state = w->d_state;
  t->pool_cap = w->pool_cap;
  t->pool_used = w->pool_used; t->n_holes = w->n_holes; t->holes_in_a = w->holes_in_a;
  t->pcount_valid = w->pcount_valid;
  auto borrow = [](DevBuf& dst, const DevBuf& src) { dst = src; dst.borrowed = true; };
  borrow(t->holes_a, w->holes_a);
  borrow(t->holes_b, w->holes_b);
  borrow(t->opaque, w->opaque);
  borrow(t->axis32, w->axis32);
  borrow(t->udens, w->udens);
  if (cudaMallocHost((void**)&t->h_res, sizeof(BuildResult)) != cudaSuccess) {
    cudaGetLastError();
    delete t;
    *rc = PX_E_OOM;
    return nullptr;
  }
  cudaEventCreate(&t->ev0);
  cudaEventCreate(&t->ev1);
  cudaEventCreate(&t->ev_fold0);
  cudaEventCreate(&t->ev_fold1);
  cudaEventCreate(&t->ev_mid);
  cudaEventCreateWithFlags(&t->ev_eval, cudaEventDisableTiming);
  cudaEventCreateWithFlags(&t->ev_done, cudaEventDisableTiming);
  *rc = reserve_build_scratch(t, P, max_ops);  // its own scratch; the shared buffers are already sized
  if (*rc != PX_OK) {
    twin_destroy(t);
    return nullptr;
  }
  return t;
}

void twin_destroy(px_world* t) { px_world_destroy(t); }

void pipeline_set(px_world* w, cudaStream_t apply, bool holes_in_a, uint32_t pool_used_bound, uint32_t n_holes_bound) {
  w->apply_stream = apply;
  w->no_retry = apply != nullptr;
  w->holes_in_a = holes_in_a;
  w->pool_used = pool_used_bound;
  w->n_holes = n_holes_bound;
}

PipelineState pipeline_begin(px_world* w) {
  PipelineState st{w->pool_used, w->n_holes, w->holes_in_a, w->derive_max, w->pairs_per_block};
  w->derive_max = 0;
  // two builds share the GPU: persistent grids sized to each build's pairs
  // (a few edits need a few blocks, not the whole GPU)
  w->pairs_per_block = PIPELINE_PAIRS_PER_BLOCK;
  return st;
}

void pipeline_end(px_world* w, const PipelineState& st, uint64_t ops, cudaStream_t s) {
  w->apply_stream = nullptr;
  w->stream = s;
  w->no_retry = false;
  w->pool_used = st.pool_used;
  w->n_holes = st.n_holes;
  w->holes_in_a = st.holes_in_a;
  w->derive_max = st.derive_max;
  w->pairs_per_block = st.pairs_per_block;
  w->ops_applied += ops;
  w->stats.ops_applied = w->ops_applied;
  w->stats.pool_used = st.pool_used;
  w->stats.n_holes = st.n_holes;
  w->derived_valid = false;
  w->free_valid = false;
  cudaMemsetAsync(&w->d_state->poisoned, 0, 4, s);  // a failed build left the world as it was
  cudaStreamSynchronize(s);
}

bool build_done(px_world* w) { return !w->in_flight || cudaEventQuery(w->ev_done) == cudaSuccess; }

void build_times(px_world* w, cudaEvent_t base, double* start_ms, double* end_ms) {
  float a = 0.f, b = 0.f;
  cudaEventElapsedTime(&a, base, w->ev0);
  cudaEventElapsedTime(&b, base, w->ev1);
  *start_ms = a;
  *end_ms = b;
}
}  // namespace px

extern "C" {

static int submit_ops_impl(px_world* w, const void* ir, size_t bytes) {
  if (!w || (!ir && bytes)) return PX_E_INVALID_ARG;
  if (w->batch_locked) return fail(w, PX_E_INVALID_ARG, "the world belongs to a batch");
  if (w->in_flight) return fail(w, PX_E_INVALID_ARG, "a build is in flight");
  if (w->uploads_pending) {  // a build that failed after its upload kernel was launched
    CU(cudaStreamSynchronize(w->stream));
    w->uploads_pending = false;
  }
  w->ops_resident = false;
  if (bytes < 32) return fail(w, PX_E_INVALID_IR, "IR shorter than its header");
  const uint32_t* h = (const uint32_t*)ir;
  if (h[0] != 0x52495850u || h[1] != 1u) return fail(w, PX_E_INVALID_IR, "not a PXIR v1 buffer");
  const size_t n_ops = h[2], n_code = h[3], n_params = h[4];
  const size_t need = 32 + n_ops * sizeof(IrOp) + n_code * 8 + n_params * 8;
  if (bytes < need) return fail(w, PX_E_INVALID_IR, "IR truncated (%zu < %zu bytes)", bytes, need);
  const IrOp* iops = (const IrOp*)((const char*)ir + 32);
  const uint32_t* code = (const uint32_t*)((const char*)ir + 32 + n_ops * sizeof(IrOp));
  // the parameters, read in place when the buffer is aligned (copied otherwise)
  const char* praw = (const char*)ir + 32 + n_ops * sizeof(IrOp) + n_code * 8;
  std::vector<double> Pcopy;
  const double* Pp = (const double*)praw;
  if ((uintptr_t)praw % alignof(double)) {
    Pcopy.resize(n_params);
    std::memcpy(Pcopy.data(), praw, n_params * 8);
    Pp = Pcopy.data();
  }

  const size_t param_base = w->params.size();
  // convert the ops in contiguous ranges on the host pool, then append the
  // ranges in order (offsets rebased)
  HostPool& pool = HostPool::get();
  const int n_chunks = n_ops < 512 ? 1 : (int)std::min<size_t>((size_t)pool.size() * 4, n_ops / 32);
  std::vector<SubmitChunk> chunks(n_chunks);
  pool.run(n_chunks, [&](int k) {
    const size_t i0 = n_ops * k / n_chunks, i1 = n_ops * (k + 1) / n_chunks;
    convert_ops(w, iops, i0, i1, code, n_code, Pp, n_params, param_base, chunks[k]);
  });
  for (auto& c : chunks)
    if (c.rc != PX_OK) return fail(w, c.rc, "%s", c.err.c_str());
  // every range's place in the world's arrays, then all ranges rebased and
  // copied at once (the IR's own parameters as one more job)
  struct Place {
    size_t code, p32, bases, ops, xp;
    uint64_t pairs;
  };
  std::vector<Place> at(n_chunks);
  Place end = {w->code.size(), w->p32.size(), w->bases.size(), w->ops.size(), param_base + n_params, w->q.pairs};
  for (int k = 0; k < n_chunks; k++) {
    const SubmitChunk& c = chunks[k];
    at[k] = end;
    end.code += c.code.size();
    end.p32 += c.p32.size();
    end.bases += c.bases.size();
    end.ops += c.ops.size();
    end.xp += c.xparams.size();
    end.pairs += c.n_pairs;
    w->q.tile_pairs += c.n_tile_pairs;
    for (uint32_t i : c.painted64) w->q.painted64.push_back((uint32_t)at[k].ops + i);
    for (uint32_t i : c.painted32) w->q.painted32.push_back((uint32_t)at[k].ops + i);
  }
  w->q.pairs = end.pairs;
  w->code.resize(end.code);
  w->code32.resize(end.code);
  w->p32.resize(end.p32);
  w->bases.resize(end.bases);
  w->ops.resize(end.ops);
  w->boxes.resize(end.ops);
  w->params.resize(end.xp);
  auto merge = [&](int k) {
    if (k == n_chunks) {
      if (n_params) std::memcpy(w->params.data() + param_base, Pp, n_params * sizeof(double));
      return;
    }
    SubmitChunk& c = chunks[k];
    const Place& pl = at[k];
    for (uint32_t i : c.xfix) c.code[i].y += (uint32_t)pl.xp;
    for (uint32_t& v : c.code32) v += (uint32_t)pl.p32;
    for (OpDev& d : c.ops) {
      d.code_off += (uint32_t)pl.code;
      d.base_off += (uint32_t)pl.bases;
      d.pair_base += pl.pairs;
      if (d.paint32_off != NO_SLOT) d.paint32_off += (uint32_t)pl.p32;
    }
    auto put = [](auto& dst, size_t pos, const auto& src) {
      if (!src.empty()) std::memcpy(dst.data() + pos, src.data(), src.size() * sizeof(src[0]));
    };
    put(w->code, pl.code, c.code);
    put(w->code32, pl.code, c.code32);
    put(w->p32, pl.p32, c.p32);
    put(w->bases, pl.bases, c.bases);
    put(w->ops, pl.ops, c.ops);
    put(w->boxes, pl.ops, c.boxes);
    put(w->params, pl.xp, c.xparams);
  };
  if (n_chunks > 1) {
    pool.run(n_chunks + 1, merge);
  } else {  // a small list: no threads
    merge(0);
    merge(1);
  }
  return PX_OK;
}

static int cost_bucket(float c) { return c >= 15.75f ? 63 : (int)(c * 4.f); }

// The host-to-device copies of one build's op tables and the clears of its
// counters (entries without a source).  One kernel does the clears and, where
// the GPU reads pageable memory through the host page tables (Grace), the
// copies too, reading the host arrays directly (a few microseconds of host
// time instead of ~10 per cudaMemcpyAsync or cudaMemsetAsync); the arrays then
// stay untouched until the build has finished (px_submit_ops and
// px_world_reset wait for it).  Elsewhere, and while a graph is captured, the
// copies are cudaMemcpyAsync.
static int issue_uploads(px_world* w, const std::vector<Upload>& ups, cudaStream_t s) {
  HostUploads hu{};
  bool reads_host = false;
  for (const Upload& u : ups) {
    if (!u.bytes) continue;
    const bool aligned = !(((uintptr_t)u.src | (uintptr_t)u.dst) & 15u);
    const bool by_kernel = aligned && hu.n < HostUploads::kMax && (!u.src || (w->host_reads && !w->capturing));
    if (by_kernel) {
      hu.e[hu.n++] = {u.src, u.dst, u.bytes, 0x01010101u * u.fill};
      reads_host = reads_host || u.src;
    } else if (u.src) {
      CU(cudaMemcpyAsync(u.dst, u.src, u.bytes, cudaMemcpyHostToDevice, s));
    } else {
      CU(cudaMemsetAsync(u.dst, u.fill, u.bytes, s));
    }
  }
  if (hu.n) {
    launch_uploads(hu, s);
    CU(cudaGetLastError());
    if (reads_host) w->uploads_pending = true;
  }
  return PX_OK;
}


// The derived upload buffers as the last kernel of a build (derive on build).
static int enqueue_build_derive(px_world* w, cudaStream_t s, const uint32_t* holes_after) {
  int rc;
  const uint64_t fcap = free_list_bound(w->pool_cap, w->derive_max);
  if ((rc = ensure(w, w->super_counts, 4 * w->ntiles)) || (rc = ensure(w, w->density, w->ncells)) ||
      (rc = ensure(w, w->free_list, 4 * fcap + 4)))
    return rc;
  DeriveArgs da{};
  da.grid = w->d_grid;
  da.pool32 = w->d_pool32;
  da.BX = w->BX; da.BY = w->BY; da.BZ = w->BZ;
  da.opaque = (const uint8_t*)w->opaque.p;
  da.udens = (const uint8_t*)w->udens.p;
  da.super_counts = (uint32_t*)w->super_counts.p;
  da.density = (uint8_t*)w->density.p;
  da.holes = holes_after;
  da.free_list = (uint32_t*)w->free_list.p;
  da.free_cap = (uint32_t)fcap;
  da.max_bricks = w->derive_max;
  da.res = (BuildResult*)w->res.p;
  // counts kept by finalize, unless the material tables changed since: then recount
  da.pcount = w->pcount_valid ? w->d_pcount : nullptr;
  da.pcount_out = w->pcount_valid ? nullptr : w->d_pcount;
  w->pcount_refresh = !w->pcount_valid;
  launch_derive(da, s);
  return PX_OK;
}

static int build_enqueue_impl(px_world* w, int mode, void* stream) {
  set_programmatic_launch(!w->capturing);
  if (!w) return PX_E_INVALID_ARG;
  if (w->batch_locked && !w->capturing) return fail(w, PX_E_INVALID_ARG, "the world belongs to a batch");
  if (w->in_flight) return fail(w, PX_E_INVALID_ARG, "a build is already in flight");
  if (mode != PX_MODE_FP64 && mode != PX_MODE_MIXED) return fail(w, PX_E_INVALID_ARG, "unknown mode %d", mode);
  cudaStream_t s = (cudaStream_t)stream;
  // the apply pass and everything after it: on the apply stream when pipelined
  cudaStream_t sa = w->apply_stream && !w->capturing ? w->apply_stream : s;
  w->stream = sa;
  const int n_ops = (int)w->ops.size();
  int rc;

  // (op, brick) pair bases (set as the ops were converted) and the tile-list bound
  const uint64_t P = w->q.pairs, tile_pairs = w->q.tile_pairs;
  std::vector<uint32_t>& painted = w->h_painted;  // float64-only paints first
  painted.assign(w->q.painted64.begin(), w->q.painted64.end());
  if (P > 0x1fffffffull) return fail(w, PX_E_QUEUE_OVERFLOW, "too many (op, brick) pairs in one build: %llu", (unsigned long long)P);
  if (n_ops >= (1 << 24)) return fail(w, PX_E_QUEUE_OVERFLOW, "too many ops in one build: %d", n_ops);
  painted.insert(painted.end(), w->q.painted32.begin(), w->q.painted32.end());
  // paint slots (one per (op, brick) pair of a painted op, 2 KiB each): every
  // painted op when they fit in 512 MiB, else the heavy kinds alone when they
  // fit, else none; ops without a slot have their paints called by the apply pass
  uint64_t n_slots = 0;
  bool inline_paints = false;
  for (int tier = 0; tier < 3; tier++) {
    n_slots = 0;
    inline_paints = false;
    // float64-only paints first: paint_kernel takes items in slot order, so the
    // slowest calls start earliest
    for (const uint32_t i : painted) {
      OpDev& o = w->ops[i];
      o.paint_slot = NO_SLOT;
      if (tier == 2 || (tier == 1 && !paint_is_heavy(o.paint_kind))) { inline_paints = true; continue; }
      const uint64_t np = (uint64_t)o.nx * o.ny * (uint64_t)(o.bz1 - o.bz0 + 1);
      o.paint_slot = (uint32_t)n_slots;
      n_slots += np;
    }
    if (n_slots * 2048 <= (512ull << 20)) break;
  }
  const uint64_t touched_bound = P < w->ncells ? P : w->ncells;
  // the host's view of the allocator state: exact, or for pipelined builds
  // (whose replay reads it from the device) upper bounds that size the buffers
  const uint32_t H = w->n_holes, U0 = w->pool_used;
  const size_t E_max = (size_t)H + 2 * P;

  // staging slots and pool bricks are reserved from a guess; a build that needs
  // more commits nothing and is retried with larger buffers (px_build_finish)
  const uint64_t stage_cap = stage_slots(w, P);
  if ((rc = grow_pool(w, (uint64_t)U0 + stage_cap, U0, s))) return rc;

  // scratch (a reallocated op table loses its resident copy)
  const void* op_bufs_before[9] = {w->d_ops.p, w->d_boxes.p, w->d_code.p, w->d_params.p, w->d_code32.p,
                                   w->d_p32.p, w->d_bases.p, w->chunk_op.p, w->chunk_op.p};
  if ((rc = ensure(w, w->d_ops, sizeof(OpDev) * (size_t)n_ops)) ||
      (rc = ensure(w, w->d_boxes, sizeof(uint2) * ((size_t)n_ops + (n_ops + 31) / 32 + (n_ops + 1) / 2))) ||
      (rc = ensure(w, w->d_code, sizeof(uint2) * w->code.size())) ||
      (rc = ensure(w, w->d_params, sizeof(double) * w->params.size())) ||
      (rc = ensure(w, w->d_code32, sizeof(uint32_t) * w->code32.size())) ||
      (rc = ensure(w, w->d_p32, sizeof(float2) * w->p32.size())) ||
      (rc = ensure(w, w->d_bases, sizeof(float2) * w->bases.size())) ||
      (rc = ensure_pair_scratch(w, P, tile_pairs, n_slots, touched_bound, E_max, stage_cap)))
    return rc;
  const uint32_t H_max = H;
  {
    const void* after[9] = {w->d_ops.p, w->d_boxes.p, w->d_code.p, w->d_params.p, w->d_code32.p,
                            w->d_p32.p, w->d_bases.p, w->chunk_op.p, w->chunk_op.p};
    for (int k = 0; k < 9; k++)
      if (after[k] != op_bufs_before[k]) w->ops_resident = false;
  }
  DevBuf& holes_in = w->holes_in_a ? w->holes_a : w->holes_b;
  DevBuf& holes_out = w->holes_in_a ? w->holes_b : w->holes_a;
  if ((rc = ensure(w, holes_in, 4 * (size_t)H + 4)) || (rc = ensure(w, holes_out, 4 * E_max + 4))) return rc;

  // upload the ops (one pinned staging copy per array)
  const unsigned long long launches0 = launch_count();
  if (!w->capturing) CU(cudaEventRecord(w->ev0, s));
  const bool upload = !w->ops_resident;
  std::vector<Upload>& ups = w->h_uploads;
  ups.clear();
  if (upload) {
    ups.push_back({w->d_ops.p, w->ops.data(), sizeof(OpDev) * (size_t)n_ops});
    {  // op boxes, then the union box of every 32 ops of the culling order (cull_kernel /
       // cull_sorted_kernel), then that order: along a Morton curve of the boxes' centres
       // (in 4-brick tiles) when the sorted kernel is used, else the op order itself
      const int n_groups = (n_ops + 31) / 32;
      // the union boxes of 32 ops of an order, and the tiles they cover in all (the
      // group tests a tile passes grow with it)
      auto group_boxes = [&](const std::vector<uint32_t>& ord, std::vector<uint2>& gb) {
        uint64_t vol = 0;
        gb.clear();
        for (int g = 0; g < n_groups; g++) {
          uint32_t lo[3] = {1023, 1023, 1023}, hi[3] = {0, 0, 0};
          bool any = false;
          for (int k = g * 32; k < n_ops && k < g * 32 + 32; k++) {
            const uint2 b = w->boxes[ord[k]];
            if (b.x >> 30) continue;
            any = true;
            for (int a = 0; a < 3; a++) {
              lo[a] = std::min(lo[a], (b.x >> (10 * a)) & 1023u);
              hi[a] = std::max(hi[a], (b.y >> (10 * a)) & 1023u);
            }
          }
          gb.push_back(any ? make_uint2(lo[0] | (lo[1] << 10) | (lo[2] << 20), hi[0] | (hi[1] << 10) | (hi[2] << 20))
                           : make_uint2(3u << 30, 0u));
          if (any) vol += (uint64_t)(hi[0] / 4 - lo[0] / 4 + 1) * (hi[1] / 4 - lo[1] / 4 + 1) * (hi[2] / 4 - lo[2] / 4 + 1);
        }
        return vol;
      };
      std::vector<uint32_t>& ord = w->h_cull_order;
      ord.resize(n_ops);
      for (int i = 0; i < n_ops; i++) ord[i] = (uint32_t)i;
      std::vector<uint2> gb_seq, gb_mc;
      const uint64_t vol_seq = group_boxes(ord, gb_seq);
      bool sorted = false;
      if (n_ops <= CULL_SORTED_MAX_OPS && n_groups > 1) {
        auto spread = [](uint32_t v) {  // 8 bits -> every third bit
          uint32_t r = 0;
          for (int k = 0; k < 8; k++) r |= ((v >> k) & 1u) << (3 * k);
          return r;
        };
        std::vector<uint32_t> key(n_ops), mc(ord);
        for (int i = 0; i < n_ops; i++) {
          const uint2 b = w->boxes[i];
          if (b.x >> 30) { key[i] = 0xffffffffu; continue; }  // no bricks: last
          uint32_t c[3];
          for (int a = 0; a < 3; a++) c[a] = ((((b.x >> (10 * a)) & 1023u) + ((b.y >> (10 * a)) & 1023u)) >> 3) & 255u;
          key[i] = spread(c[0]) | (spread(c[1]) << 1) | (spread(c[2]) << 2);
        }
        std::stable_sort(mc.begin(), mc.end(), [&](uint32_t x, uint32_t y) { return key[x] < key[y]; });
        // the spatial order where its groups cover less than half the tiles the op order's
        // do: scattered ops (the sorted kernel's bit set costs more on compact scenes)
        if (2 * group_boxes(mc, gb_mc) < vol_seq) {
          sorted = true;
          ord.swap(mc);
        }
      }
      w->cull_sorted = sorted;
      w->h_boxes.assign(w->boxes.begin(), w->boxes.end());
      const std::vector<uint2>& gb = sorted ? gb_mc : gb_seq;
      w->h_boxes.insert(w->h_boxes.end(), gb.begin(), gb.end());
      if (sorted)  // the order, two per uint2
        for (int k = 0; k < n_ops; k += 2)
          w->h_boxes.push_back(make_uint2(ord[k], k + 1 < n_ops ? ord[k + 1] : 0u));
      ups.push_back({w->d_boxes.p, w->h_boxes.data(), sizeof(uint2) * w->h_boxes.size()});
    }
    ups.push_back({w->d_code.p, w->code.data(), sizeof(uint2) * w->code.size()});
    ups.push_back({w->d_params.p, w->params.data(), sizeof(double) * w->params.size()});
    ups.push_back({w->d_code32.p, w->code32.data(), sizeof(uint32_t) * w->code32.size()});
    ups.push_back({w->d_p32.p, w->p32.data(), sizeof(float2) * w->p32.size()});
    ups.push_back({w->d_bases.p, w->bases.data(), sizeof(float2) * w->bases.size()});
  }
  // the build's counters and flags start at zero
  ups.push_back({w->res.p, nullptr, sizeof(BuildResult)});
  ups.push_back({w->work_counter.p, nullptr, 16});
  ups.push_back({w->chunk_counter.p, nullptr, 1024});
  ups.push_back({w->evt.p, nullptr, P});
  ups.push_back({w->bmark.p, nullptr, 4 * ((w->ncells + 31) / 32)});
  ups.push_back({w->replay_tmp.p, nullptr, replay_clear_bytes(P)});  // the replay's tickets and look-back flags
  ups.push_back({w->tree.p, nullptr, tree_clear_bytes(E_max), 0x7f});  // min-tree levels 1 and 2, above every depth
  if ((rc = issue_uploads(w, ups, s))) return rc;  // the op tables; the chunk order follows the cull launches

  BuildResult* res = (BuildResult*)w->res.p;
  launch_cull((const uint2*)w->d_boxes.p, n_ops, w->TX, w->TY, w->TZ, (uint32_t*)w->tile_cnt.p,
              (uint32_t*)w->tile_off.p, (uint32_t*)w->tile_ops.p, (uint2*)w->tile_boxes.p,
              (uint32_t*)w->chunk_counter.p + CULL_COUNTER, w->cull_sorted, s);
  // the classify pass's chunk order, computed while the cull kernels run
  const size_t n_chunks = (P + 31) / 32;
  if (upload) {
    // op of the first pair of every 32-pair chunk, then the order classify_kernel
    // takes the chunks in: costliest ops first (a bucket sort, stable within a bucket)
    w->h_chunk_op.resize(2 * n_chunks);
    w->h_op_bucket.resize(n_ops);
    float cc[VCLASSES] = {0.f}, cv[VQ_CLASSES] = {0.f};
    for (int i = 0; i < n_ops; i++) {
      const float c = w->ops[i].cost;
      w->h_op_bucket[i] = (uint8_t)cost_bucket(c);
      if (w->ops[i].bx0 <= w->ops[i].bx1) {
        cc[w->ops[i].vclass] = std::max(cc[w->ops[i].vclass], c);
        cv[w->ops[i].vq_class] = std::max(cv[w->ops[i].vq_class], c);
      }
    }
    // op o owns the chunks whose first pair it holds: [ceil(base_o / 32), ceil(base_o+1 / 32));
    // a chunk entry is (chunk, its first pair's op | bit 31 when all its pairs are that op's)
    auto first_chunk = [&](int i) { return (uint32_t)((w->ops[i].pair_base + 31) / 32); };
    uint32_t bucket_n[64] = {0};
    for (int i = 0; i < n_ops; i++) {
      const uint32_t c0 = first_chunk(i), c1 = i + 1 < n_ops ? first_chunk(i + 1) : (uint32_t)n_chunks;
      bucket_n[w->h_op_bucket[i]] += c1 - c0;
    }
    uint32_t at = 0;
    for (int b = 63; b >= 0; b--) {
      const uint32_t n = bucket_n[b];
      bucket_n[b] = at;
      at += n;
    }
    for (int i = 0; i < n_ops; i++) {  // each op's chunks, in order, at its bucket's next place
      const uint32_t c0 = first_chunk(i), c1 = i + 1 < n_ops ? first_chunk(i + 1) : (uint32_t)n_chunks;
      const uint64_t end = i + 1 < n_ops ? w->ops[i + 1].pair_base : P;  // the op's pairs end here
      uint32_t* dst = w->h_chunk_op.data() + 2 * (size_t)bucket_n[w->h_op_bucket[i]];
      for (uint32_t c = c0; c < c1; c++) {
        *dst++ = c;
        *dst++ = (uint32_t)i | ((uint64_t)c * 32 + 32 <= end || end >= P ? 0x80000000u : 0u);
      }
      bucket_n[w->h_op_bucket[i]] += c1 - c0;
    }
    ups.clear();
    ups.push_back({w->chunk_op.p, w->h_chunk_op.data(), 8 * n_chunks});
    // the sub-block and voxel passes take the classes costliest first
    int order[VCLASSES];
    for (int k = 0; k < VCLASSES; k++) order[k] = k;
    std::stable_sort(order, order + VCLASSES, [&](int x, int y) { return cc[x] > cc[y]; });
    for (int k = 0; k < VCLASSES; k++) w->class_order[k] = (uint8_t)order[k];
    int vorder[VQ_CLASSES];  // each group of the voxel classes costliest first
    for (int k = 0; k < VQ_CLASSES; k++) vorder[k] = k;
    for (int g = 0; g < VQ_CLASSES / 32; g++)
      std::stable_sort(vorder + 32 * g, vorder + 32 * g + 32, [&](int x, int y) { return cv[x] > cv[y]; });
    for (int k = 0; k < VQ_CLASSES; k++) w->vclass_order[k] = (uint8_t)vorder[k];
    w->vq_nonempty = 0;
    for (int i = 0; i < n_ops; i++)
      if (w->ops[i].bx0 <= w->ops[i].bx1) w->vq_nonempty |= 1u << (w->ops[i].vq_class / 32);
    if ((rc = issue_uploads(w, ups, s))) return rc;
  }
  FoldArgs fa{};
  fa.chunk_order = (const uint2*)w->chunk_op.p;
  for (int k = 0; k < VCLASSES; k++) fa.class_order[k] = w->class_order[k];
  for (int k = 0; k < VQ_CLASSES; k++) fa.vclass_order[k] = w->vclass_order[k];
  fa.vq_nonempty = w->vq_nonempty;
  fa.n_ops = (uint32_t)n_ops;
  fa.n_pairs = P;
  fa.pcode = (uint8_t*)w->pcode.p;
  fa.psub = (uint16_t*)w->psub.p;
  fa.pmask = (unsigned long long*)w->pmask.p;
  fa.chunk_counter = (uint32_t*)w->chunk_counter.p;
  fa.vitems = (uint4*)w->vitems.p;
  fa.vitems_cap = (uint32_t)(8 * P < 0xffffffffull ? 8 * P : 0xffffffffull);
  fa.vitem_counter = (uint32_t*)w->chunk_counter.p + 4;   // counters: [0] chunks, [1] paint taken,
                                                          // [2] paint pushed, [4..136] voxel, [160..193] pairs,
                                                          // [CULL_COUNTER] tile-list entries
  {  // per-class regions: the class's pairs (sub-block pass), 8 sub-blocks per pair (voxel pass)
    uint64_t per[VCLASSES] = {0}, vper[VQ_CLASSES] = {0};
    for (int i = 0; i < n_ops; i++) {
      const OpDev& o = w->ops[i];
      if (o.bx0 > o.bx1) continue;
      const uint64_t np = (uint64_t)o.nx * o.ny * (uint64_t)(o.bz1 - o.bz0 + 1);
      per[o.vclass & (VCLASSES - 1)] += np;
      vper[o.vq_class] += np;
    }
    uint64_t at = 0;
    for (int k = 0; k < VCLASSES; k++) {
      fa.pq_base[k] = (uint32_t)at;
      fa.pq_cap[k] = (uint32_t)per[k];
      at += per[k];
    }
    at = 0;
    for (int k = 0; k < VQ_CLASSES; k++) {
      fa.vq_base[k] = (uint32_t)std::min<uint64_t>(8 * at, 0xffffffffull);
      fa.vq_cap[k] = (uint32_t)std::min<uint64_t>(8 * vper[k], 0xffffffffull - fa.vq_base[k]);
      at += vper[k];
    }
  }
  fa.pitems = (uint2*)w->pitems.p;
  fa.pitem_counter = (uint32_t*)w->chunk_counter.p + 160;
  fa.rescue = (uint4*)w->rescue.p;
  fa.rescue_cap = w->rescue_cap;
  fa.paint_counter = (uint32_t*)w->chunk_counter.p + 1;
  fa.n_paint_slots = (uint32_t)n_slots;
  fa.paint_items = (uint2*)w->paint_items.p;
  fa.paint_items_cap = (uint32_t)std::min<uint64_t>(16 * n_slots, 0xffffffffull);  // float64 items come in halves
  fa.paint_item_counter = (uint32_t*)w->chunk_counter.p + 2;
  fa.pvals = (uint32_t*)w->pvals.p;
  fa.inline_paints = inline_paints ? 1 : 0;
  fa.bmark = (uint32_t*)w->bmark.p;
  fa.work = (uint32_t*)w->work.p;
  fa.ops = (const OpDev*)w->d_ops.p;
  fa.code = (const uint2*)w->d_code.p;
  fa.params = (const double*)w->d_params.p;
  fa.code32 = (const uint32_t*)w->d_code32.p;
  fa.p32 = (const float2*)w->d_p32.p;
  fa.bases = (const float2*)w->d_bases.p;
  fa.vs_lo = rd32(w->vs);
  fa.vs_hi = ru32(w->vs);
  fa.validate = w->validate;
  fa.tile_off = (const uint32_t*)w->tile_off.p;
  fa.tile_cnt = (const uint32_t*)w->tile_cnt.p;
  fa.tile_ops = (const uint32_t*)w->tile_ops.p;
  fa.tile_boxes = (const uint2*)w->tile_boxes.p;
  fa.BX = w->BX; fa.BY = w->BY; fa.BZ = w->BZ; fa.TX = w->TX; fa.TY = w->TY;
  fa.vs = w->vs;
  fa.ax32 = (const float*)w->axis32.p;
  fa.ay32 = fa.ax32 + w->dx;
  fa.az32 = fa.ay32 + w->dy;
  fa.grid = w->d_grid;
  fa.pool32 = w->d_pool32;
  fa.evt = (uint8_t*)w->evt.p;
  fa.fsrc = (int64_t*)w->fsrc.p;
  fa.staging32 = (uint32_t*)w->staging.p;
  fa.stage_cap = (uint32_t)stage_cap;
  fa.touched = (uint2*)w->touched.p;
  fa.touched_cap = (uint32_t)touched_bound;
  fa.stage_cell = (uint32_t*)w->stage_cell.p;
  fa.stage_src = (int64_t*)w->stage_src.p;
  fa.work_counter = (uint32_t*)w->work_counter.p;
  fa.res = res;
  int max_blocks = 0;  // persistent grids sized to the build (batched builds share the GPU)
  if (w->pairs_per_block) max_blocks = (int)std::max<uint64_t>(1, (P + w->pairs_per_block - 1) / w->pairs_per_block);
  if (!w->capturing) CU(cudaEventRecord(w->ev_fold0, s));
  launch_fold(fa, mode, w->n_sms, s, w->capturing ? nullptr : w->ev_mid, max_blocks, sa, w->ev_eval);
  s = sa;  // the rest of the build follows the apply pass
  if (!w->capturing) CU(cudaEventRecord(w->ev_fold1, s));

  ReplayArgs ra{};
  ra.P = P; ra.E_max = E_max; ra.H_max = H_max; ra.state = w->d_state;
  ra.evt = (const uint8_t*)w->evt.p;
  ra.fsrc = (const int64_t*)w->fsrc.p;
  ra.holes_in = (const uint32_t*)holes_in.p;
  ra.pos = (uint32_t*)w->pos.p;
  ra.etype = (uint8_t*)w->etype.p;
  ra.ew = (unsigned long long*)w->ew.p;
  ra.depth = (int32_t*)w->depth.p;
  ra.tree = (int32_t*)w->tree.p;
  ra.tl = tree_levels(E_max);
  ra.holes_out = (uint32_t*)holes_out.p;
  ra.res = res;
  ra.t = replay_temp(w->replay_tmp.p, P);
  launch_replay(ra, s);

  FinalizeArgs& fn = w->fin;
  fn.touched = (const uint2*)w->touched.p;
  fn.staging32 = (const uint32_t*)w->staging.p;
  fn.stage_cell = (const uint32_t*)w->stage_cell.p;
  fn.stage_src = (const int64_t*)w->stage_src.p;
  fn.pos = (const uint32_t*)w->pos.p;
  fn.ew = (const unsigned long long*)w->ew.p;
  fn.state = w->d_state;
  fn.holes_out = (uint32_t*)holes_out.p;
  fn.grid = w->d_grid;
  fn.pool32 = w->d_pool32;
  fn.pool_cap = w->pool_cap;
  fn.res = res;
  fn.opaque = (const uint8_t*)w->opaque.p;
  fn.pcount = w->d_pcount;
  launch_finalize(fn, (uint32_t)touched_bound, s);
  if (w->derive_max && (rc = enqueue_build_derive(w, s, (const uint32_t*)holes_out.p))) return rc;
  CU(cudaGetLastError());
  w->stats.kernel_launches = (uint32_t)(launch_count() - launches0);
  if (!w->capturing) CU(cudaEventRecord(w->ev1, s));
  CU(cudaMemcpyAsync(w->h_res, res, sizeof(BuildResult), cudaMemcpyDeviceToHost, s));
  if (!w->capturing) CU(cudaEventRecord(w->ev_done, s));
  w->in_flight = true;
  w->last_P = P;
  w->last_stage_cap = (uint32_t)stage_cap;
  w->last_touched_cap = (uint32_t)touched_bound;
  w->last_mode = mode;
  w->last_H = H;
  w->last_U0 = U0;
  return PX_OK;
}

}  // extern "C"

namespace {
// Counters of a finished build (device result block) into the world's stats.
void fill_stats(px_world* w, const BuildResult& r) {
  w->stats.pairs = w->last_P;
  w->stats.brick_evals = r.c.brick_evals;
  w->stats.sub_evals = r.c.sub_evals;
  w->stats.voxel_evals = r.c.voxel_evals;
  w->stats.paint_evals = r.c.paint_evals;
  w->stats.rescued = r.c.rescued;
  w->stats.alloc_events = r.c.alloc_events;
  w->stats.free_events = r.c.free_events;
  {
    double me;
    unsigned long long bits = r.max_err_bits;
    std::memcpy(&me, &bits, 8);
    w->stats.max_abs_err32 = me;
  }
  w->stats.violations = r.c.violations;
  w->stats.rescued_brick = r.c.resc_brick;
  w->stats.rescued_sub = r.c.resc_sub;
  w->stats.rescued_voxel = r.c.resc_vox;
  w->stats.rescued_polygon = r.c.resc_poly;
  w->stats.rescued_paint = (uint32_t)r.c.resc_paint;
  w->stats.status = r.status;
}

}  // namespace

extern "C" {

static int build_finish_impl(px_world* w) {
  if (!w) return PX_E_INVALID_ARG;
  if (!w->in_flight) return PX_OK;
  w->in_flight = false;
  CU(cudaEventSynchronize(w->ev_done));  // the result block (later work on the stream may still run)
  w->uploads_pending = false;
  const BuildResult& r = *w->h_res;
  float ms = 0.f, fold_ms = 0.f;
  cudaEventElapsedTime(&ms, w->ev0, w->ev1);
  cudaEventElapsedTime(&fold_ms, w->ev_fold0, w->ev_fold1);
  w->stats.fold_ms = fold_ms;
  float cls_ms = 0.f;
  cudaEventElapsedTime(&cls_ms, w->ev_fold0, w->ev_mid);
  w->stats.classify_ms = cls_ms;
  w->stats.build_ms = ms;
  fill_stats(w, r);
  // transactional retries: nothing was committed
  // a build that commits nothing poisons the device state (WorldState); retries clear it
  auto clear_poison = [&] { return cudaMemsetAsync(&w->d_state->poisoned, 0, 4, w->stream); };
  if (w->no_retry && (r.status & (ST_NO_COMMIT | ST_POOL_OVERFLOW))) {  // pipelined: later builds are queued
    w->retries = 0;
    return fail(w, PX_E_QUEUE_OVERFLOW, "pipelined build failed: device status 0x%x", r.status);
  }
  if ((r.status & ST_RESCUE_OVERFLOW) && w->retries < 2) {  // more left to float64 than the rescue list holds
    CU(clear_poison());
    w->rescue_cap = std::max(w->rescue_cap, r.n_rescue + r.n_rescue / 4 + 1024);
    w->retries++;
    w->ops_resident = true;
    int rc = px_build_enqueue(w, w->last_mode, w->stream);
    if (rc == PX_OK) rc = px_build_finish(w);
    w->retries = 0;
    return rc;
  }
  if ((r.status & ST_STAGE_OVERFLOW) && r.stage_count > w->last_stage_cap && w->retries < 2) {
    CU(clear_poison());
    w->stage_hint = (uint64_t)r.stage_count + r.stage_count / 4 + 64;
    w->retries++;
    w->ops_resident = true;  // the op tables uploaded by this attempt are still on the device
    int rc = px_build_enqueue(w, w->last_mode, w->stream);
    if (rc == PX_OK) rc = px_build_finish(w);
    w->retries = 0;
    return rc;
  }
  if ((r.status & ST_POOL_OVERFLOW) && !(r.status & ST_NO_COMMIT) && w->retries < 2) {
    w->retries++;
    int rc = grow_pool(w, (uint64_t)r.pool_used + r.pool_used / 4 + 64, w->last_U0, w->stream);
    if (rc) { w->retries = 0; return rc; }
    BuildResult* dres = (BuildResult*)w->res.p;
    CU(clear_poison());
    const uint32_t st2 = r.status & ~(uint32_t)ST_POOL_OVERFLOW;
    CU(cudaMemcpyAsync(&dres->status, &st2, 4, cudaMemcpyHostToDevice, w->stream));
    w->fin.pool32 = w->d_pool32;
    w->fin.pcount = w->d_pcount;
    w->fin.pool_cap = w->pool_cap;
    launch_finalize(w->fin, w->last_touched_cap, w->stream);
    if (w->derive_max) {  // the holes the replay wrote are the other buffer of the pair
      DevBuf& holes_after = w->holes_in_a ? w->holes_b : w->holes_a;
      if ((rc = enqueue_build_derive(w, w->stream, (const uint32_t*)holes_after.p))) { w->retries = 0; return rc; }
    }
    CU(cudaGetLastError());
    CU(cudaMemcpyAsync(w->h_res, dres, sizeof(BuildResult), cudaMemcpyDeviceToHost, w->stream));
    CU(cudaEventRecord(w->ev_done, w->stream));
    w->in_flight = true;
    rc = px_build_finish(w);
    w->retries = 0;
    return rc;
  }
  w->retries = 0;
  if (r.status & (ST_NO_COMMIT | ST_POOL_OVERFLOW)) {
    w->pcount_refresh = false;
    if (!w->shares_state) {  // nothing was committed: the world stays as it was, ready for the next build
      CU(clear_poison());
      CU(cudaStreamSynchronize(w->stream));
    }
    return fail(w, PX_E_QUEUE_OVERFLOW, "device status 0x%x (stage %u of %u, max pool index %u of %u)", r.status,
                r.stage_count, w->last_stage_cap, r.max_pool_index, w->pool_cap);
  }
  // the build is committed: holes/pool counters move to the new state
  w->pool_used = r.pool_used;
  w->n_holes = r.n_holes;
  w->holes_in_a = !w->holes_in_a;
  w->ops_applied += w->ops.size();
  w->last_ops.swap(w->ops);
  w->last_boxes.swap(w->boxes);
  w->last_code.swap(w->code);
  w->last_params.swap(w->params);
  w->last_code32.swap(w->code32);
  w->last_p32.swap(w->p32);
  w->last_bases.swap(w->bases);
  std::swap(w->last_q, w->q);
  w->q.clear();
  w->code32.clear();
  w->p32.clear();
  w->bases.clear();
  w->ops.clear();
  w->boxes.clear();
  w->code.clear();
  w->params.clear();
  w->derived_valid = w->derive_max != 0;  // derive on build: super, density and free list are current
  w->free_valid = w->derive_max != 0;
  if (w->pcount_refresh) w->pcount_valid = true;  // that derive recounted every referenced brick
  w->pcount_refresh = false;
  w->free_over = (r.status & ST_FREE_CAP) != 0;
  w->free_len = r.free_len;
  w->stats.ops_applied = w->ops_applied;
  w->stats.pool_used = w->pool_used;
  w->stats.n_holes = w->n_holes;
  w->stats.pool_capacity = w->pool_cap;
  if (r.status & ST_RANGE) return fail(w, PX_E_RANGE, "a paint function received an argument outside its supported range");
  return PX_OK;
}

int px_build(px_world* w, int mode, void* stream) {
  int rc = px_build_enqueue(w, mode, stream);
  if (rc) return rc;
  return px_build_finish(w);
}

int px_set_validation(px_world* w, int on) {
  if (!w) return PX_E_INVALID_ARG;
  w->validate = on ? 1 : 0;
  return PX_OK;
}

static int world_reset_impl(px_world* w, int requeue_last_ops, void* stream) {
  if (!w) return PX_E_INVALID_ARG;
  if (w->batch_locked && !w->capturing) return fail(w, PX_E_INVALID_ARG, "the world belongs to a batch");
  if (w->in_flight) return fail(w, PX_E_INVALID_ARG, "a build is in flight");
  if (w->uploads_pending) {  // a build that failed after its upload kernel was launched
    CU(cudaStreamSynchronize(w->stream));
    w->uploads_pending = false;
  }
  CU(cudaMemsetAsync(w->d_grid, 0, w->ncells * 4, (cudaStream_t)stream));
  CU(cudaMemsetAsync(w->d_state, 0, sizeof(WorldState), (cudaStream_t)stream));
  w->pool_used = 0;
  w->n_holes = 0;
  w->derived_valid = false;
  w->free_valid = false;
  if (requeue_last_ops) {
    if (!w->ops.empty()) return fail(w, PX_E_INVALID_ARG, "ops are already queued");
    w->ops = w->last_ops;
    w->boxes = w->last_boxes;
    w->code = w->last_code;
    w->params = w->last_params;
    w->code32 = w->last_code32;
    w->p32 = w->last_p32;
    w->bases = w->last_bases;
    w->q = w->last_q;
    w->ops_resident = true;  // the device tables of the last build still hold them
  }
  return PX_OK;
}

int px_read_grid(px_world* w, uint32_t* dst, size_t n) {
  if (!w || !dst || n < w->ncells) return PX_E_INVALID_ARG;
  CU(cudaMemcpy(dst, w->d_grid, w->ncells * 4, cudaMemcpyDeviceToHost));
  return PX_OK;
}
int px_read_pool(px_world* w, uint16_t* dst, size_t n) {
  if (!w || (!dst && w->pool_used) || n < (size_t)w->pool_used * 512) return PX_E_INVALID_ARG;
  if (w->pool_used) CU(cudaMemcpy(dst, w->d_pool32, (size_t)w->pool_used * 1024, cudaMemcpyDeviceToHost));
  return PX_OK;
}
int px_read_holes(px_world* w, uint32_t* dst, size_t n) {
  if (!w || n < w->n_holes) return PX_E_INVALID_ARG;
  DevBuf& cur = w->holes_in_a ? w->holes_a : w->holes_b;
  if (w->n_holes) CU(cudaMemcpy(dst, cur.p, (size_t)w->n_holes * 4, cudaMemcpyDeviceToHost));
  return PX_OK;
}

int px_derive(px_world* w) {
  if (!w) return PX_E_INVALID_ARG;
  int rc;
  size_t nsup = w->ntiles;
  if ((rc = ensure(w, w->super_counts, 4 * nsup)) || (rc = ensure(w, w->density, w->ncells))) return rc;
  DeriveArgs da{};
  da.grid = w->d_grid;
  da.pool32 = w->d_pool32;
  da.BX = w->BX; da.BY = w->BY; da.BZ = w->BZ;
  da.opaque = (const uint8_t*)w->opaque.p;
  da.udens = (const uint8_t*)w->udens.p;
  da.super_counts = (uint32_t*)w->super_counts.p;
  da.density = (uint8_t*)w->density.p;
  da.pcount = w->pcount_valid ? w->d_pcount : nullptr;
  da.pcount_out = w->pcount_valid ? nullptr : w->d_pcount;
  launch_derive(da, 0);
  CU(cudaGetLastError());
  CU(cudaDeviceSynchronize());
  w->derived_valid = true;
  w->pcount_valid = true;
  return PX_OK;
}
int px_read_super(px_world* w, uint32_t* dst, size_t n) {
  if (!w || !dst || n < w->ntiles) return PX_E_INVALID_ARG;
  if (!w->derived_valid) { int rc = px_derive(w); if (rc) return rc; }
  CU(cudaMemcpy(dst, w->super_counts.p, w->ntiles * 4, cudaMemcpyDeviceToHost));
  return PX_OK;
}
int px_read_density(px_world* w, uint8_t* dst, size_t n) {
  if (!w || !dst || n < w->ncells) return PX_E_INVALID_ARG;
  if (!w->derived_valid) { int rc = px_derive(w); if (rc) return rc; }
  CU(cudaMemcpy(dst, w->density.p, w->ncells, cudaMemcpyDeviceToHost));
  return PX_OK;
}
// GpuWorld.ts:55-60, 103-109
int px_read_free_list(px_world* w, uint32_t max_bricks, uint32_t* dst, size_t n, uint32_t* out_len) {
  if (!w) return PX_E_INVALID_ARG;
  if (w->free_valid && max_bricks == w->derive_max) {  // built on the device by the last build
    if (w->free_over)
      return fail(w, PX_E_OOM, "the scene needs %u bricks but the pool holds fewer", (unsigned)w->pool_used);
    if (out_len) *out_len = w->free_len;
    if (!dst) return PX_OK;
    if (n < w->free_len) return PX_E_INVALID_ARG;
    if (w->free_len) CU(cudaMemcpy(dst, w->free_list.p, (size_t)w->free_len * 4, cudaMemcpyDeviceToHost));
    return PX_OK;
  }
  uint64_t used = w->pool_used;
  uint64_t cap = used + 98304 > used * 2 ? used + 98304 : used * 2;
  if (cap > max_bricks) cap = max_bricks;
  if (used > cap) return fail(w, PX_E_OOM, "the scene needs %llu bricks but the pool holds %llu", (unsigned long long)used, (unsigned long long)cap);
  uint64_t len = w->n_holes + (cap - used);
  if (out_len) *out_len = (uint32_t)len;
  if (!dst) return PX_OK;
  if (n < len) return PX_E_INVALID_ARG;
  int rc = px_read_holes(w, dst, n);
  if (rc) return rc;
  for (uint64_t i = 0; i < cap - used; i++) dst[w->n_holes + i] = (uint32_t)(cap - 1 - i);
  return PX_OK;
}

int px_get_stats(px_world* w, px_stats* out) {
  if (!w || !out) return PX_E_INVALID_ARG;
  *out = w->stats;
  out->pool_used = w->pool_used;
  out->n_holes = w->n_holes;
  out->pool_capacity = w->pool_cap;
  out->ops_applied = w->ops_applied;
  return PX_OK;
}

int px_world_info(px_world* w, int dims[3], double* vpm) {
  if (!w) return PX_E_INVALID_ARG;
  if (dims) { dims[0] = w->dx; dims[1] = w->dy; dims[2] = w->dz; }
  if (vpm) *vpm = w->vpm;
  return PX_OK;
}

int px_device_view_get(px_world* w, px_device_view* out) {
  if (!w || !out) return PX_E_INVALID_ARG;
  out->grid = w->d_grid;
  out->pool = (const uint16_t*)w->d_pool32;
  DevBuf& cur = w->holes_in_a ? w->holes_a : w->holes_b;
  out->holes = (const uint32_t*)cur.p;
  out->super_counts = w->derived_valid ? (const uint32_t*)w->super_counts.p : nullptr;
  out->density = w->derived_valid ? (const uint8_t*)w->density.p : nullptr;
  out->free_list = w->free_valid && !w->free_over ? (const uint32_t*)w->free_list.p : nullptr;
  out->free_len = w->free_valid && !w->free_over ? w->free_len : 0u;
  out->pad = 0;
  return PX_OK;
}

int px_set_derive_on_build(px_world* w, uint32_t max_bricks) {
  if (!w) return PX_E_INVALID_ARG;
  if (w->in_flight || w->batch_locked) return fail(w, PX_E_INVALID_ARG, "the world is busy");
  w->derive_max = max_bricks;
  w->free_valid = false;
  return PX_OK;
}

int px_reserve_pool(px_world* w, uint64_t bricks) {
  if (!w) return PX_E_INVALID_ARG;
  if (w->in_flight || w->batch_locked) return fail(w, PX_E_INVALID_ARG, "the world is busy");
  return grow_pool(w, bricks, w->pool_used, nullptr);
}

const char* px_last_error(px_world* w) { return w ? w->err.c_str() : "null world"; }

int px_probe_peak(int fp64, float* tflops) {
  if (!tflops) return PX_E_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return PX_E_NO_DEVICE; }
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  *tflops = probe_fma_tflops(fp64, sms);
  return cudaGetLastError() == cudaSuccess ? PX_OK : PX_E_CUDA;
}

int px_check_sqrt_bounds(uint32_t lo_bits, uint32_t hi_bits, uint64_t* n_bad, uint32_t* first_bad) {
  if (!n_bad || !first_bad || lo_bits > hi_bits || hi_bits >= 0x7f800000u) return PX_E_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) { cudaGetLastError(); return PX_E_NO_DEVICE; }
  unsigned long long nb = 0;
  if (check_sqrt_bounds(lo_bits, hi_bits, &nb, first_bad)) return PX_E_CUDA;
  *n_bad = nb;
  return PX_OK;
}

// ---------------------------------------------------------------------------
// Batched builds: the rebuild of many worlds (each from its last op list)
// captured once into one CUDA graph over several streams and relaunched as a
// single graph.  Small scenes run side by side on the GPU; each scene's
// persistent grids are sized to its pairs (pairs_per_block).

struct px_batch {
  std::vector<px_world*> worlds;
  std::vector<cudaStream_t> streams;
  std::vector<cudaEvent_t> joins;
  cudaEvent_t fork = nullptr, t0 = nullptr, t1 = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int mode = 0;
  std::string err;
};

namespace {

int batch_fail(px_batch* b, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  b->err = buf;
  return code;
}

void batch_free(px_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (cudaStream_t s : b->streams) cudaStreamDestroy(s);
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->t0) cudaEventDestroy(b->t0);
  if (b->t1) cudaEventDestroy(b->t1);
  for (px_world* w : b->worlds) w->batch_locked = false;
  delete b;
}

// Host state of a world across the capture (capture runs nothing).
struct WorldSaved {
  uint32_t pool_used, n_holes;
  bool holes_in_a, derived_valid, free_valid;
  uint32_t ppb;
};

}  // namespace

static int batch_create_impl(px_world* const* worlds, size_t n, int mode, uint32_t n_streams, uint32_t pairs_per_block,
                    px_batch** out) {
  if (!out) return PX_E_INVALID_ARG;
  *out = nullptr;
  if (!worlds || n == 0 || n_streams == 0 || n_streams > 256 || (mode != PX_MODE_FP64 && mode != PX_MODE_MIXED))
    return PX_E_INVALID_ARG;
  for (size_t i = 0; i < n; i++) {
    px_world* w = worlds[i];
    if (!w || w->batch_locked || w->in_flight || !w->ops.empty() || w->last_ops.empty()) return PX_E_INVALID_ARG;
    for (size_t j = 0; j < i; j++)
      if (worlds[j] == w) return PX_E_INVALID_ARG;
  }
  px_batch* b = new px_batch;
  b->worlds.assign(worlds, worlds + n);
  b->mode = mode;
  // largest builds first, dealt round-robin over the streams
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
    return b->worlds[x]->last_ops.size() * b->worlds[x]->ncells > b->worlds[y]->last_ops.size() * b->worlds[y]->ncells;
  });
  // one real rebuild per world first, so that every buffer the captured
  // rebuild touches already has its size (nothing allocates while capturing)
  for (size_t i = 0; i < n; i++) {
    px_world* w = b->worlds[i];
    const uint32_t keep = w->pairs_per_block;
    w->pairs_per_block = pairs_per_block;
    int rc = px_world_reset(w, 1, nullptr);
    if (rc == PX_OK) rc = px_build(w, mode, nullptr);
    w->pairs_per_block = keep;
    if (rc != PX_OK) {  // px_last_error(w) tells why
      delete b;
      return rc;
    }
  }
  if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&b->t0) != cudaSuccess || cudaEventCreate(&b->t1) != cudaSuccess) {
    cudaGetLastError();
    batch_free(b);
    return PX_E_CUDA;
  }
  for (uint32_t k = 0; k < n_streams; k++) {
    cudaStream_t st;
    cudaEvent_t ev;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) { cudaGetLastError(); batch_free(b); return PX_E_CUDA; }
    b->streams.push_back(st);
    if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) { cudaGetLastError(); batch_free(b); return PX_E_CUDA; }
    b->joins.push_back(ev);
  }
  std::vector<WorldSaved> saved(n);
  for (size_t i = 0; i < n; i++) {
    px_world* w = b->worlds[i];
    saved[i] = {w->pool_used, w->n_holes, w->holes_in_a, w->derived_valid, w->free_valid, w->pairs_per_block};
  }
  cudaStream_t origin = b->streams[0];
  int rc = PX_OK;
  if (cudaStreamBeginCapture(origin, cudaStreamCaptureModeThreadLocal) != cudaSuccess) { cudaGetLastError(); batch_free(b); return PX_E_CUDA; }
  cudaEventRecord(b->fork, origin);
  for (uint32_t k = 1; k < n_streams; k++) cudaStreamWaitEvent(b->streams[k], b->fork, 0);
  for (size_t q = 0; q < n && rc == PX_OK; q++) {
    px_world* w = b->worlds[order[q]];
    cudaStream_t st = b->streams[q % n_streams];
    w->capturing = true;
    w->batch_locked = true;
    w->pairs_per_block = pairs_per_block;
    w->batch_holes_in_a = w->holes_in_a;
    rc = px_world_reset(w, 1, st);
    if (rc == PX_OK) rc = px_build_enqueue(w, mode, st);
    w->capturing = false;
    w->in_flight = false;  // captured, not launched
    if (rc != PX_OK) batch_fail(b, rc, "world %zu: %s", order[q], w->err.c_str());
  }
  for (uint32_t k = 1; k < n_streams; k++) {
    cudaEventRecord(b->joins[k], b->streams[k]);
    cudaStreamWaitEvent(origin, b->joins[k], 0);
  }
  const cudaError_t ce = cudaStreamEndCapture(origin, &b->graph);
  // the worlds keep their built state until the graph runs
  for (size_t i = 0; i < n; i++) {
    px_world* w = b->worlds[i];
    w->pool_used = saved[i].pool_used;
    w->n_holes = saved[i].n_holes;
    w->holes_in_a = saved[i].holes_in_a;
    w->derived_valid = saved[i].derived_valid;
    w->free_valid = saved[i].free_valid;
    w->pairs_per_block = saved[i].ppb;
    w->ops.clear(); w->boxes.clear(); w->code.clear(); w->params.clear();
    w->code32.clear(); w->p32.clear(); w->bases.clear();
    w->q.clear();
  }
  if (rc == PX_OK && ce != cudaSuccess) rc = batch_fail(b, PX_E_CUDA, "capture: %s", cudaGetErrorString(ce));
  if (rc == PX_OK && cudaGraphInstantiate(&b->exec, b->graph, 0) != cudaSuccess)
    rc = batch_fail(b, PX_E_CUDA, "graph instantiation failed");
  if (rc != PX_OK) {
    cudaGetLastError();
    batch_free(b);
    return rc;
  }
  *out = b;
  return PX_OK;
}

int px_batch_run(px_batch* b, void* stream, float* device_ms) {
  if (!b) return PX_E_INVALID_ARG;
  cudaStream_t s = (cudaStream_t)stream;
  if (cudaEventRecord(b->t0, s) != cudaSuccess || cudaGraphLaunch(b->exec, s) != cudaSuccess ||
      cudaEventRecord(b->t1, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) {
    const cudaError_t e = cudaGetLastError();
    return batch_fail(b, PX_E_CUDA, "graph launch: %s", cudaGetErrorString(e));
  }
  if (device_ms) cudaEventElapsedTime(device_ms, b->t0, b->t1);
  int first = PX_OK;
  for (size_t i = 0; i < b->worlds.size(); i++) {
    px_world* w = b->worlds[i];
    const BuildResult& r = *w->h_res;
    fill_stats(w, r);
    w->stats.build_ms = 0.f;
    if (r.status & (ST_NO_COMMIT | ST_POOL_OVERFLOW)) {
      if (first == PX_OK) first = batch_fail(b, PX_E_QUEUE_OVERFLOW, "world %zu: device status 0x%x", i, r.status);
      cudaMemset(&w->d_state->poisoned, 0, 4);  // the world stays as it was
      continue;
    }
    w->pool_used = r.pool_used;
    w->n_holes = r.n_holes;
    w->holes_in_a = !w->batch_holes_in_a;  // the captured build wrote the other holes buffer
    w->derived_valid = w->derive_max != 0;
    w->free_valid = w->derive_max != 0;
    w->free_over = (r.status & ST_FREE_CAP) != 0;
    w->free_len = r.free_len;
    if (w->pcount_refresh) w->pcount_valid = true;  // the captured derive recounts every referenced brick
    w->ops_applied += w->last_ops.size();
    w->stats.ops_applied = w->ops_applied;
    w->stats.pool_used = w->pool_used;
    w->stats.n_holes = w->n_holes;
    w->stats.pool_capacity = w->pool_cap;
    if ((r.status & ST_RANGE) && first == PX_OK)
      first = batch_fail(b, PX_E_RANGE, "world %zu: a paint function received an argument outside its supported range", i);
  }
  return first;
}

void px_batch_destroy(px_batch* b) {
  if (!b) return;
  if (b->streams.size()) cudaStreamSynchronize(b->streams[0]);
  batch_free(b);
}

const char* px_batch_last_error(px_batch* b) { return b ? b->err.c_str() : "null batch"; }

}  // extern "C"

extern "C" {

int px_world_create(int dx, int dy, int dz, double vpm, uint32_t initial_pool_bricks, px_world** out) {
  return guarded(nullptr, [&] { return world_create_impl(dx, dy, dz, vpm, initial_pool_bricks, out); });
}

int px_submit_ops(px_world* w, const void* ir, size_t bytes) {
  return guarded(w, [&] { return submit_ops_impl(w, ir, bytes); });
}

int px_build_enqueue(px_world* w, int mode, void* stream) {
  return guarded(w, [&] { return build_enqueue_impl(w, mode, stream); });
}

int px_build_finish(px_world* w) {
  return guarded(w, [&] { return build_finish_impl(w); });
}

int px_world_reset(px_world* w, int requeue_last_ops, void* stream) {
  return guarded(w, [&] { return world_reset_impl(w, requeue_last_ops, stream); });
}

int px_batch_create(px_world* const* worlds, size_t n, int mode, uint32_t n_streams, uint32_t pairs_per_block,
                    px_batch** out) {
  return guarded(nullptr, [&] { return batch_create_impl(worlds, n, mode, n_streams, pairs_per_block, out); });
}

}  // extern "C"
