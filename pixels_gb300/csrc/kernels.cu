// Voxeliser kernels for sm_103a (GB300).
//
// Pipeline of one build (all on one stream, no host round trip):
//   cull      one warp per 4^3-brick tile scans the op list (ballot) and keeps
//             the ops whose brick box overlaps the tile, in op order.
//   fold      persistent warps, one brick at a time: the brick's 512 voxels live
//             in registers (two voxels per lane per z slice); the warp applies
//             the brick's ops in order exactly as apply() does (shapes.ts:353-412):
//             brick classify, 4^3 sub-block classify, boundary voxels, paint,
//             uniform shortcuts, compaction.  Pool alloc/free events are
//             recorded per (op, brick) pair; bricks that end non-uniform are
//             written to a staging area.
//   replay    parallel replay of the LIFO pool allocator (VoxelWorld.ts:112-127)
//             over the events in (op, cell) order: clamped depth scan, match
//             of each pop to its push (previous-smaller-value search on a
//             32-ary min tree), pointer chasing of recycled indices.
//   finalize  staging -> pool at the replayed indices (16-byte vector copies),
//             grid entries.
//   derive    super-grid counts and density bytes (GpuWorld.ts:90-101).
#include <algorithm>
#include <cstdio>
#include "px_internal.cuh"
#include "sdf64.cuh"
#include "sdf32.cuh"
#include "paint.cuh"
#include "paint32.cuh"

namespace px {

#define FULLMASK 0xffffffffu

// CTAs per SM the two build kernels are compiled for (register budget)
#ifndef PX_CLASSIFY_MINB
#define PX_CLASSIFY_MINB 3
#endif
#ifndef PX_SUB_MINB
#define PX_SUB_MINB PX_CLASSIFY_MINB
#endif
#ifndef PX_VOXEL_MINB
#define PX_VOXEL_MINB 3
#endif
#ifndef PX_CLASSIFY64_MINB
#define PX_CLASSIFY64_MINB 2
#endif
#ifndef PX_FOLD_MINB
#define PX_FOLD_MINB 3
#endif
#ifndef PX_VSIMPLE_MINB
#define PX_VSIMPLE_MINB 4
#endif
#ifndef PX_VWIDE_MINB
#define PX_VWIDE_MINB 3
#endif
#ifndef PX_PAINT_MINB
#define PX_PAINT_MINB 3
#endif
#ifndef PX_VAFF_MINB
#define PX_VAFF_MINB 3
#endif

// kernel launches issued by the host wrappers (reported per build)
static unsigned long long g_launches = 0;
unsigned long long launch_count() { return g_launches; }

// Programmatic dependent launch: the kernels of a build are launched so that
// each may be scheduled while its predecessor drains.  Every such kernel starts
// with pdl_prologue(): it waits until the preceding grid has completed and its
// memory is visible (griddepcontrol.wait), then lets its own successor launch
// once all of its CTAs have started (griddepcontrol.launch_dependents).
__device__ __forceinline__ void pdl_prologue() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// The staging area lives between the apply pass and finalize only: its stores
// ask L2 to keep the lines (evict_last), and finalize, once it has read a staged
// brick, drops its lines from L2 without writing them back (discard.global.L2),
// so that the bricks need not travel through DRAM twice.
__device__ __forceinline__ unsigned long long l2_keep_policy() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ void st_keep(uint32_t* p, uint32_t v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.b32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}
// p: a 128-byte aligned line whose data is no longer wanted
__device__ __forceinline__ void l2_discard_line(const void* p) {
  asm volatile("discard.global.L2 [%0], 128;" ::"l"(p) : "memory");
}
// Launched from the host one by one, the overlap hides most of each launch's
// latency; inside a captured graph (whose launches are already back to back)
// it measured slower, so captures launch plainly (set_programmatic_launch).
static thread_local bool g_pdl = true;
void set_programmatic_launch(bool on) { g_pdl = on; }
template <typename... KArgs, typename... Args>
static void launch_pdl(void (*k)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = g_pdl ? 1 : 0;
  ++g_launches;
  cudaLaunchKernelEx(&cfg, k, args...);
}

// ---------------------------------------------------------------------------
// cull

__device__ __forceinline__ bool box_overlaps_tile(uint2 b, int tx, int ty, int tz) {
  int x0 = b.x & 1023, y0 = (b.x >> 10) & 1023, z0 = (b.x >> 20) & 1023;
  int x1 = b.y & 1023, y1 = (b.y >> 10) & 1023, z1 = (b.y >> 20) & 1023;
  if (b.x >> 30) return false;  // op with an empty voxel range
  return x0 <= tx * 4 + 3 && x1 >= tx * 4 && y0 <= ty * 4 + 3 && y1 >= ty * 4 && z0 <= tz * 4 + 3 && z1 >= tz * 4;
}

// The op boxes are followed by one union box per 32 consecutive ops: a warp
// tests the 32-op groups first and only the ops of groups that overlap its
// tile (a two-level culling hierarchy; scene ops come object by object, so
// groups are compact).
// One warp per tile, eight tiles per block: the tile's ops are counted, the
// block reserves room for its eight lists with one atomic, and each warp writes
// its list (op order) and the op boxes beside it.  The lists lie in reservation
// order; tile_off / tile_cnt locate them.
__global__ void __launch_bounds__(256) cull_kernel(const uint2* __restrict__ boxes, int n_ops, int TX, int TY, int TZ,
                                                   uint32_t* tile_cnt, uint32_t* tile_off, uint32_t* tile_ops,
                                                   uint2* tile_boxes, uint32_t* counter) {
  pdl_prologue();
  __shared__ uint32_t s_cnt[8], s_base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n_tiles = TX * TY * TZ;
  const int n_groups = (n_ops + 31) / 32;
  const uint2* __restrict__ gboxes = boxes + n_ops;
  const int tile = blockIdx.x * 8 + warp;
  const bool valid = tile < n_tiles;
  int tz = 0, ty = 0, tx = 0;
  if (valid) {
    tz = tile / (TX * TY);
    const int r = tile - tz * TX * TY;
    ty = r / TX;
    tx = r - ty * TX;
  }
  uint32_t cnt = 0;
  if (valid) {
    for (int g0 = 0; g0 < n_groups; g0 += 32) {
      const int gi = g0 + lane;
      uint32_t gm = __ballot_sync(FULLMASK, gi < n_groups && box_overlaps_tile(__ldg(gboxes + gi), tx, ty, tz));
      while (gm) {
        const int i = (g0 + __ffs(gm) - 1) * 32 + lane;
        gm &= gm - 1;
        const bool ov = i < n_ops && box_overlaps_tile(__ldg(boxes + i), tx, ty, tz);
        cnt += __popc(__ballot_sync(FULLMASK, ov));
      }
    }
  }
  if (lane == 0) s_cnt[warp] = cnt;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t sum = 0;
    for (int k = 0; k < 8; k++) sum += s_cnt[k];
    s_base = sum ? atomicAdd(counter, sum) : 0u;
  }
  __syncthreads();
  if (!valid) return;
  uint32_t pos = s_base;
  for (int k = 0; k < warp; k++) pos += s_cnt[k];
  if (lane == 0) {
    tile_cnt[tile] = cnt;
    tile_off[tile] = pos;
  }
  if (!cnt) return;
  for (int g0 = 0; g0 < n_groups; g0 += 32) {
    const int gi = g0 + lane;
    uint32_t gm = __ballot_sync(FULLMASK, gi < n_groups && box_overlaps_tile(__ldg(gboxes + gi), tx, ty, tz));
    while (gm) {
      const int i = (g0 + __ffs(gm) - 1) * 32 + lane;
      gm &= gm - 1;
      const uint2 b = i < n_ops ? __ldg(boxes + i) : make_uint2(3u << 30, 0u);
      const bool ov = i < n_ops && box_overlaps_tile(b, tx, ty, tz);
      const uint32_t m = __ballot_sync(FULLMASK, ov);
      if (ov) {
        const uint32_t at = pos + __popc(m & ((1u << lane) - 1u));
        tile_ops[at] = (uint32_t)i;
        tile_boxes[at] = b;  // the op's brick box beside it, for the apply pass
      }
      pos += __popc(m);
    }
  }
}

// The same lists with the ops grouped in space: the host orders the ops along a
// Morton curve of their box centres and stores one union box per 32 of that order
// (order[] after the group boxes), so that a group's box is compact even where
// consecutive ops lie far apart (scattered primitives).  A warp marks its tile's
// ops in a bit set in shared memory (one bit per op) and then writes them in op
// order from it.  W: words of the bit set (ops / 32, rounded up).
__global__ void __launch_bounds__(256) cull_sorted_kernel(const uint2* __restrict__ boxes, int n_ops, int TX, int TY,
                                                          int TZ, int W, uint32_t* tile_cnt, uint32_t* tile_off,
                                                          uint32_t* tile_ops, uint2* tile_boxes, uint32_t* counter) {
  pdl_prologue();
  extern __shared__ uint32_t s_bits[];  // [8][W]
  __shared__ uint32_t s_cnt[8], s_base;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int n_tiles = TX * TY * TZ;
  const int n_groups = (n_ops + 31) / 32;
  const uint2* __restrict__ gboxes = boxes + n_ops;
  const uint32_t* __restrict__ order = reinterpret_cast<const uint32_t*>(boxes + n_ops + n_groups);
  uint32_t* bits = s_bits + (size_t)warp * W;
  const int tile = blockIdx.x * 8 + warp;
  const bool valid = tile < n_tiles;
  int tz = 0, ty = 0, tx = 0;
  if (valid) {
    tz = tile / (TX * TY);
    const int r = tile - tz * TX * TY;
    ty = r / TX;
    tx = r - ty * TX;
  }
  for (int k = lane; k < W; k += 32) bits[k] = 0u;
  __syncwarp();
  if (valid) {
    for (int g0 = 0; g0 < n_groups; g0 += 32) {
      const int gi = g0 + lane;
      uint32_t gm = __ballot_sync(FULLMASK, gi < n_groups && box_overlaps_tile(__ldg(gboxes + gi), tx, ty, tz));
      while (gm) {
        const int k = (g0 + __ffs(gm) - 1) * 32 + lane;
        gm &= gm - 1;
        if (k < n_ops) {
          const uint32_t i = __ldg(order + k);
          if (box_overlaps_tile(__ldg(boxes + i), tx, ty, tz)) atomicOr(bits + (i >> 5), 1u << (i & 31));
        }
      }
    }
  }
  __syncwarp();
  uint32_t cnt = 0;
  for (int k = lane; k < W; k += 32) cnt += __popc(bits[k]);
#pragma unroll
  for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(FULLMASK, cnt, o);
  if (lane == 0) s_cnt[warp] = valid ? cnt : 0u;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t sum = 0;
    for (int k = 0; k < 8; k++) sum += s_cnt[k];
    s_base = sum ? atomicAdd(counter, sum) : 0u;
  }
  __syncthreads();
  if (!valid) return;
  uint32_t pos = s_base;
  for (int k = 0; k < warp; k++) pos += s_cnt[k];
  if (lane == 0) {
    tile_cnt[tile] = cnt;
    tile_off[tile] = pos;
  }
  // the ops in order: lane l writes the ops of word w0 + l after those of the words before it
  for (int w0 = 0; w0 < W && cnt; w0 += 32) {
    const uint32_t word = w0 + lane < W ? bits[w0 + lane] : 0u;
    const uint32_t c = __popc(word);
    uint32_t incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t t = __shfl_up_sync(FULLMASK, incl, o);
      if (lane >= o) incl += t;
    }
    uint32_t at = pos + incl - c;
    for (uint32_t m = word; m; m &= m - 1) {
      const uint32_t i = (uint32_t)(w0 + lane) * 32u + (uint32_t)(__ffs(m) - 1);
      tile_ops[at] = i;
      tile_boxes[at] = __ldg(boxes + i);  // the op's brick box beside it, for the apply pass
      at++;
    }
    pos += __shfl_sync(FULLMASK, incl, 31);
  }
}

void launch_cull(const uint2* boxes, int n_ops, int TX, int TY, int TZ, uint32_t* tile_cnt, uint32_t* tile_off,
                 uint32_t* tile_ops, uint2* tile_boxes, uint32_t* counter, bool sorted, cudaStream_t s) {
  const int n_tiles = TX * TY * TZ;
  const int W = (n_ops + 31) / 32;
  if (sorted)
    launch_pdl(cull_sorted_kernel, dim3((n_tiles + 7) / 8), dim3(256), (size_t)8 * W * 4, s, boxes, n_ops, TX, TY, TZ,
               W, tile_cnt, tile_off, tile_ops, tile_boxes, counter);
  else
    launch_pdl(cull_kernel, dim3((n_tiles + 7) / 8), dim3(256), 0, s, boxes, n_ops, TX, TY, TZ, tile_cnt, tile_off,
               tile_ops, tile_boxes, counter);
}

// ---------------------------------------------------------------------------
// fold

enum { ST_EMPTY = 0, ST_UNIF = 1, ST_MIXED = 2 };

struct WarpCounters {
  uint32_t brick, sub, vox, alloc, free_;
};

// The float32 path's rare events -- rescues and validation mismatches --
// counted into the build's counters where they happen (no per-lane counters
// held in registers through the work loops).
struct LaneStats {
  BuildResult* res;
  __device__ __forceinline__ void viol() { atomicAdd(&res->c.violations, 1ull); }
  // a float64 rescue at level `what` (0 voxel, 1 brick, 2 sub-block); amb: an
  // undecided polygon crossing test; err: |mid(d32) - d64| (negative: none)
  __device__ __noinline__ void rescue(int what, bool amb, float err) {
    atomicAdd(&res->c.rescued, 1ull);
    atomicAdd(what == 1 ? &res->c.resc_brick : what == 2 ? &res->c.resc_sub : &res->c.resc_vox, 1ull);
    if (amb) atomicAdd(&res->c.resc_poly, 1ull);
    else if (err > 0.f) atomicMax(&res->max_err_bits, (unsigned long long)__double_as_longlong((double)err));
  }
};

// Work items taken by a warp from a shared counter, several per atomic (one
// counter for the whole grid: fewer same-address atomics).
struct WorkBatch {
  uint32_t at = 0, end = 0;
  __device__ __forceinline__ uint32_t next(uint32_t* counter, uint32_t batch, int lane) {
    if (at == end) {
      uint32_t b = 0;
      if (lane == 0) b = atomicAdd(counter, batch);
      at = __shfl_sync(FULLMASK, b, 0);
      end = at + batch;
    }
    return at++;
  }
};

// The next work ticket of a warp, requested one item ahead: lane 0 issues the
// atomic when the current item starts and the warp reads its result when the
// item is done, so the atomic's latency (one counter for the whole grid) hides
// behind the item's work.
struct NextTicket {
  uint32_t raw = 0;
  __device__ __forceinline__ void issue(uint32_t* counter, uint32_t n, int lane) {
    if (lane == 0) raw = atomicAdd(counter, n);
  }
  __device__ __forceinline__ uint32_t get() const { return __shfl_sync(FULLMASK, raw, 0); }
};

// Decisions of apply() from a float32 interval (thresholds certified on the host):
// brick/sub-block: 0 = outside (skip), 1 = partial, 2 = full, 3 = undecided.
__device__ __forceinline__ int classify32(Iv d, const float* thr, int base) {
  if (d.lo > thr[base + 0]) return 0;
  if (!(d.hi <= thr[base + 1])) return 3;
  if (d.hi < thr[base + 2]) return 2;
  if (d.lo >= thr[base + 3]) return 1;
  return 3;
}
__device__ __forceinline__ int classify64(double d, double half_diag) {
  if (d > half_diag) return 0;
  return d < -half_diag ? 2 : 1;
}

// The float32 point (relative to the op anchor) of voxel-space offset k * vs
// from the brick's first voxel centre, enclosing the reference's float64 point.
__device__ __forceinline__ Iv koff(float k, float vs_lo, float vs_hi) { return {__fmul_rd(k, vs_lo), __fmul_ru(k, vs_hi)}; }

// The shape at the reference's point (t * vs per axis, t in voxel units).  Out
// of line so that no float64 product is hoisted into the float32 path.
__device__ __noinline__ double sdf64_at(const uint2* __restrict__ code, int clen, const double* __restrict__ params,
                                        double vs, float tx, float ty, float tz) {
  return sdf64(code, clen, params, (double)tx * vs, (double)ty * vs, (double)tz * vs);
}

// Evaluate one shape at one point: float64 directly, or float32 interval with
// a float64 rescue when the interval cannot decide.  (tx, ty, tz) are the
// reference's point in voxel units (ox + 4, sx + 2 or x + 0.5, exact in
// float32); the float64 point (t * vs) is only formed when float64 runs.
// `what`: 0 voxel (returns 1 = inside), 1 brick, 2 sub-block (return the
// classification: 0 outside, 1 partial, 2 full).
template <int MODE>
__device__ __forceinline__ int eval_decide(const FoldArgs& a, const OpDev* O, const uint2* code, int clen, bool use32,
                                           const Iv* bo, float kx, float ky, float kz, float tx, float ty, float tz,
                                           int what, LaneStats& ls, bool count = true, Iv* dout = nullptr) {
  const int base = what == 1 ? T_BSK_HI : T_SSK_HI;
  if (MODE == 1 && use32) {
    bool amb = false;
    Iv px_ = iadd(bo[0], koff(kx, a.vs_lo, a.vs_hi)), py_ = iadd(bo[1], koff(ky, a.vs_lo, a.vs_hi)),
       pz_ = iadd(bo[2], koff(kz, a.vs_lo, a.vs_hi));
    Iv d = sdf32i(code, a.code32 + O->code_off, clen, reinterpret_cast<const Iv*>(a.p32), px_, py_, pz_, O->thr[T_M], amb);
    int r;
    if (what == 0) r = amb ? 3 : (d.lo > O->thr[T_V_HI] ? 0 : (d.hi <= O->thr[T_V_LO] ? 1 : 3));
    else r = amb ? 3 : classify32(d, O->thr, base);
    if (dout) *dout = d;
    if (r != 3 && !a.validate) return r;
    double d64 = sdf64_at(code, clen, a.params, a.vs, tx, ty, tz);
    if (dout && (amb || r == 3)) {  // the exact value lies within M of the float64 one
      const double M64 = MIXED_MARGIN;
      *dout = {__double2float_rd(d64 - M64), __double2float_ru(d64 + M64)};
    }
    const double M = MIXED_MARGIN;
    if (a.validate && !amb && !((double)d.lo - M <= d64 && d64 <= (double)d.hi + M) && count) ls.viol();
    if (r == 3 && count) {
      const double e = fabs(0.5 * ((double)d.lo + (double)d.hi) - d64);
      ls.rescue(what, amb, e == e ? (float)e : -1.f);
    }
    if (what == 0) return d64 > 0.0 ? 0 : 1;
    return classify64(d64, what == 1 ? O->bhd : O->shd);
  }
  const double vs = a.vs;
  const double X = (double)tx * vs, Y = (double)ty * vs, Z = (double)tz * vs;
  const double d = (O->flags & OPF_DEEP) ? sdf64_deep(code, clen, a.params, X, Y, Z) : sdf64(code, clen, a.params, X, Y, Z);
  if (what == 0) return d > 0.0 ? 0 : 1;
  return classify64(d, what == 1 ? O->bhd : O->shd);
}

// Bits i (0..3) of a 4-voxel row starting at voxel s that lie in the run [lo, hi].
__device__ __forceinline__ uint32_t run4(int s, int lo, int hi) {
  const int a0 = max(lo - s, 0), b0 = min(hi - s, 3);
  return a0 > b0 ? 0u : (2u << b0) - (1u << a0);
}
// Inside-mask of a lone box's 4^3 sub-block at voxel (sx, sy, sz) from its
// per-axis runs (OPF_BOX_RANGES): bit lx | ly << 2 | lz << 4.
__device__ __forceinline__ unsigned long long box_mask(const OpDev* O, int sx, int sy, int sz) {
  const uint32_t xb = run4(sx, O->vr[0], O->vr[1]), yb = run4(sy, O->vr[2], O->vr[3]),
                 zb = run4(sz, O->vr[4], O->vr[5]);
  const uint32_t ys = (yb & 1u) | ((yb & 2u) << 3) | ((yb & 4u) << 6) | ((yb & 8u) << 9);  // bit ly -> 4 ly
  const unsigned long long zs =
      (zb & 1ull) | ((unsigned long long)(zb & 2u) << 15) | ((unsigned long long)(zb & 4u) << 30) |
      ((unsigned long long)(zb & 8u) << 45);  // bit lz -> 16 lz
  return (unsigned long long)(xb * ys) * zs;
}

// The float64 side of a mixed-mode voxel decision taken from the interval d
// (r: 0 outside, 1 inside, 3 undecided; amb: a polygon crossing test was
// undecided): the rescue, or in validation mode the enclosure check.
// Returns the decision, whether the enclosure failed, and |mid(d) - d64|
// (-1 when not a rescue, or for an undecided crossing test).
struct VoxelF64 {
  int inside, viol;
  float err;
};
__device__ __noinline__ VoxelF64 voxel_f64(const double* __restrict__ params, double vs, int validate,
                                           const uint2* code, int clen, Iv d, bool amb, int r, float tx, float ty,
                                           float tz) {
  const double d64 = sdf64_at(code, clen, params, vs, tx, ty, tz);
  const double M = MIXED_MARGIN;
  VoxelF64 out;
  out.inside = d64 > 0.0 ? 0 : 1;
  out.viol = validate && !amb && !((double)d.lo - M <= d64 && d64 <= (double)d.hi + M);
  out.err = -1.f;
  if (r == 3 && !amb) {
    const double e = fabs(0.5 * ((double)d.lo + (double)d.hi) - d64);
    out.err = e == e ? (float)e : 0.f;
  }
  return out;
}

__device__ __forceinline__ void brick_of_pair(const OpDev* O, unsigned long long p, int& bx, int& by, int& bz) {
  const uint32_t local = (uint32_t)(p - O->pair_base);
  const uint32_t nxy = (uint32_t)(O->nx * O->ny);
  const uint64_t ixy = O->inv_nxy, ix = O->inv_nx;  // 0: a divisor of 1
  const uint32_t zq = ixy ? (uint32_t)__umul64hi(local, ixy) : local, r = local - zq * nxy;
  const uint32_t yq = ix ? (uint32_t)__umul64hi(r, ix) : r;
  bz = O->bz0 + (int)zq;
  by = O->by0 + (int)yq;
  bx = O->bx0 + (int)(r - yq * (uint32_t)O->nx);
}

__device__ __forceinline__ void brick_bases(const FoldArgs& a, const OpDev* O, int bx, int by, int bz, Iv* bo) {
  const float2* bt = a.bases + O->base_off;
  float2 b0 = __ldg(bt + (bx - O->bx0)), b1 = __ldg(bt + O->nx + (by - O->by0)),
         b2 = __ldg(bt + O->nx + O->ny + (bz - O->bz0));
  bo[0] = {b0.x, b0.y};
  bo[1] = {b1.x, b1.y};
  bo[2] = {b2.x, b2.y};
}

// The point through a rotation of the shape's frame (shapes.ts:263-320 on
// intervals, in the centre-radius form of lin2): p holds the pivot's two
// coordinates, cos and sin.
__device__ __forceinline__ void rot32(uint32_t op, const Iv* __restrict__ p, Iv& x, Iv& y, Iv& z) {
  const Iv p0 = ldp(p, 0), p1 = ldp(p, 1), c = ldp(p, 2), sn = ldp(p, 3), nsn = ineg(sn);
  if (op == OP_ROT_Y) {
    const Iv dx = isub(x, p0), dz = isub(z, p1);
    x = lin2(p0, c, dx, sn, dz);
    z = lin2(p1, nsn, dx, c, dz);
  } else if (op == OP_ROT_X) {
    const Iv dy = isub(y, p0), dz = isub(z, p1);
    y = lin2(p0, c, dy, sn, dz);
    z = lin2(p1, nsn, dy, c, dz);
  } else {
    const Iv dx = isub(x, p0), dy = isub(y, p1);
    x = lin2(p0, c, dx, sn, dy);
    y = lin2(p1, nsn, dx, c, dy);
  }
}

// Apply a lean program's stage (LP_* kinds): one rotation, or (AFF) a composed run.
template <bool AFF>
__device__ __forceinline__ void stage32(uint32_t kind, const Iv* __restrict__ p, Iv& x, Iv& y, Iv& z) {
  if (AFF && kind == LP_AFFINE) aff32(p, x, y, z);
  else if (kind) rot32(OP_ROT_X - 1 + kind, p, x, y, z);
}

// A lean program (LP_* forms) at one point in float32 intervals, without the
// interpreter's value stack and rotation frames; amb: a polygon crossing test
// the intervals could not settle.  One copy of the primitive and stage code
// serves both primitives of forms 2 and 3.
__device__ __forceinline__ Iv lean_point(const FoldArgs& a, const OpDev* V, Iv x, Iv y, Iv z, float M, bool& amb) {
  const Iv* __restrict__ P = reinterpret_cast<const Iv*>(a.p32);
  const uint32_t l0 = *reinterpret_cast<const uint32_t*>(V->lp), l1 = *reinterpret_cast<const uint32_t*>(V->lp + 4);
  const uint32_t form = l0 & 0xffu, comb = (l0 >> 8) & 0xffu, ioff = l1 >> 24, kinds = (l1 >> 16) & 0xffu;
  const uint32_t* c32 = a.code32 + V->code_off;
  const uint2* cw = a.code + V->code_off;
  Iv v = {0.f, 0.f}, xs = x, ys = y, zs = z;
#pragma unroll 1
  for (uint32_t k = 0; k < (form > 1 ? 2u : 1u); k++) {
    const uint32_t ip = k ? l0 >> 24 : (l0 >> 16) & 0xffu;
    if (k == 0 || form == 3) {  // the stage: instruction 0, or the second primitive's own
      xs = x; ys = y; zs = z;
      const uint32_t ks = k ? kinds >> 4 : kinds & 15u, is = k ? (l1 >> 8) & 0xffu : 0u;
      if (ks) stage32<true>(ks, P + (__ldg(c32 + is) & C32_OFF), xs, ys, zs);
    }
    const uint32_t w = __ldg(&cw[ip].x);
    const Iv u = prim32(w & 0xffu, (int)(w >> 8), P + (__ldg(c32 + ip) & C32_OFF), xs, ys, zs, M, amb);
    v = k == 0 ? u : comb == LP_NEGMAX ? imax(v, ineg(u)) : comb == LP_MAX ? imax(v, u) : imin(v, u);
  }
  if (ioff != LP_NONE) v = iadd(v, ldp(P + (__ldg(c32 + ioff) & C32_OFF), 0));  // offset (penthouse.ts:250)
  return v;
}

// The rest of the brick pass for one pair per lane (`valid`), its class cls
// known: the pair's class byte, the apply pass's brick bit, the paint items of
// a full pair of a painted op, the sub-block work item of a partial pair.
// Warp-collective.
template <int MODE>
__device__ __forceinline__ void classify_finish(const FoldArgs& a, bool valid, uint32_t o, const OpDev* O,
                                                unsigned long long p, int bx, int by, int bz, int cls, int lane,
                                                uint32_t& st_local) {
  bool first = false;  // the first pair to mark its brick: it lists the brick for the apply pass
  if (valid) {
    a.pcode[p] = (uint8_t)cls;
    if (cls != PC_SKIP) {  // the apply pass visits this brick
      const size_t ci = (size_t)bx + (size_t)a.BX * ((size_t)by + (size_t)a.BY * (size_t)bz);
      first = !(atomicOr(a.bmark + (ci >> 5), 1u << (ci & 31)) & (1u << (ci & 31)));
    }
  }
  // the apply pass's brick list, packed coordinates bx | by << 10 | bz << 20: bricks
  // of tiles with more than 8 ops from the front, the others from the back
  const bool heavy = first && __ldg(a.tile_cnt + (bx >> 2) + a.TX * ((by >> 2) + a.TY * (bz >> 2))) > 8u;
#pragma unroll
  for (int e = 0; e < 2; e++) {
    const uint32_t wm = __ballot_sync(FULLMASK, first && heavy == (e == 0));
    if (!wm) continue;
    uint32_t base = 0;
    if (lane == 0) {
      base = atomicAdd(a.work_counter + 1 + e, (uint32_t)__popc(wm));
      atomicAdd(&a.res->n_work, (uint32_t)__popc(wm));
    }
    base = __shfl_sync(FULLMASK, base, 0) + __popc(wm & ((1u << lane) - 1u));
    if (first && heavy == (e == 0))
      a.work[e ? (uint32_t)a.touched_cap - base : base] = (uint32_t)bx | ((uint32_t)by << 10) | ((uint32_t)bz << 20);
  }
  // a full pair of a painted op: its 8 sub-blocks go to the paint pass
  const bool fullp = valid && cls == PC_FULL && O->paint_slot != NO_SLOT;
  if (__any_sync(FULLMASK, fullp)) {
    const bool back = MODE == 1 && O->paint32_off != NO_SLOT;
#pragma unroll
    for (int e = 0; e < 2; e++) {  // front: 16 half sub-blocks per pair; back: the pair (bit 30)
      const uint32_t fm = __ballot_sync(FULLMASK, fullp && back == (e == 1));
      if (!fm) continue;
      const uint32_t per = e ? 1u : 16u;
      uint32_t pb = 0;
      if (lane == 0) pb = atomicAdd(a.paint_item_counter + e, per * __popc(fm));
      pb = __shfl_sync(FULLMASK, pb, 0);
      if (fullp && back == (e == 1)) {
        const uint32_t at = pb + per * __popc(fm & ((1u << lane) - 1u));
        for (uint32_t q = 0; q < per; q++)
          if (at + q < a.paint_items_cap) {
            if (e) a.paint_items[a.paint_items_cap - 1 - (at + q)] = make_uint2(o | (1u << 30), (uint32_t)(p << 3));
            else a.paint_items[at + q] = make_uint2(o | ((q & 1u) << 31), (uint32_t)(p << 3) | (q >> 1));
          }
      }
    }
  }
  // partial pairs go to the sub-block pass, one queue region per shape class
  const bool part = valid && cls == PC_PARTIAL;
  const uint32_t pm = __ballot_sync(FULLMASK, part);
  if (part) {
    const uint32_t k = O->vclass & (VCLASSES - 1);
    const uint32_t grp = __match_any_sync(pm, k);
    const int leader = __ffs(grp) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(&a.pitem_counter[1 + k], (uint32_t)__popc(grp));
    base = __shfl_sync(grp, base, leader);
    const uint32_t slot = base + __popc(grp & ((1u << lane) - 1u));
    if (slot < a.pq_cap[k]) a.pitems[a.pq_base[k] + slot] = make_uint2(o, (uint32_t)p);
    else st_local |= ST_STAGE_OVERFLOW;
  }
}

// Classification of every (op, brick) pair — apply()'s SDF tests, which do not
// depend on the world's state (shapes.ts:358-366, 382-394):
//   bricks: one pair per lane (32 consecutive pairs, mostly one op);
//   sub-blocks: 4 partial pairs x 8 sub-blocks per pass;
// partial sub-blocks go to a queue that voxel_kernel drains one at a time
// (64 voxels on 32 lanes), which keeps the heavy voxel work evenly spread.
template <int MODE>
__global__ void __launch_bounds__(256, MODE == 1 ? PX_CLASSIFY_MINB : PX_CLASSIFY64_MINB) classify_kernel(FoldArgs a) {
  pdl_prologue();
  const int lane = threadIdx.x & 31;
  LaneStats ls = {a.res};
  uint32_t n_brick = 0;
  uint32_t st_local = 0;
  const unsigned long long P = a.n_pairs;
  const uint32_t n_chunks = (uint32_t)((P + 31) / 32);
  NextTicket tk;
  tk.issue(a.chunk_counter, 1u, lane);
  for (;;) {
    const uint32_t take = tk.get();
    if (take >= n_chunks) break;
    tk.issue(a.chunk_counter, 1u, lane);
    const uint2 ce = __ldg(a.chunk_order + take);
    const uint32_t chunk = ce.x;
    const unsigned long long p = (unsigned long long)chunk * 32 + lane;
    const bool valid = p < P;
    uint32_t o = ce.y & 0x7fffffffu;
    if (!(ce.y >> 31)) {  // the chunk spans several ops (at most 32 start in it; warp-uniform)
      // lane j holds the first pair of op o + 1 + j; a lane's op is o plus the number of
      // those at or below its pair (sorted: a binary search over the lanes, by shuffles)
      const unsigned long long pb =
          o + 1 + (uint32_t)lane < a.n_ops ? __ldg(&a.ops[o + 1 + lane].pair_base) : ~0ull;
      // (33 possible counts: six halvings; every lane shuffles each time, from lane <= 31)
      uint32_t lo = 0, hi = 32;
#pragma unroll
      for (int k = 0; k < 6; k++) {
        const uint32_t mid = min((lo + hi) >> 1, 31u);
        const unsigned long long v = __shfl_sync(FULLMASK, pb, (int)mid);
        if (lo < hi) {
          if (v <= p) lo = mid + 1;
          else hi = mid;
        }
      }
      o += lo;
    }
    const OpDev* O = a.ops + o;
    int bx = 0, by = 0, bz = 0, cls = PC_SKIP;
    // a pair outside its op's bricks cannot happen; if it did, it would be reported, not used
    const bool in_op = valid && p >= O->pair_base &&
                       p - O->pair_base < (unsigned long long)O->nx * O->ny * (unsigned long long)(O->bz1 - O->bz0 + 1);
    if (valid && !in_op) atomicOr(&a.res->status, (uint32_t)ST_CHAIN);
    if (in_op) {
      brick_of_pair(O, p, bx, by, bz);
      const int flags = O->flags;
      const bool contained = (flags & OPF_CONTAINS) && bx >= O->cbx0 && bx <= O->cbx1 && by >= O->cby0 &&
                             by <= O->cby1 && bz >= O->cbz0 && bz <= O->cbz1;
      if (contained) {
        cls = PC_FULL;
      } else {
        const bool use32 = MODE == 1 && !(flags & OPF_FP64_ONLY);
        Iv bo[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
        if (use32) brick_bases(a, O, bx, by, bz, bo);
        cls = 3;
        if (MODE == 1 && use32 && O->lp[LP_FORM] && !a.validate) {  // a lean program: no interpreter
          bool amb = false;
          const Iv k = koff(3.5f, a.vs_lo, a.vs_hi);
          const Iv d = lean_point(a, O, iadd(bo[0], k), iadd(bo[1], k), iadd(bo[2], k), O->thr[T_M], amb);
          if (!amb) cls = classify32(d, O->thr, T_BSK_HI);
        }
        if (cls == 3)  // the interpreter, with the float64 rescue
          cls = eval_decide<MODE>(a, O, a.code + O->code_off, (int)O->code_len, use32, bo, 3.5f, 3.5f, 3.5f,
                                  (float)(bx * 8 + 4), (float)(by * 8 + 4), (float)(bz * 8 + 4), 1, ls);
        n_brick++;
      }
    }
    classify_finish<MODE>(a, valid, o, O, p, bx, by, bz, cls, lane, st_local);
  }
  uint32_t nb = n_brick, stw = st_local;
#pragma unroll
  for (int o2 = 16; o2; o2 >>= 1) {
    nb += __shfl_xor_sync(FULLMASK, nb, o2);
    stw |= __shfl_xor_sync(FULLMASK, stw, o2);
  }
  if (lane == 0) {
    if (nb) atomicAdd(&a.res->c.brick_evals, (unsigned long long)nb);
    if (stw) atomicOr(&a.res->status, stw);
  }
}

// The rest of the sub-block pass for one sub-block per lane (`have`), its class
// scls known: the voxel mask of a lone box's partial sub-block (per-axis runs),
// the paint items of a covered sub-block of a painted op, the Lipschitz decision
// of a partial sub-block (mixed form) and its voxel work item.  Warp-collective.
template <int MODE>
__device__ __forceinline__ void sub_finish(const FoldArgs& a, bool have, uint32_t oo, unsigned long long pp, int pbx,
                                           int pby, int pbz, int s, int scls, Iv dc, bool boxr, int lane,
                                           uint32_t& st_local) {
  if (boxr && scls == PC_PARTIAL)
    a.pmask[pp * 8 + s] = box_mask(a.ops + oo, pbx * 8 + (s & 1) * 4, pby * 8 + ((s >> 1) & 1) * 4,
                                   pbz * 8 + ((s >> 2) & 1) * 4);
  const bool paint = have && scls != PC_SKIP && a.ops[oo].paint_slot != NO_SLOT;
  if (__any_sync(FULLMASK, paint)) {  // the covered sub-blocks of a painted op go to the paint pass
    const bool back = MODE == 1 && a.ops[oo].paint32_off != NO_SLOT;
#pragma unroll
    for (int e = 0; e < 2; e++) {  // front: two half sub-blocks; back: the sub-block
      const uint32_t qm = __ballot_sync(FULLMASK, paint && back == (e == 1));
      if (!qm) continue;
      const uint32_t per = e ? 1u : 2u;
      uint32_t pb = 0;
      if (lane == 0) pb = atomicAdd(a.paint_item_counter + e, per * __popc(qm));
      pb = __shfl_sync(FULLMASK, pb, 0);
      const uint32_t at = pb + per * __popc(qm & ((1u << lane) - 1u));
      if (paint && back == (e == 1)) {
        if (e) {
          if (at < a.paint_items_cap) a.paint_items[a.paint_items_cap - 1 - at] = make_uint2(oo, (uint32_t)(pp << 3) | (uint32_t)s);
        } else {
          for (uint32_t h = 0; h < 2; h++)
            if (at + h < a.paint_items_cap) a.paint_items[at + h] = make_uint2(oo | (h << 31), (uint32_t)(pp << 3) | (uint32_t)s);
        }
      }
    }
  }
  // mixed form: a partial sub-block whose centre value is farther from 0 than
  // every voxel's distance bound (Lipschitz) has all its voxels decided
  bool lipd = false;
  if (MODE == 1 && have && scls == PC_PARTIAL && !boxr && !a.validate) {
    const float l3 = a.ops[oo].lip[3];
    if (dc.lo > l3 || dc.hi < -l3) {
      a.pmask[pp * 8 + s] = dc.lo > l3 ? 0ull : ~0ull;
      lipd = true;
    }
  }
  const bool push = have && scls == PC_PARTIAL && !boxr && !lipd;
  const uint32_t vm = __ballot_sync(FULLMASK, push);
  if (push) {  // one append per shape class present among the pushing lanes
    const uint32_t k = a.ops[oo].vq_class;
    const uint32_t grp = __match_any_sync(vm, k);
    const int leader = __ffs(grp) - 1;
    uint32_t vb = 0;
    if (lane == leader) vb = atomicAdd(&a.vitem_counter[1 + k], (uint32_t)__popc(grp));
    vb = __shfl_sync(grp, vb, leader);
    const uint32_t slot = vb + __popc(grp & ((1u << lane) - 1u));
    if (slot < a.vq_cap[k])
      a.vitems[a.vq_base[k] + slot] =
          make_uint4(oo, (uint32_t)(pp << 3) | (uint32_t)s, __float_as_uint(dc.lo), __float_as_uint(dc.hi));
    else st_local |= ST_STAGE_OVERFLOW;
  }
}

// Sub-block classes of the partial pairs (shapes.ts:382-389): four pairs per
// warp pass (8 lanes each, one sub-block per lane), pairs taken in shape-class
// order like the voxel work.  Writes the pair's 2-bit sub-block classes, the
// voxel masks of lone boxes (per-axis runs), and queues the partial sub-blocks.
template <int MODE>
__global__ void __launch_bounds__(256, MODE == 1 ? PX_SUB_MINB : PX_CLASSIFY64_MINB) sub_kernel(FoldArgs a) {
  pdl_prologue();
  const int lane = threadIdx.x & 31;
  LaneStats ls = {a.res};
  uint32_t st_local = 0;
  // the classes' item counts in the order they are taken, as an inclusive prefix over lanes
  const int my_cls = lane < VCLASSES ? a.class_order[lane] : 0;
  uint32_t incl = lane < VCLASSES ? min(__ldg(&a.pitem_counter[1 + my_cls]), a.pq_cap[my_cls]) : 0u;
  const uint32_t own = incl;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(FULLMASK, incl, o);
    if (lane >= o) incl += t;
  }
  const uint32_t n_items = __shfl_sync(FULLMASK, incl, 31);
  const int g = lane >> 3, s = lane & 7;
  NextTicket tk;
  tk.issue(&a.pitem_counter[0], 4u, lane);
  for (;;) {
    const uint32_t base = tk.get();
    if (base >= n_items) break;
    tk.issue(&a.pitem_counter[0], 4u, lane);
    // the class and queue position of each of the pass's four items
    uint32_t my_k = 0, my_first = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int kq = __popc(__ballot_sync(FULLMASK, lane < VCLASSES && incl <= base + q));
      const uint32_t fq = __shfl_sync(FULLMASK, incl - own, kq & 31);
      if (g == q) { my_k = (uint32_t)kq; my_first = fq; }
    }
    const uint32_t it = base + (uint32_t)g;
    const bool have = it < n_items;
    uint32_t oo = 0;
    unsigned long long pp = 0;
    int pbx = 0, pby = 0, pbz = 0, scls = PC_SKIP;
    bool boxr = false;
    Iv dc = {-INFINITY, INFINITY};  // enclosure of the sub-block centre's value (mixed form)
    if (have) {
      const uint2 item = __ldg(a.pitems + a.pq_base[a.class_order[my_k]] + (it - my_first));
      oo = item.x;
      pp = item.y;
      const OpDev* Q = a.ops + oo;
      brick_of_pair(Q, pp, pbx, pby, pbz);
      boxr = (Q->flags & OPF_BOX_RANGES) && !a.validate;
      const bool use32 = MODE == 1 && !(Q->flags & OPF_FP64_ONLY);
      Iv bo[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      if (use32) brick_bases(a, Q, pbx, pby, pbz, bo);
      const int sxb = s & 1, syb = (s >> 1) & 1, szb = (s >> 2) & 1;
      scls = 3;
      if (MODE == 1 && use32 && Q->lp[LP_FORM] && !a.validate) {  // a lean program: no interpreter
        bool amb = false;
        dc = lean_point(a, Q, iadd(bo[0], koff(4.f * sxb + 1.5f, a.vs_lo, a.vs_hi)),
                        iadd(bo[1], koff(4.f * syb + 1.5f, a.vs_lo, a.vs_hi)),
                        iadd(bo[2], koff(4.f * szb + 1.5f, a.vs_lo, a.vs_hi)), Q->thr[T_M], amb);
        if (!amb) scls = classify32(dc, Q->thr, T_SSK_HI);
      }
      if (scls == 3)  // the interpreter, with the float64 rescue
        scls = eval_decide<MODE>(a, Q, a.code + Q->code_off, (int)Q->code_len, use32, bo, 4.f * sxb + 1.5f,
                                 4.f * syb + 1.5f, 4.f * szb + 1.5f, (float)(pbx * 8 + sxb * 4 + 2),
                                 (float)(pby * 8 + syb * 4 + 2), (float)(pbz * 8 + szb * 4 + 2), 2, ls, true,
                                 MODE == 1 && use32 ? &dc : nullptr);
    }
    uint32_t code16 = (uint32_t)scls << (2 * s);
    code16 |= __shfl_xor_sync(FULLMASK, code16, 1);
    code16 |= __shfl_xor_sync(FULLMASK, code16, 2);
    code16 |= __shfl_xor_sync(FULLMASK, code16, 4);
    if (s == 0 && have) a.psub[pp] = (uint16_t)code16;
    sub_finish<MODE>(a, have, oo, pp, pbx, pby, pbz, s, scls, dc, boxr, lane, st_local);
  }
  uint32_t stw = st_local;
#pragma unroll
  for (int o2 = 16; o2; o2 >>= 1) stw |= __shfl_xor_sync(FULLMASK, stw, o2);
  if (lane == 0 && stw) atomicOr(&a.res->status, stw);
}

// Mixed form: a voxel's decision from its sub-block centre's value dc, when the
// SDF's Lipschitz bound settles it (0 outside, 1 inside, 3 undecided); (ox, oy,
// oz) is the voxel's offset in the sub-block, 0..3 per axis.
__device__ __forceinline__ int lip_decide(const OpDev* O, Iv dc, int ox, int oy, int oz) {
  const int k = (ox == 0 || ox == 3) + (oy == 0 || oy == 3) + (oz == 0 || oz == 3);  // axes at 1.5 voxels
  const float t = O->lip[k];
  return dc.lo > t ? 0 : (dc.hi < -t ? 1 : 3);
}

// Voxel inside-masks of the queued partial sub-blocks: one sub-block per warp
// pass, 64 voxel SDFs on 32 lanes, two ballots (shapes.ts:390-394), any
// program (the bytecode interpreters); a voxel its float32 interval cannot
// decide is evaluated in float64 in line.  Groups G0 .. G1 of the voxel queue, one
// after the other (the mixed form sends the lean programs' groups to
// voxel_lean_kernel and this kernel the rest; the float64 form every group here).
template <int MODE, int G0, int G1>
__global__ void __launch_bounds__(256, MODE == 1 ? PX_VOXEL_MINB : PX_CLASSIFY64_MINB) voxel_kernel(FoldArgs a) {
  pdl_prologue();
  const int lane = threadIdx.x & 31;
  LaneStats ls = {a.res};
#pragma unroll 1
  for (int g = G0; g <= G1; g++) {
  uint32_t* const taken = &a.vitem_counter[VQ_TAKEN + g];
  // the group's classes' item counts in the order they are taken, as an inclusive prefix over lanes
  const int my_cls = a.vclass_order[32 * g + lane];
  uint32_t incl = min(__ldg(&a.vitem_counter[1 + my_cls]), a.vq_cap[my_cls]);
  const uint32_t own = incl;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(FULLMASK, incl, o);
    if (lane >= o) incl += t;
  }
  const uint32_t n_items = __shfl_sync(FULLMASK, incl, 31);
  NextTicket tk;
  tk.issue(taken, 1, lane);
  for (;;) {
    const uint32_t it = tk.get();
    if (it >= n_items) break;
    tk.issue(taken, 1, lane);
    const int k = __popc(__ballot_sync(FULLMASK, incl <= it));  // class of item `it`
    const uint32_t first = __shfl_sync(FULLMASK, incl - own, k);
    const uint4 item = __ldg(a.vitems + a.vq_base[a.vclass_order[32 * g + k]] + (it - first));
    const Iv dcen = {__uint_as_float(item.z), __uint_as_float(item.w)};  // the sub-block centre's value
    const OpDev* V = a.ops + item.x;
    const unsigned long long vp = item.y >> 3;
    const int ss = item.y & 7;
    int vbx, vby, vbz;
    brick_of_pair(V, vp, vbx, vby, vbz);
    const bool use32 = MODE == 1 && !(V->flags & OPF_FP64_ONLY);
    Iv bo[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    if (use32) brick_bases(a, V, vbx, vby, vbz, bo);
    const int sxo = (ss & 1) * 4, syo = ((ss >> 1) & 1) * 4, szo = ((ss >> 2) & 1) * 4;
    const uint2* code = a.code + V->code_off;
    const int clen = (int)V->code_len;
    unsigned long long m;
    if (MODE == 1 && use32 && (V->flags & OPF_Y_SEPARABLE)) {
      // lane = column (x, z) of the sub-block and a pair of y rows: one pass, the x/z work once
      const int col = lane & 15, yh = lane >> 4;
      const int lx = sxo + (col & 3), lz = szo + (col >> 2), ly0 = syo + 2 * yh;
      bool amb = false;
      const Iv X = iadd(bo[0], koff((float)lx, a.vs_lo, a.vs_hi)), Z = iadd(bo[2], koff((float)lz, a.vs_lo, a.vs_hi));
      const Iv Y0 = iadd(bo[1], koff((float)ly0, a.vs_lo, a.vs_hi)), Y1 = iadd(bo[1], koff((float)(ly0 + 1), a.vs_lo, a.vs_hi));
      const int lip0 = lip_decide(V, dcen, col & 3, 2 * yh, col >> 2), lip1 = lip_decide(V, dcen, col & 3, 2 * yh + 1, col >> 2);
      Iv2 d = {{0.f, 0.f}, {0.f, 0.f}};
      if (lip0 == 3 || lip1 == 3 || a.validate)
        d = sdf32i_y2(code, a.code32 + V->code_off, clen, reinterpret_cast<const Iv*>(a.p32), X, Y0, Y1, Z, V->thr[T_M], amb);
      uint32_t lo = 0, hi = 0;
#pragma unroll
      for (int k = 0; k < 2; k++) {
        const Iv dk = k ? d.b : d.a;
        const int lipk = k ? lip1 : lip0;
        int inside = lipk;
        if (lipk == 3 || a.validate) {
          inside = amb ? 3 : (dk.lo > V->thr[T_V_HI] ? 0 : (dk.hi <= V->thr[T_V_LO] ? 1 : 3));
          if (inside == 3 || a.validate) {
            const VoxelF64 f = voxel_f64(a.params, a.vs, a.validate, code, clen, dk, amb, inside,
                                         (float)(vbx * 8 + lx) + 0.5f, (float)(vby * 8 + ly0 + k) + 0.5f,
                                         (float)(vbz * 8 + lz) + 0.5f);
            if (f.viol) ls.viol();
            if (inside == 3) ls.rescue(0, amb, f.err);
            inside = f.inside;
          }
          if (lipk != 3 && inside != lipk) ls.viol();  // validation: the bound disagreed with the evaluation
        }
        const int bit = (col & 3) | ((2 * yh + k) << 2) | ((col >> 2) << 4);  // voxel index in the sub-block
        if (inside == 1) {
          if (bit < 32) lo |= 1u << bit;
          else hi |= 1u << (bit - 32);
        }
      }
      m = (unsigned long long)__reduce_or_sync(FULLMASK, lo) | ((unsigned long long)__reduce_or_sync(FULLMASK, hi) << 32);
    } else {
      uint32_t bal[2];
#pragma unroll
      for (int r = 0; r < 2; r++) {
        const int e = r * 32 + lane;
        const int lx = sxo + (e & 3), lyv = syo + ((e >> 2) & 3), lz = szo + (e >> 4);
        const int lipd = MODE == 1 && use32 ? lip_decide(V, dcen, e & 3, (e >> 2) & 3, e >> 4) : 3;
        int inside = lipd;
        if (lipd == 3 || a.validate) {
          inside = eval_decide<MODE>(a, V, code, clen, use32, bo, (float)lx, (float)lyv, (float)lz,
                                     (float)(vbx * 8 + lx) + 0.5f, (float)(vby * 8 + lyv) + 0.5f,
                                     (float)(vbz * 8 + lz) + 0.5f, 0, ls);
          if (lipd != 3 && inside != lipd) ls.viol();  // validation: the bound disagreed with the evaluation
        }
        bal[r] = __ballot_sync(FULLMASK, inside == 1);
      }
      m = (unsigned long long)bal[0] | ((unsigned long long)bal[1] << 32);
    }
    // a lone box's sub-block is queued only in validation mode: check its runs
    if ((V->flags & OPF_BOX_RANGES) && lane == 0 && box_mask(V, vbx * 8 + sxo, vby * 8 + syo, vbz * 8 + szo) != m)
      ls.viol();
    if (lane == 0) a.pmask[vp * 8 + ss] = m;
  }
  }
}

// Voxel inside-masks of the queued partial sub-blocks of the lean programs --
// one or two primitives under a rotation, a composed run of rotations or none
// (LP_* forms): 88% of the penthouse's non-box voxel work, all of the
// rotated synthetic scenes' -- in the mixed form: the same decisions as
// voxel_kernel (shapes.ts:390-394), without the interpreters' value stack and
// rotation frames.  Lane = voxel column (x, z) of the sub-block and a pair of
// y rows; unrotated primitives extruded along y (or rotated about y) share
// their x/z work between the two voxels.
// VALIDATE (validation mode) evaluates every voxel in float64 too, in line.
// Otherwise a voxel the interval cannot decide goes to the rescue list, which
// voxel_kernel<1, ...> resolves in float64 first, and counts as outside until
// then (no call in this kernel: every value live across one would be saved to
// local memory).
// G: the group of the voxel queue (VQ_NARROW, VQ_AFFINE or VQ_WIDE), each
// compiled with only its forms' live values.
template <bool VALIDATE, int G>
__global__ void __launch_bounds__(256, G == VQ_WIDE ? PX_VWIDE_MINB : G == VQ_AFFINE ? PX_VAFF_MINB : PX_VSIMPLE_MINB)
    voxel_lean_kernel(FoldArgs a) {
  constexpr bool WIDE = G == VQ_WIDE, AFF = G != VQ_NARROW;
  pdl_prologue();
  const int lane = threadIdx.x & 31;
  LaneStats ls = {a.res};
  uint32_t* const taken = &a.vitem_counter[VQ_TAKEN + G];
  const int my_cls = a.vclass_order[32 * G + lane];
  uint32_t incl = min(__ldg(&a.vitem_counter[1 + my_cls]), a.vq_cap[my_cls]);
  const uint32_t own = incl;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(FULLMASK, incl, o);
    if (lane >= o) incl += t;
  }
  const uint32_t n_items = __shfl_sync(FULLMASK, incl, 31);
  const int col = lane & 15, yh = lane >> 4;
  const Iv* __restrict__ P = reinterpret_cast<const Iv*>(a.p32);
  NextTicket tk;
  tk.issue(taken, 1, lane);
  for (;;) {
    const uint32_t it = tk.get();
    if (it >= n_items) break;
    tk.issue(taken, 1, lane);
    const int k = __popc(__ballot_sync(FULLMASK, incl <= it));  // class of item `it`
    const uint32_t first = __shfl_sync(FULLMASK, incl - own, k);
    const uint4 item = __ldg(a.vitems + a.vq_base[a.vclass_order[32 * G + k]] + (it - first));
    const Iv dcen = {__uint_as_float(item.z), __uint_as_float(item.w)};  // the sub-block centre's value
    const OpDev* V = a.ops + item.x;
    const unsigned long long vp = item.y >> 3;
    const int ss = item.y & 7;
    int vbx, vby, vbz;
    brick_of_pair(V, vp, vbx, vby, vbz);
    Iv bo[3];
    brick_bases(a, V, vbx, vby, vbz, bo);
    const int sxo = (ss & 1) * 4, syo = ((ss >> 1) & 1) * 4, szo = ((ss >> 2) & 1) * 4;
    const int lx = sxo + (col & 3), lz = szo + (col >> 2), ly0 = syo + 2 * yh;
    const int lip0 = lip_decide(V, dcen, col & 3, 2 * yh, col >> 2), lip1 = lip_decide(V, dcen, col & 3, 2 * yh + 1, col >> 2);
    const float M = V->thr[T_M];
    bool amb0 = false, amb1 = false;  // a polygon crossing test the interval could not settle, per voxel
    Iv2 d = {{0.f, 0.f}, {0.f, 0.f}};
    if (lip0 == 3 || lip1 == 3 || VALIDATE) {
      const uint2 lpw = make_uint2(*reinterpret_cast<const uint32_t*>(V->lp), *reinterpret_cast<const uint32_t*>(V->lp + 4));
      const uint32_t form = WIDE ? lpw.x & 0xffu : 1u, comb = (lpw.x >> 8) & 0xffu, ip1 = (lpw.x >> 16) & 0xffu,
                     ip2 = lpw.x >> 24, is2 = (lpw.y >> 8) & 0xffu, kinds = (lpw.y >> 16) & 0xffu,
                     ioff = lpw.y >> 24;
      const uint32_t k1 = kinds & 15u, k2 = WIDE ? kinds >> 4 : 0u;
      const uint32_t* c32 = a.code32 + V->code_off;
      const uint2* cw = a.code + V->code_off;
      const uint32_t w1 = __ldg(&cw[ip1].x), w2 = form > 1 ? __ldg(&cw[ip2].x) : 0u;
      const uint32_t p1 = w1 & 0xffu, p2 = w2 & 0xffu;
      const Iv* pr1 = P + (__ldg(c32 + ip1) & C32_OFF);
      const Iv* pr2 = P + (__ldg(c32 + (form > 1 ? ip2 : ip1)) & C32_OFF);
      const Iv* ps1 = P + (__ldg(c32) & C32_OFF);  // the first stage is instruction 0
      const Iv* ps2 = P + (__ldg(c32 + (k2 ? is2 : 0u)) & C32_OFF);
      const Iv x = iadd(bo[0], koff((float)lx, a.vs_lo, a.vs_hi)), z = iadd(bo[2], koff((float)lz, a.vs_lo, a.vs_hi));
      const Iv y0 = iadd(bo[1], koff((float)ly0, a.vs_lo, a.vs_hi)), y1 = iadd(bo[1], koff((float)(ly0 + 1), a.vs_lo, a.vs_hi));
      auto combine = [&](Iv u, Iv v) -> Iv {
        return comb == LP_NEGMAX ? imax(u, ineg(v)) : comb == LP_MAX ? imax(u, v) : imin(u, v);
      };
      // y-extruded primitives, unrotated or rotated about y: x and z are shared by both voxels
      const bool ysep = (k1 == 0 || k1 == 2) && (k2 == 0 || k2 == 2) && op_is_y_separable(p1) &&
                        (form == 1 || op_is_y_separable(p2));
      if (ysep) {
        bool amb = false;  // the column's polygon work is shared by both voxels
        Iv x1 = x, z1 = z, yd = y0;
        if (k1) rot32(OP_ROT_Y, ps1, x1, yd, z1);
        d = prim32_y2(p1, (int)(w1 >> 8), pr1, x1, y0, y1, z1, M, amb);
        if (form > 1) {
          Iv x2 = x1, z2 = z1;
          if (form == 3) {
            x2 = x; z2 = z;
            if (k2) rot32(OP_ROT_Y, ps2, x2, yd, z2);
          }
          const Iv2 e = prim32_y2(p2, (int)(w2 >> 8), pr2, x2, y0, y1, z2, M, amb);
          d = {combine(d.a, e.a), combine(d.b, e.b)};
        }
        amb0 = amb1 = amb;
      } else {
#pragma unroll 1
        for (int q = 0; q < 2; q++) {
          bool ambq = false;  // each voxel's own crossing tests
          Iv x1 = x, y1q = q ? y1 : y0, z1 = z;
          stage32<AFF>(k1, ps1, x1, y1q, z1);
          Iv v = prim32(p1, (int)(w1 >> 8), pr1, x1, y1q, z1, M, ambq);
          if (form == 2) {
            v = combine(v, prim32(p2, (int)(w2 >> 8), pr2, x1, y1q, z1, M, ambq));
          } else if (form == 3) {
            Iv x2 = x, y2q = q ? y1 : y0, z2 = z;
            stage32<AFF>(k2, ps2, x2, y2q, z2);
            v = combine(v, prim32(p2, (int)(w2 >> 8), pr2, x2, y2q, z2, M, ambq));
          }
          if (q) { d.b = v; amb1 = ambq; } else { d.a = v; amb0 = ambq; }
        }
      }
      if (ioff != LP_NONE) {  // offset (penthouse.ts:250)
        const Iv o = ldp(P + (__ldg(c32 + ioff) & C32_OFF), 0);
        d = {iadd(d.a, o), iadd(d.b, o)};
      }
    }
    const uint2* code = a.code + V->code_off;
    const int clen = (int)V->code_len;
    uint32_t lo = 0, hi = 0, resc = 0;  // resc: bit q, voxel q of this lane left to float64
#pragma unroll
    for (int q = 0; q < 2; q++) {
      const Iv dk = q ? d.b : d.a;
      const bool amb = q ? amb1 : amb0;
      const int lipk = q ? lip1 : lip0;
      int inside = lipk;
      if (lipk == 3 || VALIDATE) {
        inside = amb ? 3 : (dk.lo > V->thr[T_V_HI] ? 0 : (dk.hi <= V->thr[T_V_LO] ? 1 : 3));
        if constexpr (VALIDATE) {
          const VoxelF64 f = voxel_f64(a.params, a.vs, 1, code, clen, dk, amb, inside,
                                       (float)(vbx * 8 + lx) + 0.5f, (float)(vby * 8 + ly0 + q) + 0.5f,
                                       (float)(vbz * 8 + lz) + 0.5f);
          if (f.viol) ls.viol();
          if (inside == 3) ls.rescue(0, amb, f.err);
          inside = f.inside;
          if (lipk != 3 && inside != lipk) ls.viol();  // the bound disagreed with the evaluation
        } else if (inside == 3) {  // resolved in float64 after the work loop; outside until then
          resc |= 1u << q;
          inside = 0;
        }
      }
      const int bit = (col & 3) | ((2 * yh + q) << 2) | ((col >> 2) << 4);  // voxel index in the sub-block
      if (inside == 1) {
        if (bit < 32) lo |= 1u << bit;
        else hi |= 1u << (bit - 32);
      }
    }
    const unsigned long long m =
        (unsigned long long)__reduce_or_sync(FULLMASK, lo) | ((unsigned long long)__reduce_or_sync(FULLMASK, hi) << 32);
    // a lone box's sub-block is queued only in validation mode: check its runs
    if (VALIDATE && (V->flags & OPF_BOX_RANGES) && lane == 0 &&
        box_mask(V, vbx * 8 + sxo, vby * 8 + syo, vbz * 8 + szo) != m)
      ls.viol();
    if (lane == 0) a.pmask[vp * 8 + ss] = m;
    if (!VALIDATE) {  // undecided voxels to the rescue list, one atomic per warp
      const uint32_t nr = __popc(resc);
      const uint32_t tot = __reduce_add_sync(FULLMASK, nr);
      if (tot) {
        uint32_t at = nr;  // this lane's first entry: an exclusive prefix over the lanes
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const uint32_t t = __shfl_up_sync(FULLMASK, at, o);
          if (lane >= o) at += t;
        }
        at -= nr;
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&a.res->n_rescue, tot);
        base = __shfl_sync(FULLMASK, base, 0);
#pragma unroll
        for (int q = 0; q < 2; q++) {
          if (!((resc >> q) & 1u)) continue;
          const Iv dk = q ? d.b : d.a;
          const bool amb = q ? amb1 : amb0;
          const int bit = (col & 3) | ((2 * yh + q) << 2) | ((col >> 2) << 4);
          const uint4 e = make_uint4(item.x | ((uint32_t)bit << 24) | (amb ? 1u << 30 : 0u), item.y,
                                     __float_as_uint(dk.lo), __float_as_uint(dk.hi));
          const uint32_t r = base + at++;
          if (r < a.rescue_cap) a.rescue[r] = e;
          else atomicOr(&a.res->status, (uint32_t)ST_RESCUE_OVERFLOW);
        }
      }
    }
  }
}

// One paint call at voxel (x, y, z) of the world, in float64 (the paint kinds
// that paint_kernel does not evaluate ahead).  Out of line, so that the apply
// loop holds no float64 values.  Returns the value (a u16 for these kinds) with
// PV_RANGE for a range error and PV_VIOL for a validation mismatch.
constexpr uint32_t PV_VIOL = 0x40000000u;
__device__ __noinline__ uint32_t paint_at_voxel(const double* __restrict__ params, double vs, int validate,
                                                const OpDev* O, int x, int y, int z) {
  double PX = (x + 0.5) * vs, PY = (y + 0.5) * vs, PZ = (z + 0.5) * vs;
  if (O->flags & OPF_PAINT_FRAME) {  // localPaint (penthouse.ts:88-91)
    const double fpx = O->frame[0], fpz = O->frame[1], c = O->frame[2], sn = O->frame[3];
    const double dx = PX - fpx, dz = PZ - fpz;
    PX = fpx + c * dx + sn * dz;
    PZ = fpz - sn * dx + c * dz;
  }
  uint32_t st = 0;
  const uint32_t v = paint_eval(O->paint_kind, params + O->paint_off, PX, PY, PZ, st);
  const bool viol = validate && v != paint_eval_cr(O->paint_kind, params + O->paint_off, PX, PY, PZ, st);
  return (v & 0xffffu) | (st & ST_RANGE ? PV_RANGE : 0u) | (viol ? PV_VIOL : 0u);
}

// One paint call of op O at voxel (lx, ly, lz) of brick (bx, by, bz) as the paint
// pass stores it (value | PV_RANGE): the certified float32 evaluation first in
// the mixed form (bo: the brick's float32 bases, unused for the noise kind),
// else float64; validation mode evaluates both and counts mismatches in viol.
template <int MODE>
__device__ __forceinline__ uint32_t paint_voxel(const FoldArgs& a, const OpDev* O, int bx, int by, int bz, const Iv* bo,
                                                int lx, int ly, int lz, uint32_t& resc, uint32_t& viol) {
  const uint32_t pk = O->paint_kind;
  uint32_t v = 0, st = 0;
  bool done = false;
  if (MODE == 1 && O->paint32_off != NO_SLOT) {
    if (pk == PK_NOISE)
      done = noise32(a.p32 + O->paint32_off, __ldg(a.ax32 + bx * 8 + lx), __ldg(a.ay32 + by * 8 + ly),
                     __ldg(a.az32 + bz * 8 + lz), v);
    else
      done = paint32(pk, a.p32 + O->paint32_off, iadd(bo[0], koff((float)lx, a.vs_lo, a.vs_hi)),
                     iadd(bo[1], koff((float)ly, a.vs_lo, a.vs_hi)), iadd(bo[2], koff((float)lz, a.vs_lo, a.vs_hi)), v);
    if (!done) resc++;
  }
  if (!done || a.validate) {  // float64 (validation: also the correctly rounded decision)
    const uint32_t pr = paint_at_voxel(a.params, a.vs, a.validate, O, bx * 8 + lx, by * 8 + ly, bz * 8 + lz);
    if (pr & PV_VIOL) viol++;
    if (!done) {
      v = pr & 0xffffu;
      if (pr & PV_RANGE) st |= ST_RANGE;
    } else if (v != (pr & 0xffffu)) {
      viol++;
    }
  }
  return (v & 0xffffu) | (st & ST_RANGE ? PV_RANGE : 0u);
}

// Paint calls ahead of the apply pass: the covered sub-blocks of the painted
// ops' pairs (queued by the classify and sub-block passes), one 4^3 sub-block
// per warp pass, two voxels per lane, every voxel the op's shape covers (whether
// the reference then paints it depends on the world's state, which fold_kernel
// knows).  Values go to the pair's slot in
// voxel index order.  Spreading these calls over the whole GPU keeps one
// warp from evaluating a painted brick's 512 calls alone.  Mixed mode tries the
// certified float32 evaluation first (paint32.cuh).
// Mixed form: first the voxels the lean voxel kernels left undecided (the rescue
// list), one per thread, in float64 (shapes.ts:393): the inside ones are ORed
// into their sub-block masks, and a painted op's paint value is stored for them
// here.  Entry r goes to block r mod gridDim.x, so a warp holds few (an FP64
// instruction of a sparse warp is far quicker than a full one: FP64 runs at 1/64
// of the float32 rate) and the float64 chains overlap the paint work.  A paint
// item of the same sub-block may read its mask before or after the OR: it then
// paints the voxel too or leaves it out, and either way stores the same value.
template <int MODE>
__global__ void __launch_bounds__(256, PX_PAINT_MINB) paint_kernel(FoldArgs a) {
  pdl_prologue();
  const int lane = threadIdx.x & 31;
  uint32_t resc = 0, viol = 0;
  if (MODE == 1) {
    LaneStats ls = {a.res};
    const uint32_t n_resc = min(__ldcg(&a.res->n_rescue), a.rescue_cap);
    for (uint32_t r = blockIdx.x + gridDim.x * threadIdx.x; r < n_resc; r += gridDim.x * blockDim.x) {
      const uint4 ri = __ldcg(a.rescue + r);
      const OpDev* R = a.ops + (ri.x & 0xffffffu);
      const int bit = (int)((ri.x >> 24) & 63u);
      const bool ramb = (ri.x >> 30) & 1u;
      const unsigned long long rp = ri.y >> 3;
      const int rs = ri.y & 7;
      int rbx, rby, rbz;
      brick_of_pair(R, rp, rbx, rby, rbz);
      const int lx = (rs & 1) * 4 + (bit & 3), ly = ((rs >> 1) & 1) * 4 + ((bit >> 2) & 3), lz = ((rs >> 2) & 1) * 4 + (bit >> 4);
      const Iv dk = {__uint_as_float(ri.z), __uint_as_float(ri.w)};
      const VoxelF64 f = voxel_f64(a.params, a.vs, 0, a.code + R->code_off, (int)R->code_len, dk, ramb, 3,
                                   (float)(rbx * 8 + lx) + 0.5f, (float)(rby * 8 + ly) + 0.5f, (float)(rbz * 8 + lz) + 0.5f);
      ls.rescue(0, ramb, f.err);
      if (!f.inside) continue;
      atomicOr(a.pmask + rp * 8 + rs, 1ull << bit);
      if (R->paint_slot == NO_SLOT) continue;
      Iv bo[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
      if (R->paint32_off != NO_SLOT && R->paint_kind != PK_NOISE) brick_bases(a, R, rbx, rby, rbz, bo);
      a.pvals[(size_t)(R->paint_slot + (uint32_t)(rp - R->pair_base)) * 512 + (uint32_t)(lx | (ly << 3) | (lz << 6))] =
          paint_voxel<MODE>(a, R, rbx, rby, rbz, bo, lx, ly, lz, resc, viol);
    }
  }
  // float64 paints (the front of the queue) first, then the certified float32 ones
  const uint32_t n_front = min(__ldg(a.paint_item_counter), a.paint_items_cap);
  const uint32_t n_items = n_front + min(__ldg(a.paint_item_counter + 1), a.paint_items_cap - n_front);
  WorkBatch wb;
  for (;;) {
    const uint32_t it = wb.next(a.paint_counter, 2, lane);
    if (it >= n_items) break;
    const uint2 item = __ldg(a.paint_items + (it < n_front ? it : a.paint_items_cap - 1 - (it - n_front)));
    // a float64 item (the front) is half a sub-block: voxel rows r = bit 31 of its op field;
    // a float32 item (the back) a sub-block, or with bit 30 a whole full pair (8 sub-blocks)
    const int r0 = it < n_front ? (int)(item.x >> 31) : 0, r1 = it < n_front ? r0 + 1 : 2;
    const bool whole = it >= n_front && ((item.x >> 30) & 1u);
    const OpDev* O = a.ops + (item.x & 0xffffffu);
    const unsigned long long pair = item.y >> 3;
    const int s0 = (int)(item.y & 7u);
    const uint32_t slot = O->paint_slot + (uint32_t)(pair - O->pair_base);
    const int cls = whole ? (int)PC_FULL : (int)__ldg(a.pcode + pair);
    int bx, by, bz;
    brick_of_pair(O, pair, bx, by, bz);
    const uint32_t pk = O->paint_kind;
    const bool try32 = MODE == 1 && O->paint32_off != NO_SLOT;
    Iv bo[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
    if (try32 && pk != PK_NOISE) brick_bases(a, O, bx, by, bz, bo);
#pragma unroll 1
    for (int s = whole ? 0 : s0; s <= (whole ? 7 : s0); s++) {
      unsigned long long m = ~0ull;
      if (cls != PC_FULL) {
        const uint32_t c = (__ldg(a.psub + pair) >> (2 * s)) & 3u;
        m = c == PC_FULL ? ~0ull : c == PC_PARTIAL ? __ldcg(a.pmask + pair * 8 + s) : 0ull;
      }
#pragma unroll 1
      for (int r = r0; r < r1; r++) {
        const int e = r * 32 + lane;
        if (!((m >> e) & 1ull)) continue;
        const int lx = (s & 1) * 4 + (e & 3), ly = ((s >> 1) & 1) * 4 + ((e >> 2) & 3), lz = ((s >> 2) & 1) * 4 + (e >> 4);
        a.pvals[(size_t)slot * 512 + (uint32_t)(lx | (ly << 3) | (lz << 6))] =
            paint_voxel<MODE>(a, O, bx, by, bz, bo, lx, ly, lz, resc, viol);
      }
    }
  }
#pragma unroll
  for (int o2 = 16; o2; o2 >>= 1) {
    resc += __shfl_xor_sync(FULLMASK, resc, o2);
    viol += __shfl_xor_sync(FULLMASK, viol, o2);
  }
  if (lane == 0) {
    if (resc) atomicAdd(&a.res->c.resc_paint, (unsigned long long)resc);
    if (viol) atomicAdd(&a.res->c.violations, (unsigned long long)viol);
  }
}

// Lane layout of a brick in registers: lane owns the voxel pair
// (x0, y, z) / (x0 + 1, y, z) with x0 = 2 (lane & 3), y = lane >> 2, in
// register j = z.  Voxel index li = x | y << 3 | z << 6 (VoxelWorld.ts:60), so
// register j of the warp is the contiguous 128-byte slice pool[64 j .. 64 j + 63].
// The warp applies its brick's ops in order, as apply() does (shapes.ts:367-412),
// using the pair classifications.
// One tile-list entry of a brick, looked up for the apply loop: the op, its
// (op, brick) pair and that pair's classes, and the op fields the loop needs.
struct FoldEntry {
  unsigned long long pr;
  uint32_t oi, meta, pval, pslot, sc;
  int cls;
};

__device__ __forceinline__ FoldEntry fold_entry(const FoldArgs& a, uint32_t idx, int bx, int by, int bz) {
  FoldEntry f = {0ull, 0u, 0u, 0u, NO_SLOT, 0u, PC_SKIP};
  f.oi = __ldg(a.tile_ops + idx);
  const uint2 bb = __ldg(a.tile_boxes + idx);  // the op's brick box
  const int x0 = bb.x & 1023, y0 = (bb.x >> 10) & 1023, z0 = (bb.x >> 20) & 1023;
  const int x1 = bb.y & 1023, y1 = (bb.y >> 10) & 1023, z1 = (bb.y >> 20) & 1023;
  if (bx >= x0 && bx <= x1 && by >= y0 && by <= y1 && bz >= z0 && bz <= z1) {
    const OpDev* o = a.ops + f.oi;
    f.pr = o->pair_base + (unsigned long long)(((bz - z0) * (y1 - y0 + 1) + (by - y0)) * (x1 - x0 + 1) + (bx - x0));
    f.cls = __ldg(a.pcode + f.pr);
    f.sc = __ldg(a.psub + f.pr);  // meaningful for partial pairs only
    f.meta = (uint32_t)o->kind | ((uint32_t)o->flags << 8) | ((uint32_t)o->paint_kind << 16);
    f.pval = o->paint_value;
    f.pslot = o->paint_slot == NO_SLOT ? NO_SLOT : o->paint_slot + (uint32_t)(f.pr - o->pair_base);
  }
  return f;
}

// INLINE: some painted op has no paint slot (paint values past the slot
// budget), so paint calls happen here too; otherwise the apply loop calls nothing.
// A warp takes four bricks at a time; lanes 8j..8j+7 look up the first eight
// tile-list entries of brick j together (all four bricks' lookups in flight at
// once), then the bricks are applied one after the other.
template <bool INLINE>
__global__ void __launch_bounds__(256, PX_FOLD_MINB) fold_kernel(FoldArgs a) {
  pdl_prologue();
  __shared__ unsigned long long smask[8][8];
  __shared__ __align__(16) unsigned long long spm[8][32][8];  // voxel masks of the looked-up partial pairs
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int lx0 = (lane & 3) * 2, ly = lane >> 2;
  const uint32_t grp = (uint32_t)lane >> 3, ent = (uint32_t)lane & 7u;
  WarpCounters wc = {0, 0, 0, 0, 0};
  uint32_t paint_calls = 0, paint_viol = 0;
  uint32_t st_local = 0;
  const uint32_t n_front = __ldg(a.work_counter + 1), n_work = n_front + __ldg(a.work_counter + 2);

  for (;;) {
    uint32_t wbase = 0;
    if (lane == 0) wbase = atomicAdd(a.work_counter, 4u);
    wbase = __shfl_sync(FULLMASK, wbase, 0);
    if (wbase >= n_work) break;
    const uint32_t n_here = min(4u, n_work - wbase);
    uint32_t q_pk = 0, q_g = 0, q_toff = 0, q_tcnt = 0;
    FoldEntry q = {0ull, 0u, 0u, 0u, NO_SLOT, 0u, PC_SKIP};
    if (grp < n_here) {
      const uint32_t wi = wbase + grp;
      q_pk = __ldg(a.work + (wi < n_front ? wi : a.touched_cap - (wi - n_front)));
      const uint32_t bx = q_pk & 1023u, by = (q_pk >> 10) & 1023u, bz = q_pk >> 20;
      q_g = a.grid[bx + (uint32_t)a.BX * (by + (uint32_t)a.BY * bz)];
      const uint32_t tile = (bx >> 2) + (uint32_t)a.TX * ((by >> 2) + (uint32_t)a.TY * (bz >> 2));
      q_toff = __ldg(a.tile_off + tile);
      q_tcnt = __ldg(a.tile_cnt + tile);
      if (ent < q_tcnt) q = fold_entry(a, q_toff + ent, (int)bx, (int)by, (int)bz);
    }
    if (q.cls == PC_PARTIAL) {  // its pair's voxel masks, copied to shared memory while the bricks load
      const uint32_t dst = (uint32_t)__cvta_generic_to_shared(&spm[wib][lane][0]);
      const unsigned long long* srcp = a.pmask + q.pr * 8;
#pragma unroll
      for (int k = 0; k < 4; k++)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst + 16 * k), "l"(srcp + 2 * k) : "memory");
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    const uint32_t m_all = __ballot_sync(FULLMASK, q.cls != PC_SKIP);  // shapes.ts:364 skips the rest
    uint32_t t_ci = 0, t_tag = 0;  // lane j: brick j's touched-list entry
    bool t_dirty = false;
    asm volatile("cp.async.wait_all;\n" ::: "memory");
    __syncwarp();

    for (uint32_t j = 0; j < n_here; j++) {
      const uint32_t pk = __shfl_sync(FULLMASK, q_pk, 8 * j);
      const uint32_t g = __shfl_sync(FULLMASK, q_g, 8 * j);
      const uint32_t toff = __shfl_sync(FULLMASK, q_toff, 8 * j), tcnt = __shfl_sync(FULLMASK, q_tcnt, 8 * j);
      const int bx = (int)(pk & 1023u), by = (int)((pk >> 10) & 1023u), bz = (int)(pk >> 20);
      const uint32_t ci = (uint32_t)bx + (uint32_t)a.BX * ((uint32_t)by + (uint32_t)a.BY * (uint32_t)bz);
      const int ox = bx * 8, oy = by * 8, oz = bz * 8;

      // current brick contents (VoxelWorld.ts:55-61)
      int state = ST_EMPTY;
      uint32_t uval = 0;
      uint32_t vox[8];
      long long src = -1;  // pool identity: >= 0 pair of the last alloc, < 0 -(old index + 1)
      bool dirty = false;
      if (g == 0) {
#pragma unroll
        for (int k = 0; k < 8; k++) vox[k] = 0;
      } else if (g & UNIFORM) {
        state = ST_UNIF; uval = g & 0xffffu;
#pragma unroll
        for (int k = 0; k < 8; k++) vox[k] = uval | (uval << 16);
      } else {
        state = ST_MIXED; src = -(long long)(g - 1) - 1;
        const uint32_t* pb = a.pool32 + (size_t)(g - 1) * 256;
#pragma unroll
        for (int k = 0; k < 8; k++) vox[k] = pb[32 * k + lane];
      }

      // apply the op whose entry lane `b` holds (`pm`: its voxel masks are in spm[wib][b])
      auto apply = [&](const FoldEntry& f, int b, bool pm) {
        const unsigned long long pair = __shfl_sync(FULLMASK, f.pr, b);
        const int cls = __shfl_sync(FULLMASK, f.cls, b);
        const uint32_t mt = __shfl_sync(FULLMASK, f.meta, b);
        const uint32_t pv = __shfl_sync(FULLMASK, f.pval, b);
        const uint32_t slot = __shfl_sync(FULLMASK, f.pslot, b);
        const uint32_t o_idx = __shfl_sync(FULLMASK, f.oi, b);
        const uint32_t psc = __shfl_sync(FULLMASK, f.sc, b);
        const bool full = cls == PC_FULL;
        const int kind = (int)(mt & 0xffu);
        const uint32_t pk_ = mt >> 16;
        const bool constPaint = pk_ == PK_CONST;
        // uniform shortcuts (shapes.ts:367-374)
        int set_u = -1;
        if (full) {
          if (kind == KIND_ADD && constPaint) set_u = (int)pv;
          else if (kind == KIND_CARVE) set_u = 0;
          else if (kind == KIND_PAINT && state == ST_EMPTY) return;
          else if (kind == KIND_PAINT && constPaint && state == ST_UNIF) set_u = (int)pv;
        }
        if (set_u >= 0) {  // setBrickUniform (VoxelWorld.ts:89-97)
          if (state == ST_MIXED) {
            if (lane == 0) { a.evt[pair] = 2; a.fsrc[pair] = src; }
            wc.free_++;
          }
          const uint32_t v = (uint32_t)set_u;
          state = v == 0 ? ST_EMPTY : ST_UNIF;
          uval = v; src = -1;
#pragma unroll
          for (int k = 0; k < 8; k++) vox[k] = v | (v << 16);
          dirty = true;
          return;
        }
        if (kind == KIND_PAINT && state == ST_EMPTY) return;

        // sub-block and voxel classes (shapes.ts:382-394), computed by classify_kernel
        if (!full) {
          if (lane < 8) {
            const uint32_t c = (psc >> (2 * lane)) & 3u;
            smask[wib][lane] = c == PC_FULL      ? ~0ull
                               : c != PC_PARTIAL ? 0ull
                               : pm              ? spm[wib][b][lane]
                                                 : __ldg(a.pmask + pair * 8 + lane);
          }
          wc.sub += 8;
          wc.vox += 64 * __popc(psc & ~(psc >> 1) & 0x5555u);  // sub-blocks of class PC_PARTIAL (01)
        } else if (lane < 8) {
          smask[wib][lane] = ~0ull;
        }
        __syncwarp();

        // write voxels (shapes.ts:395-405)
        bool changed = false;
        if (constPaint || kind == KIND_CARVE) {
          // one value for every covered voxel (carve: air; a const paint is a u16, so the
          // unstored value equals the stored one): whole voxel pairs at a time.  Bit 2j + h
          // of lb is voxel (x0 + h, y, j) of this lane.
          const int base = (lx0 & 3) | ((ly & 3) << 2);
          const int s0 = (lx0 >> 2) | ((ly >> 2) << 1);
          const unsigned long long m0 = smask[wib][s0], m1 = smask[wib][s0 + 4];
          uint32_t lb = 0;
#pragma unroll
          for (int jj = 0; jj < 4; jj++) {
            lb |= (uint32_t)((m0 >> (base + 16 * jj)) & 3ull) << (2 * jj);
            lb |= (uint32_t)((m1 >> (base + 16 * jj)) & 3ull) << (2 * jj + 8);
          }
          const uint32_t v = kind == KIND_CARVE ? 0u : pv;
          const uint32_t vv = v | (v << 16);
#pragma unroll
          for (int k = 0; k < 8; k++) {
            const uint32_t two = (lb >> (2 * k)) & 3u;
            uint32_t keep = ((two & 1u) ? 0xffffu : 0u) | ((two & 2u) ? 0xffff0000u : 0u);
            if (kind == KIND_PAINT)  // Paint recolours non-air voxels only
              keep &= ((vox[k] & 0xffffu) ? 0xffffu : 0u) | ((vox[k] & 0xffff0000u) ? 0xffff0000u : 0u);
            const uint32_t nv = (vox[k] & ~keep) | (vv & keep);
            changed = changed || nv != vox[k];
            vox[k] = nv;
          }
        } else {
#pragma unroll
          for (int k = 0; k < 8; k++) {
            const int s = (lx0 >> 2) | ((ly >> 2) << 1) | ((k >> 2) << 2);
            const int e0 = (lx0 & 3) | ((ly & 3) << 2) | ((k & 3) << 4);
            const unsigned long long ms = smask[wib][s];
#pragma unroll
            for (int h = 0; h < 2; h++) {
              if (!((ms >> (e0 + h)) & 1ull)) continue;
              const uint32_t cur = (vox[k] >> (16 * h)) & 0xffffu;
              uint32_t next;
              if (kind == KIND_PAINT && cur == 0) continue;
              else if (slot != NO_SLOT) {  // evaluated by paint_kernel
                const uint32_t pvv = __ldg(a.pvals + (size_t)slot * 512 + (uint32_t)((lx0 + h) | (ly << 3) | (k << 6)));
                if (pvv & PV_RANGE) st_local |= ST_RANGE;
                next = pvv & 0xffffu;
                paint_calls++;
              } else {
                if constexpr (INLINE) {
                  const uint32_t pv2 = paint_at_voxel(a.params, a.vs, a.validate, a.ops + o_idx, ox + lx0 + h, oy + ly, oz + k);
                  if (pv2 & PV_RANGE) st_local |= ST_RANGE;
                  if (pv2 & PV_VIOL) paint_viol++;
                  next = pv2 & 0xffffu;
                  paint_calls++;
                } else {  // every painted op has a slot in this build
                  st_local |= ST_CHAIN;
                  next = cur;
                }
              }
              if (next != cur) {  // Uint16Array store; the comparison uses the unstored value
                vox[k] = (vox[k] & ~(0xffffu << (16 * h))) | ((next & 0xffffu) << (16 * h));
                changed = true;
              }
            }
          }
        }
        __syncwarp();
        if (!__any_sync(FULLMASK, changed)) return;
        dirty = true;
        uint8_t ev = 0;
        if (state != ST_MIXED) {  // editableBrick -> allocBrick (VoxelWorld.ts:103-122)
          ev = 1; src = (long long)pair; state = ST_MIXED;
          wc.alloc++;
        }
        // compactCell (VoxelWorld.ts:147-156)
        const uint32_t v0 = __shfl_sync(FULLMASK, vox[0] & 0xffffu, 0);
        const uint32_t vv = v0 | (v0 << 16);
        bool eq = true;
#pragma unroll
        for (int k = 0; k < 8; k++) eq = eq && vox[k] == vv;
        if (__all_sync(FULLMASK, eq)) {
          if (lane == 0) a.fsrc[pair] = src;
          ev |= 2;
          wc.free_++;
          state = v0 == 0 ? ST_EMPTY : ST_UNIF;
          uval = v0; src = -1;
        }
        if (lane == 0) a.evt[pair] = ev;
      };

      // entries 0..7 of the tile list, looked up above by lanes 8j..8j+7
      for (uint32_t m = (m_all >> (8 * j)) & 0xffu; m; m &= m - 1) apply(q, (int)(8 * j) + __ffs(m) - 1, true);
      // the rest of a longer list, 32 entries per pass
      for (uint32_t c0 = 8; c0 < tcnt; c0 += 32) {
        FoldEntry f = {0ull, 0u, 0u, 0u, NO_SLOT, 0u, PC_SKIP};
        if (c0 + lane < tcnt) f = fold_entry(a, toff + c0 + lane, bx, by, bz);
        for (uint32_t m = __ballot_sync(FULLMASK, f.cls != PC_SKIP); m; m &= m - 1) apply(f, __ffs(m) - 1, false);
      }

      if (!dirty) continue;
      // the grid entry is committed by finalize, so a failed build leaves the world intact
      uint32_t tag;
      if (state == ST_EMPTY) {
        tag = 0;
      } else if (state == ST_UNIF) {
        tag = UNIFORM | uval;
      } else {
        uint32_t slot = 0;
        if (lane == 0) slot = atomicAdd(&a.res->stage_count, 1u);
        slot = __shfl_sync(FULLMASK, slot, 0);
        if (slot >= a.stage_cap) {
          st_local |= ST_STAGE_OVERFLOW;
        } else {
          uint32_t* dst = a.staging32 + (size_t)slot * 256;
          const unsigned long long keep = l2_keep_policy();
#pragma unroll
          for (int k = 0; k < 8; k++) st_keep(dst + 32 * k + lane, vox[k], keep);
          if (lane == 0) { a.stage_cell[slot] = ci; a.stage_src[slot] = src; }
        }
        tag = TAG_STAGED | (slot & 0x3fffffffu);
      }
      if (lane == (int)j) { t_ci = ci; t_tag = tag; t_dirty = true; }
    }
    // the group's touched-list entries, one append per group
    const uint32_t dm = __ballot_sync(FULLMASK, t_dirty);
    if (dm) {
      uint32_t t0 = 0;
      if (lane == 0) t0 = atomicAdd(&a.res->touched_count, (uint32_t)__popc(dm));
      t0 = __shfl_sync(FULLMASK, t0, 0);
      if (t_dirty) {
        const uint32_t t = t0 + (uint32_t)__popc(dm & ((1u << lane) - 1u));
        if (t < a.touched_cap) a.touched[t] = make_uint2(t_ci, t_tag);
        else st_local |= ST_STAGE_OVERFLOW;
      }
    }
  }
  if (lane == 0) {
    if (wc.sub) atomicAdd(&a.res->c.sub_evals, (unsigned long long)wc.sub);
    if (wc.vox) atomicAdd(&a.res->c.voxel_evals, (unsigned long long)wc.vox);
    if (wc.alloc) atomicAdd(&a.res->c.alloc_events, (unsigned long long)wc.alloc);
    if (wc.free_) atomicAdd(&a.res->c.free_events, (unsigned long long)wc.free_);
  }
  uint32_t pc = paint_calls, stw = st_local, pvl = paint_viol;
#pragma unroll
  for (int o2 = 16; o2; o2 >>= 1) {
    pc += __shfl_xor_sync(FULLMASK, pc, o2);
    pvl += __shfl_xor_sync(FULLMASK, pvl, o2);
    stw |= __shfl_xor_sync(FULLMASK, stw, o2);
  }
  if (lane == 0) {
    if (pc) atomicAdd(&a.res->c.paint_evals, (unsigned long long)pc);
    if (pvl) atomicAdd(&a.res->c.violations, (unsigned long long)pvl);
    if (stw) atomicOr(&a.res->status, stw);
  }
}

void launch_fold(const FoldArgs& a, int mode, int n_sms, cudaStream_t s, cudaEvent_t mid, int max_blocks,
                 cudaStream_t s_apply, cudaEvent_t eval_done) {
  auto grid = [&](int per_sm) { return max_blocks > 0 && max_blocks < n_sms * per_sm ? max_blocks : n_sms * per_sm; };
  if (mode == 1) {
    launch_pdl(classify_kernel<1>, dim3(grid(PX_CLASSIFY_MINB)), dim3(256), 0, s, a);
    launch_pdl(sub_kernel<1>, dim3(grid(PX_SUB_MINB)), dim3(256), 0, s, a);
    if (a.vq_nonempty & (1u << VQ_NARROW)) {
      if (a.validate) launch_pdl(voxel_lean_kernel<true, VQ_NARROW>, dim3(grid(PX_VSIMPLE_MINB)), dim3(256), 0, s, a);
      else launch_pdl(voxel_lean_kernel<false, VQ_NARROW>, dim3(grid(PX_VSIMPLE_MINB)), dim3(256), 0, s, a);
    }
    if (a.vq_nonempty & (1u << VQ_AFFINE)) {
      if (a.validate) launch_pdl(voxel_lean_kernel<true, VQ_AFFINE>, dim3(grid(PX_VAFF_MINB)), dim3(256), 0, s, a);
      else launch_pdl(voxel_lean_kernel<false, VQ_AFFINE>, dim3(grid(PX_VAFF_MINB)), dim3(256), 0, s, a);
    }
    if (a.vq_nonempty & (1u << VQ_WIDE)) {
      if (a.validate) launch_pdl(voxel_lean_kernel<true, VQ_WIDE>, dim3(grid(PX_VWIDE_MINB)), dim3(256), 0, s, a);
      else launch_pdl(voxel_lean_kernel<false, VQ_WIDE>, dim3(grid(PX_VWIDE_MINB)), dim3(256), 0, s, a);
    }
    launch_pdl(voxel_kernel<1, VQ_GENERIC, VQ_GENERIC>, dim3(grid(PX_VOXEL_MINB)), dim3(256), 0, s, a);
  } else {
    launch_pdl(classify_kernel<0>, dim3(grid(PX_CLASSIFY64_MINB)), dim3(256), 0, s, a);
    launch_pdl(sub_kernel<0>, dim3(grid(PX_CLASSIFY64_MINB)), dim3(256), 0, s, a);
    launch_pdl(voxel_kernel<0, VQ_NARROW, VQ_GENERIC>, dim3(grid(PX_CLASSIFY64_MINB)), dim3(256), 0, s, a);
  }
  // the mixed form's paint pass also resolves the lean voxel kernels' rescue list
  if (mode == 1) launch_pdl(paint_kernel<1>, dim3(grid(4)), dim3(256), 0, s, a);
  else if (a.n_paint_slots) launch_pdl(paint_kernel<0>, dim3(grid(4)), dim3(256), 0, s, a);
  if (mid) cudaEventRecord(mid, s);
  if (s_apply != s) {  // the apply pass waits for these passes on its own stream
    cudaEventRecord(eval_done, s);
    cudaStreamWaitEvent(s_apply, eval_done, 0);
    s = s_apply;
  }
  if (a.inline_paints) launch_pdl(fold_kernel<true>, dim3(grid(PX_FOLD_MINB)), dim3(256), 0, s, a);
  else launch_pdl(fold_kernel<false>, dim3(grid(PX_FOLD_MINB)), dim3(256), 0, s, a);
}

// ---------------------------------------------------------------------------
// scan building blocks of the allocator replay's single-pass look-back scans

__device__ __forceinline__ int4 shfl_up_any(int4 v, int o) {
  return make_int4(__shfl_up_sync(FULLMASK, v.x, o), __shfl_up_sync(FULLMASK, v.y, o), __shfl_up_sync(FULLMASK, v.z, o),
                   0);
}
__device__ __forceinline__ int4 shfl_any(int4 v, int l) {
  return make_int4(__shfl_sync(FULLMASK, v.x, l), __shfl_sync(FULLMASK, v.y, l), __shfl_sync(FULLMASK, v.z, l), 0);
}

// A run of events: x its count, (y, z) = (a, c) its clamped stack-depth map:
// after the run, a stack of depth d has depth max(c, d + a).  Applying x then y
// gives (x.a + y.a, max(y.c, x.c + y.a)).  A push is (1, -inf); a pop is
// (-1, 0): on an empty stack it allocates a fresh brick instead.
struct EventOp {
  typedef int4 T;
  __device__ static T identity() { return make_int4(0, 0, -(1 << 30), 0); }
  __device__ static T combine(T x, T y) { return make_int4(x.x + y.x, x.y + y.y, max(y.z, x.z + y.y), 0); }
  __device__ static T push() { return make_int4(1, 1, -(1 << 30), 0); }
  __device__ static T pop() { return make_int4(1, -1, 0, 0); }
};
// Min-tree entries before any event (the byte value 0x7f of their clear),
// above every depth.
constexpr int32_t NO_DEPTH = 0x7f7f7f7f;

// Exclusive scan of one value per thread across the block; returns the
// thread's exclusive prefix and the block total.
template <class Op>
__device__ typename Op::T block_exclusive(typename Op::T v, typename Op::T* sh, typename Op::T& total) {
  typedef typename Op::T T;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = shfl_up_any(x, o);
    if (lane >= o) x = Op::combine(y, x);
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    T s = lane < nw ? sh[lane] : Op::identity();
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T y = shfl_up_any(s, o);
      if (lane >= o) s = Op::combine(y, s);
    }
    if (lane < nw) sh[lane] = s;
  }
  __syncthreads();
  T wp = w ? sh[w - 1] : Op::identity();
  total = sh[nw - 1];
  T ex = shfl_up_any(x, 1);
  if (lane == 0) ex = Op::identity();
  __syncthreads();
  return Op::combine(wp, ex);
}

// Decoupled look-back: each block takes the next tile by ticket (so every
// earlier tile is already running or done), publishes its aggregate, reads its
// predecessors' inclusive prefixes (or aggregates, while those are pending) from
// nearest to farthest, publishes its own inclusive prefix and writes its
// outputs.  Flags: 0 pending, 1 aggregate, 2 prefix.  Waits give up after
// SCAN_SPIN_LIMIT polls (an error status, no hang).
constexpr uint32_t SCAN_SPIN_LIMIT = 1u << 24;

template <class T>
__device__ __forceinline__ void scan_publish(T* slot, uint32_t* flag, T v, uint32_t f) {
  __stcg(slot, v);
  __threadfence();
  *(volatile uint32_t*)flag = f;
}
__device__ __forceinline__ int4 scan_peek(const int4* p) { return __ldcg(p); }

// ---------------------------------------------------------------------------
// replay of the LIFO pool allocator (VoxelWorld.ts:112-127) over the build's
// alloc/free events in (op, cell) order -- the order of the reference's loop --
// in three kernels:
//   event_scan    one look-back scan over the (op, brick) pairs: the position
//                 of each pair's events, the events themselves (a pop per
//                 allocation, a push per free, the H holes before the build as
//                 the first pushes), the stack depth after each event (a
//                 clamped prefix scan: a pop that finds the stack empty takes
//                 poolUsed++ instead, its rank read off the same scan) and the
//                 min tree over the depths;
//   match         each event's link towards its pool index: a pop at depth D
//                 takes the push that last filled slot D (the event after the
//                 last earlier event of depth < D, found in the min tree); a
//                 push frees its brick's index, the index of that brick's last
//                 allocation.  The pushes no later event undercuts are the holes
//                 after the build;
//   resolve       the links followed to pool indices (finalize turns the holes'
//                 event indices into their pool indices).

constexpr unsigned long long KNOWN = 1ull << 63;    // ew: a resolved pool index
constexpr unsigned long long PAIRREF = 1ull << 62;  // ew of a push: the pair of its brick's last allocation
enum : uint8_t { EV_PUSH = 0, EV_POP = 1, EV_NONE = 0xff };
constexpr int RP_THREADS = PX_REPLAY_THREADS, RP_ITEMS = 8;
static_assert(RP_THREADS * RP_ITEMS == REPLAY_TILE, "a tile is one block pass");

// Decoupled look-back of tile `tile`, by warp 0: publishes the tile's
// aggregate, combines its predecessors' (inclusive prefixes where published,
// aggregates while those are pending, 32 tiles per step, nearest first) and
// publishes the tile's inclusive prefix.  Returns the exclusive prefix.
template <class Op>
__device__ typename Op::T lookback(uint32_t tile, typename Op::T total, typename Op::T* agg, typename Op::T* incl,
                                   uint32_t* flags, uint32_t* status) {
  typedef typename Op::T T;
  const int lane = threadIdx.x & 31;
  T prefix = Op::identity();
  if (tile == 0) {
    if (lane == 0) scan_publish(incl, flags, total, 2u);
    return prefix;
  }
  if (lane == 0) scan_publish(agg + tile, flags + tile, total, 1u);
  long long hi = (long long)tile - 1;
  uint32_t spins = 0;
  for (;;) {
    const long long j = hi - 31 + lane;  // lane 31 reads the nearest tile of the window
    const uint32_t f = j >= 0 ? *(volatile uint32_t*)(flags + j) : 2u;  // before tile 0: the identity
    if (__any_sync(FULLMASK, f == 0)) {
      if (++spins > SCAN_SPIN_LIMIT) {  // cannot happen: earlier tiles publish unconditionally
        if (lane == 0) atomicOr(status, (uint32_t)ST_CHAIN);
        break;
      }
      continue;
    }
    __threadfence();
    T v = j >= 0 ? scan_peek(f == 2 ? incl + j : agg + j) : Op::identity();
    const uint32_t im = __ballot_sync(FULLMASK, f == 2);
    if (lane < (im ? 31 - __clz(im) : 0)) v = Op::identity();  // tiles before the nearest prefix
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {  // ordered combination of the window
      const T y = shfl_up_any(v, o);
      if (lane >= o) v = Op::combine(y, v);
    }
    prefix = Op::combine(shfl_any(v, 31), prefix);
    if (im) break;
    hi -= 32;
  }
  if (lane == 0) scan_publish(incl + tile, flags + tile, Op::combine(prefix, total), 2u);
  return prefix;
}

__device__ __forceinline__ size_t level_size(size_t E, int l) {
  size_t n = E;
  for (int i = 0; i < l; i++) n = (n + 31) >> 5;
  return n;
}

// The replay's first kernel: one single-pass look-back over the (op, brick)
// pairs whose tile aggregate is an EventOp -- the tile's event count and the
// depth map of its events -- so that each thread knows, for its pairs, the
// position of their events and the stack as they find it.  It writes the
// events (a pop per allocation, a push per free, the H holes before the build
// as the first pushes), the depth after each event, the fresh allocations'
// pool indices (a pop on the empty stack takes poolUsed + the number of fresh
// allocations before it, which is max(c - a, 0) of the depth map of all events
// before it) and the min tree: levels 1 and 2 by atomicMin on entries cleared
// to NO_DEPTH (an entry's events may come from two tiles), the levels above by
// the block that finishes last.
__global__ void __launch_bounds__(RP_THREADS) event_scan_kernel(ReplayArgs a) {
  pdl_prologue();
  __shared__ int4 sh[32];
  __shared__ int4 s_prefix;
  __shared__ uint32_t s_tile;
  __shared__ bool s_last;
  // the committed state: no build writes it until this one commits
  const uint32_t H = __ldcg(&a.state->n_holes), U0 = __ldcg(&a.state->pool_used);
  if (threadIdx.x == 0) s_tile = atomicAdd(&a.t.counters[0], 1u);
  __syncthreads();
  const uint32_t tile = s_tile;
  const size_t P = a.P, n_tiles = (P + REPLAY_TILE - 1) / REPLAY_TILE;
  int32_t* const L1 = a.tl.n >= 1 ? a.tree + a.tl.off[0] : nullptr;
  int32_t* const L2 = a.tl.n >= 2 ? a.tree + a.tl.off[1] : nullptr;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.res->h_before = H;
    a.res->u_before = U0;
    if (P == 0) { a.res->n_events = H; a.res->n_fresh = 0; }
  }
  if (tile < n_tiles) {
    const size_t k0 = (size_t)tile * REPLAY_TILE + (size_t)threadIdx.x * RP_ITEMS;
    uint32_t ev8[2] = {0u, 0u};  // the event codes of the thread's 8 pairs, a byte each
    if (k0 + RP_ITEMS <= P) {
      const uint2 u = *reinterpret_cast<const uint2*>(a.evt + k0);
      ev8[0] = u.x; ev8[1] = u.y;
    } else {
#pragma unroll
      for (int j = 0; j < RP_ITEMS; j++)
        if (k0 + j < P) ev8[j >> 2] |= (uint32_t)a.evt[k0 + j] << (8 * (j & 3));
    }
    int4 acc = EventOp::identity();
#pragma unroll
    for (int j = 0; j < RP_ITEMS; j++) {
      const uint32_t ev = (ev8[j >> 2] >> (8 * (j & 3))) & 3u;
      if (ev & 1u) acc = EventOp::combine(acc, EventOp::pop());
      if (ev & 2u) acc = EventOp::combine(acc, EventOp::push());
    }
    int4 total;
    const int4 pre_block = block_exclusive<EventOp>(acc, sh, total);
    if (threadIdx.x < 32) {
      const int4 pf = lookback<EventOp>(tile, total, a.t.agg, a.t.incl, a.t.flag, &a.res->status);
      if (threadIdx.x == 0) s_prefix = pf;
    }
    __syncthreads();
    // the events before this thread's first: the H holes (pushes), then those of the earlier pairs
    int4 run = EventOp::combine(make_int4(0, (int)H, -(1 << 30), 0), EventOp::combine(s_prefix, pre_block));
    uint32_t pos = (uint32_t)run.x;  // events of the pairs before k0 (after the holes)
    const uint32_t B0 = __shfl_sync(FULLMASK, H + pos, 0) >> 10;  // the warp's events lie in level-2 blocks B0, B0 + 1
    int32_t m1 = NO_DEPTH, m2lo = NO_DEPTH, m2hi = NO_DEPTH;
    long long b1 = -1;
#pragma unroll
    for (int j = 0; j < RP_ITEMS; j++) {
      const size_t k = k0 + j;
      if (k >= P) break;
      const uint32_t ev = (ev8[j >> 2] >> (8 * (j & 3))) & 3u;
      if (ev & 1u) a.pos[k] = pos;  // read only for allocations (a push's brick, a staged brick)
#pragma unroll
      for (int t = 0; t < 2; t++) {
        if (!((ev >> t) & 1u)) continue;
        const size_t e = (size_t)H + pos;
        if (t == 0) {  // editableBrick -> allocBrick: a pop; on the empty stack, a fresh brick
          const bool fresh = max(run.z, run.y) == 0;
          a.etype[e] = EV_POP;
          a.ew[e] = fresh ? KNOWN | (unsigned long long)(U0 + (uint32_t)max(run.z - run.y, 0)) : 0ull;
          run = EventOp::combine(run, EventOp::pop());
        } else {  // setBrickUniform / compactCell: a push of the brick's index
          const long long src = a.fsrc[k];
          a.etype[e] = EV_PUSH;
          a.ew[e] = src >= 0 ? PAIRREF | (unsigned long long)src : KNOWN | (unsigned long long)(-(src + 1));
          run = EventOp::combine(run, EventOp::push());
        }
        const int32_t d = max(run.z, run.y);
        a.depth[e] = d;
        if ((long long)(e >> 5) != b1) {
          if (b1 >= 0 && L1) atomicMin(L1 + b1, m1);
          b1 = (long long)(e >> 5);
          m1 = d;
        } else {
          m1 = min(m1, d);
        }
        if ((uint32_t)(e >> 10) == B0) m2lo = min(m2lo, d);
        else m2hi = min(m2hi, d);
        pos++;
      }
    }
    if (b1 >= 0 && L1) atomicMin(L1 + b1, m1);
    if (L2) {
      const int32_t lo = __reduce_min_sync(FULLMASK, m2lo), hi = __reduce_min_sync(FULLMASK, m2hi);
      if (lane == 0 && lo != NO_DEPTH) atomicMin(L2 + B0, lo);
      if (lane == 0 && hi != NO_DEPTH) atomicMin(L2 + B0 + 1, hi);
    }
    if (tile == n_tiles - 1 && threadIdx.x == RP_THREADS - 1) {
      a.res->n_events = H + pos;
      a.res->n_fresh = (uint32_t)max(run.z - run.y, 0);
    }
  }
  // the holes before the build: the first H pushes, known indices, depth i + 1 (every block takes a share)
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < H; i += (size_t)gridDim.x * blockDim.x) {
    a.etype[i] = EV_PUSH;
    a.ew[i] = KNOWN | a.holes_in[i];
    a.depth[i] = (int32_t)(i + 1);
    if (L1 && (i & 31) == 0) atomicMin(L1 + (i >> 5), (int32_t)(i + 1));  // a block's smallest hole depth
    if (L2 && (i & 1023) == 0) atomicMin(L2 + (i >> 10), (int32_t)(i + 1));
  }
  // the levels above 2: by the block that finishes last
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&a.t.counters[2], 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last || a.tl.n < 3) return;
  __threadfence();
  const size_t E = __ldcg(&a.res->n_events);
  for (int l = 3; l <= a.tl.n; l++) {
    const size_t nb = level_size(E, l - 1), n = level_size(E, l);
    const int32_t* below = a.tree + a.tl.off[l - 2];
    int32_t* lev = a.tree + a.tl.off[l - 1];
    for (size_t c = warp; c < n; c += RP_THREADS / 32) {
      const size_t i = c * 32 + lane;
      const int32_t m = __reduce_min_sync(FULLMASK, i < nb ? __ldcg(below + i) : 0x7fffffff);
      if (lane == 0) lev[c] = m;
    }
    __threadfence();
    __syncthreads();
  }
}

// Bit q of the result: entry 32 b + q of level L is below D, for q <= qmax
// (the block's 32 entries as eight 16-byte loads; levels are 128-byte aligned
// and padded to whole blocks).
__device__ __forceinline__ uint32_t block_below(const int32_t* L, long long b, int D, int qmax) {
  const int4* p = reinterpret_cast<const int4*>(L + b * 32);
  int4 v[8];
#pragma unroll
  for (int k = 0; k < 8; k++) v[k] = __ldcg(p + k);
  uint32_t m = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    m |= (uint32_t)(v[k].x < D) << (4 * k);
    m |= (uint32_t)(v[k].y < D) << (4 * k + 1);
    m |= (uint32_t)(v[k].z < D) << (4 * k + 2);
    m |= (uint32_t)(v[k].w < D) << (4 * k + 3);
  }
  return qmax >= 31 ? m : m & ((2u << qmax) - 1u);
}

// Largest i < e with depth[i] < D (or -1): climb the min tree to the nearest
// block holding a smaller value, then descend to its last such leaf.
__device__ long long prev_less(const int32_t* depth, const int32_t* tree, const TreeLevels& tl, size_t E, size_t e, int D) {
  long long i = (long long)e - 1;
  int lev = 0;
  long long found = -1;
  while (i >= 0) {
    const int32_t* L = lev == 0 ? depth : tree + tl.off[lev - 1];
    const long long start = i & ~31ll;
    const uint32_t m = block_below(L, start >> 5, D, (int)(i - start));
    if (m) { found = start + 31 - __clz(m); break; }
    if (start == 0 || lev == tl.n) return -1;
    i = (start >> 5) - 1;
    lev++;
  }
  if (found < 0) return -1;
  while (lev > 0) {
    lev--;
    const int32_t* L = lev == 0 ? depth : tree + tl.off[lev - 1];
    const long long n = (long long)level_size(E, lev);
    const uint32_t m = block_below(L, found, D, (int)min(31ll, n - 1 - found * 32));
    if (!m) return -1;  // cannot happen: the parent's minimum is below D
    found = found * 32 + 31 - __clz(m);
  }
  return found;
}

// Whether some i > e (i < E) has depth[i] < D: the rest of e's block at each
// level, climbing; at the top level, every entry to the right.
__device__ bool next_less_exists(const int32_t* depth, const int32_t* tree, const TreeLevels& tl, size_t E, size_t e,
                                 int D) {
  size_t i = e + 1;  // the first entry to check at level lev
  for (int lev = 0;; lev++) {
    const size_t n = level_size(E, lev);
    if (i >= n) return false;
    const int32_t* L = lev == 0 ? depth : tree + tl.off[lev - 1];
    for (size_t b = i >> 5;; b++) {
      uint32_t m = block_below(L, (long long)b, D, 31);
      if (b == (i >> 5)) m &= ~((1u << (i & 31)) - 1u);  // entries from i on
      if (b * 32 + 32 > n) m &= (1u << (n - b * 32)) - 1u;  // entries below n
      if (m) return true;
      if (lev < tl.n || b * 32 + 32 >= n) break;  // below the top level: one block, then climb
    }
    if (lev == tl.n) return false;
    i = (i >> 5) + 1;  // the blocks wholly to the right, one level up
  }
}

// Each event's link towards its pool index: a pop (not fresh) takes the value of
// the push that last filled its slot (it links past that push), a push of a brick
// allocated in this build links to that allocation's pop; fresh pops, old indices
// and the holes before the build are known already.  Links always lead to
// earlier events; resolve follows them.
// A push that no later event undercuts is the hole of its slot after the build:
// holes_out[slot] receives the push's event index (finalize turns it into the
// pool index).
__global__ void __launch_bounds__(256) match_events_kernel(ReplayArgs a) {
  pdl_prologue();
  const size_t E = a.res->n_events;
  const uint32_t H = a.res->h_before;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.res->n_holes = E ? (uint32_t)a.depth[E - 1] : 0u;
    a.res->pool_used = a.res->u_before + a.res->n_fresh;
  }
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (size_t)gridDim.x * blockDim.x) {
    const unsigned long long w = __ldcg(a.ew + e);
    if (a.etype[e] == EV_PUSH) {
      if (!(w & KNOWN)) a.ew[e] = (unsigned long long)H + a.pos[w & ~PAIRREF];  // the brick's allocation
      const int d = a.depth[e];
      if (!next_less_exists(a.depth, a.tree, a.tl, E, e, d)) a.holes_out[d - 1] = (uint32_t)e;
    } else if (!(w & KNOWN)) {
      const int D = e ? a.depth[e - 1] : 0;  // >= 1: a pop at depth 0 is fresh, known already
      const size_t p = (size_t)(prev_less(a.depth, a.tree, a.tl, E, e, D) + 1);  // the push that filled slot D
      // the pop takes that push's value: link past the push, to its known index or to its
      // brick's allocation (an earlier pop).  The push's word is read while this kernel may
      // be rewriting it, so it comes in either form.
      const unsigned long long q = __ldcg(a.ew + p);
      a.ew[e] = (q & KNOWN) ? q : (q & PAIRREF) ? (unsigned long long)H + a.pos[q & ~PAIRREF] : q;
    }
  }
}

// Each event's pool index: follow the links (each to an earlier event) to a
// known index, storing it back, so that walks running at the same time cut
// each other's chains short (a pool slot reused many times in one build makes
// a long chain).
__global__ void __launch_bounds__(256) resolve_events_kernel(ReplayArgs a) {
  pdl_prologue();
  const size_t E = a.res->n_events;
  for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (size_t)gridDim.x * blockDim.x) {
    unsigned long long w = *((volatile unsigned long long*)a.ew + e);
    if (w & KNOWN) continue;
    size_t p = (size_t)w;
    for (size_t steps = 0;; steps++) {
      const unsigned long long q = *((volatile unsigned long long*)a.ew + p);
      if (q & KNOWN) { w = q; break; }
      if ((size_t)q >= p || steps > E) {  // cannot happen: links lead to earlier events
        atomicOr(&a.res->status, (uint32_t)ST_CHAIN);
        w = KNOWN;
        break;
      }
      p = (size_t)q;
    }
    a.ew[e] = w;
  }
}

TreeLevels tree_levels(size_t E_max) {
  TreeLevels tl;
  tl.n = 0;
  size_t n = E_max, off = 0;
  while (n > 32 && tl.n < 8) {
    n = (n + 31) / 32;
    tl.off[tl.n++] = off;
    off += (n + 31) & ~(size_t)31;  // levels start on 128-byte boundaries (whole blocks are loaded)
  }
  return tl;
}

size_t tree_clear_bytes(size_t E_max) {
  size_t n = E_max, off = 0;
  for (int l = 0; l < 2 && n > 32; l++) {  // levels 1 and 2, laid out as tree_levels lays them out
    n = (n + 31) / 32;
    off += (n + 31) & ~(size_t)31;
  }
  return 4 * off;
}

static size_t al16(size_t b) { return (b + 15) & ~(size_t)15; }
// layout: counters[8], flags (cleared); aggregates, inclusive prefixes
ReplayTemp replay_temp(void* base, uint64_t P) {
  const size_t tp = P / REPLAY_TILE + 2;
  char* c = (char*)base;
  ReplayTemp t;
  t.counters = (uint32_t*)c; c += 32;
  t.flag = (uint32_t*)c; c += al16(4 * tp);
  t.agg = (int4*)c; c += 16 * tp;
  t.incl = (int4*)c;
  return t;
}
size_t replay_clear_bytes(uint64_t P) { return 32 + al16(4 * (P / REPLAY_TILE + 2)); }
size_t replay_temp_bytes(uint64_t P) { return replay_clear_bytes(P) + 32 * (P / REPLAY_TILE + 2); }

void launch_replay(const ReplayArgs& a, cudaStream_t s) {
  int dev = 0, n_sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t p_tiles = (a.P + REPLAY_TILE - 1) / REPLAY_TILE;
  const size_t h_blocks = std::min<size_t>(((size_t)a.H_max + RP_THREADS - 1) / RP_THREADS, (size_t)n_sms * 4);
  launch_pdl(event_scan_kernel, dim3((unsigned)std::max<size_t>(1, std::max(p_tiles, h_blocks))), dim3(RP_THREADS), 0,
             s, a);
  const size_t rb = std::min<size_t>((a.E_max + 255) / 256, (size_t)n_sms * 8);
  launch_pdl(match_events_kernel, dim3((unsigned)std::max<size_t>(1, rb)), dim3(256), 0, s, a);
  launch_pdl(resolve_events_kernel, dim3((unsigned)std::max<size_t>(1, rb)), dim3(256), 0, s, a);
}

// ---------------------------------------------------------------------------
// finalize: staging -> pool at the replayed indices, grid entries

#ifndef PX_FIN_BRICKS
#define PX_FIN_BRICKS 8
#endif
constexpr int FIN_BRICKS = PX_FIN_BRICKS;  // touched bricks per warp pass of finalize (at most 32)
static_assert(FIN_BRICKS >= 1 && FIN_BRICKS <= 32, "one brick per lane");

__global__ void __launch_bounds__(256) finalize_kernel(FinalizeArgs a) {
  __shared__ uint8_t op_s[256];
  op_s[threadIdx.x] = a.opaque[threadIdx.x];  // 256 threads
  pdl_prologue();
  __syncthreads();
  // commit only a complete build (every staging slot written, every pool index within
  // the pool) that follows committed builds; the first thread records the outcome
  const bool after_failure = __ldcg(&a.state->poisoned) != 0;
  if (after_failure || (a.res->status & ST_NO_COMMIT) || a.res->pool_used > a.pool_cap) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      if (after_failure) atomicOr(&a.res->status, (uint32_t)ST_CHAIN);
      else if (!(a.res->status & ST_NO_COMMIT)) atomicOr(&a.res->status, (uint32_t)ST_POOL_OVERFLOW);
      a.state->poisoned = 1u;
    }
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {  // nothing below reads the state
    a.state->pool_used = a.res->pool_used;
    a.state->n_holes = a.res->n_holes;
  }
  const uint32_t H = a.res->h_before;
  // the holes after the build: their pushes' event indices become pool indices
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x, nh = a.res->n_holes; k < nh; k += gridDim.x * blockDim.x)
    a.holes_out[k] = (uint32_t)(__ldcg(a.ew + a.holes_out[k]) & 0xffffffffull);
  const int lane = threadIdx.x & 31;
  const uint32_t n = a.res->touched_count;
  // FIN_BRICKS touched bricks per warp pass: each of the first lanes resolves one
  // brick's pool index (a chain of dependent loads), then the warp copies the
  // staged bricks four at a time (eight 16-byte loads in flight per lane).  Few
  // bricks per pass keep many warps' chains and copies in flight at once.
  const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t base = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * FIN_BRICKS; base < n;
       base += n_warps * FIN_BRICKS) {
    const uint32_t t = base + lane;
    uint32_t cell = 0, slot = 0, idx = 0;
    bool staged = false;
    if (lane < FIN_BRICKS && t < n) {
      const uint2 e = a.touched[t];
      cell = e.x;
      if (!(e.y & TAG_STAGED) || (e.y & UNIFORM)) {
        a.grid[e.x] = e.y;
      } else {
        slot = e.y & 0x3fffffffu;
        const long long src = a.stage_src[slot];
        if (src >= 0) {
          const unsigned long long w = a.ew[H + a.pos[src]];
          if (!(w & KNOWN)) atomicOr(&a.res->status, (uint32_t)ST_CHAIN);
          else { idx = (uint32_t)(w & 0xffffffffull); staged = true; }
        } else {
          idx = (uint32_t)(-(src + 1));
          staged = true;
        }
      }
    }
    uint32_t mx = staged ? idx : 0u;
#pragma unroll
    for (int o = 16; o; o >>= 1) mx = max(mx, __shfl_xor_sync(FULLMASK, mx, o));
    if (lane == 0 && mx) atomicMax(&a.res->max_pool_index, mx);
    if (staged) a.grid[cell] = idx + 1;
    uint32_t sm = __ballot_sync(FULLMASK, staged);
    while (sm) {
      int src_l[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        src_l[q] = -1;
        if (sm) { src_l[q] = __ffs(sm) - 1; sm &= sm - 1; }
      }
      uint4 v[4][2];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (src_l[q] < 0) continue;
        const uint32_t sl = __shfl_sync(FULLMASK, slot, src_l[q]);
        const uint4* s4 = reinterpret_cast<const uint4*>(a.staging32 + (size_t)sl * 256);
        v[q][0] = s4[lane];
        v[q][1] = s4[lane + 32];
      }
      // each brick's opaque, non-air voxels (16 per lane), two bricks per 32-bit word
      uint32_t cnt2[2] = {0u, 0u};
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (src_l[q] < 0) continue;
        const uint32_t w8[8] = {v[q][0].x, v[q][0].y, v[q][0].z, v[q][0].w, v[q][1].x, v[q][1].y, v[q][1].z, v[q][1].w};
        uint32_t c = 0;
#pragma unroll
        for (int k = 0; k < 8; k++) {
          const uint32_t lo = w8[k] & 0xffffu, hi = w8[k] >> 16;
          c += (lo != 0 && op_s[lo & 0xffu]) + (hi != 0 && op_s[hi & 0xffu]);
        }
        cnt2[q >> 1] += c << (16 * (q & 1));
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        cnt2[0] += __shfl_xor_sync(FULLMASK, cnt2[0], o);
        cnt2[1] += __shfl_xor_sync(FULLMASK, cnt2[1], o);
      }
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (src_l[q] < 0) continue;
        const uint32_t di = __shfl_sync(FULLMASK, idx, src_l[q]);
        uint4* d4 = reinterpret_cast<uint4*>(a.pool32 + (size_t)di * 256);
        d4[lane] = v[q][0];
        d4[lane + 32] = v[q][1];
        if (lane == 0) a.pcount[di] = (uint16_t)((cnt2[q >> 1] >> (16 * (q & 1))) & 0xffffu);
      }
      // every lane's loads of these staged bricks have returned (their values are
      // stored): their eight 128-byte lines each leave L2 unwritten
      __syncwarp();
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (src_l[q] < 0) continue;
        const uint32_t sl = __shfl_sync(FULLMASK, slot, src_l[q]);
        if (lane < 8) l2_discard_line(a.staging32 + (size_t)sl * 256 + 32 * lane);
      }
    }
  }
}

void launch_finalize(const FinalizeArgs& a, uint32_t touched_cap, cudaStream_t s) {
  int dev = 0, n_sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&n_sms, cudaDevAttrMultiProcessorCount, dev);
  // a grid-stride loop over the touched bricks (their count is known on the device
  // only): at most four blocks per SM, fewer when the bound is small
  const size_t b = ((size_t)touched_cap + 8 * FIN_BRICKS - 1) / (8 * FIN_BRICKS);
  const int blocks = (int)std::max<size_t>(1, std::min<size_t>(b, (size_t)n_sms * 4));
  launch_pdl(finalize_kernel, dim3(blocks), dim3(256), 0, s, a);
}

// ---------------------------------------------------------------------------
// derive: super-grid counts and density (GpuWorld.ts:90-101, VoxelWorld.ts:159-170)

__global__ void __launch_bounds__(256) derive_kernel(DeriveArgs a) {
  pdl_prologue();
  // a build that committed nothing leaves the world (and its derived buffers) as they were
  if (a.res && (a.res->status & (ST_NO_COMMIT | ST_POOL_OVERFLOW))) return;
  const uint32_t* __restrict__ grid = a.grid;
  const uint32_t* __restrict__ pool32 = a.pool32;
  const int BX = a.BX, BY = a.BY, BZ = a.BZ;
  const uint8_t* __restrict__ opaque = a.opaque;
  const uint8_t* __restrict__ udens = a.udens;
  uint32_t* super_counts = a.super_counts;
  uint8_t* density = a.density;
  __shared__ uint8_t op_s[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) op_s[i] = opaque[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int SX = (BX + 3) / 4, SY = (BY + 3) / 4, SZ = (BZ + 3) / 4;
  const int n_super = SX * SY * SZ;
  for (int sc = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; sc < n_super; sc += (gridDim.x * blockDim.x) >> 5) {
    const int sz = sc / (SX * SY), r = sc - sz * SX * SY, sy = r / SX, sx = r - sy * SX;
    uint32_t nz = 0;
    uint32_t mixed_g[2] = {0, 0};
    size_t mixed_ci[2] = {0, 0};
    bool is_mixed[2] = {false, false};
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int k = lane + 32 * h;
      const int bx = sx * 4 + (k & 3), by = sy * 4 + ((k >> 2) & 3), bz = sz * 4 + (k >> 4);
      if (bx < BX && by < BY && bz < BZ) {
        const size_t ci = (size_t)bx + (size_t)BX * ((size_t)by + (size_t)BY * bz);
        const uint32_t g = grid[ci];
        nz += g != 0;
        if (g == 0) density[ci] = 0;
        else if (g & UNIFORM) density[ci] = udens[g & 0xffu];
        else if (a.pcount) density[ci] = (uint8_t)px_round(((double)__ldg(a.pcount + (g - 1)) / 512.0) * 255.0);
        else { is_mixed[h] = true; mixed_g[h] = g; mixed_ci[h] = ci; }
      }
    }
#pragma unroll
    for (int h = 0; h < 2; h++) {
      uint32_t mm = __ballot_sync(FULLMASK, is_mixed[h]);
      while (mm) {
        const int src = __ffs(mm) - 1;
        mm &= mm - 1;
        const uint32_t g = __shfl_sync(FULLMASK, mixed_g[h], src);
        const unsigned long long ci = __shfl_sync(FULLMASK, (unsigned long long)mixed_ci[h], src);
        const uint32_t* b = pool32 + (size_t)(g - 1) * 256;
        uint32_t cnt = 0;
#pragma unroll
        for (int j = 0; j < 8; j++) {
          uint32_t w = b[32 * j + lane];
          uint32_t v0 = w & 0xffffu, v1 = w >> 16;
          cnt += (v0 != 0 && op_s[v0 & 0xffu]) + (v1 != 0 && op_s[v1 & 0xffu]);
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(FULLMASK, cnt, o);
        if (lane == 0) {
          density[ci] = (uint8_t)px_round(((double)cnt / 512.0) * 255.0);
          if (a.pcount_out) a.pcount_out[g - 1] = (uint16_t)cnt;
        }
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) nz += __shfl_xor_sync(FULLMASK, nz, o);
    if (lane == 0) super_counts[sc] = nz;
  }
  // the GPU free list (GpuWorld.ts:103-109): holes inside the used range in
  // push order, then every index above it, from the top of the pool down
  if (!a.free_list) return;
  const uint32_t used = a.res ? a.res->pool_used : 0u, n_holes = a.res ? a.res->n_holes : 0u;
  const uint64_t cap = free_list_bound(used, a.max_bricks);
  const uint64_t len = used <= cap ? (uint64_t)n_holes + (cap - used) : 0ull;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (used > cap || len > a.free_cap) atomicOr(&a.res->status, (uint32_t)ST_FREE_CAP);
    a.res->free_len = used > cap || len > a.free_cap ? 0u : (uint32_t)len;
  }
  if (used > cap || len > a.free_cap) return;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (uint64_t)gridDim.x * blockDim.x)
    a.free_list[i] = i < n_holes ? __ldg(a.holes + i) : (uint32_t)(cap - 1 - (i - n_holes));
}

// A build's op-table uploads (read straight from the host arrays: pageable
// memory the GPU reads through the host page tables) and counter clears in one
// launch: entry blockIdx.y, 16-byte words, then the last bytes of an entry.
__global__ void __launch_bounds__(256) upload_kernel(HostUploads u) {
  pdl_prologue();
  const HostUploads::Entry& e = u.e[blockIdx.y];
  const size_t n16 = e.bytes >> 4;
  const uint4* src = reinterpret_cast<const uint4*>(e.src);
  uint4* dst = reinterpret_cast<uint4*>(e.dst);
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src ? src[i] : make_uint4(e.fill, e.fill, e.fill, e.fill);
  if (blockIdx.x == 0 && threadIdx.x < (e.bytes & 15u)) {
    const size_t k = (n16 << 4) + threadIdx.x;
    static_cast<unsigned char*>(e.dst)[k] = src ? static_cast<const unsigned char*>(e.src)[k] : (unsigned char)e.fill;
  }
}
void launch_uploads(const HostUploads& u, cudaStream_t s) {
  if (u.n == 0) return;
  launch_pdl(upload_kernel, dim3(32, (unsigned)u.n), dim3(256), 0, s, u);
}

void launch_derive(const DeriveArgs& a, cudaStream_t s) {
  const int n_super = ((a.BX + 3) / 4) * ((a.BY + 3) / 4) * ((a.BZ + 3) / 4);
  const size_t b = ((size_t)n_super * 32 + 255) / 256;
  launch_pdl(derive_kernel, dim3((unsigned)(b < 65535 ? b : 65535)), dim3(256), 0, s, a);
}

// ---------------------------------------------------------------------------
// check of the square-root bounds of the float32 interval evaluator: every
// float v in [lo_bits, hi_bits] against the IEEE directed square roots
// (sqrt_lo(v) <= sqrt_rd(v) and sqrt_hi(v) >= sqrt_ru(v)); counts failures and
// keeps the smallest failing bit pattern.

__global__ void __launch_bounds__(256) sqrt_bounds_kernel(uint32_t lo_bits, uint32_t hi_bits,
                                                          unsigned long long* bad, uint32_t* first_bad) {
  uint32_t n_bad = 0;
  for (uint64_t b = (uint64_t)lo_bits + (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; b <= hi_bits;
       b += (uint64_t)gridDim.x * blockDim.x) {
    const float v = __uint_as_float((uint32_t)b);
    if (sqrt_lo(v) > __fsqrt_rd(v) || sqrt_hi(v) < __fsqrt_ru(v)) {
      n_bad++;
      atomicMin(first_bad, (uint32_t)b);
    }
  }
  if (n_bad) atomicAdd(bad, (unsigned long long)n_bad);
}

int check_sqrt_bounds(uint32_t lo_bits, uint32_t hi_bits, unsigned long long* n_bad, uint32_t* first_bad) {
  unsigned long long* d_bad = nullptr;
  if (cudaMalloc((void**)&d_bad, 16) != cudaSuccess) return 1;
  uint32_t* d_first = (uint32_t*)(d_bad + 1);
  cudaMemset(d_bad, 0, 8);
  cudaMemset(d_first, 0xff, 4);
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  sqrt_bounds_kernel<<<sms * 8, 256>>>(lo_bits, hi_bits, d_bad, d_first);
  cudaMemcpy(n_bad, d_bad, 8, cudaMemcpyDeviceToHost);
  cudaMemcpy(first_bad, d_first, 4, cudaMemcpyDeviceToHost);
  const cudaError_t e = cudaGetLastError();
  cudaFree(d_bad);
  return e == cudaSuccess ? 0 : 1;
}

// ---------------------------------------------------------------------------
// peak probe: dependent FMA chains on every SM (roofline denominators)

template <typename T>
__global__ void __launch_bounds__(256) fma_probe_kernel(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + (T)1, x2 = x0 + (T)2, x3 = x0 + (T)3, x4 = x0 + (T)4, x5 = x0 + (T)5,
    x6 = x0 + (T)6, x7 = x0 + (T)7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int k = 0; k < 16; k++) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  T r = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (r == (T)-1.2345) out[threadIdx.x] = r;  // keeps the chains alive
}

float probe_fma_tflops(int fp64, int n_sms) {
  void* out = nullptr;
  cudaMalloc(&out, 1024 * 8);
  const int blocks = n_sms * 8, threads = 256;
  const int iters = fp64 ? 64 : 4096;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 0.f;
  for (int rep = 0; rep < 4; rep++) {
    cudaEventRecord(e0);
    if (fp64) fma_probe_kernel<double><<<blocks, threads>>>((double*)out, iters, 0.999999, 1e-7);
    else fma_probe_kernel<float><<<blocks, threads>>>((float*)out, iters, 0.999999f, 1e-7f);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
    float tf = (float)(flops / (ms * 1e-3) / 1e12);
    if (rep > 0 && tf > best) best = tf;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  return best;
}

}  // namespace px
