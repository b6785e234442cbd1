// Shared definitions of the voxeliser's host runtime and kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace px {

constexpr uint32_t UNIFORM = 0x80000000u;  // VoxelWorld.ts:13
constexpr int BRICK = 8;
constexpr int BRICK_VOXELS = 512;
constexpr int TILE = 4;                    // tiles are the 4^3-brick super cells (GpuWorld.ts:52)
constexpr int MAX_STACK = 4;               // SDF value-stack depth the register evaluators hold
constexpr int MAX_ROT = 3;                 // nested rotation frames they hold
// Deeper programs (nested CSG / rotation trees) run on the float64 evaluator
// with a stack in local memory (sdf64_deep), up to these depths.
constexpr int DEEP_MAX_STACK = 32;
constexpr int DEEP_MAX_ROT = 16;
constexpr int MAX_AXIS_BRICKS = 1023;      // op brick boxes pack 10 bits per axis

// op kinds (shapes.ts:325-330)
enum : uint8_t { KIND_ADD = 0, KIND_CARVE = 1, KIND_PAINT = 2 };

// SDF bytecode opcodes (pixels_gb300/ir.py)
enum : uint32_t {
  OP_BOX = 1, OP_ROUNDBOX = 2, OP_SPHERE = 3, OP_ELLIPSOID = 4,
  OP_CYL_X = 5, OP_CYL_Y = 6, OP_CYL_Z = 7, OP_CAPSULE = 8,
  OP_TORUS_X = 9, OP_TORUS_Y = 10, OP_TORUS_Z = 11,
  OP_LATHE_SOLID = 12, OP_LATHE_SHELL = 13, OP_PRISM = 14, OP_STADIUM = 15,
  OP_ROT_X = 20, OP_ROT_Y = 21, OP_ROT_Z = 22, OP_ROT_END = 23,
  OP_OFFSET = 24, OP_NEGMAX = 25, OP_MAX = 26, OP_MIN = 27,
};

// paint kinds
enum : uint16_t {
  PK_CONST = 0, PK_CHIP = 1, PK_TUFTED = 2, PK_CARD = 3, PK_WHITE = 4, PK_BLACK = 5,
  PK_VASE = 6, PK_PAINTING = 7, PK_NOISE = 8, PK_COUNT = 9,
};
constexpr int PAINT_NPARAMS[PK_COUNT] = {0, 5, 3, 4, 2, 2, 5, 37, 8};

enum : uint8_t { OPF_CONTAINS = 1, OPF_HAS_SLACK = 2, OPF_PAINT_FRAME = 4, OPF_DEEP = 0x10, OPF_Y_SEPARABLE = 0x20,
                 OPF_BOX_RANGES = 0x40, OPF_FP64_ONLY = 0x80 };
constexpr uint8_t OPF_FROM_IR = OPF_CONTAINS | OPF_HAS_SLACK | OPF_PAINT_FRAME;  // flags an op list may set

// Mixed mode: margin between the exact value of an expression on the float64
// inputs and the reference's float64 result (valid for |values| <= 2^10 m).
constexpr double MIXED_MARGIN = 0x1p-30;
constexpr double MIXED_MAX_COORD = 1024.0;

// per-op float32 thresholds of the mixed mode (certified comparisons)
enum { T_BSK_HI, T_BSK_LO, T_BFU_HI, T_BFU_LO, T_SSK_HI, T_SSK_LO, T_SFU_HI, T_SFU_LO, T_V_HI, T_V_LO, T_M, T_COUNT };

// device status bits (first error wins for the reported code)
enum : uint32_t {
  ST_OK = 0, ST_STAGE_OVERFLOW = 1, ST_POOL_OVERFLOW = 2, ST_RANGE = 4, ST_CHAIN = 8,
  ST_FREE_CAP = 16,  // derive: poolUsed exceeds the GPU pool capacity (GpuWorld.ts:59 throws)
  ST_RESCUE_OVERFLOW = 32,  // the list of voxels left to float64 ran out of room (the build commits nothing)
};
// a build's failures: it commits nothing and the host retries with larger buffers or reports
constexpr uint32_t ST_NO_COMMIT = ST_STAGE_OVERFLOW | ST_CHAIN | ST_RESCUE_OVERFLOW;

// PXIR op record (128 bytes, pixels_gb300/ir.py OP_DTYPE)
struct IrOp {
  uint8_t kind, flags;
  uint16_t paint_kind;
  uint32_t paint_value, paint_param, code_begin, code_len, pad0;
  double mn[3], mx[3], slack;
  double frame[4];
  double pad1[2];
};
static_assert(sizeof(IrOp) == 128, "PXIR op is 128 bytes");

// An op as the kernels see it.
struct OpDev {
  int32_t bx0, by0, bz0, bx1, by1, bz1;  // brick box (inclusive), from apply()'s voxel range
  int32_t nx, ny;                        // box extent in bricks (x, y)
  uint64_t pair_base;                    // index of the op's first (op, brick) pair
  // ceil(2^64 / nx) and ceil(2^64 / (nx ny)) (0 for a divisor of 1): a pair's brick
  // row and slab by one 64-bit high multiply instead of a division (brick_of_pair)
  uint64_t inv_nx, inv_nxy;
  uint32_t code_off, code_len;           // SDF bytecode (uint2 records)
  uint32_t paint_off;                    // paint parameters (doubles)
  uint8_t kind, flags;
  uint16_t paint_kind;
  uint32_t paint_value;
  uint32_t vclass;                       // sub-block work class (VCLASSES): first primitive, y-extruded
  uint32_t vq_class;                     // voxel work class (VQ_CLASSES): 32 per VQ_* group
  // a program of the lean voxel kernel (LP_* forms; lp[LP_FORM] == 0: not one): instruction
  // indices within the op of its primitives, stages and offset, and the stages' kinds
  uint8_t lp[8];
  double bhd, shd;                       // brickHalfDiag, subHalfDiag (shapes.ts:349-350)
  double mn[3], mx[3];                   // contains box (boxes only)
  double frame[4];                       // paint frame px, pz, cos, sin
  double anchor[3];                      // mixed mode: origin of the op's float32 coordinates
  float thr[12];                         // mixed mode thresholds (T_*)
  int32_t cbx0, cby0, cbz0, cbx1, cby1, cbz1;  // bricks the box fully contains (contains(), shapes.ts:47-48,360)
  uint32_t base_off;                     // mixed mode: float32 first-voxel-centre offsets per brick row
  float cost;                            // relative cost of one evaluation (work order only)
  // OPF_BOX_RANGES (a lone axis-aligned box): per axis, the first and last voxel
  // whose centre the reference's float64 box SDF puts inside on that axis
  int32_t vr[6];                         // x lo, x hi, y lo, y hi, z lo, z hi (empty: lo > hi)
  // paints evaluated ahead of the apply pass (paint_kernel): the op's first
  // paint slot (one slot of 512 values per (op, brick) pair), or NO_SLOT
  uint32_t paint_slot;
  // mixed mode: float32 parameters of the certified paint evaluation (p32 index), or NO_SLOT
  uint32_t paint32_off;
  // mixed mode: a voxel of a partial sub-block is outside if the sub-block centre's
  // value exceeds lip[k], inside if it is below -lip[k] (k: the voxel's distance class
  // from the centre; every shape's SDF is Lipschitz with constant <= its slack)
  float lip[4];
};
constexpr uint32_t NO_SLOT = 0xffffffffu;
// paint kinds whose calls are the most expensive (transcendentals, Math.hypot):
// chip stack, tufted, vase, painting.  Their calls are evaluated ahead of the
// apply pass whenever the slots fit; the other kinds when all painted ops fit.
__host__ __device__ constexpr bool paint_is_heavy(uint32_t k) {
  return k == PK_CHIP || k == PK_TUFTED || k == PK_VASE || k == PK_PAINTING;
}
// a precomputed paint value with a paint argument out of range (ST_RANGE)
constexpr uint32_t PV_RANGE = 0x80000000u;

struct BuildCounters {
  unsigned long long brick_evals, sub_evals, voxel_evals, paint_evals, rescued;
  unsigned long long alloc_events, free_events;
  unsigned long long violations;  // validation mode: float64 results outside the float32 enclosure
  unsigned long long resc_brick, resc_sub, resc_vox, resc_poly;  // rescues by level; polygon-test ambiguity
  unsigned long long resc_paint;  // mixed mode: paint calls the float32 path could not decide
};

// The world's allocator state on the device (VoxelWorld.poolUsed and the
// free-list length), written by the finalize kernel of each build that commits
// and read by the next build's allocator replay, so that builds can be queued
// before the previous one has returned to the host.  A build that commits
// nothing sets `poisoned`; every later build then commits nothing either,
// until the host clears it.
struct WorldState {
  uint32_t pool_used, n_holes, poisoned, pad;
};

// Small device block read back after every build.
struct BuildResult {
  uint32_t status;
  uint32_t n_events;     // H + N
  uint32_t pool_used;    // after the build
  uint32_t n_holes;      // after the build
  uint32_t stage_count;  // bricks that end as pool bricks and were touched (staging slots wanted)
  uint32_t touched_count;  // bricks whose grid entry the build rewrites
  uint32_t n_work;       // bricks with at least one (op, brick) pair that is not skipped
  uint32_t n_fresh;
  uint32_t max_pool_index;
  BuildCounters c;
  unsigned long long max_err_bits;  // max |mid(d32) - d64| over rescued evaluations (double bits, >= 0)
  uint32_t free_len;     // derive: length of the GPU free list (GpuWorld.ts:103-111, C_FREE_TOP)
  uint32_t n_rescue;     // voxels the float32 pass left to float64 (voxel_lean_kernel), pushed
  uint32_t h_before;     // holes before the build (from the WorldState)
  uint32_t u_before;     // poolUsed before the build
  uint32_t pad2;
};

// Pair classification (state independent): class per (op, brick) pair, the 8
// sub-block classes of partial pairs, and voxel inside-masks of partial sub-blocks.
enum : uint8_t { PC_SKIP = 0, PC_PARTIAL = 1, PC_FULL = 2 };

// Work items of the sub-block and voxel passes are grouped by the op's shape
// (its first primitive, and whether it runs the y-extruded evaluation), so
// that warps draining a queue at the same time run the same code.
constexpr int VCLASSES = 32;
// The voxel queue has four groups of 32 classes, each drained by its own
// kernel: VQ_NARROW, lean programs of one primitive under at most one rotation
// (by primitive and rotation), VQ_AFFINE, one primitive under a composed run of
// rotations (by primitive), VQ_WIDE, the two-primitive lean programs (by first
// primitive and form), and VQ_GENERIC, every other program (by sub-block class),
// drained by the interpreter kernel.
enum { VQ_NARROW = 0, VQ_AFFINE = 1, VQ_WIDE = 2, VQ_GENERIC = 3 };
constexpr int VQ_CLASSES = 128;
constexpr int VQ_TAKEN = 1 + VQ_CLASSES;  // vitem_counter[VQ_TAKEN + group]: items the group's kernel took
constexpr int CULL_COUNTER = 200;         // chunk_counter[CULL_COUNTER]: tile-list entries reserved by cull_kernel

// Programs of the lean voxel kernels, by form:
//   1  [stage] prim [stage end] [offset]
//   2  [stage] prim prim comb [stage end] [offset]           (one stage for both)
//   3  [stage] prim [stage end] [stage] prim [stage end] comb [offset]
// A stage is one rotation (kind 1-3: about x, y, z) or a run of rotations the
// float32 parameters hold composed into one affine map (kind 4); comb is a
// subtract step, an intersection or a union.
enum { LP_FORM, LP_COMB, LP_P1, LP_P2, LP_S1, LP_S2, LP_KINDS, LP_OFF };
enum : uint8_t { LP_NEGMAX = 1, LP_MAX = 2, LP_MIN = 3, LP_NONE = 0xff, LP_AFFINE = 4 };
// code32 flags of the float32 path: a run of rotations (not all about y) composed
// into an affine map on its first rotation; its other rotations and all but the
// first of its ends are skipped
constexpr uint32_t C32_SKIP = 1u << 31, C32_AFFINE = 1u << 30, C32_OFF = (1u << 30) - 1;

struct FoldArgs {
  const uint2* chunk_order;  // the 32-pair chunks in the order classify_kernel takes them (costliest ops
                             // first): (chunk, op containing its first pair | 1 << 31 when that op holds
                             // all of the chunk's pairs)
  uint8_t class_order[VCLASSES];  // the order the sub-block pass takes its classes in
  uint8_t vclass_order[VQ_CLASSES];  // the order the voxel passes take theirs, group by group
  uint32_t vq_nonempty;              // bit g: group g has work (its kernel is launched)
  uint32_t n_ops;
  unsigned long long n_pairs;
  uint8_t* pcode;             // per pair: PC_*
  uint16_t* psub;             // per partial pair: 2 bits per sub-block (PC_*)
  unsigned long long* pmask;  // per partial pair: 8 inside-masks (bit = x&3 | (y&3)<<2 | (z&3)<<4)
  uint32_t* chunk_counter;
  // voxels whose float32 interval cannot decide them, left by voxel_lean_kernel to
  // paint_kernel<1> (which resolves them in float64 first): (op | voxel bit << 24 |
  // undecided-crossing-test << 30, pair << 3 | sub-block, interval lo, hi bits)
  uint4* rescue;
  uint32_t rescue_cap;
  uint4* vitems;              // partial sub-blocks to classify voxel by voxel: (op, pair << 3 | sub,
                              // bits of the centre value's enclosure lo, hi)
  uint32_t vitems_cap;
  uint32_t* vitem_counter;    // [1 + k] items pushed to class k, [VQ_TAKEN + g] items taken from group g
  uint32_t vq_base[VQ_CLASSES], vq_cap[VQ_CLASSES];  // per-class regions of vitems
  uint2* pitems;              // partial pairs for the sub-block pass: (op, pair)
  uint32_t* pitem_counter;    // [0] items taken, [1 + k] items pushed to class k
  uint32_t pq_base[VCLASSES], pq_cap[VCLASSES];  // per-class regions of pitems
  uint32_t* paint_counter;    // paint_kernel items taken
  uint32_t n_paint_slots;     // (op, brick) pairs of painted ops with a slot
  uint2* paint_items;         // sub-blocks to paint: (op, pair << 3 | sub-block), from classify and sub;
                              // float64 paints from the front, certified float32 ones from the back
  uint32_t paint_items_cap;
  uint32_t* paint_item_counter;  // items pushed: [0] at the front, [1] at the back
  uint32_t* pvals;            // 512 paint values per slot (voxel index order); PV_RANGE flags
  int inline_paints;          // some painted op has no slot: fold_kernel calls its paints itself
  uint32_t* bmark;            // one bit per brick: some pair of it is not skipped (classify_kernel)
  uint32_t* work;             // those bricks, listed by their first marking pair: bricks of tiles with more
                              // than 8 ops from the front, the others from the back (touched_cap down)
  const OpDev* ops;
  const uint2* code;
  const double* params;
  const uint32_t* code32;     // per instruction: offset of its float32 interval parameters
  const float2* p32;          // float32 interval parameters (lo, hi)
  const float2* bases;        // per op and axis: (b*8 + 0.5)*vs - anchor as a float32 interval
  float vs_lo, vs_hi;         // float32 enclosure of the voxel size
  // float32 roundings of the voxel centres' float64 coordinates ((i + 0.5) * vs), per axis
  const float *ax32, *ay32, *az32;
  int validate;               // mixed mode: also evaluate float64 everywhere and count violations
  const uint32_t* tile_off;
  const uint32_t* tile_cnt;
  const uint32_t* tile_ops;
  const uint2* tile_boxes;    // the brick box of each tile_ops entry (packed like the op boxes)
  int BX, BY, BZ, TX, TY;
  double vs;
  uint32_t* grid;
  const uint32_t* pool32;     // pool viewed as voxel pairs
  uint8_t* evt;               // per pair: 1 = alloc, 2 = free, 3 = both
  int64_t* fsrc;              // per pair with a free: pair of the brick's last alloc, or -(old index + 1)
  uint32_t* staging32;
  uint32_t stage_cap;
  uint32_t* stage_cell;
  int64_t* stage_src;
  uint2* touched;             // (cell, final tag): 0, UNIFORM|v, or STAGED|slot
  uint32_t touched_cap;
  uint32_t* work_counter;     // [0] apply-pass takes, [1] front bricks, [2] back bricks
  BuildResult* res;
};

// touched-list tag of a brick that ends as a pool brick: its staging slot
constexpr uint32_t TAG_STAGED = 0x40000000u;

// Host-side launch wrappers (kernels.cu)
// counter: a zeroed word (the tile lists' reservation count).  sorted: boxes holds
// the op boxes, the union boxes of 32 ops in the order after them, then that order
// (cull_sorted_kernel, up to CULL_SORTED_MAX_OPS ops); else the union boxes of 32
// consecutive ops
constexpr int CULL_SORTED_MAX_OPS = 47 * 1024;  // 8 warps x ops / 8 bytes of shared memory: 47 KiB
void launch_cull(const uint2* boxes, int n_ops, int TX, int TY, int TZ, uint32_t* tile_cnt, uint32_t* tile_off,
                 uint32_t* tile_ops, uint2* tile_boxes, uint32_t* counter, bool sorted, cudaStream_t s);
// max_blocks > 0 caps the persistent grids (builds sharing the GPU)
// The evaluation passes (classify .. paint) go on s; the apply pass on s_apply,
// after eval_done is recorded on s (s_apply == s: one stream, no event).
void launch_fold(const FoldArgs& a, int mode, int n_sms, cudaStream_t s, cudaEvent_t mid, int max_blocks,
                 cudaStream_t s_apply, cudaEvent_t eval_done);



// The allocator replay's look-back scratch: counters and flags (cleared by
// every build: replay_clear_bytes from `counters`) and the published tile
// aggregates and inclusive prefixes (event count and depth map, x/y/z).
struct ReplayTemp {
  uint32_t* counters;  // [0] pair-tile tickets, [2] blocks done
  uint32_t* flag;      // per pair tile (0 pending, 1 aggregate, 2 prefix)
  int4* agg;
  int4* incl;
};
// threads per block of the replay's event scan (128, 256 and 512 measured: 128
// gave the fastest build, by 0.5-1%)
#ifndef PX_REPLAY_THREADS
#define PX_REPLAY_THREADS 128
#endif
constexpr int REPLAY_TILE = PX_REPLAY_THREADS * 8;  // pairs per look-back tile (a block, 8 per thread)
// bytes of the replay scratch for P pairs, and of its cleared part
size_t replay_temp_bytes(uint64_t P);
size_t replay_clear_bytes(uint64_t P);
ReplayTemp replay_temp(void* base, uint64_t P);

struct TreeLevels {
  size_t off[8];  // offsets (in int32) of levels 1.. in the tree buffer
  int n;          // levels above the depth array
};
TreeLevels tree_levels(size_t E_max);
// bytes of levels 1 and 2 of the min tree, which every build clears to the
// byte value 0x7f before the replay fills them by atomicMin
size_t tree_clear_bytes(size_t E_max);

struct ReplayArgs {
  size_t P;                 // pairs
  size_t E_max;             // bound of H + 2P (H: holes before the build)
  uint32_t H_max;           // bound of H (launch sizes only)
  const WorldState* state;  // H and poolUsed before the build, copied to res->h_before / u_before
  const uint8_t* evt;
  const int64_t* fsrc;
  const uint32_t* holes_in;
  uint32_t* pos;            // P: first event of each pair that allocates (after the H initial holes)
  uint8_t* etype;           // E_max
  unsigned long long* ew;   // E_max: the pool index of each event once resolved (KNOWN | index)
  int32_t* depth;           // E_max (+ 32): stack depth after each event
  int32_t* tree;            // levels of the min tree above depth
  TreeLevels tl;
  uint32_t* holes_out;      // >= E_max
  BuildResult* res;
  ReplayTemp t;
};
void launch_replay(const ReplayArgs& a, cudaStream_t s);

struct FinalizeArgs {
  const uint2* touched;
  const uint32_t* staging32;
  const uint32_t* stage_cell;
  const int64_t* stage_src;
  const uint32_t* pos;
  const unsigned long long* ew;
  uint32_t* holes_out;      // the holes after the build: event indices in, pool indices out
  WorldState* state;        // committed: the build's poolUsed and hole count
  uint32_t* grid;
  uint32_t* pool32;
  uint32_t pool_cap;
  BuildResult* res;
  // per pool brick: its opaque, non-air voxels (cellDensity's count, VoxelWorld.ts:163-169),
  // written for every brick the build writes to the pool
  const uint8_t* opaque;
  uint16_t* pcount;
};
void launch_finalize(const FinalizeArgs& a, uint32_t touched_cap, cudaStream_t s);

// Host-to-device copies and device clears done by one kernel: an entry with a
// source copies it (read straight from host memory: only where the device
// reports pageable memory access through the host page tables), one without
// zeroes its destination.  Sources and destinations 16-byte aligned.
struct HostUploads {
  static constexpr int kMax = 16;
  struct Entry {
    const void* src;
    void* dst;
    size_t bytes;
    uint32_t fill;  // without a source: the byte value of the clear, in all four bytes
  } e[kMax];
  int n;
};
void launch_uploads(const HostUploads& u, cudaStream_t s);

// Derived upload buffers of a world (GpuWorld.ts:52-109): super-grid counts,
// density bytes and, when free_list is set, the GPU free list -- the holes in
// push order, then cap - 1 down to poolUsed, cap = min(max_bricks,
// max(used + 98304, 2 used)).  With res set the kernel is the last step of a
// build: poolUsed and the hole count come from the build's result, and a
// build that committed nothing derives nothing.
struct DeriveArgs {
  const uint32_t* grid;
  const uint32_t* pool32;
  int BX, BY, BZ;
  const uint8_t* opaque;
  const uint8_t* udens;
  uint32_t* super_counts;
  uint8_t* density;
  const uint32_t* holes;  // the world's holes after the build
  uint32_t* free_list;    // nullptr: no free list
  uint32_t free_cap;      // entries free_list holds
  uint32_t max_bricks;
  BuildResult* res;
  // pool bricks' opaque counts: read from pcount when it holds every referenced
  // brick's count (kept by the builds' finalize), else counted from the pool and
  // written to pcount_out
  const uint16_t* pcount;
  uint16_t* pcount_out;
};
void launch_derive(const DeriveArgs& a, cudaStream_t s);
// entries the GPU free list of a pool of `pool_cap` bricks can need
__host__ __device__ inline uint64_t free_list_bound(uint64_t pool_cap, uint64_t max_bricks) {
  const uint64_t c = pool_cap + 98304 > 2 * pool_cap ? pool_cap + 98304 : 2 * pool_cap;
  return c < max_bricks ? c : max_bricks;
}

// Build kernels launched by this thread overlap their predecessors' tails
// (programmatic dependent launch) unless switched off (graph captures).
void set_programmatic_launch(bool on);
float probe_fma_tflops(int fp64, int n_sms);
// failures of the float32 evaluator's square-root bounds over float bit patterns [lo_bits, hi_bits]
int check_sqrt_bounds(uint32_t lo_bits, uint32_t hi_bits, unsigned long long* n_bad, uint32_t* first_bad);
unsigned long long launch_count();

}  // namespace px

struct px_world;
namespace px {
// Serving (px_api.cu): allocate ahead the scratch of any build of at most P
// (op, brick) pairs and max_ops one-instruction ops without paint slots, and
// the pool room its staging guess needs; the staging slots such a build
// reserves.
int reserve_build_scratch(px_world* w, uint64_t P, uint32_t max_ops);
uint64_t build_stage_slots(const px_world* w, uint64_t P);
// Pipelined builds (serving): a twin of a world over the same grid, pool,
// opaque counts, free list and device state, with build scratch of its own,
// so that one build's evaluation passes can run on the device while the
// other's apply pass does.  Builds on either commit to the shared world in the
// order their apply passes are queued on the apply stream.
px_world* twin_create(px_world* w, uint64_t P, uint32_t max_ops, int* rc);
void twin_destroy(px_world* t);
// Queue settings of a pipelined world: the apply pass on `apply` (NULL: the
// build's stream), no retries, and the host's view of the shared allocator
// state before the build (holes parity, bounds of poolUsed and the hole count).
void pipeline_set(px_world* w, cudaStream_t apply, bool holes_in_a, uint32_t pool_used_bound, uint32_t n_holes_bound);
// The committed allocator state a pipeline starts from (and ends with).
struct PipelineState {
  uint32_t pool_used, n_holes;
  bool holes_in_a;
  uint32_t derive_max;  // the world's derive-on-build setting, off while pipelined
  uint32_t pairs_per_block;  // the world's persistent-grid sizing, restored after the pipeline
};
PipelineState pipeline_begin(px_world* w);
// After the last pipelined build: the world takes over the committed state,
// counts `ops` more ops applied, clears a poisoned device state and restores
// derive on build.
void pipeline_end(px_world* w, const PipelineState& st, uint64_t ops, cudaStream_t s);
// The build's result block is on the host (px_build_finish would not wait).
bool build_done(px_world* w);
// Device times (ms since `base`) of the last finished build's first and last kernels.
void build_times(px_world* w, cudaEvent_t base, double* start_ms, double* end_ms);

}  // namespace px
