/*
 * pixels_gb300 — C ABI of the GB300 scene voxeliser.
 *
 * Drop-in for the reference's world-building path (paths relative to the
 * reference project):
 *   - the sparse voxel store          src/world/VoxelWorld.ts:15-187
 *   - the rasteriser and its Builder  src/world/shapes.ts:334-414, :417-431
 *   - the derived upload buffers      src/gpu/GpuWorld.ts:52-113
 * A host binding (Python ctypes in this repository; an N-API addon for the
 * TypeScript host) records Builder.add/carve/paint calls as
 * a PXIR op list, submits it, and builds on the GPU.  All device memory is
 * owned by the world handle.  Functions return a PX_* status; no C++ exception
 * crosses this boundary; px_last_error() describes the last failure.
 * One host thread per handle.
 */
#ifndef PIXELS_GB300_H
#define PIXELS_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define PX_OK 0
#define PX_E_INVALID_ARG 1    /* bad handle, size or mode */
#define PX_E_INVALID_IR 2     /* malformed op list (bounds, bytecode, NaN/inf parameters) */
#define PX_E_OOM 3            /* device or host allocation failed */
#define PX_E_QUEUE_OVERFLOW 4 /* a device work list ran out of room */
#define PX_E_TIMEOUT 5        /* a bounded device wait gave up */
#define PX_E_CUDA 6           /* CUDA runtime error */
#define PX_E_RANGE 7          /* a paint function got an argument outside its supported range */
#define PX_E_NO_DEVICE 8      /* no CUDA device */
#define PX_E_TOO_LARGE 9      /* input larger than a fixed-size buffer of the library allows */

/* build modes */
#define PX_MODE_FP64 0   /* every decision in float64, as JavaScript numbers */
#define PX_MODE_MIXED 1  /* float32 evaluation, float64 rescue within a certified error bound */

#define PX_UNIFORM 0x80000000u /* grid flag of a uniform brick (VoxelWorld.ts:13) */

typedef struct px_world px_world;

typedef struct px_stats {
  uint64_t ops_applied;      /* ops built into this world so far */
  uint64_t pairs;            /* (op, brick) pairs of the last build */
  uint64_t brick_evals;      /* SDF evaluations at brick centres (last build) */
  uint64_t sub_evals;        /* ... at 4^3 sub-block centres */
  uint64_t voxel_evals;      /* ... at voxel centres */
  uint64_t paint_evals;      /* paint-function calls */
  uint64_t rescued;          /* float32 evaluations re-done in float64 (mixed mode) */
  uint64_t alloc_events;     /* pool allocations replayed */
  uint64_t free_events;      /* pool frees replayed */
  uint32_t pool_used;        /* VoxelWorld.poolUsed */
  uint32_t n_holes;          /* VoxelWorld.freeList.length */
  uint32_t pool_capacity;    /* bricks the device pool can hold */
  uint32_t status;           /* device status bits of the last build */
  double max_abs_err32;      /* max |d32 - d64| seen by rescued evaluations (mixed mode) */
  float build_ms;            /* device time of the last build */
  float fold_ms;             /* device time of its classify + apply kernels */
  uint32_t kernel_launches;  /* kernels the last build launched */
  uint32_t pad;
  uint64_t violations;       /* validation mode: float64 results outside their float32 enclosure */
  uint64_t rescued_brick, rescued_sub, rescued_voxel;  /* rescues by level (mixed mode) */
  uint64_t rescued_polygon;  /* ... of which a polygon crossing test was undecided */
  float classify_ms;         /* device time of the classify and voxel kernels */
  uint32_t rescued_paint;    /* mixed mode: paint calls the float32 path left to float64 */
} px_stats;

/* Device addresses of the world's buffers (valid until the next build or destroy). */
typedef struct px_device_view {
  const uint32_t* grid;      /* bx*by*bz */
  const uint16_t* pool;      /* pool_used * 512 */
  const uint32_t* holes;     /* n_holes, push order */
  const uint32_t* super_counts; /* ceil(bx/4)*ceil(by/4)*ceil(bz/4), after px_derive */
  const uint8_t* density;    /* bx*by*bz, after px_derive */
  const uint32_t* free_list; /* free_len entries: the GPU free list of the last build (derive on build), else NULL */
  uint32_t free_len;
  uint32_t pad;
} px_device_view;

/* new VoxelWorld(dx, dy, dz, initialPoolBricks) at a voxel density (VoxelWorld.ts:35-45;
   VOXEL_SIZE = 1/vpm, config.ts:12-13).  dx, dy, dz: positive multiples of 8. */
int px_world_create(int dx, int dy, int dz, double vpm, uint32_t initial_pool_bricks, px_world** out);
void px_world_destroy(px_world* w);

/* Queue ops (PXIR bytes, pixels_gb300/ir.py) — Builder.add/carve/paint (shapes.ts:417-431). */
int px_submit_ops(px_world* w, const void* ir, size_t bytes);

/* Run every queued op, in order, as apply() would (shapes.ts:334-414), on `stream`
   (a cudaStream_t, NULL = default stream).  px_build waits for the result;
   px_build_enqueue only launches, px_build_finish waits and reports. */
int px_build(px_world* w, int mode, void* stream);
int px_build_enqueue(px_world* w, int mode, void* stream);
int px_build_finish(px_world* w);

/* Empty the world (all air, poolUsed = 0, no holes), like a fresh VoxelWorld of the
   same dims.  requeue_last_ops = 1 queues the ops of the last build again, reusing
   their device copies (rebuilding a scene without re-uploading it). */
int px_world_reset(px_world* w, int requeue_last_ops, void* stream);

/* Reads into caller memory (grid: VoxelWorld.grid; pool: pool[0 .. poolUsed*512);
   holes: freeBricks(), VoxelWorld.ts:173-175). n = capacity of dst in elements. */
int px_read_grid(px_world* w, uint32_t* dst, size_t n);
int px_read_pool(px_world* w, uint16_t* dst, size_t n);
int px_read_holes(px_world* w, uint32_t* dst, size_t n);

/* Derived upload buffers (GpuWorld.ts:52-113): super-grid counts, density
   (red channel of the density texture) and the GPU free list for a pool of
   capacity min(max_bricks, max(used + 98304, 2 used)). */
int px_derive(px_world* w);
int px_read_super(px_world* w, uint32_t* dst, size_t n);
int px_read_density(px_world* w, uint8_t* dst, size_t n);
int px_read_free_list(px_world* w, uint32_t max_bricks, uint32_t* dst, size_t n, uint32_t* out_len);

/* Derive on build: with max_bricks > 0 every later build ends, on the device and
   on its stream, with the super-grid counts, the density bytes and the GPU free
   list for a device limit of max_bricks pool bricks (GpuWorld.ts:55-60,90-111:
   the free list is the holes in push order, then cap - 1 down to poolUsed), so
   a build leaves every upload buffer in HBM with no host step.  px_read_super /
   px_read_density / px_read_free_list (with the same max_bricks) then copy them
   out.  A world whose poolUsed exceeds the capacity gets no free list
   (px_read_free_list returns PX_E_OOM, as GpuWorld.ts:59 throws).  0 turns it
   off (the derived buffers are then computed when first read). */
int px_set_derive_on_build(px_world* w, uint32_t max_bricks);

/* The same super-grid counts and density bytes as px_derive, from a grid (bx*by*bz
   entries, bricks) and a pool (n_pool_bricks * 512 voxels) that the caller holds
   on the current device, written into caller-held device buffers super_counts
   (ceil(bx/4)*ceil(by/4)*ceil(bz/4)) and density (bx*by*bz); the material tables
   are host arrays of 256 bytes (as px_set_material_tables).  No counterpart in
   the reference (GpuWorld.ts:90-101 computes these with its world); this entry
   point exists for callers that must not allocate device memory once they run
   (fixed device budgets, frame loops): it allocates nothing and uses a fixed
   scratch area of 2 MiB + 256 bytes inside the library, which limits
   n_pool_bricks to PX_NOALLOC_MAX_POOL_BRICKS (larger: PX_E_TOO_LARGE, no GPU
   work).  The first call on each device looks up that area, with the device
   current; make it before any stream capture on that device, and do not call
   it on a device reset (cudaDeviceReset) since that first call.  grid, pool
   and super_counts must be 4-byte aligned (else PX_E_INVALID_ARG, no GPU
   work).  All calls share the area, so calls that overlap in time race:
   serialise them.  Returns after the work on `stream` has finished;
   PX_E_INVALID_ARG also when the grid names a pool brick >= n_pool_bricks
   (that cell's density is written as 0). */
#define PX_NOALLOC_MAX_POOL_BRICKS 1048576u
int px_derive_noalloc(const uint32_t* grid, const uint16_t* pool, int bx, int by, int bz, uint32_t n_pool_bricks,
                      const uint8_t* opaque256, const uint8_t* uniform_density256, uint32_t* super_counts,
                      uint8_t* density, void* stream);

/* snapToEmissive (GpuWorld.ts:165-174) for n light anchors of the built world in
   one launch: xyz / out_xyz hold n voxel coordinates (x, y, z) each; every anchor
   moves to the first voxel of the cubes of radius 0, 1, 2 around it (z, then y,
   then x outermost first, each from -r to r) whose material emits, else stays.
   emission256[id]: 0 no emission, 1 emits, 2 no such material (the reference
   throws there: PX_E_INVALID_ARG).  packLights (GpuWorld.ts:141-162) lays the
   result out on the host. */
int px_snap_anchors(px_world* w, const int32_t* xyz, size_t n, const uint8_t* emission256, int32_t* out_xyz);

/* Material tables for the density pass: opaque[id] (OPAQUE, VoxelWorld.ts:190-196) and the
   density of a uniform brick of material id (VoxelWorld.ts:162).  256 bytes each. */
int px_set_material_tables(px_world* w, const uint8_t* opaque256, const uint8_t* uniform_density256);

/* Validation mode for the mixed form (testing aid, slow): every float32
   evaluation is also done in float64 and checked against its enclosure;
   stats.violations counts failures (must stay 0). */
int px_set_validation(px_world* w, int on);

int px_get_stats(px_world* w, px_stats* out);
/* Grow the device pool to at least `bricks` bricks now (the contents are kept),
   so that later builds do not stop to grow it; GpuWorld.ts:57 sizes the GPU
   pool to max(used + 98304, 2 used) at upload in the same spirit. */
int px_reserve_pool(px_world* w, uint64_t bricks);
int px_device_view_get(px_world* w, px_device_view* out);
/* Dims (voxels) and voxel density of a world. */
int px_world_info(px_world* w, int dims[3], double* vpm);

/* ---- serving: subtract-edits on a resident world (continuous batching) ----
   The game's carve as the rasteriser sees it: Builder.carve of a sphere
   (shapes.ts:65-72) or capsule (shapes.ts:114-128), appended to the world's
   op history (shapes.ts:423-426). */
#define PX_EDIT_SPHERE 0
#define PX_EDIT_CAPSULE 1
typedef struct px_edit {
  uint32_t shape;      /* PX_EDIT_SPHERE (centre a) or PX_EDIT_CAPSULE (segment a-b) */
  uint32_t pad;
  double a[3], b[3];
  double r;            /* radius in metres (capsules clamp to 0.9 voxel, shapes.ts:115) */
} px_edit;
typedef struct px_edit_result {
  uint64_t id;         /* index into the edits array */
  uint32_t status;     /* PX_OK, or PX_E_OOM when the edit cannot fit the pool budget */
  uint32_t batch;      /* build step that applied it */
  double arrival_s, start_s, done_s;  /* seconds since the run started */
  double dev_start_ms, dev_end_ms;    /* its build step's first and last kernel on the device,
                                         ms since the run started on the device */
} px_edit_result;
/* Serve `n` edits arriving at arrival_s[i] (seconds from now): a producer
   releases them in real time; each build step takes every released edit, in
   arrival order, up to max_batch, whose worst-case pool growth (bricks in its
   box) fits pool_budget_bricks minus the live bricks (and the steps still in
   flight), and builds them together on the resident world.  Steps overlap on
   the device: a step's evaluation passes (classify, sub-block, voxel, paint:
   independent of the world's state) run on `stream` while the previous step's
   apply pass, allocator replay and commit run on a second stream; steps commit
   in admission order, so the world equals the edits applied one after another
   (shapes.ts:423-426).  Before the first edit the pool is reserved to
   min(pool_budget_bricks, max(used + 98304, 2 used)) bricks (GpuWorld.ts:57).
   applied_order (n entries, may be NULL) receives the edit indices in the
   order applied.  Blocks until every edit is applied or rejected; a step that
   fails (PX_E_QUEUE_OVERFLOW) ends the run with the world as it was before it. */
int px_serve_run(px_world* w, const px_edit* edits, const double* arrival_s, size_t n, uint32_t max_batch,
                 uint64_t pool_budget_bricks, int mode, void* stream, px_edit_result* results,
                 uint64_t* applied_order, size_t* n_applied);
const char* px_last_error(px_world* w);

/* ---- batched builds: many scenes in one CUDA graph ----
   No counterpart in the reference (it builds one world); the per-scene result
   is the reference's apply() loop over that scene's ops (shapes.ts:334-431).
   px_batch_create takes worlds that each hold a built scene (px_build done,
   no ops queued), rebuilds each once from its last op list to size every
   buffer, then captures the rebuild of all of them (reset + the same ops) into
   one graph over n_streams streams (1-256), largest scenes first; pairs_per_block
   sizes each scene's persistent grids to its (op, brick) pairs (0: whole GPU
   per kernel).  px_batch_run launches the graph on `stream`, waits, and
   updates every world (reads work as after px_build); device_ms (may be NULL)
   receives the graph's device time.  While a batch exists its worlds cannot
   be rebuilt, reset or destroyed (PX_E_INVALID_ARG; destroy is ignored). */
typedef struct px_batch px_batch;
int px_batch_create(px_world* const* worlds, size_t n, int mode, uint32_t n_streams, uint32_t pairs_per_block,
                    px_batch** out);
int px_batch_run(px_batch* b, void* stream, float* device_ms);
void px_batch_destroy(px_batch* b);
const char* px_batch_last_error(px_batch* b);

/* Measurement utility (no counterpart in the reference): dependent-FMA
   throughput of this GPU's CUDA cores in TFLOP/s, float64 (fp64 = 1) or
   float32 (fp64 = 0) — the denominators of the voxeliser's ALU roofline. */
int px_probe_peak(int fp64, float* tflops);

/* Self-check of the mixed form's float32 square-root bounds (no counterpart in
   the reference): for every float whose bit pattern lies in [lo_bits, hi_bits]
   (positive, finite), the lower and upper bounds the interval evaluator uses
   must enclose the IEEE directed square roots of this GPU; n_bad receives the
   failures (must be 0) and first_bad the smallest failing bit pattern. */
int px_check_sqrt_bounds(uint32_t lo_bits, uint32_t hi_bits, uint64_t* n_bad, uint32_t* first_bad);

#ifdef __cplusplus
}
#endif
#endif /* PIXELS_GB300_H */
