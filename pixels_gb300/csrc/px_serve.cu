// Serving: continuous batching of subtract-edits on a resident world.
//
// The game's carve is a Carve op of a sphere or capsule (shapes.ts:65-72,
// 114-128, 423-426).  A producer thread releases requests at their arrival
// times; the serving loop takes every released request (in arrival order, up
// to max_batch) whose worst-case pool growth fits the free pool, builds them in
// one incremental build on the resident world (the same kernels as a scene
// build, starting from the world's current grid, pool and free list), and
// stamps their completion.  Requests that arrive while a batch is on the GPU
// join the next batch.  The world after any sequence of batches equals the
// reference applying the same carves one after another in admission order.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <atomic>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "../../include/pixels_gb300.h"
#include "px_internal.cuh"

using namespace px;

namespace {

using clock_t_ = std::chrono::steady_clock;

double secs(clock_t_::time_point t0, clock_t_::time_point t) { return std::chrono::duration<double>(t - t0).count(); }

// PXIR encoding of one carve (the constructors of shapes.ts, float64 as in JS)
void encode_carve(const px_edit& e, double vs, std::vector<IrOp>& ops, std::vector<uint32_t>& code,
                  std::vector<double>& params) {
  IrOp o;
  std::memset(&o, 0, sizeof o);
  o.kind = KIND_CARVE;
  o.flags = 0;
  o.paint_kind = PK_CONST;
  o.paint_value = 0;
  o.code_begin = (uint32_t)(code.size() / 2);
  o.code_len = 1;
  o.slack = 1.0;
  o.frame[2] = 1.0;
  const uint32_t off = (uint32_t)params.size();
  if (e.shape == PX_EDIT_SPHERE) {  // shapes.ts:65-72
    const double cx = e.a[0], cy = e.a[1], cz = e.a[2], r = e.r;
    params.insert(params.end(), {cx, cy, cz, r});
    code.push_back(OP_SPHERE);
    code.push_back(off);
    o.mn[0] = cx - r; o.mn[1] = cy - r; o.mn[2] = cz - r;
    o.mx[0] = cx + r; o.mx[1] = cy + r; o.mx[2] = cz + r;
  } else {  // shapes.ts:114-128
    const double min_line_r = 0.9 * vs;
    const double r = e.r > min_line_r ? e.r : min_line_r;
    const double ax = e.a[0], ay = e.a[1], az = e.a[2];
    const double bax = e.b[0] - ax, bay = e.b[1] - ay, baz = e.b[2] - az;
    double bb = bax * bax + bay * bay + baz * baz;
    if (bb == 0 || bb != bb) bb = 1e-12;
    params.insert(params.end(), {ax, ay, az, bax, bay, baz, bb, r});
    code.push_back(OP_CAPSULE);
    code.push_back(off);
    const double* b = e.b;
    o.mn[0] = std::min(ax, b[0]) - r; o.mn[1] = std::min(ay, b[1]) - r; o.mn[2] = std::min(az, b[2]) - r;
    o.mx[0] = std::max(ax, b[0]) + r; o.mx[1] = std::max(ay, b[1]) + r; o.mx[2] = std::max(az, b[2]) + r;
  }
  ops.push_back(o);
}

// Bricks an edit can touch (the brick box of apply(), shapes.ts:341-347): the
// most pool bricks it can add.
uint64_t brick_bound(const px_edit& e, double vs, int dx, int dy, int dz) {
  double lo[3], hi[3];
  double r = e.r;
  if (e.shape == PX_EDIT_SPHERE) {
    for (int k = 0; k < 3; k++) { lo[k] = e.a[k] - r; hi[k] = e.a[k] + r; }
  } else {
    r = std::max(r, 0.9 * vs);
    for (int k = 0; k < 3; k++) { lo[k] = std::min(e.a[k], e.b[k]) - r; hi[k] = std::max(e.a[k], e.b[k]) + r; }
  }
  const int dims[3] = {dx, dy, dz};
  uint64_t n = 1;
  for (int k = 0; k < 3; k++) {
    double v0 = std::max(0.0, std::floor(lo[k] / vs - 0.5)), v1 = std::min((double)dims[k] - 1, std::ceil(hi[k] / vs + 0.5));
    if (v0 > v1) return 0;
    n *= (uint64_t)(((int)v1 >> 3) - ((int)v0 >> 3) + 1);
  }
  return n;
}

}  // namespace

extern "C" {

static int serve_run_impl(px_world* w, const px_edit* edits, const double* arrival_s, size_t n, uint32_t max_batch,
                 uint64_t pool_budget_bricks, int mode, void* stream, px_edit_result* results, uint64_t* applied_order,
                 size_t* n_applied) {
  if (!w || (!edits && n) || (!arrival_s && n) || (!results && n) || max_batch == 0) return PX_E_INVALID_ARG;
  int dims[3];
  double vpm;
  px_world_info(w, dims, &vpm);
  const double vs = 1 / vpm;
  px_stats st;
  px_get_stats(w, &st);
  {  // the pool the serving loop works in, allocated before the clock starts (GpuWorld.ts:57)
    const uint64_t used = st.pool_used;
    uint64_t cap = std::max<uint64_t>(used + 98304, 2 * used);
    if (cap > pool_budget_bricks) cap = pool_budget_bricks;
    const int rc0 = px_reserve_pool(w, cap);
    if (rc0 != PX_OK) return rc0;
  }
  // The build scratch of the largest batch the stream can form (the max_batch
  // largest edits' pairs, at most kPairBudget), also allocated before the clock:
  // a step that had to allocate device memory would stall the loop for a
  // millisecond or more.  A batch is closed before its pairs pass that budget.
  constexpr uint64_t kPairBudget = 1ull << 22;
  uint64_t pair_budget = 0;
  {
    std::vector<uint64_t> nb(n);
    for (size_t i = 0; i < n; i++) nb[i] = brick_bound(edits[i], vs, dims[0], dims[1], dims[2]);
    const size_t top = std::min<size_t>(n, max_batch);
    std::partial_sort(nb.begin(), nb.begin() + top, nb.end(), std::greater<uint64_t>());
    for (size_t i = 0; i < top; i++) pair_budget += nb[i];
    pair_budget = std::min(std::max<uint64_t>(pair_budget, 1), kPairBudget);
    const int rc0 = reserve_build_scratch(w, pair_budget, max_batch);
    if (rc0 != PX_OK) return rc0;
    px_get_stats(w, &st);
  }
  uint64_t pool_cap = st.pool_capacity;

  // arrival order
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; i++) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return arrival_s[x] < arrival_s[y]; });
  for (size_t i = 0; i < n; i++) {
    results[i].id = i;
    results[i].status = PX_OK;
    results[i].batch = 0;
    results[i].arrival_s = arrival_s[i];
    results[i].start_s = results[i].done_s = -1;
    results[i].dev_start_ms = results[i].dev_end_ms = -1;
  }

  // Two world objects over the one resident world (the twin has build scratch
  // of its own), builds alternating between them: a step's evaluation passes
  // run on s_eval while the previous step's apply pass runs on s_apply.
  int trc = PX_OK;
  px_world* twin = twin_create(w, pair_budget, max_batch, &trc);
  if (!twin) return trc;
  cudaStream_t s_eval = (cudaStream_t)stream, s_apply = nullptr;
  cudaEvent_t base = nullptr;
  if (cudaStreamCreateWithFlags(&s_apply, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&base) != cudaSuccess) {
    cudaGetLastError();
    if (s_apply) cudaStreamDestroy(s_apply);
    twin_destroy(twin);
    return PX_E_CUDA;
  }
  cudaEventRecord(base, s_eval);
  px_world* W[2] = {w, twin};
  PipelineState committed = pipeline_begin(w);  // the allocator state of the last finished step

  // producer: releases requests at their arrival times
  std::mutex mu;
  std::condition_variable cv;
  std::atomic<size_t> released{0};
  std::atomic<bool> stop{false};
  const auto t0 = clock_t_::now();
  std::thread producer([&] {
    for (size_t k = 0; k < n; k++) {
      const double t = arrival_s[order[k]];
      std::this_thread::sleep_until(t0 + std::chrono::duration_cast<clock_t_::duration>(std::chrono::duration<double>(t)));
      if (stop.load()) return;
      {
        std::lock_guard<std::mutex> g(mu);
        released.store(k + 1);
      }
      cv.notify_one();
    }
  });

  struct Step {
    std::vector<size_t> edits;
    uint64_t bound;       // the most pool bricks it can add
    int world;            // W index
    double start;
    uint32_t id;
    size_t n_ops;
  };
  std::vector<Step> flight;  // at most two steps in flight, oldest first
  size_t next = 0, applied = 0;
  uint32_t batch_id = 0;
  uint64_t ops_done = 0;
  bool parity = committed.holes_in_a;  // holes buffer the next queued step reads
  int rc = PX_OK;
  std::vector<IrOp> ops;
  std::vector<uint32_t> code;
  std::vector<double> params;
  std::vector<unsigned char> ir;

  auto finish_oldest = [&]() {
    Step stp = std::move(flight.front());
    flight.erase(flight.begin());
    px_world* x = W[stp.world];
    const int brc = px_build_finish(x);
    const double done = secs(t0, clock_t_::now());
    double d0 = -1, d1 = -1;
    build_times(x, base, &d0, &d1);
    if (brc == PX_OK && rc == PX_OK) {
      px_stats xs;
      px_get_stats(x, &xs);
      committed.pool_used = xs.pool_used;
      committed.n_holes = xs.n_holes;
      committed.holes_in_a = !committed.holes_in_a;  // the step wrote the other holes buffer
      ops_done += stp.n_ops;
    } else if (rc == PX_OK) {
      rc = brc;  // later queued steps commit nothing (the device state is poisoned)
    }
    for (size_t i : stp.edits) {
      results[i].start_s = stp.start;
      results[i].done_s = done;
      results[i].dev_start_ms = d0;
      results[i].dev_end_ms = d1;
      results[i].batch = stp.id;
      results[i].status = (uint32_t)(rc == PX_OK ? PX_OK : PX_E_QUEUE_OVERFLOW);
      if (rc == PX_OK) {
        if (applied_order) applied_order[applied] = i;
        applied++;
      }
    }
  };

  while ((next < n && rc == PX_OK) || !flight.empty()) {
    if (flight.size() == 2 || rc != PX_OK) {  // both world objects busy (or draining after a failure)
      finish_oldest();
      continue;
    }
    if (flight.empty() && released.load() <= next && next < n) {  // idle: sleep until a request arrives
      std::unique_lock<std::mutex> g(mu);
      cv.wait(g, [&] { return released.load() > next; });
    }
    const size_t avail = released.load();
    if (next >= n) {
      finish_oldest();
      continue;
    }
    if (avail <= next) {  // nothing new: the step in flight finishes unless a request arrives first
      if (build_done(W[flight.front().world])) finish_oldest();
      else std::this_thread::yield();
      continue;
    }
    // admit in arrival order while the free pool holds the worst case of this
    // step and of the step still in flight
    uint64_t in_flight = 0;
    for (const Step& f : flight) in_flight += f.bound;
    const uint64_t live = (uint64_t)committed.pool_used - committed.n_holes;
    const uint64_t used_bound = (uint64_t)committed.pool_used + in_flight;
    std::vector<size_t> batch;
    ops.clear();
    code.clear();
    params.clear();
    uint64_t bound = 0;
    while (next < avail && batch.size() < max_batch) {
      const size_t i = order[next];
      const uint64_t b = brick_bound(edits[i], vs, dims[0], dims[1], dims[2]);
      const bool fits = live + in_flight + bound + b <= pool_budget_bricks &&
                        used_bound + build_stage_slots(w, bound + b) <= pool_cap && bound + b <= pair_budget;
      if (!fits) {
        if (batch.empty() && flight.empty()) {  // cannot fit even alone on an idle world: reject
          results[i].status = PX_E_OOM;
          results[i].done_s = secs(t0, clock_t_::now());
          next++;
          continue;
        }
        break;  // wait for the next step (or for the step in flight to commit)
      }
      bound += b;
      batch.push_back(i);
      encode_carve(edits[i], vs, ops, code, params);
      next++;
    }
    if (batch.empty()) {
      if (!flight.empty()) finish_oldest();
      continue;
    }
    const double start = secs(t0, clock_t_::now());
    ir.assign(32 + ops.size() * sizeof(IrOp) + code.size() * 4 + params.size() * 8, 0);
    uint32_t hdr[8] = {0x52495850u, 1u, (uint32_t)ops.size(), (uint32_t)(code.size() / 2), (uint32_t)params.size(), 0, 0, 0};
    std::memcpy(ir.data(), hdr, 32);
    std::memcpy(ir.data() + 32, ops.data(), ops.size() * sizeof(IrOp));
    std::memcpy(ir.data() + 32 + ops.size() * sizeof(IrOp), code.data(), code.size() * 4);
    std::memcpy(ir.data() + 32 + ops.size() * sizeof(IrOp) + code.size() * 4, params.data(), params.size() * 8);
    const int wi = (int)(batch_id & 1u);
    px_world* x = W[wi];
    pipeline_set(x, s_apply, parity, (uint32_t)std::min<uint64_t>(used_bound, pool_cap),
                 (uint32_t)std::min<uint64_t>((uint64_t)committed.n_holes + in_flight, pool_cap));
    int erc = px_submit_ops(x, ir.data(), ir.size());
    if (erc == PX_OK) erc = px_build_enqueue(x, mode, s_eval);
    if (erc != PX_OK) {
      rc = erc;
      for (size_t i : batch) {
        results[i].status = (uint32_t)erc;
        results[i].done_s = secs(t0, clock_t_::now());
      }
      continue;
    }
    parity = !parity;
    flight.push_back(Step{std::move(batch), bound, wi, start, batch_id, ops.size()});
    batch_id++;
  }
  stop.store(true);
  producer.join();
  cudaStreamSynchronize(s_apply);
  pipeline_end(w, committed, ops_done, s_eval);
  twin_destroy(twin);
  cudaStreamDestroy(s_apply);
  cudaEventDestroy(base);
  if (n_applied) *n_applied = applied;
  return rc;
}

// host exceptions (thread or allocation failures) never cross the C ABI
int px_serve_run(px_world* w, const px_edit* edits, const double* arrival_s, size_t n, uint32_t max_batch,
                 uint64_t pool_budget_bricks, int mode, void* stream, px_edit_result* results, uint64_t* applied_order,
                 size_t* n_applied) {
  try {
    return serve_run_impl(w, edits, arrival_s, n, max_batch, pool_budget_bricks, mode, stream, results, applied_order, n_applied);
  } catch (const std::bad_alloc&) {
    return PX_E_OOM;
  } catch (...) {
    return PX_E_CUDA;
  }
}

}  // extern "C"
