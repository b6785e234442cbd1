// px_derive_noalloc: the derived upload buffers (super-grid counts and the
// density bytes of GpuWorld.ts:90-101, VoxelWorld.ts:159-170) computed from a
// grid and pool the caller holds on the device, into output buffers the
// caller holds, without allocating any device memory.
//
// Who needs it: a caller that has fixed its device memory before it starts
// working and cannot let a library take more afterwards — a renderer that
// sizes all of its buffers once at upload and shares the GPU with other
// programs, a frame loop in which an allocation can stall the device for the
// length of a frame, or a process running under a hard device-memory cap.
// px_derive needs a world handle, whose buffers are allocated (and grown) by
// this library; this entry point needs none.
//
// Scratch: one opaque-voxel count per pool brick and a status block, kept in
// the fixed-size array below (2 MiB + 256 bytes, allocated once when the
// library's device code is loaded), so the entry point's footprint is known in
// advance.  It limits the pool to PX_NOALLOC_MAX_POOL_BRICKS bricks (1 GiB of
// pool); larger pools are refused with PX_E_TOO_LARGE before any GPU work.
//
// Set-up: the first call on each device, with that device current, looks up
// the array's device address (cudaGetSymbolAddress) and keeps it for later
// calls on that device.  Make the first call on a device before any stream
// capture is begun on it.  The kept address belongs to the device's current
// context: after cudaDeviceReset (which unloads the library's device code) the
// array may live elsewhere, so this entry point is not to be called on a
// device that has been reset since its first call.
//
// Alignment: the pool is read as 32-bit voxel pairs and the grid and super
// counts as 32-bit words, so those three addresses must be multiples of 4
// bytes (a uint16 pool that starts at an odd element is refused with
// PX_E_INVALID_ARG before any GPU work).
//
// Every call shares the one array: calls that overlap in time (from several
// host threads, or on several streams) race on it and may return wrong
// results.  Callers serialise them.  Each call clears the status block before
// its kernels run; the counts are written for every pool brick before they
// are read, so they need no clearing.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/pixels_gb300.h"
#include "jsmath.cuh"

namespace {

constexpr uint32_t MAX_POOL_BRICKS = PX_NOALLOC_MAX_POOL_BRICKS;
constexpr size_t STATUS_BYTES = 256;  // status block; keeps the counts 256-byte aligned
constexpr size_t SCRATCH_BYTES = STATUS_BYTES + sizeof(uint16_t) * (size_t)MAX_POOL_BRICKS;
constexpr int MAX_DEVICES = 64;

// The only scratch of px_derive_noalloc.  Host code never uses this name as a
// device address: the address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_derive_scratch[SCRATCH_BYTES];

struct Status {            // first bytes of the scratch
  uint32_t bad;            // 1 if a grid entry names a pool brick >= n_pool
  uint32_t pad;
  unsigned long long first_bad_cell;  // smallest such cell index
};

struct Tables {  // passed by value (512 bytes of kernel parameters)
  uint8_t opaque[256];
  uint8_t udens[256];
};

constexpr uint32_t FULL = 0xffffffffu;
constexpr uint32_t UNIFORM_FLAG = 0x80000000u;

// Pass 1: opaque, non-air voxels of every pool brick (one warp per brick,
// 8 coalesced 128-byte rows of voxel pairs).
__global__ void __launch_bounds__(256) noalloc_count_kernel(const uint32_t* __restrict__ pool32, uint32_t n_pool,
                                                            Tables t, uint16_t* __restrict__ counts) {
  __shared__ uint8_t op_s[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) op_s[i] = t.opaque[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b < n_pool; b += warps) {
    const uint32_t* p = pool32 + (size_t)b * 256;
    uint32_t cnt = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      const uint32_t w = p[32 * j + lane];
      const uint32_t v0 = w & 0xffffu, v1 = w >> 16;
      cnt += (v0 != 0 && op_s[v0 & 0xffu]) + (v1 != 0 && op_s[v1 & 0xffu]);
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) cnt += __shfl_xor_sync(FULL, cnt, o);
    if (lane == 0) counts[b] = (uint16_t)cnt;
  }
}

// Pass 2: one warp per super cell (4x4x4 bricks, two per lane): the count of
// non-empty bricks, and each brick's density byte — 0 for air, the material's
// table value for a uniform brick, Math.round(n / 512 * 255) for a pool brick.
__global__ void __launch_bounds__(256) noalloc_cells_kernel(const uint32_t* __restrict__ grid, int BX, int BY, int BZ,
                                                            uint32_t n_pool, Tables t,
                                                            const uint16_t* __restrict__ counts, Status* status,
                                                            uint32_t* __restrict__ super_counts,
                                                            uint8_t* __restrict__ density) {
  __shared__ uint8_t ud_s[256];
  for (int i = threadIdx.x; i < 256; i += blockDim.x) ud_s[i] = t.udens[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int SX = (BX + 3) / 4, SY = (BY + 3) / 4, SZ = (BZ + 3) / 4;
  const long long n_super = (long long)SX * SY * SZ;
  const long long warps = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long sc = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; sc < n_super; sc += warps) {
    const int sz = (int)(sc / ((long long)SX * SY));
    const int rem = (int)(sc - (long long)sz * SX * SY);
    const int sy = rem / SX, sx = rem - sy * SX;
    uint32_t nz = 0;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int k = lane + 32 * h;
      const int bx = sx * 4 + (k & 3), by = sy * 4 + ((k >> 2) & 3), bz = sz * 4 + (k >> 4);
      if (bx < BX && by < BY && bz < BZ) {
        const size_t ci = (size_t)bx + (size_t)BX * ((size_t)by + (size_t)BY * (size_t)bz);
        const uint32_t g = grid[ci];
        uint8_t d = 0;
        if (g != 0) {
          nz++;
          if (g & UNIFORM_FLAG) {
            d = ud_s[g & 0xffu];
          } else if (g - 1 < n_pool) {
            d = (uint8_t)px_round(((double)counts[g - 1] / 512.0) * 255.0);
          } else {  // a pool index outside the caller's pool: report it, read nothing
            atomicExch(&status->bad, 1u);
            atomicMin(&status->first_bad_cell, (unsigned long long)ci);
          }
        }
        density[ci] = d;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) nz += __shfl_xor_sync(FULL, nz, o);
    if (lane == 0) super_counts[sc] = nz;
  }
}

std::mutex g_setup_mu;
void* g_scratch_addr[MAX_DEVICES];

// Device address of the scratch on the current device (set-up on first use).
int scratch_for_current_device(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return PX_E_NO_DEVICE;
  }
  if (dev < 0 || dev >= MAX_DEVICES) return PX_E_INVALID_ARG;
  std::lock_guard<std::mutex> g(g_setup_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_derive_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return PX_E_CUDA;
    }
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return PX_OK;
}

}  // namespace

extern "C" int px_derive_noalloc(const uint32_t* grid, const uint16_t* pool, int bx, int by, int bz,
                                 uint32_t n_pool_bricks, const uint8_t* opaque256, const uint8_t* uniform_density256,
                                 uint32_t* super_counts, uint8_t* density, void* stream) {
  if (!grid || !super_counts || !density || !opaque256 || !uniform_density256 || (n_pool_bricks && !pool) ||
      bx <= 0 || by <= 0 || bz <= 0)
    return PX_E_INVALID_ARG;
  if (n_pool_bricks > MAX_POOL_BRICKS) return PX_E_TOO_LARGE;
  if (((uintptr_t)grid & 3u) || ((uintptr_t)pool & 3u) || ((uintptr_t)super_counts & 3u)) return PX_E_INVALID_ARG;
  void* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc != PX_OK) return rc;
  Status* status = (Status*)scratch;
  uint16_t* counts = (uint16_t*)((unsigned char*)scratch + STATUS_BYTES);
  cudaStream_t s = (cudaStream_t)stream;

  Tables t;
  for (int i = 0; i < 256; i++) {
    t.opaque[i] = opaque256[i];
    t.udens[i] = uniform_density256[i];
  }
  // the status block starts clear: bad = 0, first_bad_cell = all ones
  if (cudaMemsetAsync(&status->bad, 0, 8, s) != cudaSuccess ||
      cudaMemsetAsync(&status->first_bad_cell, 0xff, 8, s) != cudaSuccess) {
    cudaGetLastError();
    return PX_E_CUDA;
  }
  if (n_pool_bricks) {
    const uint32_t blocks = (n_pool_bricks + 7) / 8;  // 8 warps per block, one brick per warp
    noalloc_count_kernel<<<blocks < 65535 ? blocks : 65535, 256, 0, s>>>((const uint32_t*)pool, n_pool_bricks, t, counts);
  }
  const long long n_super = (long long)((bx + 3) / 4) * ((by + 3) / 4) * ((bz + 3) / 4);
  const long long blocks = (n_super + 7) / 8;
  noalloc_cells_kernel<<<(int)(blocks < 65535 ? blocks : 65535), 256, 0, s>>>(grid, bx, by, bz, n_pool_bricks, t, counts,
                                                                              status, super_counts, density);
  if (cudaGetLastError() != cudaSuccess) return PX_E_CUDA;
  Status out;
  if (cudaMemcpyAsync(&out, status, sizeof out, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    return PX_E_CUDA;
  }
  return out.bad ? PX_E_INVALID_ARG : PX_OK;
}
