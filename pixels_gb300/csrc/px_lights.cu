// Light anchors: snapToEmissive (GpuWorld.ts:165-174) for every anchor of the
// scene's lights in one launch on the built world.  packLights
// (GpuWorld.ts:141-162), which lays the snapped anchors out with the light
// records, stays with the host binding (pixels_gb300/lights.py).
//
// For each anchor voxel (x, y, z) the reference scans the cubes of radius
// r = 0, 1, 2 around it, z outermost, then y, then x, each from -r to r, and
// returns the first voxel whose material emits; with none it keeps (x, y, z).
// The scan reads the world as VoxelWorld.get does (GpuWorld.ts:170;
// VoxelWorld.ts:55-61): air outside the world, the uniform value of a uniform
// brick, else the pool voxel.  A non-air voxel whose material byte names no
// material makes the reference throw (mat(id) is undefined); here the call
// returns PX_E_INVALID_ARG.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "../../include/pixels_gb300.h"

namespace {

struct EmissionTable {  // 0 no emission, 1 emits, 2 no such material
  uint8_t v[256];
};

__device__ __forceinline__ uint32_t voxel_at(const uint32_t* __restrict__ grid, const uint16_t* __restrict__ pool,
                                             int dx, int dy, int dz, int x, int y, int z) {
  if (x < 0 || y < 0 || z < 0 || x >= dx || y >= dy || z >= dz) return 0;
  const int bx = dx >> 3, by = dy >> 3;
  const uint32_t g = grid[(size_t)(x >> 3) + (size_t)bx * ((size_t)(y >> 3) + (size_t)by * (size_t)(z >> 3))];
  if (g == 0) return 0;
  if (g & PX_UNIFORM) return g & 0xffffu;
  return pool[(size_t)(g - 1) * 512 + (uint32_t)((x & 7) | ((y & 7) << 3) | ((z & 7) << 6))];
}

// one thread per anchor: out = snapped voxel, status = 1 where the scan met an unknown material
__global__ void snap_kernel(const uint32_t* __restrict__ grid, const uint16_t* __restrict__ pool, int dx, int dy, int dz,
                            EmissionTable t, const int3* __restrict__ in, int n, int3* out, int* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int3 a = in[i];
  for (int r = 0; r <= 2; r++)
    for (int oz = -r; oz <= r; oz++)
      for (int oy = -r; oy <= r; oy++)
        for (int ox = -r; ox <= r; ox++) {
          const uint32_t v = voxel_at(grid, pool, dx, dy, dz, a.x + ox, a.y + oy, a.z + oz);
          if (!v) continue;
          const uint8_t e = t.v[v & 0xffu];
          if (e == 2) {
            out[i] = a;
            atomicOr(status, 1);
            return;
          }
          if (e == 1) {
            out[i] = make_int3(a.x + ox, a.y + oy, a.z + oz);
            return;
          }
        }
  out[i] = a;
}

}  // namespace

extern "C" int px_snap_anchors(px_world* w, const int32_t* xyz, size_t n, const uint8_t* emission256, int32_t* out_xyz) {
  if (!w || !emission256 || (n && (!xyz || !out_xyz)) || n > (1u << 24)) return PX_E_INVALID_ARG;
  if (n == 0) return PX_OK;
  px_device_view view;
  int dims[3];
  int rc = px_device_view_get(w, &view);
  if (rc == PX_OK) rc = px_world_info(w, dims, nullptr);
  if (rc != PX_OK) return rc;
  EmissionTable t;
  for (int k = 0; k < 256; k++) t.v[k] = emission256[k];
  void* buf = nullptr;
  const size_t bytes = n * sizeof(int3);
  if (cudaMalloc(&buf, 2 * bytes + 16) != cudaSuccess) {
    cudaGetLastError();
    return PX_E_OOM;
  }
  int3* d_in = (int3*)buf;
  int3* d_out = d_in + n;
  int* d_status = (int*)(d_out + n);
  int st = 0;
  bool ok = cudaMemcpy(d_in, xyz, bytes, cudaMemcpyHostToDevice) == cudaSuccess &&
            cudaMemset(d_status, 0, sizeof(int)) == cudaSuccess;
  if (ok) {
    snap_kernel<<<(unsigned)((n + 127) / 128), 128>>>(view.grid, view.pool, dims[0], dims[1], dims[2], t, d_in, (int)n,
                                                      d_out, d_status);
    ok = cudaGetLastError() == cudaSuccess && cudaMemcpy(out_xyz, d_out, bytes, cudaMemcpyDeviceToHost) == cudaSuccess &&
         cudaMemcpy(&st, d_status, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
  }
  cudaFree(buf);
  if (!ok) {
    cudaGetLastError();
    return PX_E_CUDA;
  }
  return st ? PX_E_INVALID_ARG : PX_OK;
}
