// Field integrals without any device allocation.
//
// Who needs this: a caller that holds a nodal field in its own device memory and
// must obtain the total amount or the boundary flux at a point where it may not
// allocate GPU memory.  Examples are a host simulation loop that runs inside a
// strict device-memory budget enforced by its own allocator (a cudaMalloc from a
// library would break the budget accounting), code that runs while other streams
// are timing-critical (cudaMalloc and cudaFree can synchronise the device), and
// callers that hand the library only pre-allocated buffers by contract.  The
// ordinary entry points (eqf_total_mass, eqf_boundary_flux) allocate their
// reduction scratch per call; this one keeps it in a fixed device array instead.
//
// The scratch is the file-scope array below: one FP64 partial sum per block of
// kNoallocBlockNodes nodes plus one slot for the total.  Every GPU that loads the
// library holds it (about 32 KB) until the process exits.  All calls share it, so
// calls that overlap on the GPU (different streams, or different host threads on
// one device) race and must be serialised by the caller.  Each slot is written
// by its block before it is read, so no part of it has to start at zero.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/eqfield.h"

namespace {

constexpr int kNoallocThreads = 256;
constexpr int kNoallocBlockNodes = 2048;
constexpr int kNoallocMaxBlocks = EQF_NOALLOC_MAX_NODES / kNoallocBlockNodes;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kNoallocMaxBlocks + 1];

__device__ __forceinline__ double block_total(double v) {
  __shared__ double red[kNoallocThreads / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) red[w] = v;
  __syncthreads();
  double t = 0.0;
  if (w == 0) {
    t = lane < kNoallocThreads / 32 ? red[lane] : 0.0;
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
  }
  return t;
}

// Partial integral over nodes [blockIdx.x * kNoallocBlockNodes, ...) of a uniform
// (nx x ny squares, spacing hx, hy) right-triangle mesh in grid order.
//   what 0: sum_k c_k * (row sum of the P1 mass matrix) = 1^T M c
//   what 1: -int grad c . n ds, each boundary edge taking the gradient of the one
//           triangle it bounds (bottom/right edges: lower-right triangle,
//           top/left edges: upper-left triangle)
__global__ void __launch_bounds__(kNoallocThreads)
    k_noalloc_partials(const double* __restrict__ u, int nx, int ny, double hx, double hy,
                       int what, double* __restrict__ part) {
  const int P = nx + 1, n = P * (ny + 1);
  const int k0 = blockIdx.x * kNoallocBlockNodes;
  const int k1 = min(n, k0 + kNoallocBlockNodes);
  double acc = 0.0;
  for (int k = k0 + threadIdx.x; k < k1; k += kNoallocThreads) {
    const int i = k / P, j = k - i * P;
    if (what == 0) {
      const double hxl = j > 0 ? hx : 0.0, hxr = j < nx ? hx : 0.0;
      const double hyd = i > 0 ? hy : 0.0, hyu = i < ny ? hy : 0.0;
      const double sx = hxl + hxr, sy = hyd + hyu;
      const double w = (2.0 * hxl * hyd + hxr * hyd + hxl * hyu + 2.0 * hxr * hyu) / 12.0 +
                       sx * sy / 24.0 + sy * sx / 24.0 + (hxr * hyu + hxl * hyd) / 12.0;
      acc += w * u[k];
    } else {
      if (i == 0 && j < nx) acc += (u[k + P + 1] - u[k + 1]) / hy * hx;
      if (i == ny && j < nx) acc += -(u[k] - u[k - P]) / hy * hx;
      if (j == 0 && i < ny) acc += (u[k + P + 1] - u[k + P]) / hx * hy;
      if (j == nx && i < ny) acc += -(u[k] - u[k - 1]) / hx * hy;
    }
  }
  const double t = block_total(acc);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// total = scale * sum of the partials in block order (one thread: fixed order)
__global__ void k_noalloc_total(double* __restrict__ part, int nblocks, double scale) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nblocks; ++b) s += part[b];
  part[kNoallocMaxBlocks] = scale * s;
}

// Device address of the scratch array, looked up once per device.
std::mutex g_lock;
double* g_scratch_ptr[kMaxDevices] = {};

int scratch_for_current_device(double** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return EQF_ERR_NO_DEVICE;
  if (dev < 0 || dev >= kMaxDevices) return EQF_ERR_INVALID;
  std::lock_guard<std::mutex> guard(g_lock);
  if (!g_scratch_ptr[dev]) {
    double* p = nullptr;
    if (cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_noalloc_scratch) != cudaSuccess ||
        !p)
      return EQF_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return EQF_OK;
}

}  // namespace

extern "C" int eqf_field_integral_noalloc(const double* d_field, int32_t nx, int32_t ny,
                                          double width, double height, int32_t what,
                                          double scale, void* stream, double* out) {
  if (!d_field || !out || nx < 1 || ny < 1 || !(width > 0.0) || !(height > 0.0) ||
      (what != 0 && what != 1))
    return EQF_ERR_INVALID;
  const long long n = ((long long)nx + 1) * ((long long)ny + 1);
  if (n > (long long)EQF_NOALLOC_MAX_NODES) return EQF_ERR_TOO_LARGE;
  double* scratch = nullptr;
  const int rc = scratch_for_current_device(&scratch);
  if (rc != EQF_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int nblocks = (int)((n + kNoallocBlockNodes - 1) / kNoallocBlockNodes);
  double hx = width / nx, hy = height / ny;
  // each launch's status comes from its own cudaLaunchKernel call: a cudaGetLastError
  // afterwards would also take (and clear) an error the caller had left pending
  void* part_args[] = {(void*)&d_field, (void*)&nx, (void*)&ny, (void*)&hx, (void*)&hy,
                       (void*)&what, (void*)&scratch};
  if (cudaLaunchKernel((const void*)k_noalloc_partials, dim3(nblocks), dim3(kNoallocThreads),
                       part_args, 0, s) != cudaSuccess)
    return EQF_ERR_CUDA;
  void* total_args[] = {(void*)&scratch, (void*)&nblocks, (void*)&scale};
  if (cudaLaunchKernel((const void*)k_noalloc_total, dim3(1), dim3(32), total_args, 0, s) !=
      cudaSuccess)
    return EQF_ERR_CUDA;
  if (cudaMemcpyAsync(out, scratch + kNoallocMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost,
                      s) != cudaSuccess)
    return EQF_ERR_CUDA;
  if (cudaStreamSynchronize(s) != cudaSuccess) return EQF_ERR_CUDA;
  return EQF_OK;
}
