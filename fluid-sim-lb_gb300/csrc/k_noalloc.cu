// k_noalloc.cu -- an allocation-free entry point: CFL() on a caller's field.
//
// Some callers cannot call cudaMalloc while they run this step: an engine
// that hands the solver pre-reserved device buffers from its own pool and
// forbids allocation inside its frame loop, or code running where an
// allocation would synchronise the device or break a real-time budget.
// For them fsim_cfl_noalloc computes FlipSimulation::CFL() (the time-step
// speed: 1/max(sqrt(0.5*gravity), max |v| over active in-box faces), v >= 1e-2)
// from a velocity field they already hold on the device, in the dense layout
// of fsim_download_field.  It allocates nothing: the per-block maxima of
// the reduction live in the file-scope device array below, which every GPU
// that loads this library holds until the process exits (4 KB + a counter).
#include <algorithm>
#include <cmath>
#include <mutex>

#include "fsim_internal.cuh"

namespace fsim {

namespace {

constexpr int kNaBlocks = 1024;  // scratch capacity: one partial per block
constexpr int kNaThreads = 256;
constexpr int kNaMaxDevices = 64;

// Scratch shared by every call on a device: per-block maxima and the
// arrival counter of the last-block finish.  Calls that overlap on the GPU
// (two streams at once) race on it.
struct NoallocScratch {
  float partial[kNaBlocks];
  unsigned int arrivals;
};
static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

// Device address of g_noalloc_scratch per device (host code may not use the
// symbol's host-side name as a device pointer).
NoallocScratch* g_scratch_ptr[kNaMaxDevices] = {};
std::mutex g_scratch_mu;

__global__ void __launch_bounds__(kNaThreads)
    k_cfl_dense(const float* __restrict__ vel, const uint8_t* __restrict__ active, int n0, int n1,
                int n2, float gravity, float* __restrict__ out, NoallocScratch* __restrict__ sc) {
  __shared__ float red[kNaThreads / 32];
  __shared__ bool last;
  const int64_t s1 = n1 + 2, s2 = n2 + 2;
  const int64_t cells = int64_t(n0) * n1 * n2;
  float vmax = 0.f;
  for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c < cells;
       c += int64_t(gridDim.x) * blockDim.x) {
    const int i = int(c / (int64_t(n1) * n2)), j = int((c / n2) % n1), k = int(c % n2);
    const int64_t o = (int64_t(i + 1) * s1 + (j + 1)) * s2 + (k + 1);
    if (!active[o]) continue;
    const float* v = vel + 3 * o;
    if (j != n1 - 1 && k != n2 - 1) vmax = fmaxf(vmax, fabsf(v[0]));
    if (i != n0 - 1 && k != n2 - 1) vmax = fmaxf(vmax, fabsf(v[1]));
    if (i != n0 - 1 && j != n1 - 1) vmax = fmaxf(vmax, fabsf(v[2]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = vmax;
  __syncthreads();
  if (threadIdx.x == 0) {
    float m = 0.f;
    for (int w = 0; w < kNaThreads / 32; ++w) m = fmaxf(m, red[w]);
    sc->partial[blockIdx.x] = m;
    __threadfence();
    last = atomicAdd(&sc->arrivals, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last || threadIdx.x != 0) return;
  __threadfence();
  float m = 0.f;
  for (unsigned b = 0; b < gridDim.x; ++b) m = fmaxf(m, __ldcg(&sc->partial[b]));
  sc->arrivals = 0u;  // leave the counter at zero for the next call
  // FlipSimulation::CFL, common/flip_simulation.cc:485-487
  float v = float(fmax(sqrt(0.5 * double(gravity)), double(m)));
  if (v < 1e-2) v = float(1e-2);
  *out = float(1.0 / double(v));
}

// Once per device, with that device current: the scratch's device address.
int scratch_for_device(int dev, NoallocScratch** out) {
  if (dev < 0 || dev >= kNaMaxDevices) return FSIM_ERR_INVALID;
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    NoallocScratch* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_noalloc_scratch);
    if (e != cudaSuccess || !p) return FSIM_ERR_CUDA;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return FSIM_OK;
}

}  // namespace

}  // namespace fsim

extern "C" {

int fsim_cfl_noalloc(const float* vel, const uint8_t* active, const int32_t dims[3],
                     float gravity, float* inv_speed, void* stream) {
  using namespace fsim;
  if (!vel || !active || !dims || !inv_speed) return FSIM_ERR_INVALID;
  for (int a = 0; a < 3; ++a) {
    if (dims[a] < 8) return FSIM_ERR_INVALID;
    if (dims[a] > 1024) return FSIM_ERR_CAPACITY;  // beyond the stated maximum
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return FSIM_ERR_NO_DEVICE;
  NoallocScratch* sc = nullptr;
  const int rc = scratch_for_device(dev, &sc);
  if (rc) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // the counter must start at zero (a previous call leaves it there; this
  // also covers a call that was interrupted)
  if (cudaMemsetAsync(&sc->arrivals, 0, sizeof(unsigned int), st) != cudaSuccess)
    return FSIM_ERR_CUDA;
  const int64_t cells = int64_t(dims[0]) * dims[1] * dims[2];
  const int grid = int(std::min<int64_t>((cells + kNaThreads - 1) / kNaThreads, kNaBlocks));
  k_cfl_dense<<<grid, kNaThreads, 0, st>>>(vel, active, dims[0], dims[1], dims[2], gravity,
                                          inv_speed, sc);
  if (cudaGetLastError() != cudaSuccess) return FSIM_ERR_CUDA;
  return FSIM_OK;
}

}  // extern "C"
