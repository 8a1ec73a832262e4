// Allocation-free max-norm of a device field (the reduction of
// sf3d_check_stability, check_stability.f90:408, with its scratch memory in a
// fixed device array instead of the Mesh's allocation).
//
// The scratch is a file-scope __device__ array of kNoAllocScratchFloats floats
// (256 KB): pass 1 writes one partial maximum and one NaN flag per CTA with
// plain stores, pass 2 (one CTA) reduces the partials and stores the result in
// the last two slots.  Every slot that is read was written earlier in the same
// call, so nothing has to start at zero.  The device address of the array is
// looked up with cudaGetSymbolAddress on the first call on each device (with
// that device current) and cached; no call allocates or frees memory.  The
// cached address belongs to the device's primary context: a caller that resets
// the device (cudaDeviceReset) between calls unloads the module and must not
// call this entry point again in that process.  A non-null stream must belong
// to the current device (checked).  Two calls that overlap in time on the same
// device (different streams or host threads) share the array and race; callers
// serialise them.
#include <math.h>
#include <mutex>
#include <string.h>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocPerThread = 64;                       // values per thread per CTA pass
constexpr long kNoAllocPerBlock = (long)kNoAllocThreads * kNoAllocPerThread;  // 16384
constexpr int kNoAllocMaxBlocks = 32768;
constexpr int kNoAllocScratchFloats = 2 * kNoAllocMaxBlocks;  // 65536 floats = 256 KB
constexpr long kNoAllocMaxValues = kNoAllocPerBlock * (kNoAllocMaxBlocks - 1);  // last CTA slot holds the result

__device__ __align__(256) float g_noalloc_scratch[kNoAllocScratchFloats];

constexpr int kMaxDevices = 64;
void* g_scratch_ptr[kMaxDevices] = {};
std::mutex g_scratch_mutex;

// pass 1: CTA b reduces values [b*16384, (b+1)*16384) into slots b (max) and
// kNoAllocMaxBlocks + b (NaN flag, 0/1 as float)
__global__ void __launch_bounds__(kNoAllocThreads) noalloc_partial_kernel(const float* __restrict__ x, long n,
                                                                          float* __restrict__ scratch) {
  __shared__ float s_max[kNoAllocThreads / 32];
  __shared__ int s_nan[kNoAllocThreads / 32];
  const long base = (long)blockIdx.x * kNoAllocPerBlock;
  float m = 0.f;
  bool nan = false;
#pragma unroll 4
  for (int q = 0; q < kNoAllocPerThread; ++q) {
    const long i = base + (long)q * kNoAllocThreads + threadIdx.x;
    if (i < n) {
      const float v = fabsf(x[i]);
      if (v != v)
        nan = true;
      else
        m = fmaxf(m, v);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  nan = __any_sync(0xffffffffu, nan);
  if ((threadIdx.x & 31) == 0) {
    s_max[threadIdx.x >> 5] = m;
    s_nan[threadIdx.x >> 5] = nan ? 1 : 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float bm = 0.f;
    int bn = 0;
    for (int w = 0; w < kNoAllocThreads / 32; ++w) {
      bm = fmaxf(bm, s_max[w]);
      bn |= s_nan[w];
    }
    scratch[blockIdx.x] = bm;
    scratch[kNoAllocMaxBlocks + blockIdx.x] = bn ? 1.f : 0.f;
  }
}

// pass 2: one CTA reduces the nblocks partials into slots kNoAllocMaxBlocks-1
// (max) and 2*kNoAllocMaxBlocks-1 (NaN flag); nblocks <= kNoAllocMaxBlocks-1
__global__ void __launch_bounds__(kNoAllocThreads) noalloc_final_kernel(int nblocks, float* __restrict__ scratch) {
  __shared__ float s_max[kNoAllocThreads / 32];
  __shared__ int s_nan[kNoAllocThreads / 32];
  float m = 0.f;
  bool nan = false;
  for (int b = threadIdx.x; b < nblocks; b += kNoAllocThreads) {
    m = fmaxf(m, scratch[b]);
    nan = nan || scratch[kNoAllocMaxBlocks + b] != 0.f;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  nan = __any_sync(0xffffffffu, nan);
  if ((threadIdx.x & 31) == 0) {
    s_max[threadIdx.x >> 5] = m;
    s_nan[threadIdx.x >> 5] = nan ? 1 : 0;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    float bm = 0.f;
    int bn = 0;
    for (int w = 0; w < kNoAllocThreads / 32; ++w) {
      bm = fmaxf(bm, s_max[w]);
      bn |= s_nan[w];
    }
    scratch[kNoAllocMaxBlocks - 1] = bm;
    scratch[2 * kNoAllocMaxBlocks - 1] = bn ? 1.f : 0.f;
  }
}

// device address of the scratch array on the current device (looked up once per device)
float* scratch_on_current_device() {
  int dev = 0;
  if (!cuda_ok(cudaGetDevice(&dev), "cudaGetDevice")) return nullptr;
  if (dev < 0 || dev >= kMaxDevices) {
    set_error(SF3D_ERR_ARG, "sf3d_field_maxabs_noalloc: device ordinal beyond 63");
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (!cuda_ok(rc, "cudaGetSymbolAddress(g_noalloc_scratch)")) return nullptr;
    g_scratch_ptr[dev] = p;
  }
  return static_cast<float*>(g_scratch_ptr[dev]);
}

}  // namespace
}  // namespace sf3d

using namespace sf3d;

extern "C" {

int sf3d_field_maxabs_noalloc(const realw* d_field, long n, void* stream, realw* max_abs) {
  if (!d_field || !max_abs) {
    set_error(SF3D_ERR_ARG, "sf3d_field_maxabs_noalloc: null pointer");
    return SF3D_ERR_ARG;
  }
  if (n <= 0 || n > kNoAllocMaxValues) {
    set_error(SF3D_ERR_ARG,
              "sf3d_field_maxabs_noalloc: n must be in [1, 536854528] (the fixed 256 KB scratch holds one partial "
              "per 16384 values)");
    return SF3D_ERR_ARG;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  if (s) {
    // the scratch address is the current device's: a stream of another device
    // would launch against it
    int sdev = -1, cur = -1;
    if (!cuda_ok(cudaStreamGetDevice(s, &sdev), "cudaStreamGetDevice") || !cuda_ok(cudaGetDevice(&cur), "cudaGetDevice"))
      return SF3D_ERR_CUDA;
    if (sdev != cur) {
      set_error(SF3D_ERR_ARG, "sf3d_field_maxabs_noalloc: the stream belongs to another device than the current one");
      return SF3D_ERR_ARG;
    }
  }
  float* scratch = scratch_on_current_device();
  if (!scratch) return SF3D_ERR_CUDA;
  const int nblocks = (int)((n + kNoAllocPerBlock - 1) / kNoAllocPerBlock);
  noalloc_partial_kernel<<<nblocks, kNoAllocThreads, 0, s>>>(d_field, n, scratch);
  noalloc_final_kernel<<<1, kNoAllocThreads, 0, s>>>(nblocks, scratch);
  if (!cuda_ok(cudaGetLastError(), "sf3d_field_maxabs_noalloc")) return SF3D_ERR_CUDA;
  float h[2] = {0.f, 0.f};
  if (!cuda_ok(cudaMemcpyAsync(&h[0], scratch + kNoAllocMaxBlocks - 1, sizeof(float), cudaMemcpyDeviceToHost, s),
               "cudaMemcpyAsync") ||
      !cuda_ok(cudaMemcpyAsync(&h[1], scratch + 2 * kNoAllocMaxBlocks - 1, sizeof(float), cudaMemcpyDeviceToHost, s),
               "cudaMemcpyAsync") ||
      !cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize"))
    return SF3D_ERR_CUDA;
  *max_abs = h[1] != 0.f ? NAN : h[0];
  return SF3D_OK;
}

}  // extern "C"
