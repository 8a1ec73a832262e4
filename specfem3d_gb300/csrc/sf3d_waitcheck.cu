// Self-check of the bounded mbarrier wait that guards every bulk copy of the
// stiffness, C-PML and adjoint kernels (sm_103a).
//
// One CTA initialises an mbarrier, announces 16 bytes of transaction that no
// copy will ever deliver (mbarrier.arrive.expect_tx with no cp.async.bulk
// behind it), and every thread waits on it with the same bounded wait the
// kernels use, here with a short caller-given limit.  The wait gives up, the
// error word is set exactly as the kernels set it, the kernel returns, and the
// host reads the word: the path a real timeout would take, run without a fault,
// a trap or an unbounded spin, and with no asynchronous copy in flight.
#include "sf3d_internal.h"

namespace sf3d {
namespace {

__global__ void bounded_wait_check_kernel(int* err, unsigned long long limit_ns, unsigned long long* waited_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    mbar_arrive_expect_tx(&bar, 16u);   // the one arrival; 16 bytes that never come
  }
  __syncthreads();
  const uint64_t t0 = global_ns();
  if (!mbar_wait_bounded(&bar, 0, limit_ns)) atomicExch(err, 1);
  if (threadIdx.x == 0) *waited_ns = global_ns() - t0;
}

}  // namespace
}  // namespace sf3d

using namespace sf3d;

extern "C" int sf3d_check_bounded_wait(double limit_s, int* timed_out, double* waited_s) {
  if (!(limit_s > 0.0) || limit_s > 2.0 || !timed_out) {
    set_error(SF3D_ERR_ARG, "sf3d_check_bounded_wait: limit in (0, 2] s and a non-null timed_out");
    return SF3D_ERR_ARG;
  }
  int* d_err = nullptr;
  unsigned long long* d_ns = nullptr;
  bool ok = alloc_zero((void**)&d_err, sizeof(int)) && alloc_zero((void**)&d_ns, sizeof(unsigned long long));
  int h_err = 0;
  unsigned long long h_ns = 0;
  if (ok) {
    bounded_wait_check_kernel<<<1, 128>>>(d_err, (unsigned long long)(limit_s * 1e9), d_ns);
    ok = cuda_ok(cudaGetLastError(), "bounded_wait_check_kernel") &&
         cuda_ok(cudaDeviceSynchronize(), "cudaDeviceSynchronize") &&
         cuda_ok(cudaMemcpy(&h_err, d_err, sizeof(int), cudaMemcpyDeviceToHost), "cudaMemcpy") &&
         cuda_ok(cudaMemcpy(&h_ns, d_ns, sizeof(h_ns), cudaMemcpyDeviceToHost), "cudaMemcpy");
  }
  cudaFree(d_err);
  cudaFree(d_ns);
  if (!ok) return SF3D_ERR_CUDA;
  *timed_out = h_err;
  if (waited_s) *waited_s = (double)h_ns * 1e-9;
  return SF3D_OK;
}
