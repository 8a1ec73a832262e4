// Misfit post-processing on the device: adjoint sources from seismograms and
// the summation of event kernels (sm_103a).
//
// Adjoint sources (utils/adjoint_sources/{waveform,traveltime,amplitude}):
// one CTA per (receiver, component) trace, FP64 throughout as the reference
// tools (real*8):
//   window  is = int((ts - t0)/dt) + 1, ie = int((te - t0)/dt) + 1 (1-based);
//   waveform    tw: cosine taper over 10 % of the window at each end
//               (create_adjsrc_waveform.f90:241-249), r = syn - dat,
//               norm = dt sum(tw r^2), adj = r tw (:262-287);
//   traveltime  tw = 1 - (2 (j - is)/(ie - is) - 1)^2, v = centred difference
//               of syn (one-sided at the ends), norm = dt sum(tw v^2),
//               adj = -v tw / norm (create_adjsrc_traveltime.f90:141-162);
//   amplitude   same window, adj = syn tw / norm (create_adjsrc_amplitude.f90:140-157);
// a component other than `component` (1-3; 0 = all) is zeroed, and so is a
// trace whose |norm| <= 1e-17.  The norms are returned per trace.
//
// Kernel summation (src/tomography/sum_kernels.f90:215-315): the event kernels
// (optionally times their source masks) accumulated in FP64 on the device,
// with the norm sum(k^2) of every event kernel before masking.
#include <math.h>

#include <algorithm>
#include <vector>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

constexpr int kTraceThreads = 256;
constexpr double kAdjEps = 1.0e-17;        // create_adjsrc_*.f90: EPS
constexpr double kAdjPi = 3.1415926;       // create_adjsrc_waveform.f90: PI as the tool declares it

__device__ double block_sum(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  for (int q = 0; q < kTraceThreads / 32; ++q) s += red[q];
  return s;
}

// window weight at 1-based sample j
__device__ double window(int kind, int j, int is, int ie, int taper) {
  if (j < is || j > ie) return 0.0;
  if (kind == 0) {
    if (j < is + taper) return (1.0 - cos(kAdjPi * 2.0 * (double)(j - is) / (double)(taper - 1))) / 2.0;
    if (j <= ie - taper) return 1.0;
    return (1.0 - cos(kAdjPi * 2.0 * (double)(ie - j) / (double)(taper - 1))) / 2.0;
  }
  const double x = 2.0 * ((double)j - is) / (double)(ie - is) - 1.0;
  return 1.0 - x * x;
}

// measured signal at 0-based sample t: waveform residual, velocity, displacement
__device__ double signal(int kind, const double* s, const double* d, int t, int nstep, double dt) {
  if (kind == 0) return s[t] - d[t];
  if (kind == 2) return s[t];
  if (t == 0) return (s[1] - s[0]) / dt;
  if (t == nstep - 1) return (s[nstep - 1] - s[nstep - 2]) / dt;
  return (s[t + 1] - s[t - 1]) / (2.0 * dt);
}

__global__ void __launch_bounds__(kTraceThreads) adjoint_source_kernel(int kind, int nstep, int is, int ie, int taper,
                                                                       double dt, int component,
                                                                       const double* __restrict__ syn,
                                                                       const double* __restrict__ dat,
                                                                       double* __restrict__ adj,
                                                                       double* __restrict__ norms) {
  __shared__ double red[kTraceThreads / 32];
  const long tr = blockIdx.x;           // trace = 3 * receiver + component
  const int comp = (int)(tr % 3) + 1;
  const double* s = syn + tr * nstep;
  const double* d = dat ? dat + tr * nstep : nullptr;
  double acc = 0.0;
  for (int t = threadIdx.x; t < nstep; t += kTraceThreads) {
    const double w = window(kind, t + 1, is, ie, taper);
    if (w != 0.0) {
      const double o = signal(kind, s, d, t, nstep, dt);
      acc += w * o * o;
    }
  }
  double norm = dt * block_sum(acc, red);
  if (component != 0 && component != comp) norm = 0.0;
  const bool keep = fabs(norm) > kAdjEps;
  for (int t = threadIdx.x; t < nstep; t += kTraceThreads) {
    double a = 0.0;
    if (keep) {
      const double w = window(kind, t + 1, is, ie, taper);
      const double o = signal(kind, s, d, t, nstep, dt);
      a = kind == 0 ? o * w : (kind == 1 ? -o * w / norm : o * w / norm);
    }
    adj[tr * nstep + t] = a;
  }
  if (threadIdx.x == 0) norms[tr] = norm;
}

__global__ void sum_event_kernel(long n, const float* __restrict__ k, const float* __restrict__ mask,
                                 double* __restrict__ total, double* __restrict__ partial) {
  __shared__ double red[kTraceThreads / 32];
  double acc = 0.0;
  for (long i = (long)blockIdx.x * kTraceThreads + threadIdx.x; i < n; i += (long)gridDim.x * kTraceThreads) {
    const double v = (double)k[i];
    acc += v * v;
    total[i] += mask ? v * (double)mask[i] : v;
  }
  const double s = block_sum(acc, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

}  // namespace
}  // namespace sf3d

using namespace sf3d;

extern "C" {

int sf3d_adjoint_sources(int kind, int nrec, int nstep, double dt, double t0, double ts, double te, int component,
                         const double* h_syn, const double* h_dat, double* h_adj, double* h_norms) {
  if (kind < 0 || kind > 2 || nrec < 1 || nstep < 3 || !(dt > 0.0) || !h_syn || !h_adj || !h_norms ||
      (kind == 0 && !h_dat) || component < 0 || component > 3) {
    set_error(SF3D_ERR_ARG, "sf3d_adjoint_sources: invalid arguments");
    return SF3D_ERR_ARG;
  }
  const int is = (int)((ts - t0) / dt) + 1, ie = (int)((te - t0) / dt) + 1;
  if (is < 1 || ie <= is || ie > nstep) {
    set_error(SF3D_ERR_ARG, "sf3d_adjoint_sources: window [ts, te] outside the trace (Error in ts, te)");
    return SF3D_ERR_ARG;
  }
  const int taper = (int)(0.1 * (ie - is));
  if (kind == 0 && taper < 2) {
    // the tool's cosine taper divides by (taper - 1): windows shorter than 20
    // samples give a division by zero there
    set_error(SF3D_ERR_ARG, "sf3d_adjoint_sources: waveform window shorter than 20 samples (taper length < 2)");
    return SF3D_ERR_ARG;
  }
  const size_t n = (size_t)3 * nrec * nstep;
  double *d_syn = nullptr, *d_dat = nullptr, *d_adj = nullptr, *d_norm = nullptr;
  bool ok = alloc_zero((void**)&d_syn, sizeof(double) * n) && alloc_zero((void**)&d_adj, sizeof(double) * n) &&
            alloc_zero((void**)&d_norm, sizeof(double) * 3 * nrec) &&
            (kind != 0 || alloc_zero((void**)&d_dat, sizeof(double) * n));
  ok = ok && cuda_ok(cudaMemcpy(d_syn, h_syn, sizeof(double) * n, cudaMemcpyHostToDevice), "cudaMemcpy") &&
       (kind != 0 || cuda_ok(cudaMemcpy(d_dat, h_dat, sizeof(double) * n, cudaMemcpyHostToDevice), "cudaMemcpy"));
  if (ok) {
    adjoint_source_kernel<<<3 * nrec, kTraceThreads>>>(kind, nstep, is, ie, taper, dt, component, d_syn, d_dat,
                                                        d_adj, d_norm);
    ok = cuda_ok(cudaGetLastError(), "adjoint_source_kernel") &&
         cuda_ok(cudaMemcpy(h_adj, d_adj, sizeof(double) * n, cudaMemcpyDeviceToHost), "cudaMemcpy") &&
         cuda_ok(cudaMemcpy(h_norms, d_norm, sizeof(double) * 3 * nrec, cudaMemcpyDeviceToHost), "cudaMemcpy");
  }
  cudaFree(d_syn); cudaFree(d_dat); cudaFree(d_adj); cudaFree(d_norm);
  return ok ? SF3D_OK : SF3D_ERR_CUDA;
}

int sf3d_sum_kernels(int nker, long n, const realw* const* h_kernels, const realw* const* h_masks, double* h_total,
                     realw* h_total_f32, double* h_norms) {
  if (nker < 1 || n < 1 || !h_kernels || !h_total || !h_norms) {
    set_error(SF3D_ERR_ARG, "sf3d_sum_kernels: invalid arguments");
    return SF3D_ERR_ARG;
  }
  for (int q = 0; q < nker; ++q)
    if (!h_kernels[q] || (h_masks && !h_masks[q])) {
      set_error(SF3D_ERR_ARG, "sf3d_sum_kernels: null kernel or mask");
      return SF3D_ERR_ARG;
    }
  const int nblocks = (int)std::min<long>((n + kTraceThreads - 1) / kTraceThreads, 2048);
  double *d_total = nullptr, *d_part = nullptr;
  float *d_k = nullptr, *d_m = nullptr;
  bool ok = alloc_zero((void**)&d_total, sizeof(double) * n) && alloc_zero((void**)&d_k, sizeof(float) * n) &&
            alloc_zero((void**)&d_part, sizeof(double) * nblocks) &&
            (!h_masks || alloc_zero((void**)&d_m, sizeof(float) * n));
  std::vector<double> part(nblocks);
  for (int q = 0; ok && q < nker; ++q) {
    ok = cuda_ok(cudaMemcpy(d_k, h_kernels[q], sizeof(float) * n, cudaMemcpyHostToDevice), "cudaMemcpy") &&
         (!h_masks || cuda_ok(cudaMemcpy(d_m, h_masks[q], sizeof(float) * n, cudaMemcpyHostToDevice), "cudaMemcpy"));
    if (!ok) break;
    sum_event_kernel<<<nblocks, kTraceThreads>>>(n, d_k, d_m, d_total, d_part);
    ok = cuda_ok(cudaGetLastError(), "sum_event_kernel") &&
         cuda_ok(cudaMemcpy(part.data(), d_part, sizeof(double) * nblocks, cudaMemcpyDeviceToHost), "cudaMemcpy");
    double s = 0.0;
    for (int b = 0; b < nblocks; ++b) s += part[b];
    h_norms[q] = s;
  }
  ok = ok && cuda_ok(cudaMemcpy(h_total, d_total, sizeof(double) * n, cudaMemcpyDeviceToHost), "cudaMemcpy");
  if (ok && h_total_f32)
    for (long i = 0; i < n; ++i) h_total_f32[i] = (float)h_total[i];
  cudaFree(d_total); cudaFree(d_part); cudaFree(d_k); cudaFree(d_m);
  return ok ? SF3D_OK : SF3D_ERR_CUDA;
}

}  // extern "C"
