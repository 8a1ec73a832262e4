// Gaussian smoothing of sensitivity kernels over the mesh (xsmooth_sem's GPU
// mode): for every GLL point of this slice, sum over the GLL points of nearby
// elements of a slice (itself or a neighbour) of
//   w = exp(-(dx^2 + dy^2) / (2 sigma_h^2) - dz^2 / (2 sigma_v^2)) * J w_i w_j w_k
// times the kernel values, and of w alone; the result is the ratio.
//
// Replaces prepare_smooth_gpu / compute_smooth_gpu / get_smooth_gpu
// (src/gpu/smooth_cuda.cu:40-248) and follows kernels/process_smooth.cu:30-194:
// an element of the other slice takes part when its centre (the mean of its first
// and last GLL points) lies within sigma_h3 horizontally and sigma_v3 vertically
// of the target element's GLL point number (element index mod 125); exponents
// below -86 give 0.  The sums are kept in FP64 across elements (the reference
// keeps them in FP32).  The reference scans every element of the other slice and
// evaluates the weights once per kernel; here the other slice's elements are
// binned on a uniform grid of cells (sigma_h3 x sigma_h3 x sigma_v3) so each
// target element scans only the cells its search box touches, and the weights of
// a point pair serve all kernels at once.
#include <math.h>

#include <vector>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

constexpr int kMaxKernels = 8;

struct SmoothState {
  int nspec_me = 0, nker = 0;
  float* x_me = nullptr;
  float* y_me = nullptr;
  float* z_me = nullptr;
  double* data_smooth = nullptr;    // (nker, 125 * nspec_me)
  double* normalisation = nullptr;  // (125 * nspec_me)
  float sigma_h2_inv = 0.f, sigma_v2_inv = 0.f;
  float h_criterion = 0.f, v_criterion = 0.f;   // sigma_h3^2, sigma_v3^2
  float sigma_h3 = 0.f, sigma_v3 = 0.f;
};

struct SmoothArgs {
  const float* x_me;
  const float* y_me;
  const float* z_me;
  const float* x_o;
  const float* y_o;
  const float* z_o;
  const float* integ;
  const float* data;               // (nker, 125 * nspec_other)
  const int* cell_start;           // (ncells + 1)
  const int* cell_elems;           // elements by cell, element order inside a cell
  int nspec_me, nspec_other, nker;
  int ncx, ncy, ncz;
  float ox, oy, oz, csh, csv;      // grid origin and cell sizes
  float sigma_h3, sigma_v3;
  float sigma_h2_inv, sigma_v2_inv, h_criterion, v_criterion;
  double* data_smooth;
  double* normalisation;
};

__device__ __forceinline__ float block_reduce(float v, bool take_max, float* scratch) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float w = __shfl_xor_sync(0xffffffffu, v, o);
    v = take_max ? fmaxf(v, w) : fminf(v, w);
  }
  const int t = threadIdx.x;
  __syncthreads();
  if ((t & 31) == 0) scratch[t >> 5] = v;
  __syncthreads();
  float r = scratch[0];
  for (int q = 1; q < (int)(blockDim.x >> 5); ++q) r = take_max ? fmaxf(r, scratch[q]) : fminf(r, scratch[q]);
  return r;
}

// One CTA (128 threads) per target element; thread = GLL point.
__global__ void __launch_bounds__(NGLL3_PAD) smooth_kernel(const SmoothArgs a) {
  extern __shared__ float s_dyn[];               // nker * 125 kernel values of one element
  __shared__ float s_mx[NGLL3_PAD], s_my[NGLL3_PAD], s_mz[NGLL3_PAD];
  __shared__ float s_ox[NGLL3_PAD], s_oy[NGLL3_PAD], s_oz[NGLL3_PAD], s_oi[NGLL3_PAD];
  __shared__ int s_list[NGLL3_PAD];
  __shared__ int s_warp[4];
  __shared__ float s_red[4];
  const int e = blockIdx.x, t = threadIdx.x;
  const bool active = t < NGLL3;
  const long me = (long)e * NGLL3 + t;
  float x = 0.f, y = 0.f, z = 0.f;
  if (active) {
    x = a.x_me[me];
    y = a.y_me[me];
    z = a.z_me[me];
  }
  s_mx[t] = x;
  s_my[t] = y;
  s_mz[t] = z;
  // search box of the element: its bounding box grown by the search radii
  const float big = 3.0e38f;
  const float xmin = block_reduce(active ? x : big, false, s_red), xmax = block_reduce(active ? x : -big, true, s_red);
  const float ymin = block_reduce(active ? y : big, false, s_red), ymax = block_reduce(active ? y : -big, true, s_red);
  const float zmin = block_reduce(active ? z : big, false, s_red), zmax = block_reduce(active ? z : -big, true, s_red);
  auto cell_lo = [](float v, float o, float c, int n) { return max(0, min(n - 1, (int)floorf((v - o) / c))); };
  const int cx0 = cell_lo(xmin - a.sigma_h3, a.ox, a.csh, a.ncx), cx1 = cell_lo(xmax + a.sigma_h3, a.ox, a.csh, a.ncx);
  const int cy0 = cell_lo(ymin - a.sigma_h3, a.oy, a.csh, a.ncy), cy1 = cell_lo(ymax + a.sigma_h3, a.oy, a.csh, a.ncy);
  const int cz0 = cell_lo(zmin - a.sigma_v3, a.oz, a.csv, a.ncz), cz1 = cell_lo(zmax + a.sigma_v3, a.oz, a.csv, a.ncz);
  // per element FP32 partial sums folded into FP64 totals: the totals gather
  // thousands of terms, which in FP32 alone would lose ~1e-5
  double acc[kMaxKernels];
#pragma unroll
  for (int k = 0; k < kMaxKernels; ++k) acc[k] = 0.0;
  double norm = 0.0;
  const long no = (long)a.nspec_other * NGLL3;
  for (int cz = cz0; cz <= cz1; ++cz)
    for (int cy = cy0; cy <= cy1; ++cy)
      for (int cx = cx0; cx <= cx1; ++cx) {
        const int c = cx + a.ncx * (cy + a.ncy * cz);
        const int beg = a.cell_start[c], end = a.cell_start[c + 1];
        for (int base = beg; base < end; base += NGLL3_PAD) {
          // each thread tests one candidate element with the target point the
          // reference's thread (element index mod 125) would use
          bool take = false;
          int o = -1;
          if (base + t < end) {
            o = a.cell_elems[base + t];
            const long f = (long)o * NGLL3;
            const float ccx = (a.x_o[f] + a.x_o[f + NGLL3 - 1]) * 0.5f;
            const float ccy = (a.y_o[f] + a.y_o[f + NGLL3 - 1]) * 0.5f;
            const float ccz = (a.z_o[f] + a.z_o[f + NGLL3 - 1]) * 0.5f;
            const int p = o % NGLL3;
            const float dh = (s_mx[p] - ccx) * (s_mx[p] - ccx) + (s_my[p] - ccy) * (s_my[p] - ccy);
            const float dv = (s_mz[p] - ccz) * (s_mz[p] - ccz);
            take = !(dh > a.h_criterion || dv > a.v_criterion);
          }
          // compact the accepted elements into s_list (warp ballots + warp offsets)
          const unsigned bal = __ballot_sync(0xffffffffu, take);
          if ((t & 31) == 0) s_warp[t >> 5] = __popc(bal);
          __syncthreads();
          int off = 0, total = 0;
          for (int q = 0; q < 4; ++q) {
            if (q < (t >> 5)) off += s_warp[q];
            total += s_warp[q];
          }
          if (take) s_list[off + __popc(bal & ((1u << (t & 31)) - 1u))] = o;
          __syncthreads();
          for (int q = 0; q < total; ++q) {
            const int oo = s_list[q];
            const long f = (long)oo * NGLL3;
            if (active) {
              s_ox[t] = a.x_o[f + t];
              s_oy[t] = a.y_o[f + t];
              s_oz[t] = a.z_o[f + t];
              s_oi[t] = a.integ[f + t];
              for (int k = 0; k < a.nker; ++k) s_dyn[k * NGLL3 + t] = a.data[k * no + f + t];
            }
            __syncthreads();
            if (active) {
              float pe[kMaxKernels];
#pragma unroll
              for (int k = 0; k < kMaxKernels; ++k) pe[k] = 0.f;
              float ne = 0.f;
              for (int j = 0; j < NGLL3; ++j) {
                const float dx = x - s_ox[j], dy = y - s_oy[j], dz = z - s_oz[j];
                const float val = -(dx * dx + dy * dy) * a.sigma_h2_inv - dz * dz * a.sigma_v2_inv;
                const float g = val < -86.0f ? 0.0f : expf(val);
                const float coef = g * s_oi[j];
                ne += coef;
#pragma unroll
                for (int k = 0; k < kMaxKernels; ++k)
                  if (k < a.nker) pe[k] = fmaf(s_dyn[k * NGLL3 + j], coef, pe[k]);
              }
              norm += (double)ne;
#pragma unroll
              for (int k = 0; k < kMaxKernels; ++k)
                if (k < a.nker) acc[k] += (double)pe[k];
            }
            __syncthreads();
          }
        }
      }
  if (active) {
    const long n = (long)a.nspec_me * NGLL3;
#pragma unroll
    for (int k = 0; k < kMaxKernels; ++k)
      if (k < a.nker) a.data_smooth[k * n + me] += acc[k];
    a.normalisation[me] += norm;
  }
}

// normalize_data (process_smooth.cu): value / sum of weights, rounded to FP32
__global__ void normalize_kernel(const double* data, const double* norm, float* out, long n, int nker) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double w = norm[i];
  if (w < 1.e-24) w = 1.0;
  for (int k = 0; k < nker; ++k) out[k * n + i] = (float)(data[k * n + i] / w);
}

SmoothState* get_smooth(long* p) {
  if (!p || !*p) {
    set_error(SF3D_ERR_STATE, "smoothing handle not prepared (prepare_smooth_gpu)");
    return nullptr;
  }
  return reinterpret_cast<SmoothState*>(*p);
}

}  // namespace
}  // namespace sf3d

using namespace sf3d;

extern "C" {

void prepare_smooth_gpu_(long* Container, realw* xstore_me, realw* ystore_me, realw* zstore_me, realw* sigma_h2,
                         realw* sigma_v2, realw* sigma_h3, realw* sigma_v3, int* nspec_me, int* nker) {
  if (!Container) return;
  *Container = 0;
  if (*nspec_me <= 0 || *nker <= 0 || *nker > kMaxKernels) {
    set_error(SF3D_ERR_ARG, "prepare_smooth_gpu: nspec_me > 0 and 1 <= nker <= 8 required");
    return;
  }
  if (!(*sigma_h2 > 0.f) || !(*sigma_v2 > 0.f)) {
    set_error(SF3D_ERR_ARG, "prepare_smooth_gpu: sigma_h2 and sigma_v2 must be positive");
    return;
  }
  SmoothState* sp = new SmoothState;
  sp->nspec_me = *nspec_me;
  sp->nker = *nker;
  sp->sigma_h2_inv = 1.0f / *sigma_h2;
  sp->sigma_v2_inv = 1.0f / *sigma_v2;
  sp->h_criterion = *sigma_h3 * *sigma_h3;
  sp->v_criterion = *sigma_v3 * *sigma_v3;
  sp->sigma_h3 = *sigma_h3;
  sp->sigma_v3 = *sigma_v3;
  const size_t n = (size_t)NGLL3 * sp->nspec_me;
  bool ok = alloc_zero((void**)&sp->x_me, sizeof(float) * n) && alloc_zero((void**)&sp->y_me, sizeof(float) * n) &&
            alloc_zero((void**)&sp->z_me, sizeof(float) * n) &&
            alloc_zero((void**)&sp->data_smooth, sizeof(double) * n * sp->nker) &&
            alloc_zero((void**)&sp->normalisation, sizeof(double) * n);
  ok = ok && cudaMemcpy(sp->x_me, xstore_me, sizeof(float) * n, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(sp->y_me, ystore_me, sizeof(float) * n, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(sp->z_me, zstore_me, sizeof(float) * n, cudaMemcpyHostToDevice) == cudaSuccess;
  if (!ok) {
    cudaFree(sp->x_me); cudaFree(sp->y_me); cudaFree(sp->z_me); cudaFree(sp->data_smooth); cudaFree(sp->normalisation);
    delete sp;
    set_error(SF3D_ERR_CUDA, "prepare_smooth_gpu: device allocation or copy failed");
    return;
  }
  *Container = reinterpret_cast<long>(sp);
}

void compute_smooth_gpu_(long* smooth_pointer, realw* data_other, realw* integ_factor, realw* xstore_other,
                         realw* ystore_other, realw* zstore_other, const int* nspec_other_f) {
  NvtxRange nvtx_range("compute_smooth_gpu");
  SmoothState* sp = get_smooth(smooth_pointer);
  if (!sp) return;
  const int nso = *nspec_other_f;
  if (nso <= 0) return;
  const size_t n = (size_t)NGLL3 * nso;
  // element centres of the other slice (mean of the first and last GLL point,
  // process_smooth.cu:84-86) and a uniform grid of cells over them
  std::vector<float> cx(nso), cy(nso), cz(nso);
  float lo[3] = {3.0e38f, 3.0e38f, 3.0e38f}, hi[3] = {-3.0e38f, -3.0e38f, -3.0e38f};
  for (int o = 0; o < nso; ++o) {
    const size_t f = (size_t)o * NGLL3;
    cx[o] = (xstore_other[f] + xstore_other[f + NGLL3 - 1]) * 0.5f;
    cy[o] = (ystore_other[f] + ystore_other[f + NGLL3 - 1]) * 0.5f;
    cz[o] = (zstore_other[f] + zstore_other[f + NGLL3 - 1]) * 0.5f;
    const float c[3] = {cx[o], cy[o], cz[o]};
    for (int d = 0; d < 3; ++d) { lo[d] = fminf(lo[d], c[d]); hi[d] = fmaxf(hi[d], c[d]); }
  }
  float csh = fmaxf(sp->sigma_h3, 1e-6f), csv = fmaxf(sp->sigma_v3, 1e-6f);
  long ncx, ncy, ncz;
  for (;;) {   // at most 4M cells: coarser cells only cost more candidate tests
    ncx = (long)floorf((hi[0] - lo[0]) / csh) + 1;
    ncy = (long)floorf((hi[1] - lo[1]) / csh) + 1;
    ncz = (long)floorf((hi[2] - lo[2]) / csv) + 1;
    if (ncx * ncy * ncz <= (1L << 22)) break;
    csh *= 2.f;
    csv *= 2.f;
  }
  const long ncell = ncx * ncy * ncz;
  std::vector<int> cell_of(nso), start(ncell + 1, 0), elems(nso);
  for (int o = 0; o < nso; ++o) {
    const long ix = std::min(ncx - 1, std::max(0L, (long)floorf((cx[o] - lo[0]) / csh)));
    const long iy = std::min(ncy - 1, std::max(0L, (long)floorf((cy[o] - lo[1]) / csh)));
    const long iz = std::min(ncz - 1, std::max(0L, (long)floorf((cz[o] - lo[2]) / csv)));
    cell_of[o] = (int)(ix + ncx * (iy + ncy * iz));
    start[cell_of[o] + 1]++;
  }
  for (long c = 0; c < ncell; ++c) start[c + 1] += start[c];
  {
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int o = 0; o < nso; ++o) elems[fill[cell_of[o]]++] = o;   // element order inside a cell
  }
  float *dx = nullptr, *dy = nullptr, *dz = nullptr, *di = nullptr, *dd = nullptr;
  int *dstart = nullptr, *delems = nullptr;
  bool ok = alloc_zero((void**)&dx, sizeof(float) * n) && alloc_zero((void**)&dy, sizeof(float) * n) &&
            alloc_zero((void**)&dz, sizeof(float) * n) && alloc_zero((void**)&di, sizeof(float) * n) &&
            alloc_zero((void**)&dd, sizeof(float) * n * sp->nker) &&
            alloc_zero((void**)&dstart, sizeof(int) * (ncell + 1)) && alloc_zero((void**)&delems, sizeof(int) * nso);
  ok = ok && cudaMemcpy(dx, xstore_other, sizeof(float) * n, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(dy, ystore_other, sizeof(float) * n, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(dz, zstore_other, sizeof(float) * n, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(di, integ_factor, sizeof(float) * n, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(dd, data_other, sizeof(float) * n * sp->nker, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(dstart, start.data(), sizeof(int) * (ncell + 1), cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(delems, elems.data(), sizeof(int) * nso, cudaMemcpyHostToDevice) == cudaSuccess;
  if (ok) {
    SmoothArgs a;
    a.x_me = sp->x_me; a.y_me = sp->y_me; a.z_me = sp->z_me;
    a.x_o = dx; a.y_o = dy; a.z_o = dz; a.integ = di; a.data = dd;
    a.cell_start = dstart; a.cell_elems = delems;
    a.nspec_me = sp->nspec_me; a.nspec_other = nso; a.nker = sp->nker;
    a.ncx = (int)ncx; a.ncy = (int)ncy; a.ncz = (int)ncz;
    a.ox = lo[0]; a.oy = lo[1]; a.oz = lo[2]; a.csh = csh; a.csv = csv;
    a.sigma_h3 = sp->sigma_h3; a.sigma_v3 = sp->sigma_v3;
    a.sigma_h2_inv = sp->sigma_h2_inv; a.sigma_v2_inv = sp->sigma_v2_inv;
    a.h_criterion = sp->h_criterion; a.v_criterion = sp->v_criterion;
    a.data_smooth = sp->data_smooth; a.normalisation = sp->normalisation;
    smooth_kernel<<<sp->nspec_me, NGLL3_PAD, sizeof(float) * NGLL3 * sp->nker>>>(a);
    ok = cuda_ok(cudaGetLastError(), "smooth_kernel") && cuda_ok(cudaDeviceSynchronize(), "smooth_kernel");
  } else {
    set_error(SF3D_ERR_CUDA, "compute_smooth_gpu: device allocation or copy failed");
  }
  cudaFree(dx); cudaFree(dy); cudaFree(dz); cudaFree(di); cudaFree(dd); cudaFree(dstart); cudaFree(delems);
}

void get_smooth_gpu_(long* smooth_pointer, realw* data_smooth) {
  SmoothState* sp = get_smooth(smooth_pointer);
  if (!sp) return;
  const long n = (long)NGLL3 * sp->nspec_me;
  float* d_out = nullptr;
  if (alloc_zero((void**)&d_out, sizeof(float) * n * sp->nker)) {
    normalize_kernel<<<(unsigned)((n + 255) / 256), 256>>>(sp->data_smooth, sp->normalisation, d_out, n, sp->nker);
    if (cuda_ok(cudaGetLastError(), "normalize_kernel"))
      SF3D_CUDA(cudaMemcpy(data_smooth, d_out, sizeof(float) * n * sp->nker, cudaMemcpyDeviceToHost));
    cudaFree(d_out);
  } else {
    set_error(SF3D_ERR_CUDA, "get_smooth_gpu: device allocation failed");
  }
  cudaFree(sp->x_me); cudaFree(sp->y_me); cudaFree(sp->z_me); cudaFree(sp->data_smooth); cudaFree(sp->normalisation);
  delete sp;
  *smooth_pointer = 0;
}

}  // extern "C"
