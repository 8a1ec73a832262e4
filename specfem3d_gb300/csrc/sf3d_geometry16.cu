// 16-bit geometric factors and moduli with per-element scales.
//
// The stiffness kernel's static per-element streams (nine metric rows of
// irregular elements, kappa and mu) are stored as FP16 with one
// (offset, scale) pair per element and array: value = offset + scale * h,
// h = (value - min) / (max - min) rounded to FP16, so h lies in [0, 1].  A row
// that is constant over the element (box-shaped elements, layered moduli) is
// stored exactly (scale 0); elsewhere the absolute error is at most
// (max - min) * 2^-12, i.e. relative to the range inside one element, not to
// the value.  Fields, memory variables and all arithmetic stay FP32.  The FP32
// arrays are kept: other kernels (Stacey, gradient, batched shots) read them.
#include <math.h>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

// one 128-thread block per 128-value row (125 valid)
__global__ void encode_rows_kernel(const float* __restrict__ src, __half* __restrict__ dst, float2* __restrict__ so) {
  __shared__ float s_min[4], s_max[4];
  const long row = blockIdx.x;
  const int t = threadIdx.x;
  const float v = t < NGLL3 ? src[row * NGLL3_PAD + t] : 0.f;
  float lo = t < NGLL3 ? v : INFINITY, hi = t < NGLL3 ? v : -INFINITY;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((t & 31) == 0) {
    s_min[t >> 5] = lo;
    s_max[t >> 5] = hi;
  }
  __syncthreads();
  lo = fminf(fminf(s_min[0], s_min[1]), fminf(s_min[2], s_min[3]));
  hi = fmaxf(fmaxf(s_max[0], s_max[1]), fmaxf(s_max[2], s_max[3]));
  const float range = hi - lo;
  const float h = (t < NGLL3 && range > 0.f) ? (v - lo) / range : 0.f;
  dst[row * NGLL3_PAD + t] = __float2half_rn(h);
  if (t == 0) so[row] = make_float2(lo, range);
}

bool encode(Mesh* mp, const float* src, long nrows, __half** dst, float2* so) {
  if (nrows <= 0) return true;
  if (!alloc_zero((void**)dst, sizeof(__half) * nrows * NGLL3_PAD)) return false;
  encode_rows_kernel<<<(unsigned)nrows, NGLL3_PAD, 0, mp->stream>>>(src, *dst, so);
  return cuda_ok(cudaGetLastError(), "encode_rows_kernel");
}

}  // namespace

void free_half_geometry(Mesh* mp) {
  for (int q = 0; q < 9; ++q) {
    cudaFree(mp->d_metric_h[q]);
    mp->d_metric_h[q] = nullptr;
  }
  cudaFree(mp->d_metric_so); cudaFree(mp->d_kappa_h); cudaFree(mp->d_mu_h);
  cudaFree(mp->d_kappa_so); cudaFree(mp->d_mu_so);
  mp->d_metric_so = nullptr; mp->d_kappa_h = nullptr; mp->d_mu_h = nullptr;
  mp->d_kappa_so = nullptr; mp->d_mu_so = nullptr;
  mp->geom_half = 0;
}

}  // namespace sf3d

using namespace sf3d;

extern "C" {

int sf3d_set_geometry_precision(long* Mesh_pointer, int bits) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (bits != 16 && bits != 32) {
    set_error(SF3D_ERR_ARG, "sf3d_set_geometry_precision: bits must be 16 or 32");
    return SF3D_ERR_ARG;
  }
  if (bits == 16 && mp->anisotropy) {
    set_error(SF3D_ERR_ARG, "sf3d_set_geometry_precision: 16-bit storage is for isotropic moduli");
    return SF3D_ERR_ARG;
  }
  if (!mp->d_kappav || !mp->d_muv) {
    set_error(SF3D_ERR_STATE, "sf3d_set_geometry_precision: prepare_fields_elastic_device not called");
    return SF3D_ERR_STATE;
  }
  SF3D_CUDA_RET(cudaStreamSynchronize(mp->stream), SF3D_ERR_CUDA);
  free_half_geometry(mp);
  if (bits == 32) return SF3D_OK;
  const long nirr = mp->nspec_irregular;
  bool ok = alloc_zero((void**)&mp->d_kappa_so, sizeof(float2) * mp->nspec) &&
            alloc_zero((void**)&mp->d_mu_so, sizeof(float2) * mp->nspec);
  if (ok && nirr > 0) ok = alloc_zero((void**)&mp->d_metric_so, sizeof(float2) * 9 * nirr);
  ok = ok && encode(mp, mp->d_kappav, mp->nspec, &mp->d_kappa_h, mp->d_kappa_so) &&
       encode(mp, mp->d_muv, mp->nspec, &mp->d_mu_h, mp->d_mu_so);
  for (int q = 0; ok && q < 9 && nirr > 0; ++q)
    ok = encode(mp, mp->d_metric[q], nirr, &mp->d_metric_h[q], mp->d_metric_so + (long)q * nirr);
  ok = ok && cuda_ok(cudaStreamSynchronize(mp->stream), "cudaStreamSynchronize");
  if (!ok) {
    free_half_geometry(mp);
    return SF3D_ERR_CUDA;
  }
  mp->geom_half = 1;
  return SF3D_OK;
}

}  // extern "C"
