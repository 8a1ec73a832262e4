// Packed static element streams of the stiffness kernel (geometric factors,
// moduli and attenuation factors) with per-element scales.
//
// For every element and each of the 17 static streams (nine metric rows of an
// irregular element, kappa, mu, factor_common and factor_common_kappa for the
// three standard linear solids) the encoder finds the minimum and maximum over
// the element's 125 GLL points:
//   * a stream that is constant over the element (box-shaped elements of a
//     structured mesh, layered moduli, per-element attenuation factors) is
//     stored as its value alone, exactly, in the element's record;
//   * a stream that varies gets a payload row of 128 values in a compact pool,
//     value = offset + scale * h with offset = (max + min) / 2 and
//     scale = (max - min) / 2, h in [-1, 1] stored as FP16 (absolute error at
//     most scale * 2^-11) or BF16 (scale * 2^-8); the FP32 pool stores the value
//     itself (offset 0, scale 1), which makes the packing lossless.
// Only varying streams cost payload bytes, so a mesh of box elements with
// per-element materials reads 160 bytes of static data per element instead of
// 8,500 (attenuation) or 5,500 (elastic).  Fields, memory variables and all
// arithmetic stay FP32.  The FP32 arrays are kept: other kernels (Stacey,
// gradient, batched shots) read them.
#include <cuda_bf16.h>
#include <math.h>

#include <vector>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

struct PackSources {
  const int* irregular;
  const float* m[9];
  const float* kappav;
  const float* muv;
  const float* fc;   // [nspec][3][128] or nullptr
  const float* fck;
};

// value of stream q at point t of element e; `present` false where the stream
// does not exist (metric of a regular element, factors without attenuation)
__device__ __forceinline__ float source_value(const PackSources& S, int q, long e, int t, bool* present) {
  *present = true;
  if (q < 9) {
    const int ir = S.irregular[e];
    if (ir < 0) { *present = false; return 0.f; }
    return S.m[q][(long)ir * NGLL3_PAD + t];
  }
  if (q == 9) return S.kappav[e * NGLL3_PAD + t];
  if (q == 10) return S.muv[e * NGLL3_PAD + t];
  const float* f = q < 14 ? S.fc : S.fck;
  if (!f) { *present = false; return 0.f; }
  return f[e * (NSLS * NGLL3_PAD) + (long)((q - 11) % 3) * NGLL3_PAD + t];
}

// pass 1, one 128-thread CTA per element: (offset, scale) and the varying mask
// of every stream, and the element's payload row count
__global__ void pack_stats_kernel(PackSources S, int format, ElemPack* __restrict__ pack, int* __restrict__ nrows) {
  __shared__ float s_lo[4], s_hi[4];
  const long e = blockIdx.x;
  const int t = threadIdx.x;
  unsigned vary = 0;
  for (int q = 0; q < kPackStreams; ++q) {
    bool present = true;
    const float v = t < NGLL3 ? source_value(S, q, e, t, &present) : 0.f;
    if (!present) {  // uniform over the CTA
      if (t == 0) pack[e].so[q] = make_float2(0.f, 0.f);
      continue;
    }
    float lo = t < NGLL3 ? v : INFINITY, hi = t < NGLL3 ? v : -INFINITY;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
      hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    __syncthreads();  // the previous stream's reads of s_lo / s_hi are done
    if ((t & 31) == 0) {
      s_lo[t >> 5] = lo;
      s_hi[t >> 5] = hi;
    }
    __syncthreads();
    lo = fminf(fminf(s_lo[0], s_lo[1]), fminf(s_lo[2], s_lo[3]));
    hi = fmaxf(fmaxf(s_hi[0], s_hi[1]), fmaxf(s_hi[2], s_hi[3]));
    if (hi > lo) {
      vary |= 1u << q;
      if (t == 0)
        pack[e].so[q] = format == kGeomPackF32 ? make_float2(0.f, 1.f) : make_float2(0.5f * (hi + lo), 0.5f * (hi - lo));
    } else if (t == 0) {
      pack[e].so[q] = make_float2(lo, 0.f);
    }
  }
  if (t == 0) {
    pack[e].vary = vary;
    nrows[e] = __popc(vary);
  }
}

// pass 2, one CTA per element: the element's first payload row and its payload values
__global__ void pack_payload_kernel(PackSources S, int format, const int* __restrict__ base, ElemPack* __restrict__ pack,
                                    void* __restrict__ pool) {
  const long e = blockIdx.x;
  const int t = threadIdx.x;
  const unsigned vary = pack[e].vary;
  const int b = base[e];
  if (t == 0) pack[e].base = b;
  for (int q = 0; q < kPackStreams; ++q) {
    if (!((vary >> q) & 1u)) continue;
    const long i = ((long)b + __popc(vary & ((1u << q) - 1u))) * NGLL3_PAD + t;
    bool present = true;
    const float v = t < NGLL3 ? source_value(S, q, e, t, &present) : 0.f;
    const float2 so = pack[e].so[q];
    const float h = t < NGLL3 ? (v - so.x) / so.y : 0.f;
    if (format == kGeomPackF16)
      static_cast<__half*>(pool)[i] = __float2half_rn(fminf(fmaxf(h, -1.f), 1.f));
    else if (format == kGeomPackBF16)
      static_cast<__nv_bfloat16*>(pool)[i] = __float2bfloat16_rn(fminf(fmaxf(h, -1.f), 1.f));
    else
      static_cast<float*>(pool)[i] = t < NGLL3 ? v : 0.f;
  }
}

size_t pool_value_bytes(int format) { return format == kGeomPackF32 ? 4 : 2; }

}  // namespace

void free_geometry_pack(Mesh* mp) {
  cudaFree(mp->d_pack);
  cudaFree(mp->d_pack_pool);
  mp->d_pack = nullptr;
  mp->d_pack_pool = nullptr;
  mp->pack_rows = 0;
  mp->geom_format = kGeomFP32;
}

}  // namespace sf3d

using namespace sf3d;

extern "C" {

int sf3d_set_geometry_format(long* Mesh_pointer, int format) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (format < kGeomFP32 || format > kGeomPackF32) {
    set_error(SF3D_ERR_ARG, "sf3d_set_geometry_format: format must be 0 (FP32 arrays), 1 (FP16), 2 (BF16) or 3 (FP32 pool)");
    return SF3D_ERR_ARG;
  }
  if (format != kGeomFP32 && mp->anisotropy) {
    set_error(SF3D_ERR_ARG, "sf3d_set_geometry_format: packed streams are for isotropic moduli");
    return SF3D_ERR_ARG;
  }
  if (!mp->d_kappav || !mp->d_muv) {
    set_error(SF3D_ERR_STATE, "sf3d_set_geometry_format: prepare_fields_elastic_device not called");
    return SF3D_ERR_STATE;
  }
  SF3D_CUDA_RET(cudaStreamSynchronize(mp->stream), SF3D_ERR_CUDA);
  free_geometry_pack(mp);
  if (format == kGeomFP32) return SF3D_OK;
  PackSources S;
  S.irregular = mp->d_irregular;
  for (int q = 0; q < 9; ++q) S.m[q] = mp->d_metric[q];
  S.kappav = mp->d_kappav;
  S.muv = mp->d_muv;
  S.fc = mp->attenuation ? mp->d_factor_common : nullptr;
  S.fck = mp->attenuation ? mp->d_factor_common_kappa : nullptr;
  const long nspec = mp->nspec;
  int* d_n = nullptr;
  bool ok = alloc_zero((void**)&mp->d_pack, sizeof(ElemPack) * nspec) && alloc_zero((void**)&d_n, sizeof(int) * nspec);
  if (ok) {
    pack_stats_kernel<<<(unsigned)nspec, NGLL3_PAD, 0, mp->stream>>>(S, format, mp->d_pack, d_n);
    ok = cuda_ok(cudaGetLastError(), "pack_stats_kernel");
  }
  // exclusive prefix sum of the payload rows per element (host; once per mesh)
  std::vector<int> n(nspec);
  long rows = 0;
  if (ok) ok = copy_sync(n.data(), d_n, sizeof(int) * nspec, cudaMemcpyDeviceToHost, mp->stream);
  if (ok) {
    for (long e = 0; e < nspec; ++e) {
      const int c = n[e];
      n[e] = (int)rows;
      rows += c;
    }
    if (rows > 0x7fffffffL) {
      set_error(SF3D_ERR_ARG, "sf3d_set_geometry_format: more than 2^31 payload rows");
      ok = false;
    }
  }
  if (ok) ok = copy_sync(d_n, n.data(), sizeof(int) * nspec, cudaMemcpyHostToDevice, mp->stream);
  if (ok) ok = alloc_zero(&mp->d_pack_pool, pool_value_bytes(format) * NGLL3_PAD * (size_t)(rows > 0 ? rows : 1));
  if (ok) {
    pack_payload_kernel<<<(unsigned)nspec, NGLL3_PAD, 0, mp->stream>>>(S, format, d_n, mp->d_pack, mp->d_pack_pool);
    ok = cuda_ok(cudaGetLastError(), "pack_payload_kernel") &&
         cuda_ok(cudaStreamSynchronize(mp->stream), "cudaStreamSynchronize");
  }
  cudaFree(d_n);
  if (!ok) {
    free_geometry_pack(mp);
    return SF3D_ERR_CUDA;
  }
  mp->pack_rows = rows;
  mp->geom_format = format;
  return SF3D_OK;
}

int sf3d_set_geometry_precision(long* Mesh_pointer, int bits) {
  if (bits != 16 && bits != 32) {
    set_error(SF3D_ERR_ARG, "sf3d_set_geometry_precision: bits must be 16 or 32");
    return SF3D_ERR_ARG;
  }
  return sf3d_set_geometry_format(Mesh_pointer, bits == 16 ? kGeomPackF16 : kGeomFP32);
}

int sf3d_geometry_pack_info(long* Mesh_pointer, long* payload_rows, long* device_bytes) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!payload_rows || !device_bytes) {
    set_error(SF3D_ERR_ARG, "sf3d_geometry_pack_info: null pointer");
    return SF3D_ERR_ARG;
  }
  *payload_rows = mp->geom_format ? mp->pack_rows : 0;
  *device_bytes = mp->geom_format ? (long)(sizeof(ElemPack) * mp->nspec +
                                           pool_value_bytes(mp->geom_format) * NGLL3_PAD * mp->pack_rows)
                                  : 0;
  return SF3D_OK;
}

}  // extern "C"
