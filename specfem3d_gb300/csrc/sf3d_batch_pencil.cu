// Batched-shots stiffness with register-blocked pencils (sm_103a).
//
// The per-point batched kernels (sf3d_batch.cu) give every thread one GLL point
// and read the five neighbours of each 5-wide contraction from shared memory:
// 90 shared loads per point and shot for the two contraction sets, which makes
// them shared-memory bound.  Here a thread owns a pencil: the five points of
// one line of the element along the direction being contracted, for one shot.
// It holds the line's values in registers and forms all five outputs of the
// contraction from them (25 FMAs per five loads instead of five per five), so
// each value crosses shared memory once per direction.  Per element and shot:
//   x pass   the thread's x-line gathered from HBM -> d/dxi at its 5 points
//   y pass   y-line from shared memory            -> d/deta
//   z pass   z-line from shared memory            -> d/dgamma, then strain,
//            stress and J sigma grad(xi) at the z-line's points (each point
//            belongs to exactly one z-line, so no other thread touches it)
//   then the transposed contractions with hprimewgll along x, y, z, the
//   weighted sum accumulated in shared memory and, in the z pass, the
//   scatter-add of the element's force into the stacked acceleration.
// Shared memory holds nine rows of 125 points x W shots with the shot
// innermost: the W lanes of a pencil read W consecutive words, and the 32/W
// pencils of a warp are consecutive in line order, whose point offsets (5, 1,
// 1, or 5, 21, 1 on a wrap) are odd, so every pass is free of bank conflicts.
// The arithmetic per point and shot is that of stiffness_kernel<ATT=0>
// (compute_forces_viscoelastic.F90:250-860): the same stress and J sigma
// grad(xi); the 5-wide contractions use the even / odd split of the derivative
// matrices (eo5: 20 operations per line of five instead of 25 FMAs, equal to
// the FMA chains up to rounding), and the sum of the three weighted contraction
// directions is formed in two steps.
#include "sf3d_internal.h"

namespace sf3d {
namespace {

constexpr int kPencils = 25;

template <int GEOM>
__device__ __forceinline__ float moduli_value(const PencilArgs& a, const ElemPack* pk, unsigned vary, int base,
                                              int q, long eo, int p) {
  if (GEOM == kGeomFP32) return __ldg((q == 9 ? a.kappav : a.muv) + eo);
  return pack_value<GEOM>(pk, a.pool, vary, base, q, p);
}

template <int GEOM>
__device__ __forceinline__ float metric_value(const PencilArgs& a, const ElemPack* pk, unsigned vary, int base, int q,
                                              int ir, int p) {
  if (GEOM == kGeomFP32) return __ldg(a.m[q] + (long)ir * NGLL3_PAD + p);
  return pack_value<GEOM>(pk, a.pool, vary, base, q, p);
}

// thread = (pencil pc, shot lane w), w fastest; CTA = one element x W shots
template <int W, int MINB, int GEOM>
__global__ void __launch_bounds__(kPencils * W, MINB) batch_pencil_kernel(const PencilArgs a) {
  extern __shared__ __align__(16) float smem[];
  float* s_gll = smem;                // hprime, hprimewgll, wgllwgll_xy, _xz, _yz (125)
  float* rows = smem + NGLL3_PAD;     // [9][125][W]
  const int tid = threadIdx.x;
  const int w = tid % W, pc = tid / W;
  const int pa = pc % NGLLX, pb = pc / NGLLX;
  const int tile = blockIdx.x % a.shot_tiles;
  const int slot = blockIdx.x / a.shot_tiles;
  // stacked-field indices in 32 bits: the host allows this kernel only while
  // 3 nglob nshots < 2^32 (pencil_fits_index32)
  const unsigned S = a.nshots;
  const unsigned shot = a.shot_offset + tile * W + w;
  const int e = a.phase ? __ldg(a.phase + slot) : slot;
  const int ir = __ldg(a.irregular + e);
  const long eb = (long)e * NGLL3_PAD;
  if (tid < NGLL3) s_gll[tid] = __ldg(a.gll + tid);
#define ROW(r, p) rows[((r) * NGLL3 + (p)) * W + w]
  const int xb = NGLLX * pa + NGLL2 * pb;   // x-line (l, pa, pb)
  const int yb = pa + NGLL2 * pb;           // y-line (pa, l, pb)
  const int zb = pa + NGLLX * pb;           // z-line (pa, pb, l)

  // ---- x pass: gather the x-line, contract along xi -----------------------------
  float u[3][NGLLX];
#pragma unroll
  for (int l = 0; l < NGLLX; ++l) {
    const unsigned gb = 3u * (unsigned)__ldg(a.ibool + eb + xb + l) * S + shot;
#pragma unroll
    for (int c = 0; c < 3; ++c) u[c][l] = a.displ[gb + c * S];
  }
  __syncthreads();  // s_gll
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float t[NGLLX];
    eo5(u[c], a.ek, t);
#pragma unroll
    for (int o = 0; o < NGLLX; ++o) {
      ROW(3 + c, xb + o) = t[o];            // rows 3-5: d/dxi
      ROW(c, xb + o) = u[c][o];             // rows 0-2: displacement
    }
  }
  __syncthreads();

  // ---- y pass: d/deta along the y-line ------------------------------------------
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float v[NGLLX];
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) v[l] = ROW(c, yb + NGLLX * l);
    float t[NGLLX];
    eo5(v, a.ek, t);
#pragma unroll
    for (int o = 0; o < NGLLX; ++o) ROW(6 + c, yb + NGLLX * o) = t[o];   // rows 6-8: d/deta
  }
  // ---- z pass: d/dgamma along the z-line (kept in registers until the stress) ---
  float t3[3][NGLLX];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float v[NGLLX];
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) v[l] = ROW(c, zb + NGLL2 * l);
    eo5(v, a.ek, t3[c]);
  }
  __syncthreads();  // rows 3-8 complete; every read of rows 0-2 done

  // ---- strain, stress and J sigma grad(xi) at the z-line's points ---------------
  // F[d][c] (contraction direction d, component c): d = 0, 1 go to row 3d + c (rows
  // 0-2 hold nothing live at these points any more, rows 3-5 were just read by this
  // thread); d = 2 stays in registers for the z-line's own transposed contraction
  const ElemPack* pk = GEOM != kGeomFP32 ? a.pack + e : nullptr;
  const unsigned vary = GEOM != kGeomFP32 ? __ldg(&pk->vary) : 0u;
  const int pbase = GEOM != kGeomFP32 ? __ldg(&pk->base) : 0;
  float fz[3][NGLLX];
#pragma unroll
  for (int o = 0; o < NGLLX; ++o) {
    const int p = zb + NGLL2 * o;
    const float t1x = ROW(3, p), t1y = ROW(4, p), t1z = ROW(5, p);
    const float t2x = ROW(6, p), t2y = ROW(7, p), t2z = ROW(8, p);
    const float t3x = t3[0][o], t3y = t3[1][o], t3z = t3[2][o];
    const float kap = moduli_value<GEOM>(a, pk, vary, pbase, 9, eb + p, p);
    const float mu = moduli_value<GEOM>(a, pk, vary, pbase, 10, eb + p, p);
    const float l2m = kap + (4.f / 3.f) * mu;
    const float lam = l2m - 2.f * mu;
    float F[9];
    if (ir >= 0) {
      float m[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) m[q] = metric_value<GEOM>(a, pk, vary, pbase, q, ir, p);
      const float xix = m[0], xiy = m[1], xiz = m[2], etax = m[3], etay = m[4], etaz = m[5];
      const float gammax = m[6], gammay = m[7], gammaz = m[8];
      const float dxx = xix * t1x + etax * t2x + gammax * t3x;
      const float dxy = xiy * t1x + etay * t2x + gammay * t3x;
      const float dxz = xiz * t1x + etaz * t2x + gammaz * t3x;
      const float dyx = xix * t1y + etax * t2y + gammax * t3y;
      const float dyy = xiy * t1y + etay * t2y + gammay * t3y;
      const float dyz = xiz * t1y + etaz * t2y + gammaz * t3y;
      const float dzx = xix * t1z + etax * t2z + gammax * t3z;
      const float dzy = xiy * t1z + etay * t2z + gammay * t3z;
      const float dzz = xiz * t1z + etaz * t2z + gammaz * t3z;
      const float sxx = l2m * dxx + lam * (dyy + dzz);
      const float syy = l2m * dyy + lam * (dxx + dzz);
      const float szz = l2m * dzz + lam * (dxx + dyy);
      const float sxy = mu * (dxy + dyx);
      const float sxz = mu * (dzx + dxz);
      const float syz = mu * (dzy + dyz);
      const float jac = 1.f / (xix * (etay * gammaz - etaz * gammay) - xiy * (etax * gammaz - etaz * gammax) +
                               xiz * (etax * gammay - etay * gammax));
      F[0] = jac * (sxx * xix + sxy * xiy + sxz * xiz);
      F[1] = jac * (sxy * xix + syy * xiy + syz * xiz);
      F[2] = jac * (sxz * xix + syz * xiy + szz * xiz);
      F[3] = jac * (sxx * etax + sxy * etay + sxz * etaz);
      F[4] = jac * (sxy * etax + syy * etay + syz * etaz);
      F[5] = jac * (sxz * etax + syz * etay + szz * etaz);
      F[6] = jac * (sxx * gammax + sxy * gammay + sxz * gammaz);
      F[7] = jac * (sxy * gammax + syy * gammay + syz * gammaz);
      F[8] = jac * (sxz * gammax + syz * gammay + szz * gammaz);
    } else {
      const float xr = a.xix_regular;
      const float dxx = xr * t1x, dxy = xr * t2x, dxz = xr * t3x;
      const float dyx = xr * t1y, dyy = xr * t2y, dyz = xr * t3y;
      const float dzx = xr * t1z, dzy = xr * t2z, dzz = xr * t3z;
      const float sxx = l2m * dxx + lam * (dyy + dzz);
      const float syy = l2m * dyy + lam * (dxx + dzz);
      const float szz = l2m * dzz + lam * (dxx + dyy);
      const float sxy = mu * (dxy + dyx);
      const float sxz = mu * (dzx + dxz);
      const float syz = mu * (dzy + dyz);
      const float js = a.jacobian_regular * xr;
      F[0] = js * sxx; F[1] = js * sxy; F[2] = js * sxz;
      F[3] = js * sxy; F[4] = js * syy; F[5] = js * syz;
      F[6] = js * sxz; F[7] = js * syz; F[8] = js * szz;
    }
#pragma unroll
    for (int q = 0; q < 6; ++q) ROW(q, p) = F[q];
#pragma unroll
    for (int c = 0; c < 3; ++c) fz[c][o] = F[6 + c];
  }
  __syncthreads();

  // ---- transposed contractions along x (rows 0-2) and y (rows 3-5), each written
  // in place along the thread's own line: the two passes touch disjoint rows, so
  // no barrier separates them
  {
    const float fac1 = s_gll[4 * NGLL2 + pa + NGLLX * pb];  // wgllwgll_yz(j, k)
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float v[NGLLX];
#pragma unroll
      for (int l = 0; l < NGLLX; ++l) v[l] = ROW(c, xb + l);
      float n[NGLLX];
      eo5(v, a.ekw, n);
#pragma unroll
      for (int o = 0; o < NGLLX; ++o) ROW(c, xb + o) = fac1 * n[o];
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      float v[NGLLX];
#pragma unroll
      for (int l = 0; l < NGLLX; ++l) v[l] = ROW(3 + c, yb + NGLLX * l);
      float n[NGLLX];
      eo5(v, a.ekw, n);
#pragma unroll
      for (int o = 0; o < NGLLX; ++o) ROW(3 + c, yb + NGLLX * o) = n[o];   // fac2 applied in the sum below
    }
  }
  __syncthreads();
  // ---- z from registers, the weighted sum (fac1 nx + fac2 ny + fac3 nz, in that
  // order and rounding) and the scatter-add ------------------------------------------
  {
    const float fac3 = s_gll[2 * NGLL2 + pa + NGLLX * pb];  // wgllwgll_xy(i, j)
    float nz[3][NGLLX];
#pragma unroll
    for (int c = 0; c < 3; ++c) eo5(fz[c], a.ekw, nz[c]);
#pragma unroll
    for (int o = 0; o < NGLLX; ++o) {
      const int p = zb + NGLL2 * o;
      const float fac2 = s_gll[3 * NGLL2 + pa + NGLLX * o];  // wgllwgll_xz(i, k)
      const unsigned gb = 3u * (unsigned)__ldg(a.ibool + eb + p) * S + shot;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float r = fmaf(fac2, ROW(3 + c, p), ROW(c, p));
        atomicAdd(a.accel + gb + c * S, -(r + fac3 * nz[c][o]));
      }
    }
  }
#undef ROW
}

template <int W, int MINB, int GEOM>
bool launch_w(const PencilArgs& a, cudaStream_t s) {
  const size_t smem = sizeof(float) * (NGLL3_PAD + 9 * NGLL3 * W);
  static bool configured = false;  // per instantiation: opt in to > 48 KB of shared memory once
  if (!configured) {
    if (!cuda_ok(cudaFuncSetAttribute(batch_pencil_kernel<W, MINB, GEOM>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                 "cudaFuncSetAttribute(batch_pencil_kernel)"))
      return false;
    configured = true;
  }
  const long nblocks = (long)a.nelem * a.shot_tiles;
  batch_pencil_kernel<W, MINB, GEOM><<<(unsigned)nblocks, kPencils * W, smem, s>>>(a);
  return true;
}

template <int GEOM>
bool launch_geom(const PencilArgs& a, int lanes, cudaStream_t s) {
  switch (lanes) {
    case 8: return launch_w<8, 4, GEOM>(a, s);
    case 16: return launch_w<16, 2, GEOM>(a, s);
    default: return launch_w<32, 1, GEOM>(a, s);
  }
}

}  // namespace

void even_odd_coefficients(const float* m, int so, int sl, float k[12]) {
  auto M = [&](int o, int l) { return (double)m[o * so + l * sl]; };
  for (int o = 0; o < 2; ++o) {
    k[5 * o + 0] = (float)(0.5 * (M(o, 0) - M(o, 4)));
    k[5 * o + 1] = (float)(0.5 * (M(o, 1) - M(o, 3)));
    k[5 * o + 2] = (float)(0.5 * (M(o, 0) + M(o, 4)));
    k[5 * o + 3] = (float)(0.5 * (M(o, 1) + M(o, 3)));
    k[5 * o + 4] = (float)M(o, 2);
  }
  k[10] = (float)M(2, 0);
  k[11] = (float)M(2, 1);
}

// lanes: shots per CTA (8, 16 or 32; divides the launch's shot count);
// geom_format: the Mesh's packed static streams (kGeomFP32: the FP32 arrays)
bool launch_batch_pencil(const PencilArgs& a, int lanes, int geom_format, cudaStream_t s) {
  if (a.nelem <= 0) return true;
  switch (geom_format) {
    case kGeomPackF16: return launch_geom<kGeomPackF16>(a, lanes, s);
    case kGeomPackBF16: return launch_geom<kGeomPackBF16>(a, lanes, s);
    case kGeomPackF32: return launch_geom<kGeomPackF32>(a, lanes, s);
    default: return launch_geom<kGeomFP32>(a, lanes, s);
  }
}

}  // namespace sf3d
