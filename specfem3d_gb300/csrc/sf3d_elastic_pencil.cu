// Elastic stiffness of one wavefield without attenuation, register-blocked
// pencils (sm_103a).
//
// The one-CTA-per-element kernel (sf3d_elastic.cu) gives every thread one GLL
// point and reads the five neighbours of each 5-wide contraction, and the
// five hprime coefficients, from shared memory.  Without attenuation a regular
// element moves only 1.5 KB of static streams, and that kernel is bound by
// instruction issue and the shared-memory pipe, not by HBM.  Here a thread owns
// a pencil: the five points of one line of an element, held in registers, so
// all five outputs of a contraction come from five loads, the coefficients are
// kernel parameters, and every value crosses shared memory once per direction.  Per element:
//   gather   the thread's z-line from HBM into shared memory
//   x pass   x-line from shared memory -> d/dxi
//   y pass   y-line from shared memory -> d/deta
//   z pass   z-line from shared memory -> d/dgamma (registers)
//   stress and J sigma grad(xi) at the z-line's points, the transposed
//   contractions along x and y in shared memory and along z in registers, and
//   the weighted sum scatter-added into accel at the z-line's points.
// A CTA holds W elements, thread = (element w, pencil pc) with the pencil
// fastest: the 25 lanes of an element gather and scatter a whole xy-plane of it
// per instruction, as the one-point-per-thread kernel does.  Shared memory
// holds nine rows of W elements at a pitch of 153 words: 153 = 25 (mod 32), so
// the lanes of a warp (one element's tail, the next one's head) address banks
// in thread order at the z-line points, where half of the shared accesses are;
// the x- and y-line accesses of warps that straddle two elements take two
// wavefronts (no pitch or assignment of lines to lanes avoids that for both).
// The element's kappa / mu (and metric) rows are prefetched into L1 at kernel
// start, since the stress stage is their first use.
// The arithmetic per point is that of stiffness_kernel<ATT=0, STRAIN=0>
// (compute_forces_viscoelastic.F90:250-860): the same stress and J sigma
// grad(xi); the 5-wide contractions use the even / odd split of the derivative
// matrices (eo5, equal to the FMA chains up to rounding), and the three weighted
// transposed contractions are summed as fac1 nx + fac2 ny + fac3 nz.
#include "sf3d_internal.h"

namespace sf3d {
namespace {

constexpr int kPencils = 25;
constexpr int kPitch = 153;   // words per element row; 153 = 25 (mod 32)

__device__ __forceinline__ void prefetch_l1(const void* p) {
  asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

template <int W, int MINB>
__global__ void __launch_bounds__(kPencils * W, MINB) elem_pencil_kernel(const ElemPencilArgs a) {
  extern __shared__ __align__(16) float smem[];
  float* s_gll = smem;                // hprime, hprimewgll, wgllwgll_xy, _xz, _yz (125)
  float* rows = smem + NGLL3_PAD;     // [9][W][kPitch]
  const int tid = threadIdx.x;
  const int pc = tid % kPencils, w = tid / kPencils;
  const int pa = pc % NGLLX, pb = pc / NGLLX;
  const int slot = blockIdx.x * W + w;
  const bool live = slot < a.nelem;   // the last CTA of a phase may hold fewer elements
  const int e = live ? (a.phase ? __ldg(a.phase + slot) : slot) : 0;
  const int ir = live ? __ldg(a.irregular + e) : -1;
  const long eb = (long)e * NGLL3_PAD;
  if (tid < NGLL3) s_gll[tid] = __ldg(a.gll + tid);
#define ROW(r, p) rows[((r) * W + w) * kPitch + (p)]
  const int xb = NGLLX * pa + NGLL2 * pb;   // x-line (l, pa, pb)
  const int yb = pa + NGLL2 * pb;           // y-line (pa, l, pb)
  const int zb = pa + NGLLX * pb;           // z-line (pa, pb, l)

  // the element's kappa / mu rows and, if irregular, its nine metric rows (128-byte
  // lines, 4 a row) are first read in the stress stage: the element's lanes
  // prefetch them into L1 now, so those reads do not wait on HBM
  if (live) {
#pragma unroll
    for (int q = pc; q < 44; q += kPencils) {
      if (q < 8)
        prefetch_l1((q < 4 ? a.kappav : a.muv) + eb + 32 * (q & 3));
      else if (ir >= 0)
        prefetch_l1(a.m[(q - 8) >> 2] + (long)ir * NGLL3_PAD + 32 * (q & 3));
    }
  }

  // ---- gather the z-line into rows 0-2 ------------------------------------------
  {
    float u[3][NGLLX];
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) {
      const long g = live ? (long)__ldg(a.ibool + eb + zb + NGLL2 * l) : 0;
#pragma unroll
      for (int c = 0; c < 3; ++c) u[c][l] = live ? a.displ[3 * g + c] : 0.f;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int o = 0; o < NGLLX; ++o) ROW(c, zb + NGLL2 * o) = u[c][o];
  }
  __syncthreads();

  // ---- x and y passes: d/dxi to rows 3-5, d/deta to rows 6-8 ------------------
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float v[NGLLX];
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) v[l] = ROW(c, xb + l);
    float t[NGLLX];
    eo5(v, a.ek, t);
#pragma unroll
    for (int o = 0; o < NGLLX; ++o) ROW(3 + c, xb + o) = t[o];
  }
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float v[NGLLX];
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) v[l] = ROW(c, yb + NGLLX * l);
    float t[NGLLX];
    eo5(v, a.ek, t);
#pragma unroll
    for (int o = 0; o < NGLLX; ++o) ROW(6 + c, yb + NGLLX * o) = t[o];
  }
  // ---- z pass: d/dgamma along the thread's own z-line, kept in registers ------
  float t3[3][NGLLX];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float v[NGLLX];
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) v[l] = ROW(c, zb + NGLL2 * l);
    eo5(v, a.ek, t3[c]);
  }
  __syncthreads();  // rows 3-8 complete; every read of rows 0-2 done

  // ---- stress and J sigma grad(xi) at the z-line's points: F[d][c] for d = 0, 1
  // to row 3d + c (rows 0-2 hold nothing live any more, rows 3-5 at these points
  // were just read by this thread), d = 2 kept in registers ----------------------
  float fz[3][NGLLX];
#pragma unroll
  for (int o = 0; o < NGLLX; ++o) {
    const int p = zb + NGLL2 * o;
    const float t1x = ROW(3, p), t1y = ROW(4, p), t1z = ROW(5, p);
    const float t2x = ROW(6, p), t2y = ROW(7, p), t2z = ROW(8, p);
    const float t3x = t3[0][o], t3y = t3[1][o], t3z = t3[2][o];
    const float kap = live ? __ldg(a.kappav + eb + p) : 0.f;
    const float mu = live ? __ldg(a.muv + eb + p) : 0.f;
    const float l2m = kap + (4.f / 3.f) * mu;
    const float lam = l2m - 2.f * mu;
    float F[9];
    if (ir >= 0) {
      float m[9];
#pragma unroll
      for (int q = 0; q < 9; ++q) m[q] = __ldg(a.m[q] + (long)ir * NGLL3_PAD + p);
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

  // ---- transposed contractions along x (rows 0-2) and y (rows 3-5), each in place
  // along the thread's own line (disjoint rows: no barrier between them) ----------
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
  // ---- z from registers, the weighted sum and the scatter-add ---------------------
  if (live) {
    const float fac3 = s_gll[2 * NGLL2 + pa + NGLLX * pb];  // wgllwgll_xy(i, j)
    float nz[3][NGLLX];
#pragma unroll
    for (int c = 0; c < 3; ++c) eo5(fz[c], a.ekw, nz[c]);
#pragma unroll
    for (int o = 0; o < NGLLX; ++o) {
      const int p = zb + NGLL2 * o;
      const float fac2 = s_gll[3 * NGLL2 + pa + NGLLX * o];  // wgllwgll_xz(i, k)
      const long g = __ldg(a.ibool + eb + p);
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        const float r = fmaf(fac2, ROW(3 + c, p), ROW(c, p));
        atomicAdd(a.accel + 3 * g + c, -(r + fac3 * nz[c][o]));
      }
    }
  }
#undef ROW
}

template <int W, int MINB>
bool launch_w(const ElemPencilArgs& a, cudaStream_t s) {
  const size_t smem = sizeof(float) * (NGLL3_PAD + 9 * kPitch * W);
  static bool configured = false;  // per instantiation: opt in to > 48 KB of shared memory once
  if (!configured) {
    if (!cuda_ok(cudaFuncSetAttribute(elem_pencil_kernel<W, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem),
                 "cudaFuncSetAttribute(elem_pencil_kernel)"))
      return false;
    configured = true;
  }
  const long nblocks = (a.nelem + W - 1) / W;
  elem_pencil_kernel<W, MINB><<<(unsigned)nblocks, kPencils * W, smem, s>>>(a);
  return true;
}

}  // namespace

// five elements per CTA (125 threads), compiled for 8 (register budget 64) or
// 7 (72) resident CTAs per SM; measured on GB300, eight elements per CTA (200
// threads, 4 or 5 CTAs/SM) ran 7-15 % slower on both no-attenuation workloads
bool launch_elem_pencil(const ElemPencilArgs& a, int blocks_per_sm, cudaStream_t s) {
  if (a.nelem <= 0) return true;
  return blocks_per_sm == 7 ? launch_w<5, 7>(a, s) : launch_w<5, 8>(a, s);
}

void run_elem_pencil(Mesh* mp, const StiffnessArgs& a, int blocks_per_sm, cudaStream_t s) {
  ElemPencilArgs q;
  memset(&q, 0, sizeof(q));
  q.nelem = a.nelem;
  q.phase = a.phase;
  q.ibool = a.ibool;
  q.irregular = a.irregular;
  for (int c = 0; c < 9; ++c) q.m[c] = a.m[c];
  q.kappav = a.kappav;
  q.muv = a.muv;
  q.gll = a.gll;
  q.xix_regular = a.xix_regular;
  q.jacobian_regular = a.jacobian_regular;
  q.displ = a.displ;
  q.accel = a.accel;
  memcpy(q.hp, mp->h_hprime, sizeof(q.hp));
  memcpy(q.hpw, mp->h_hprimewgll, sizeof(q.hpw));
  even_odd_coefficients(mp->h_hprime, 1, NGLLX, q.ek);
  even_odd_coefficients(mp->h_hprimewgll, NGLLX, 1, q.ekw);
  launch_elem_pencil(q, blocks_per_sm, s);
}

}  // namespace sf3d
