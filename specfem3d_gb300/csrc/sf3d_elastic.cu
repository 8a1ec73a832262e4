// Elastic / viscoelastic stiffness kernel (sm_103a).
//
// Computes, for every element of a phase list, the weak-form internal force
// exactly as compute_forces_viscoelastic.F90:250-860 does on the CPU:
//   gather u (and dt*v with attenuation) through ibool -> 5-wide derivative
//   contractions with hprime -> metric -> strain, isotropic stress minus the
//   memory variables -> J sigma grad(xi) -> transposed contractions with
//   hprimewgll -> weighted scatter-add (red.global.add.f32) into accel ->
//   memory-variable update (compute_element_att_memory.f90:28-157).
//
// Mapping: one 128-thread CTA per element, thread p < 125 owns GLL point
// p = i + 5j + 25k.  Every per-element HBM stream (ibool, metric, moduli,
// memory variables, strains, attenuation factors) is one aligned 512-byte row
// per array and is issued before the first barrier, so each CTA keeps its
// whole element (up to ~21 KB) in flight; the contractions exchange values
// through shared memory.  The 5-wide contractions stay on the FP32 pipes: they
// are far too small to feed the tensor cores.
#include "sf3d_internal.h"

namespace sf3d {

namespace {

// STAGE (attenuation only): the 30 memory-variable / strain / factor values of
// each point (15 KB per element) are copied into shared memory with cp.async
// instead of being held in registers from the start of the kernel to the end,
// so the kernel fits a smaller register budget (more resident CTAs per SM).
// BULK (with STAGE): thread 0 brings the same rows in with 14 bulk copies
// (cp.async.bulk, contiguous per component: R[c] 1536 B, epsilondev 512 B,
// factors 1536 B) completing on one mbarrier, so no thread spends an
// instruction or a register per row; every thread waits (bounded) on the
// mbarrier after the first barrier, where its initialisation is visible.
// Element streams are read and written exactly once per launch: with STREAM
// they carry evict-first hints (ld.global.cs / st.global.cs) so that L2 keeps
// the gathered displacement / velocity and the scattered acceleration, which
// neighbouring elements reuse.
template <bool STREAM>
__device__ __forceinline__ float ld_elem(const float* p) {
  return STREAM ? __ldcs(p) : __ldg(p);
}
template <bool STREAM>
__device__ __forceinline__ int ld_elem(const int* p) {
  return STREAM ? __ldcs(p) : __ldg(p);
}
template <bool STREAM>
__device__ __forceinline__ float ld_state(const float* p) {
  return STREAM ? __ldcs(p) : *p;
}
template <bool STREAM>
__device__ __forceinline__ void st_state(float* p, float v) {
  if (STREAM)
    __stcs(p, v);
  else
    *p = v;
}

// GEOM: kGeomFP32 reads the FP32 element arrays; the packed formats read the
// per-element records and payload rows of a.pack / a.pool instead (metric,
// kappa, mu and, with attenuation, factor_common(_kappa)).
template <bool ATT, bool STRAIN, int MINB, int GEOM = kGeomFP32, bool STAGE = false, bool ATOMIC = true,
          bool STREAM = false, bool ANISO = false, bool BULK = false>
__global__ void __launch_bounds__(NGLL3_PAD, MINB) stiffness_kernel(const StiffnessArgs a) {
  constexpr bool kBulkAtt = ATT && STAGE && BULK;   // the attenuation rows by bulk copy
  __shared__ __align__(16) float s_att[(ATT && STAGE) ? (GEOM == kGeomFP32 ? 30 : 24) : 1][NGLL3_PAD];
  __shared__ uint64_t s_bar;
  bool bulk_failed = false;
  __shared__ float s_gll[NGLL3];
  __shared__ __align__(16) float s_t[9][NGLL3_PAD];
  // the bulk-copy builds keep the displacement / velocity rows in rows 0-5 of
  // s_t (a barrier separates their last read from the first stress write): 3 KB
  // less shared memory a CTA, so one CTA more fits an SM
  constexpr bool kAlias = kBulkAtt;
  __shared__ __align__(16) float s_uv_own[kAlias ? 1 : (ATT ? 6 : 3)][NGLL3_PAD];
  float (*s_u)[NGLL3_PAD] = kAlias ? s_t : s_uv_own;
  // with attenuation a point's displacement and dt * velocity sit side by side
  // (float2): one shared load serves both gradients
  float2 (*s_uv)[NGLL3_PAD] = reinterpret_cast<float2 (*)[NGLL3_PAD]>(kAlias ? &s_t[0][0] : &s_uv_own[0][0]);

  const int t = threadIdx.x;
  const int e = a.phase ? __ldg(a.phase + blockIdx.x) : (int)blockIdx.x;
  const bool active = t < NGLL3;
  const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
  const long eo = (long)e * NGLL3_PAD + t;
  const int ir = __ldg(a.irregular + e);

  // ---- issue every HBM load of this element up front ------------------------
  int iglob = 0;
  float ux = 0.f, uy = 0.f, uz = 0.f, vx = 0.f, vy = 0.f, vz = 0.f;
  float m[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) m[q] = 0.f;
  float kap = 0.f, mu = 0.f;
  float R[6][NSLS], eold[6], fc[NSLS], fck[NSLS];
#pragma unroll
  for (int c = 0; c < 6; ++c) {
    eold[c] = 0.f;
#pragma unroll
    for (int s = 0; s < NSLS; ++s) R[c][s] = 0.f;
  }
#pragma unroll
  for (int s = 0; s < NSLS; ++s) fc[s] = fck[s] = 0.f;
  if (kBulkAtt) {
    if (t == 0) {
      constexpr int kRows = GEOM == kGeomFP32 ? 30 : 24;
      const long se0 = (long)e * (NSLS * NGLL3_PAD), ee0 = (long)e * NGLL3_PAD;
      mbar_init(&s_bar, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
      mbar_arrive_expect_tx(&s_bar, (uint32_t)(kRows * NGLL3_PAD * sizeof(float)));
#pragma unroll
      for (int c = 0; c < 6; ++c) bulk_g2s(&s_att[3 * c][0], a.R[c] + se0, NSLS * NGLL3_PAD * sizeof(float), &s_bar);
#pragma unroll
      for (int c = 0; c < 6; ++c) bulk_g2s(&s_att[18 + c][0], a.eps[c] + ee0, NGLL3_PAD * sizeof(float), &s_bar);
      if (GEOM == kGeomFP32) {
        bulk_g2s(&s_att[24][0], a.fc + se0, NSLS * NGLL3_PAD * sizeof(float), &s_bar);
        bulk_g2s(&s_att[27][0], a.fck + se0, NSLS * NGLL3_PAD * sizeof(float), &s_bar);
      }
    }
  }
  if (ATT && STAGE && !BULK && active) {
    // rows: R[c][s] -> 3c+s (0..17), epsilondev[c] -> 18+c, factor_common[s] -> 24+s,
    // factor_common_kappa[s] -> 27+s (FP32 geometry only: the packed formats read
    // the factors from the element record where they are used).  Each thread copies
    // (4-byte cp.async) and later reads only its own point's column, so no barrier
    // is needed, and the copies stay in flight through the first contraction set.
    const long se = (long)e * (NSLS * NGLL3_PAD) + t, ee = (long)e * NGLL3_PAD + t;
#pragma unroll
    for (int row = 0; row < (GEOM == kGeomFP32 ? 30 : 24); ++row) {
      const float* src;
      if (row < 18) src = a.R[row / 3] + se + (row % 3) * NGLL3_PAD;
      else if (row < 24) src = a.eps[row - 18] + ee;
      else if (row < 27) src = a.fc + se + (row - 24) * NGLL3_PAD;
      else src = a.fck + se + (row - 27) * NGLL3_PAD;
      cp_async4(&s_att[row][t], src);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
  }
  if (active) {
    iglob = ld_elem<STREAM>(a.ibool + eo);
    if (GEOM != kGeomFP32) {
      const ElemPack* pk = a.pack + e;
      const unsigned vary = __ldg(&pk->vary);
      const int base = __ldg(&pk->base);
      kap = pack_value<GEOM>(pk, a.pool, vary, base, 9, t);
      mu = pack_value<GEOM>(pk, a.pool, vary, base, 10, t);
      if (ir >= 0) {
#pragma unroll
        for (int q = 0; q < 9; ++q) m[q] = pack_value<GEOM>(pk, a.pool, vary, base, q, t);
      }
      if (ATT && !STAGE) {
#pragma unroll
        for (int s = 0; s < NSLS; ++s) {
          fc[s] = pack_value<GEOM>(pk, a.pool, vary, base, 11 + s, t);
          fck[s] = pack_value<GEOM>(pk, a.pool, vary, base, 14 + s, t);
        }
      }
    } else {
      kap = ld_elem<STREAM>(a.kappav + eo);
      mu = ld_elem<STREAM>(a.muv + eo);
      if (ir >= 0) {
        const long mo = (long)ir * NGLL3_PAD + t;
#pragma unroll
        for (int q = 0; q < 9; ++q) m[q] = ld_elem<STREAM>(a.m[q] + mo);
      }
    }
    if (ATT && !STAGE) {
      const long so = (long)e * (NSLS * NGLL3_PAD) + t;
#pragma unroll
      for (int c = 0; c < 6; ++c)
#pragma unroll
        for (int s = 0; s < NSLS; ++s) R[c][s] = ld_state<STREAM>(a.R[c] + so + s * NGLL3_PAD);
#pragma unroll
      for (int c = 0; c < 6; ++c) eold[c] = ld_state<STREAM>(a.eps[c] + eo);
      if (GEOM == kGeomFP32) {
#pragma unroll
        for (int s = 0; s < NSLS; ++s) {
          fc[s] = ld_elem<STREAM>(a.fc + so + s * NGLL3_PAD);
          fck[s] = ld_elem<STREAM>(a.fck + so + s * NGLL3_PAD);
        }
      }
    }
    ux = a.displ[3L * iglob];
    uy = a.displ[3L * iglob + 1];
    uz = a.displ[3L * iglob + 2];
    if (ATT) {
      vx = a.deltat * a.veloc[3L * iglob];
      vy = a.deltat * a.veloc[3L * iglob + 1];
      vz = a.deltat * a.veloc[3L * iglob + 2];
    }
  }
  if (t < NGLL3) s_gll[t] = __ldg(a.gll + t);
  if (ATT) {
    s_uv[0][t] = make_float2(ux, vx);
    s_uv[1][t] = make_float2(uy, vy);
    s_uv[2][t] = make_float2(uz, vz);
  } else {
    s_u[0][t] = ux;
    s_u[1][t] = uy;
    s_u[2][t] = uz;
  }
  __syncthreads();

  // ---- gradient, strain, stress ---------------------------------------------
  float epsl[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  float t1x = 0.f, t2x = 0.f, t3x = 0.f, t1y = 0.f, t2y = 0.f, t3y = 0.f, t1z = 0.f, t2z = 0.f, t3z = 0.f;
  float a1x = 0.f, a2x = 0.f, a3x = 0.f, a1y = 0.f, a2y = 0.f, a3y = 0.f, a1z = 0.f, a2z = 0.f, a3z = 0.f;
  if (active) {
    const float* hp = s_gll;  // hprime(i2,i1) = hp[i2 + 5 i1]
    if (ATT) {
      // gradients of u and of dt v in one loop; the strain of u + dt v is their sum
      float b1x = 0.f, b2x = 0.f, b3x = 0.f, b1y = 0.f, b2y = 0.f, b3y = 0.f, b1z = 0.f, b2z = 0.f, b3z = 0.f;
#pragma unroll
      for (int l = 0; l < NGLLX; ++l) {
        const float h1 = hp[i + NGLLX * l], h2 = hp[j + NGLLX * l], h3 = hp[k + NGLLX * l];
        const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
        float2 q;
        q = s_uv[0][p1]; t1x = fmaf(q.x, h1, t1x); b1x = fmaf(q.y, h1, b1x);
        q = s_uv[1][p1]; t1y = fmaf(q.x, h1, t1y); b1y = fmaf(q.y, h1, b1y);
        q = s_uv[2][p1]; t1z = fmaf(q.x, h1, t1z); b1z = fmaf(q.y, h1, b1z);
        q = s_uv[0][p2]; t2x = fmaf(q.x, h2, t2x); b2x = fmaf(q.y, h2, b2x);
        q = s_uv[1][p2]; t2y = fmaf(q.x, h2, t2y); b2y = fmaf(q.y, h2, b2y);
        q = s_uv[2][p2]; t2z = fmaf(q.x, h2, t2z); b2z = fmaf(q.y, h2, b2z);
        q = s_uv[0][p3]; t3x = fmaf(q.x, h3, t3x); b3x = fmaf(q.y, h3, b3x);
        q = s_uv[1][p3]; t3y = fmaf(q.x, h3, t3y); b3y = fmaf(q.y, h3, b3y);
        q = s_uv[2][p3]; t3z = fmaf(q.x, h3, t3z); b3z = fmaf(q.y, h3, b3z);
      }
      a1x = t1x + b1x; a2x = t2x + b2x; a3x = t3x + b3x;
      a1y = t1y + b1y; a2y = t2y + b2y; a3y = t3y + b3y;
      a1z = t1z + b1z; a2z = t2z + b2z; a3z = t3z + b3z;
    } else {
#pragma unroll
      for (int l = 0; l < NGLLX; ++l) {
        const float h1 = hp[i + NGLLX * l], h2 = hp[j + NGLLX * l], h3 = hp[k + NGLLX * l];
        const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
        t1x = fmaf(s_u[0][p1], h1, t1x); t1y = fmaf(s_u[1][p1], h1, t1y); t1z = fmaf(s_u[2][p1], h1, t1z);
        t2x = fmaf(s_u[0][p2], h2, t2x); t2y = fmaf(s_u[1][p2], h2, t2y); t2z = fmaf(s_u[2][p2], h2, t2z);
        t3x = fmaf(s_u[0][p3], h3, t3x); t3y = fmaf(s_u[1][p3], h3, t3y); t3z = fmaf(s_u[2][p3], h3, t3z);
      }
    }
  }
  if (kAlias) __syncthreads();  // every read of s_uv done: s_t may be written
  if (active) {
    const float xr = a.xix_regular;
    const float xix = m[0], xiy = m[1], xiz = m[2], etax = m[3], etay = m[4], etaz = m[5];
    const float gammax = m[6], gammay = m[7], gammaz = m[8];
    float dxx, dxy, dxz, dyx, dyy, dyz, dzx, dzy, dzz;
    if (ir >= 0) {
      dxx = xix * t1x + etax * t2x + gammax * t3x;
      dxy = xiy * t1x + etay * t2x + gammay * t3x;
      dxz = xiz * t1x + etaz * t2x + gammaz * t3x;
      dyx = xix * t1y + etax * t2y + gammax * t3y;
      dyy = xiy * t1y + etay * t2y + gammay * t3y;
      dyz = xiz * t1y + etaz * t2y + gammaz * t3y;
      dzx = xix * t1z + etax * t2z + gammax * t3z;
      dzy = xiy * t1z + etay * t2z + gammay * t3z;
      dzz = xiz * t1z + etaz * t2z + gammaz * t3z;
    } else {
      dxx = xr * t1x; dxy = xr * t2x; dxz = xr * t3x;
      dyx = xr * t1y; dyy = xr * t2y; dyz = xr * t3y;
      dzx = xr * t1z; dzy = xr * t2z; dzz = xr * t3z;
    }
    if (STRAIN) {
      float sxx, sxy, sxz, syx, syy, syz, szx, szy, szz;
      if (ATT) {
        if (ir >= 0) {
          sxx = xix * a1x + etax * a2x + gammax * a3x;
          sxy = xiy * a1x + etay * a2x + gammay * a3x;
          sxz = xiz * a1x + etaz * a2x + gammaz * a3x;
          syx = xix * a1y + etax * a2y + gammax * a3y;
          syy = xiy * a1y + etay * a2y + gammay * a3y;
          syz = xiz * a1y + etaz * a2y + gammaz * a3y;
          szx = xix * a1z + etax * a2z + gammax * a3z;
          szy = xiy * a1z + etay * a2z + gammay * a3z;
          szz = xiz * a1z + etaz * a2z + gammaz * a3z;
        } else {
          sxx = xr * a1x; sxy = xr * a2x; sxz = xr * a3x;
          syx = xr * a1y; syy = xr * a2y; syz = xr * a3y;
          szx = xr * a1z; szy = xr * a2z; szz = xr * a3z;
        }
      } else {
        sxx = dxx; sxy = dxy; sxz = dxz; syx = dyx; syy = dyy; syz = dyz; szx = dzx; szy = dzy; szz = dzz;
      }
      const float templ = (1.f / 3.f) * (sxx + syy + szz);
      epsl[5] = sxx + syy + szz;
      epsl[0] = sxx - templ;
      epsl[1] = syy - templ;
      epsl[2] = 0.5f * (sxy + syx);
      epsl[3] = 0.5f * (szx + sxz);
      epsl[4] = 0.5f * (szy + syz);
      if (a.eps_trace_over_3) a.eps_trace_over_3[eo] = templ;
    }
    float sig_xx, sig_yy, sig_zz, sig_xy, sig_xz, sig_yz;
    if (ANISO) {
      // sigma = C eps in the reference's Voigt arrangement
      // (compute_forces_viscoelastic.F90:578-611); the memory variables below
      // still take mu and kappa, as the reference does
      float c[21];
#pragma unroll
      for (int q = 0; q < 21; ++q) c[q] = ld_elem<STREAM>(a.c[q] + eo);
      const float c11 = c[0], c12 = c[1], c13 = c[2], c14 = c[3], c15 = c[4], c16 = c[5], c22 = c[6];
      const float c23 = c[7], c24 = c[8], c25 = c[9], c26 = c[10], c33 = c[11], c34 = c[12], c35 = c[13];
      const float c36 = c[14], c44 = c[15], c45 = c[16], c46 = c[17], c55 = c[18], c56 = c[19], c66 = c[20];
      const float exy = dxy + dyx, exz = dzx + dxz, eyz = dzy + dyz;
      sig_xx = c11 * dxx + c16 * exy + c12 * dyy + c15 * exz + c14 * eyz + c13 * dzz;
      sig_yy = c12 * dxx + c26 * exy + c22 * dyy + c25 * exz + c24 * eyz + c23 * dzz;
      sig_zz = c13 * dxx + c36 * exy + c23 * dyy + c35 * exz + c34 * eyz + c33 * dzz;
      sig_xy = c16 * dxx + c66 * exy + c26 * dyy + c56 * exz + c46 * eyz + c36 * dzz;
      sig_xz = c15 * dxx + c56 * exy + c25 * dyy + c55 * exz + c45 * eyz + c35 * dzz;
      sig_yz = c14 * dxx + c46 * exy + c24 * dyy + c45 * exz + c44 * eyz + c34 * dzz;
    } else {
      const float l2m = kap + (4.f / 3.f) * mu;
      const float lam = l2m - 2.f * mu;
      sig_xx = l2m * dxx + lam * (dyy + dzz);
      sig_yy = l2m * dyy + lam * (dxx + dzz);
      sig_zz = l2m * dzz + lam * (dxx + dyy);
      sig_xy = mu * (dxy + dyx);
      sig_xz = mu * (dzx + dxz);
      sig_yz = mu * (dzy + dyz);
    }
    if (ATT && STAGE && !BULK) asm volatile("cp.async.wait_all;" ::: "memory");
    // every bulk-copied row is needed from here on (first use: the
    // memory-variable sums of the stress)
    if (kBulkAtt && !mbar_wait_bounded(&s_bar, 0)) {
      bulk_failed = true;  // the results of this element are not valid; the host is told
      if (a.err) atomicExch(a.err, 1);
    }
    if (ATT) {
      float sR[6];
#pragma unroll
      for (int c = 0; c < 6; ++c)
        sR[c] = STAGE ? s_att[3 * c][t] + s_att[3 * c + 1][t] + s_att[3 * c + 2][t] : R[c][0] + R[c][1] + R[c][2];
      sig_xx = sig_xx - sR[0] - sR[5];
      sig_yy = sig_yy - sR[1] - sR[5];
      sig_zz = sig_zz + sR[0] + sR[1] - sR[5];
      sig_xy -= sR[2];
      sig_xz -= sR[3];
      sig_yz -= sR[4];
    }
    if (ir >= 0) {
      // the device recomputes J = 1/det(d xi / d x) from the stored metric
      const float jac = 1.f / (xix * (etay * gammaz - etaz * gammay) - xiy * (etax * gammaz - etaz * gammax) +
                               xiz * (etax * gammay - etay * gammax));
      s_t[0][t] = jac * (sig_xx * xix + sig_xy * xiy + sig_xz * xiz);
      s_t[1][t] = jac * (sig_xy * xix + sig_yy * xiy + sig_yz * xiz);
      s_t[2][t] = jac * (sig_xz * xix + sig_yz * xiy + sig_zz * xiz);
      s_t[3][t] = jac * (sig_xx * etax + sig_xy * etay + sig_xz * etaz);
      s_t[4][t] = jac * (sig_xy * etax + sig_yy * etay + sig_yz * etaz);
      s_t[5][t] = jac * (sig_xz * etax + sig_yz * etay + sig_zz * etaz);
      s_t[6][t] = jac * (sig_xx * gammax + sig_xy * gammay + sig_xz * gammaz);
      s_t[7][t] = jac * (sig_xy * gammax + sig_yy * gammay + sig_yz * gammaz);
      s_t[8][t] = jac * (sig_xz * gammax + sig_yz * gammay + sig_zz * gammaz);
    } else {
      const float js = a.jacobian_regular * xr;
      s_t[0][t] = js * sig_xx; s_t[1][t] = js * sig_xy; s_t[2][t] = js * sig_xz;
      s_t[3][t] = js * sig_xy; s_t[4][t] = js * sig_yy; s_t[5][t] = js * sig_yz;
      s_t[6][t] = js * sig_xz; s_t[7][t] = js * sig_yz; s_t[8][t] = js * sig_zz;
    }
  }
  __syncthreads();

  // ---- transposed contractions and scatter-add --------------------------------
  if (active) {
    const float* hpw = s_gll + NGLL2;  // hprimewgll(i2,i1) = hpw[i2 + 5 i1]
    float n1x = 0.f, n2x = 0.f, n3x = 0.f, n1y = 0.f, n2y = 0.f, n3y = 0.f, n1z = 0.f, n2z = 0.f, n3z = 0.f;
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) {
      const float f1 = hpw[l + NGLLX * i], f2 = hpw[l + NGLLX * j], f3 = hpw[l + NGLLX * k];
      const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
      n1x = fmaf(s_t[0][p1], f1, n1x); n1y = fmaf(s_t[1][p1], f1, n1y); n1z = fmaf(s_t[2][p1], f1, n1z);
      n2x = fmaf(s_t[3][p2], f2, n2x); n2y = fmaf(s_t[4][p2], f2, n2y); n2z = fmaf(s_t[5][p2], f2, n2z);
      n3x = fmaf(s_t[6][p3], f3, n3x); n3y = fmaf(s_t[7][p3], f3, n3y); n3z = fmaf(s_t[8][p3], f3, n3z);
    }
    const float fac1 = s_gll[4 * NGLL2 + j + NGLLX * k];  // wgllwgll_yz(j,k)
    const float fac2 = s_gll[3 * NGLL2 + i + NGLLX * k];  // wgllwgll_xz(i,k)
    const float fac3 = s_gll[2 * NGLL2 + i + NGLLX * j];  // wgllwgll_xy(i,j)
    const float ax = fac1 * n1x + fac2 * n2x + fac3 * n3x;
    const float ay = fac1 * n1y + fac2 * n2y + fac3 * n3y;
    const float az = fac1 * n1z + fac2 * n2z + fac3 * n3z;
    if (ATOMIC) {
      atomicAdd(a.accel + 3L * iglob, -ax);
      atomicAdd(a.accel + 3L * iglob + 1, -ay);
      atomicAdd(a.accel + 3L * iglob + 2, -az);
    } else {
      // one colour: no other element of this launch touches iglob
      a.accel[3L * iglob] -= ax;
      a.accel[3L * iglob + 1] -= ay;
      a.accel[3L * iglob + 2] -= az;
    }

    if (ATT) {
      const long so = (long)e * (NSLS * NGLL3_PAD) + t;
      const float fkap = kap, fmu = mu;
      if (STAGE) {
#pragma unroll
        for (int c = 0; c < 6; ++c) eold[c] = s_att[18 + c][t];
      }
#pragma unroll
      for (int s = 0; s < NSLS; ++s) {
        const float al = a.alpha[s], be = a.beta[s], ga = a.gamma[s];
        float fcs = 0.f, fcks = 0.f;
        if (STAGE && GEOM != kGeomFP32) {
          const ElemPack* pk = a.pack + e;
          const unsigned vary = __ldg(&pk->vary);
          const int base = __ldg(&pk->base);
          fcs = pack_value<GEOM>(pk, a.pool, vary, base, 11 + s, t);
          fcks = pack_value<GEOM>(pk, a.pool, vary, base, 14 + s, t);
        } else if (STAGE) {
          fcs = s_att[24 + s][t];
          fcks = s_att[27 + s][t];
        } else {
          fcs = fc[s];
          fcks = fck[s];
        }
        const float fk = fkap * fcks;
        const float r5 = STAGE ? s_att[15 + s][t] : R[5][s];
        st_state<STREAM>(a.R[5] + so + s * NGLL3_PAD, al * r5 + fk * (be * eold[5] + ga * epsl[5]));
        const float fm = fmu * fcs;
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          const float rc = STAGE ? s_att[3 * c + s][t] : R[c][s];
          st_state<STREAM>(a.R[c] + so + s * NGLL3_PAD, al * rc + fm * (be * eold[c] + ga * epsl[c]));
        }
      }
    }
    if (STRAIN) {
      if (ATT) st_state<STREAM>(a.eps[5] + eo, epsl[5]);
#pragma unroll
      for (int c = 0; c < 5; ++c)
        if (a.eps[c]) st_state<STREAM>(a.eps[c] + eo, epsl[c]);
    }
  }
  // a bulk copy still in flight must land before the CTA's shared memory is
  // released: wait once more, with the same bound
  if (kBulkAtt && bulk_failed) mbar_wait_bounded(&s_bar, 0);
}

// MINB_NOATT: the register budget of the builds without attenuation (no memory
// variables: they fit more CTAs per SM than the attenuation build of the variant)
template <int MINB, int GEOM, bool STAGE = false, bool STREAM = false, bool BULK = false, int MINB_NOATT = MINB>
void launch_minb(const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s) {
  dim3 grid(a.nelem), block(NGLL3_PAD);
  if (att)
    stiffness_kernel<true, true, MINB, GEOM, STAGE, true, STREAM, false, BULK><<<grid, block, 0, s>>>(a);
  else if (store_strain)
    stiffness_kernel<false, true, MINB_NOATT, GEOM, false, true, STREAM><<<grid, block, 0, s>>>(a);
  else
    stiffness_kernel<false, false, MINB_NOATT, GEOM, false, true, STREAM><<<grid, block, 0, s>>>(a);
}

template <int MINB, bool STAGE = false, bool BULK = false>
void launch_packed(const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s, int geom) {
  if (geom == kGeomPackF16)
    launch_minb<MINB, kGeomPackF16, STAGE, false, BULK>(a, att, store_strain, s);
  else if (geom == kGeomPackBF16)
    launch_minb<MINB, kGeomPackBF16, STAGE, false, BULK>(a, att, store_strain, s);
  else
    launch_minb<MINB, kGeomPackF32, STAGE, false, BULK>(a, att, store_strain, s);
}

}  // namespace

// blocks_per_sm: the register budget the kernel is compiled for (4..7 CTAs of
// 128 threads per SM; more CTAs keep more elements' loads in flight, fewer
// let the compiler keep every load of an element in registers).  The packed
// geometry builds exist for 6 and 7 CTAs/SM, and with cp.async-staged memory
// variables for 8, 9 and 10.
void launch_stiffness(const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s, int blocks_per_sm,
                      int geom_format, bool staged, bool streaming, bool bulk) {
  if (a.nelem <= 0) return;
  if (bulk && geom_format == kGeomFP32) {
    // 20.5 KB of shared memory and 64 / 56 / 48 registers a thread: 8, 9 or 10 CTAs/SM;
    // without attenuation (nothing to stage) 8, 10 or 12 CTAs/SM
    if (blocks_per_sm >= 10)
      launch_minb<10, kGeomFP32, true, false, true, 12>(a, att, store_strain, s);
    else if (blocks_per_sm == 9)
      launch_minb<9, kGeomFP32, true, false, true, 10>(a, att, store_strain, s);
    else
      launch_minb<8, kGeomFP32, true, false, true, 8>(a, att, store_strain, s);
    return;
  }
  if (geom_format != kGeomFP32 && bulk) {
    // 24 bulk-copied rows (factors from the element record): 20.5 KB of shared
    // memory, 64 / 56 / 48 registers a thread for 8, 9 or 10 CTAs/SM
    if (blocks_per_sm >= 10)
      launch_packed<10, true, true>(a, att, store_strain, s, geom_format);
    else if (blocks_per_sm == 9)
      launch_packed<9, true, true>(a, att, store_strain, s, geom_format);
    else
      launch_packed<8, true, true>(a, att, store_strain, s, geom_format);
    return;
  }
  if (geom_format != kGeomFP32 && staged) {
    // staged memory variables and record-resident constants leave 48-64
    // registers a thread (no spills): 8, 9 or 10 CTAs/SM of 20.5 KB shared memory
    if (blocks_per_sm >= 10)
      launch_packed<10, true>(a, att, store_strain, s, geom_format);
    else if (blocks_per_sm == 9)
      launch_packed<9, true>(a, att, store_strain, s, geom_format);
    else
      launch_packed<8, true>(a, att, store_strain, s, geom_format);
    return;
  }
  if (streaming) {
    if (blocks_per_sm == 7)
      launch_minb<7, kGeomFP32, false, true>(a, att, store_strain, s);
    else
      launch_minb<6, kGeomFP32, false, true>(a, att, store_strain, s);
    return;
  }
  if (staged) {
    // cp.async-staged memory variables (attenuation); without attenuation the
    // same register budgets of the plain build
    if (blocks_per_sm == 8)
      launch_minb<8, kGeomFP32, true>(a, att, store_strain, s);
    else if (blocks_per_sm == 7)
      launch_minb<7, kGeomFP32, true>(a, att, store_strain, s);
    else
      launch_minb<6, kGeomFP32, true>(a, att, store_strain, s);
    return;
  }
  if (geom_format != kGeomFP32) {
    if (blocks_per_sm == 7)
      launch_packed<7>(a, att, store_strain, s, geom_format);
    else
      launch_packed<6>(a, att, store_strain, s, geom_format);
    return;
  }
  switch (blocks_per_sm) {
    case 5: launch_minb<5, kGeomFP32>(a, att, store_strain, s); break;
    case 6: launch_minb<6, kGeomFP32>(a, att, store_strain, s); break;
    case 7: launch_minb<7, kGeomFP32>(a, att, store_strain, s); break;
    default: launch_minb<4, kGeomFP32>(a, att, store_strain, s); break;
  }
}

template <int MINB>
void launch_aniso_minb(const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s) {
  dim3 grid(a.nelem), block(NGLL3_PAD);
  if (att)
    stiffness_kernel<true, true, MINB, kGeomFP32, false, true, false, true><<<grid, block, 0, s>>>(a);
  else if (store_strain)
    stiffness_kernel<false, true, MINB, kGeomFP32, false, true, false, true><<<grid, block, 0, s>>>(a);
  else
    stiffness_kernel<false, false, MINB, kGeomFP32, false, true, false, true><<<grid, block, 0, s>>>(a);
}

// blocks_per_sm: 4, 5 or 6 resident CTAs (the register budget of the 21 extra moduli)
void launch_stiffness_aniso(const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s, int blocks_per_sm) {
  if (a.nelem <= 0) return;
  if (blocks_per_sm >= 6)
    launch_aniso_minb<6>(a, att, store_strain, s);
  else if (blocks_per_sm == 5)
    launch_aniso_minb<5>(a, att, store_strain, s);
  else
    launch_aniso_minb<4>(a, att, store_strain, s);
}

void launch_stiffness_colored(const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s) {
  if (a.nelem <= 0) return;
  dim3 grid(a.nelem), block(NGLL3_PAD);
  if (att)
    stiffness_kernel<true, true, 6, kGeomFP32, false, false><<<grid, block, 0, s>>>(a);
  else if (store_strain)
    stiffness_kernel<false, true, 6, kGeomFP32, false, false><<<grid, block, 0, s>>>(a);
  else
    stiffness_kernel<false, false, 6, kGeomFP32, false, false><<<grid, block, 0, s>>>(a);
}

}  // namespace sf3d
