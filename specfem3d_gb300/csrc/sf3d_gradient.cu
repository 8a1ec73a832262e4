// Checkpointed discrete-adjoint gradient of a waveform misfit (sm_103a).
//
// The reference computes sensitivity kernels (SIMULATION_TYPE = 3) by running
// the adjoint wavefield forward in reversed time next to a backward
// reconstruction of the forward field from stored Stacey boundary values
// (iterate_time.F90:219-330, compute_forces_viscoelastic_calling_routine.F90:443-686,
// compute_kernels.f90:67-226), or, with UNDO_ATTENUATION_AND_OR_PML, by
// recomputing the forward field from snapshots (iterate_time_undoatt.F90:29-632).
// This module follows the second route, entirely in HBM:
//
//   forward  : the fused elastic step of sf3d_iterate_time from rest; the raw
//              step state (displ, veloc, accel before the mass matrix) is
//              copied to a checkpoint slot every `every` steps;
//   backward : for each segment, last to first, the forward steps of the
//              segment are recomputed from its checkpoint, storing the
//              displacement and the force of every step; then the exact
//              transpose of each Newmark step is applied in reverse order.
//
// With the explicit Newmark step (n -> n+1)
//     ut = u + dt v + dt^2/2 a,   vt = v + dt/2 a,
//     a' = M^-1 (f - K ut - B vt),   v' = vt + dt/2 a',   u' = ut,
// (K: stiffness, B: Stacey damping, M: mass incl. its Stacey term, all
// symmetric) and misfit J = sum_n r_n(u_n), the transpose step is
//     uh' += dJ/du'                         (receiver residual, transposed interpolation)
//     p    = -M^-1 (ah' + dt/2 vh')
//     uth  = uh' + K p,   vth = vh' + B p
//     uh   = uth,  vh = dt uth + vth,  ah = dt^2/2 uth + dt/2 vth
// and the gradient contributions of the step are
//     dJ/dkappa_(e,p) += w_p J_p tr eps(p) tr eps(ut)
//     dJ/dmu_(e,p)    += w_p J_p 2 dev eps(p) : dev eps(ut)
//     dJ/drho_(e,p)   += w_p J_p p . a'           (mass-matrix dependence)
// accumulated in FP64 per GLL point.  K p and B p reuse the forward stiffness
// and Stacey kernels (both operators are symmetric).  These are the reference's
// kernel formulas (compute_kernels.f90:151-186: kappa from the strain traces,
// mu from the deviatoric strains, rho from the acceleration-displacement
// product) evaluated on the discrete adjoint field, so the gradient is the
// exact derivative of the discrete misfit for model perturbations that leave
// the Stacey faces unchanged.
#include <math.h>
#include <string.h>

#include <vector>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

// uh(iglob) += sum over receivers of h_xi h_eta h_gamma nu^T residual(:, r, slot)
__global__ void adj_residual_kernel(int nrec, const int* __restrict__ ispec_rec, const float* __restrict__ hx,
                                    const float* __restrict__ he, const float* __restrict__ hg,
                                    const float* __restrict__ nu, const int* __restrict__ ibool,
                                    const float* __restrict__ residual, int slot, float* __restrict__ uh) {
  const int r = blockIdx.x, t = threadIdx.x;
  if (r >= nrec || t >= NGLL3) return;
  const int e = ispec_rec[r];
  const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
  const float h = hx[5 * r + i] * he[5 * r + j] * hg[5 * r + k];
  const float* res = residual + 3L * (r + (long)nrec * slot);
  const float* n = nu + 9 * r;  // nu(3,3) column-major: seismogram = nu u
  const float w0 = n[0] * res[0] + n[1] * res[1] + n[2] * res[2];
  const float w1 = n[3] * res[0] + n[4] * res[1] + n[5] * res[2];
  const float w2 = n[6] * res[0] + n[7] * res[1] + n[8] * res[2];
  const int g = ibool[(long)e * NGLL3_PAD + t];
  atomicAdd(uh + 3L * g, h * w0);
  atomicAdd(uh + 3L * g + 1, h * w1);
  atomicAdd(uh + 3L * g + 2, h * w2);
}

// p = -M^-1 (ah + dt/2 vh); clears the K p and B p accumulators
__global__ void adj_p_kernel(const float* __restrict__ vh, const float* __restrict__ ah,
                             const float* __restrict__ rmx, const float* __restrict__ rmy,
                             const float* __restrict__ rmz, long nglob, float dt2, float* __restrict__ p,
                             float* __restrict__ kp, float* __restrict__ bp) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * nglob) return;
  const long g = i / 3;
  const int c = (int)(i - 3 * g);
  const float rm = c == 0 ? __ldg(rmx + g) : (c == 1 ? __ldg(rmy + g) : __ldg(rmz + g));
  p[i] = -rm * (ah[i] + dt2 * vh[i]);
  kp[i] = 0.f;
  bp[i] = 0.f;
}

// kp = -K p and bp = -B p: uth = uh - kp, vth = vh - bp; back through the
// predictor; then p of the previous step, -M^-1 (ah + dt/2 vh), from the new
// adjoints (the residual enters uh only, so p does not depend on it), and the
// K p / B p accumulators cleared for that step.  The adjoint of the
// acceleration is used only through p, so it is not stored.
__global__ void adj_update_kernel(float* __restrict__ uh, float* __restrict__ vh, float* __restrict__ kp,
                                  float* __restrict__ bp, float* __restrict__ p, const float* __restrict__ rmx,
                                  const float* __restrict__ rmy, const float* __restrict__ rmz, long nglob,
                                  float dt, float dt2, float dtsq2) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * nglob) return;
  const float ut = uh[i] - kp[i];
  const float vt = vh[i] - bp[i];
  const float vn = dt * ut + vt;
  const float an = dtsq2 * ut + dt2 * vt;
  uh[i] = ut;
  vh[i] = vn;
  const long g = i / 3;
  const int c = (int)(i - 3 * g);
  const float rm = c == 0 ? __ldg(rmx + g) : (c == 1 ? __ldg(rmy + g) : __ldg(rmz + g));
  p[i] = -rm * (an + dt2 * vn);
  kp[i] = 0.f;
  bp[i] = 0.f;
}

// The same update when K p and B p were scatter-added straight into the adjoint
// fields (uh already holds uh - kp, vh holds vh - bp): vh and p of the previous
// step, no accumulators to read or clear.
// Four consecutive values per thread (16-byte accesses), thread n4 also taking
// the tail; n = 3 * nglob < 2^31.
__global__ void adj_update_direct_kernel(const float* __restrict__ uh, float* __restrict__ vh,
                                         float* __restrict__ p, const float* __restrict__ rmx,
                                         const float* __restrict__ rmy, const float* __restrict__ rmz, int n,
                                         float dt, float dt2, float dtsq2) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int n4 = n >> 2;
  if (q > n4) return;
  auto one = [&](float ut, float vt, int i, float& vn, float& pn) {
    vn = dt * ut + vt;
    const float an = dtsq2 * ut + dt2 * vt;
    const int g = i / 3;
    const int c = i - 3 * g;
    const float rm = c == 0 ? __ldg(rmx + g) : (c == 1 ? __ldg(rmy + g) : __ldg(rmz + g));
    pn = -rm * (an + dt2 * vn);
  };
  if (q == n4) {
    for (int i = 4 * n4; i < n; ++i) one(uh[i], vh[i], i, vh[i], p[i]);
    return;
  }
  const int i0 = 4 * q;
  const float4 u4 = reinterpret_cast<const float4*>(uh)[q];
  const float4 v4 = reinterpret_cast<const float4*>(vh)[q];
  float4 vn, pn;
  one(u4.x, v4.x, i0, vn.x, pn.x);
  one(u4.y, v4.y, i0 + 1, vn.y, pn.y);
  one(u4.z, v4.z, i0 + 2, vn.z, pn.z);
  one(u4.w, v4.w, i0 + 3, vn.w, pn.w);
  reinterpret_cast<float4*>(vh)[q] = vn;
  reinterpret_cast<float4*>(p)[q] = pn;
}

struct GradArgs {
  int nelem;
  const int* phase;
  const int* ibool;
  const int* irregular;
  const float* m[9];
  const float* gll;
  float xix_regular, jacobian_regular;
  float w[NGLLX];
  float uscale;        // power of two bringing the forward field near 1
  const float* p;      // adjoint field p_n
  const float* u;      // forward displacement after step n
  const float* araw;   // forward force after step n (before the mass matrix)
  const float* rmx;
  const float* rmy;
  const float* rmz;
  double* g_rho;
  double* g_kappa;
  double* g_mu;
  const float* kappav; // fused form: moduli and the K p accumulator
  const float* muv;
  float* kp;           // K p scatter target, kp_sign times the force: -1 into the
  float kp_sign;       // kp accumulator, +1 straight into the adjoint displacement
  int* err;            // kernel error word (a bounded wait that timed out)
};

// Local derivatives (d/dxi, d/deta, d/dgamma of each component) of two fields
// staged in shared memory, t of s and q of r, in one loop: each hprime
// coefficient is read from shared memory once for both fields; every output is
// the same 5-term FMA chain as a loop over one field would form.
__device__ __forceinline__ void local_grad_pair(const float (*s)[NGLL3_PAD], const float (*r)[NGLL3_PAD],
                                            const float* hp, int i, int j, int k, float t[3][3], float q[3][3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) t[c][0] = t[c][1] = t[c][2] = q[c][0] = q[c][1] = q[c][2] = 0.f;
#pragma unroll
  for (int l = 0; l < NGLLX; ++l) {
    const float h1 = hp[i + NGLLX * l], h2 = hp[j + NGLLX * l], h3 = hp[k + NGLLX * l];
    const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      t[c][0] = fmaf(s[c][p1], h1, t[c][0]);
      t[c][1] = fmaf(s[c][p2], h2, t[c][1]);
      t[c][2] = fmaf(s[c][p3], h3, t[c][2]);
      q[c][0] = fmaf(r[c][p1], h1, q[c][0]);
      q[c][1] = fmaf(r[c][p2], h2, q[c][1]);
      q[c][2] = fmaf(r[c][p3], h3, q[c][2]);
    }
  }
}

// One CTA per element, thread = GLL point: strains of p and u, FP64 accumulation.
__global__ void __launch_bounds__(NGLL3_PAD) grad_accum_kernel(const GradArgs a) {
  __shared__ float s_h[NGLL2];
  __shared__ float s_p[3][NGLL3_PAD];
  __shared__ float s_u[3][NGLL3_PAD];
  const int t = threadIdx.x;
  const int e = a.phase ? __ldg(a.phase + blockIdx.x) : (int)blockIdx.x;
  const bool active = t < NGLL3;
  const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
  const long eo = (long)e * NGLL3_PAD + t;
  float pa = 0.f;
  if (t < NGLL2) s_h[t] = __ldg(a.gll + t);
  if (active) {
    const int g = __ldg(a.ibool + eo);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      s_p[c][t] = a.p[3L * g + c];
      s_u[c][t] = a.u[3L * g + c] * a.uscale;
    }
    pa = s_p[0][t] * (a.araw[3L * g] * a.uscale * __ldg(a.rmx + g)) +
         s_p[1][t] * (a.araw[3L * g + 1] * a.uscale * __ldg(a.rmy + g)) +
         s_p[2][t] * (a.araw[3L * g + 2] * a.uscale * __ldg(a.rmz + g));
  }
  __syncthreads();
  if (!active) return;
  float tp[3][3], tu[3][3];
  local_grad_pair(s_p, s_u, s_h, i, j, k, tp, tu);
  const int ir = __ldg(a.irregular + e);
  // d[c][x]: derivative of component c along x, y, z
  float dp[3][3], du[3][3], jac;
  if (ir >= 0) {
    float m[9];
    const long mo = (long)ir * NGLL3_PAD + t;
#pragma unroll
    for (int q = 0; q < 9; ++q) m[q] = __ldg(a.m[q] + mo);
    // m = xix xiy xiz etax etay etaz gammax gammay gammaz
#pragma unroll
    for (int c = 0; c < 3; ++c) {
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        dp[c][x] = m[x] * tp[c][0] + m[3 + x] * tp[c][1] + m[6 + x] * tp[c][2];
        du[c][x] = m[x] * tu[c][0] + m[3 + x] * tu[c][1] + m[6 + x] * tu[c][2];
      }
    }
    jac = 1.f / (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                 m[2] * (m[3] * m[7] - m[4] * m[6]));
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        dp[c][x] = a.xix_regular * tp[c][x];
        du[c][x] = a.xix_regular * tu[c][x];
      }
    jac = a.jacobian_regular;
  }
  const float trp = dp[0][0] + dp[1][1] + dp[2][2];
  const float tru = du[0][0] + du[1][1] + du[2][2];
  float dd = 0.f;
#pragma unroll
  for (int x = 0; x < 3; ++x) dd += (dp[x][x] - trp * (1.f / 3.f)) * (du[x][x] - tru * (1.f / 3.f));
  const float exy_p = 0.5f * (dp[0][1] + dp[1][0]), exz_p = 0.5f * (dp[0][2] + dp[2][0]),
              eyz_p = 0.5f * (dp[1][2] + dp[2][1]);
  const float exy_u = 0.5f * (du[0][1] + du[1][0]), exz_u = 0.5f * (du[0][2] + du[2][0]),
              eyz_u = 0.5f * (du[1][2] + du[2][1]);
  dd += 2.f * (exy_p * exy_u + exz_p * exz_u + eyz_p * eyz_u);
  // the step's products in FP32, their time integration in FP64 (GB300's FP64 pipe
  // is narrow: 3 conversions + 3 adds per point instead of the whole product chain)
  const float wj = (a.w[i] * a.w[j] * a.w[k]) * jac;
  a.g_kappa[eo] += (double)(wj * trp * tru);
  a.g_mu[eo] += (double)(wj * 2.f * dd);
  a.g_rho[eo] += (double)(wj * pa);
}

// Fused form of one element's part of the transposed step: K p (the elastic
// stiffness applied to p, arithmetic of stiffness_kernel<ATT=0>) scatter-added
// into kp, and the gradient contributions of grad_accum_kernel, from one gather
// of p and one set of p derivatives.  The element's three FP64 gradient rows
// (3 KB) come into shared memory by bulk copy at the start, so their load
// latency runs under the gathers; every thread waits for them (bounded) where
// it adds its contributions.
// Register budget of 10 CTAs/SM (48 registers, no spills; 11 KB of shared
// memory a CTA): measured against 6 and 8 CTAs/SM, the most resident elements
// hide the gathers best (reverse sweep 3.96 / 3.88 / 3.84 s per shot).
__global__ void __launch_bounds__(NGLL3_PAD, 10) adj_stiffness_grad_kernel(const GradArgs a) {
  __shared__ float s_gll[NGLL3];
  __shared__ float s_p[3][NGLL3_PAD];
  __shared__ float s_u[3][NGLL3_PAD];
  __shared__ float s_t[9][NGLL3_PAD];
  __shared__ __align__(16) double s_g[3][NGLL3_PAD];   // rho, kappa, mu
  __shared__ uint64_t s_bar;
  const int t = threadIdx.x;
  const int e = a.phase ? __ldg(a.phase + blockIdx.x) : (int)blockIdx.x;
  const bool active = t < NGLL3;
  const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
  const long eo = (long)e * NGLL3_PAD + t;
  float pa = 0.f, kap = 0.f, mu = 0.f;
  int g = 0;
  bool bulk_failed = false;
  if (t == 0) {
    const long eb = (long)e * NGLL3_PAD;
    mbar_init(&s_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    mbar_arrive_expect_tx(&s_bar, (uint32_t)(3 * NGLL3_PAD * sizeof(double)));
    bulk_g2s(&s_g[0][0], a.g_rho + eb, NGLL3_PAD * sizeof(double), &s_bar);
    bulk_g2s(&s_g[1][0], a.g_kappa + eb, NGLL3_PAD * sizeof(double), &s_bar);
    bulk_g2s(&s_g[2][0], a.g_mu + eb, NGLL3_PAD * sizeof(double), &s_bar);
  }
  if (active) {
    s_gll[t] = __ldg(a.gll + t);
    g = __ldg(a.ibool + eo);
    kap = __ldg(a.kappav + eo);
    mu = __ldg(a.muv + eo);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      s_p[c][t] = a.p[3L * g + c];
      s_u[c][t] = a.u[3L * g + c] * a.uscale;
    }
    pa = s_p[0][t] * (a.araw[3L * g] * a.uscale * __ldg(a.rmx + g)) +
         s_p[1][t] * (a.araw[3L * g + 1] * a.uscale * __ldg(a.rmy + g)) +
         s_p[2][t] * (a.araw[3L * g + 2] * a.uscale * __ldg(a.rmz + g));
  }
  __syncthreads();
  const int ir = __ldg(a.irregular + e);
  if (active) {
    float tp[3][3], tu[3][3];
    local_grad_pair(s_p, s_u, s_gll, i, j, k, tp, tu);
    float dp[3][3], du[3][3], jac, m[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) m[q] = 0.f;
    if (ir >= 0) {
      const long mo = (long)ir * NGLL3_PAD + t;
#pragma unroll
      for (int q = 0; q < 9; ++q) m[q] = __ldg(a.m[q] + mo);
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          dp[c][x] = m[x] * tp[c][0] + m[3 + x] * tp[c][1] + m[6 + x] * tp[c][2];
          du[c][x] = m[x] * tu[c][0] + m[3 + x] * tu[c][1] + m[6 + x] * tu[c][2];
        }
      jac = 1.f / (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                   m[2] * (m[3] * m[7] - m[4] * m[6]));
    } else {
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          dp[c][x] = a.xix_regular * tp[c][x];
          du[c][x] = a.xix_regular * tu[c][x];
        }
      jac = a.jacobian_regular;
    }
    // gradient contributions
    const float trp = dp[0][0] + dp[1][1] + dp[2][2];
    const float tru = du[0][0] + du[1][1] + du[2][2];
    float dd = 0.f;
#pragma unroll
    for (int x = 0; x < 3; ++x) dd += (dp[x][x] - trp * (1.f / 3.f)) * (du[x][x] - tru * (1.f / 3.f));
    const float exy_p = 0.5f * (dp[0][1] + dp[1][0]), exz_p = 0.5f * (dp[0][2] + dp[2][0]),
                eyz_p = 0.5f * (dp[1][2] + dp[2][1]);
    const float exy_u = 0.5f * (du[0][1] + du[1][0]), exz_u = 0.5f * (du[0][2] + du[2][0]),
                eyz_u = 0.5f * (du[1][2] + du[2][1]);
    dd += 2.f * (exy_p * exy_u + exz_p * exz_u + eyz_p * eyz_u);
    // products in FP32, time integration in FP64 (as grad_accum_kernel)
    const float wj = (a.w[i] * a.w[j] * a.w[k]) * jac;
    if (!mbar_wait_bounded(&s_bar, 0)) {
      bulk_failed = true;  // this element's gradient is not valid; the host is told
      if (a.err) atomicExch(a.err, 1);
    }
    a.g_kappa[eo] = s_g[1][t] + (double)(wj * trp * tru);
    a.g_mu[eo] = s_g[2][t] + (double)(wj * 2.f * dd);
    a.g_rho[eo] = s_g[0][t] + (double)(wj * pa);
    // stress of p (stiffness_kernel<ATT=0> arithmetic)
    const float dxx = dp[0][0], dxy = dp[0][1], dxz = dp[0][2];
    const float dyx = dp[1][0], dyy = dp[1][1], dyz = dp[1][2];
    const float dzx = dp[2][0], dzy = dp[2][1], dzz = dp[2][2];
    const float l2m = kap + (4.f / 3.f) * mu;
    const float lam = l2m - 2.f * mu;
    const float sxx = l2m * dxx + lam * (dyy + dzz);
    const float syy = l2m * dyy + lam * (dxx + dzz);
    const float szz = l2m * dzz + lam * (dxx + dyy);
    const float sxy = mu * (dxy + dyx);
    const float sxz = mu * (dzx + dxz);
    const float syz = mu * (dzy + dyz);
    if (ir >= 0) {
      const float xix = m[0], xiy = m[1], xiz = m[2], etax = m[3], etay = m[4], etaz = m[5];
      const float gammax = m[6], gammay = m[7], gammaz = m[8];
      s_t[0][t] = jac * (sxx * xix + sxy * xiy + sxz * xiz);
      s_t[1][t] = jac * (sxy * xix + syy * xiy + syz * xiz);
      s_t[2][t] = jac * (sxz * xix + syz * xiy + szz * xiz);
      s_t[3][t] = jac * (sxx * etax + sxy * etay + sxz * etaz);
      s_t[4][t] = jac * (sxy * etax + syy * etay + syz * etaz);
      s_t[5][t] = jac * (sxz * etax + syz * etay + szz * etaz);
      s_t[6][t] = jac * (sxx * gammax + sxy * gammay + sxz * gammaz);
      s_t[7][t] = jac * (sxy * gammax + syy * gammay + syz * gammaz);
      s_t[8][t] = jac * (sxz * gammax + syz * gammay + szz * gammaz);
    } else {
      const float js = a.jacobian_regular * a.xix_regular;
      s_t[0][t] = js * sxx; s_t[1][t] = js * sxy; s_t[2][t] = js * sxz;
      s_t[3][t] = js * sxy; s_t[4][t] = js * syy; s_t[5][t] = js * syz;
      s_t[6][t] = js * sxz; s_t[7][t] = js * syz; s_t[8][t] = js * szz;
    }
  }
  __syncthreads();
  if (active) {
    const float* hpw = s_gll + NGLL2;
    float n1x = 0.f, n2x = 0.f, n3x = 0.f, n1y = 0.f, n2y = 0.f, n3y = 0.f, n1z = 0.f, n2z = 0.f, n3z = 0.f;
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) {
      const float f1 = hpw[l + NGLLX * i], f2 = hpw[l + NGLLX * j], f3 = hpw[l + NGLLX * k];
      const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
      n1x = fmaf(s_t[0][p1], f1, n1x); n1y = fmaf(s_t[1][p1], f1, n1y); n1z = fmaf(s_t[2][p1], f1, n1z);
      n2x = fmaf(s_t[3][p2], f2, n2x); n2y = fmaf(s_t[4][p2], f2, n2y); n2z = fmaf(s_t[5][p2], f2, n2z);
      n3x = fmaf(s_t[6][p3], f3, n3x); n3y = fmaf(s_t[7][p3], f3, n3y); n3z = fmaf(s_t[8][p3], f3, n3z);
    }
    const float fac1 = s_gll[4 * NGLL2 + j + NGLLX * k];
    const float fac2 = s_gll[3 * NGLL2 + i + NGLLX * k];
    const float fac3 = s_gll[2 * NGLL2 + i + NGLLX * j];
    atomicAdd(a.kp + 3L * g, a.kp_sign * (fac1 * n1x + fac2 * n2x + fac3 * n3x));
    atomicAdd(a.kp + 3L * g + 1, a.kp_sign * (fac1 * n1y + fac2 * n2y + fac3 * n3y));
    atomicAdd(a.kp + 3L * g + 2, a.kp_sign * (fac1 * n1z + fac2 * n2z + fac3 * n3z));
  }
  // a bulk copy still in flight must land before the CTA's shared memory is
  // released: wait once more, with the same bound
  if (bulk_failed) mbar_wait_bounded(&s_bar, 0);
}

bool alloc_f(float** d, size_t n) { return alloc_zero((void**)d, sizeof(float) * n); }

}  // namespace

void free_grad(Mesh* mp) {
  GradState* G = mp->grad;
  if (!G) return;
  cudaFree(G->ckpt); cudaFree(G->seg_u); cudaFree(G->seg_a);
  cudaFree(G->adj_u); cudaFree(G->adj_v); cudaFree(G->adj_a);
  cudaFree(G->p); cudaFree(G->kp); cudaFree(G->bp); cudaFree(G->residual);
  cudaFree(G->g_rho); cudaFree(G->g_kappa); cudaFree(G->g_mu);
  delete G;
  mp->grad = nullptr;
}

namespace {

bool grad_ready(Mesh* mp) {
  if (!mp->grad) return set_error(SF3D_ERR_STATE, "sf3d_gradient_setup not called");
  if (mp->num_phase_ispec <= 0) return set_error(SF3D_ERR_STATE, "phase element lists not prepared");
  default_phase_counts(mp);
  return true;
}

void save_state(Mesh* mp, float* dst, cudaStream_t s) {
  const size_t n3 = 3ull * mp->nglob;
  cudaMemcpyAsync(dst, mp->f.displ, sizeof(float) * n3, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(dst + n3, mp->f.veloc, sizeof(float) * n3, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(dst + 2 * n3, mp->f.accel, sizeof(float) * n3, cudaMemcpyDeviceToDevice, s);
}

void load_state(Mesh* mp, const float* src, cudaStream_t s) {
  const size_t n3 = 3ull * mp->nglob;
  cudaMemcpyAsync(mp->f.displ, src, sizeof(float) * n3, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(mp->f.veloc, src + n3, sizeof(float) * n3, cudaMemcpyDeviceToDevice, s);
  cudaMemcpyAsync(mp->f.accel, src + 2 * n3, sizeof(float) * n3, cudaMemcpyDeviceToDevice, s);
}

void zero_state(Mesh* mp, cudaStream_t s) {
  const size_t n3 = 3ull * mp->nglob;
  cudaMemsetAsync(mp->f.displ, 0, sizeof(float) * n3, s);
  cudaMemsetAsync(mp->f.veloc, 0, sizeof(float) * n3, s);
  cudaMemsetAsync(mp->f.accel, 0, sizeof(float) * n3, s);
}

// One transposed Newmark step n (0-based): u = displacement after step n,
// araw = force after step n.
void adjoint_step(Mesh* mp, int n, const float* u, const float* araw, float dt, float dt2, float dtsq2) {
  GradState* G = mp->grad;
  cudaStream_t s = mp->stream;
  const long n3 = 3L * mp->nglob;
  if (mp->nrec_local > 0)
    adj_residual_kernel<<<mp->nrec_local, NGLL3_PAD, 0, s>>>(mp->nrec_local, mp->d_ispec_rec, mp->d_hxir,
                                                             mp->d_hetar, mp->d_hgammar, mp->d_nu_rec, mp->d_ibool,
                                                             G->residual, n, G->adj_u);
  // p (and with the separate kernels kp, bp) of this step were produced by the
  // previous transposed step (or the start of the sweep).  The fused kernel adds
  // B p and K p straight into the adjoint velocity and displacement: they are
  // read only by the update below, so its kp and bp reads and clears go away.
  if (G->fused)
    launch_stacey(mp, G->p, G->adj_v, s, 1.f);
  else
    launch_stacey(mp, G->p, G->bp, s);
  Fields tmp;
  tmp.displ = G->p;
  tmp.veloc = G->p;
  tmp.accel = G->kp;
  for (int iphase = 1; iphase <= 2; ++iphase) {
    StiffnessArgs a = stiffness_args(mp, tmp, iphase, dt, false, false, false);
    if (a.nelem <= 0) continue;
    if (!G->fused) run_stiffness(mp, a, false, false, s);
    GradArgs ga;
    memset(&ga, 0, sizeof(ga));
    ga.nelem = a.nelem;
    ga.phase = a.phase;
    ga.ibool = mp->d_ibool;
    ga.irregular = mp->d_irregular;
    for (int q = 0; q < 9; ++q) ga.m[q] = mp->d_metric[q];
    ga.gll = mp->d_gll;
    ga.xix_regular = mp->xix_regular;
    ga.jacobian_regular = mp->jacobian_regular;
    for (int q = 0; q < NGLLX; ++q) ga.w[q] = G->wgll[q];
    ga.uscale = G->u_scale;
    ga.p = G->p;
    ga.u = u;
    ga.araw = araw;
    ga.rmx = mp->d_rmassx;
    ga.rmy = mp->d_rmassy;
    ga.rmz = mp->d_rmassz;
    ga.g_rho = G->g_rho;
    ga.g_kappa = G->g_kappa;
    ga.g_mu = G->g_mu;
    ga.kappav = mp->d_kappav;
    ga.muv = mp->d_muv;
    ga.kp = G->fused ? G->adj_u : G->kp;
    ga.kp_sign = G->fused ? 1.f : -1.f;
    ga.err = mp->d_kerr;
    if (G->fused)
      adj_stiffness_grad_kernel<<<a.nelem, NGLL3_PAD, 0, s>>>(ga);
    else
      grad_accum_kernel<<<a.nelem, NGLL3_PAD, 0, s>>>(ga);
  }
  if (G->fused)
    adj_update_direct_kernel<<<nblk((n3 >> 2) + 1, 256), 256, 0, s>>>(G->adj_u, G->adj_v, G->p, mp->d_rmassx,
                                                                      mp->d_rmassy, mp->d_rmassz, (int)n3, dt,
                                                                      dt2, dtsq2);
  else
    adj_update_kernel<<<nblk(n3, 256), 256, 0, s>>>(G->adj_u, G->adj_v, G->kp, G->bp, G->p, mp->d_rmassx,
                                                    mp->d_rmassy, mp->d_rmassz, mp->nglob, dt, dt2, dtsq2);
}

}  // namespace
}  // namespace sf3d

using namespace sf3d;

extern "C" {

int sf3d_gradient_setup(long* Mesh_pointer, int nstep, int checkpoint_every, double* device_bytes) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!mp->f.displ) { set_error(SF3D_ERR_STATE, "prepare_fields_elastic_device not called"); return SF3D_ERR_STATE; }
  if (mp->anisotropy) {
    set_error(SF3D_ERR_ARG, "sf3d_gradient: the gradient is for isotropic rho, kappa, mu");
    return SF3D_ERR_ARG;
  }
  if (mp->attenuation) {
    set_error(SF3D_ERR_ARG, "sf3d_gradient: attenuation is not supported (elastic misfit gradient only)");
    return SF3D_ERR_ARG;
  }
  if (mp->pml) {
    set_error(SF3D_ERR_UNSUPPORTED, "sf3d_gradient: C-PML layers are not supported in the adjoint sweep");
    return SF3D_ERR_UNSUPPORTED;
  }
  if (3L * mp->nglob >= (1L << 31)) {
    // the sweep's vector passes index the (3, NGLOB) arrays in 32 bits
    set_error(SF3D_ERR_ARG, "sf3d_gradient: 3 * NGLOB must stay below 2^31");
    return SF3D_ERR_ARG;
  }
  if (mp->has_acoustic) {
    set_error(SF3D_ERR_ARG, "sf3d_gradient: acoustic elements are not supported");
    return SF3D_ERR_ARG;
  }
  if (nstep < 1 || checkpoint_every < 1) { set_error(SF3D_ERR_ARG, "sf3d_gradient: nstep and checkpoint_every must be >= 1"); return SF3D_ERR_ARG; }
  if (mp->nrec_local > 0 && (!mp->d_seismo_d || mp->nlength_seismogram < nstep)) {
    set_error(SF3D_ERR_ARG, "sf3d_gradient: the displacement seismogram buffer must hold nstep samples");
    return SF3D_ERR_ARG;
  }
  if (mp->nsources > 0 && (!mp->d_stf_table || mp->stf_nstep < nstep)) {
    set_error(SF3D_ERR_STATE, "sf3d_set_stf_table must cover nstep");
    return SF3D_ERR_STATE;
  }
  free_grad(mp);
  GradState* G = new GradState();
  mp->grad = G;
  G->nstep = nstep;
  G->every = checkpoint_every < nstep ? checkpoint_every : nstep;
  const int nseg = (nstep + G->every - 1) / G->every;
  G->nckpt = nseg - 1;  // segment 0 starts from rest
  const size_t n3 = 3ull * mp->nglob;
  const size_t npt = (size_t)mp->nspec * NGLL3_PAD;
  bool ok = true;
  if (G->nckpt > 0) ok = ok && alloc_f(&G->ckpt, (size_t)G->nckpt * 3 * n3);
  G->seg_stride = (n3 + 3) & ~(size_t)3;
  ok = ok && alloc_f(&G->seg_u, (size_t)G->every * G->seg_stride) &&
       alloc_f(&G->seg_a, (size_t)G->every * G->seg_stride);
  ok = ok && alloc_f(&G->adj_u, n3) && alloc_f(&G->adj_v, n3) && alloc_f(&G->adj_a, n3);
  ok = ok && alloc_f(&G->p, n3) && alloc_f(&G->kp, n3) && alloc_f(&G->bp, n3);
  ok = ok && alloc_f(&G->residual, 3ull * (mp->nrec_local > 0 ? mp->nrec_local : 1) * nstep);
  ok = ok && alloc_zero((void**)&G->g_rho, sizeof(double) * npt) && alloc_zero((void**)&G->g_kappa, sizeof(double) * npt) &&
       alloc_zero((void**)&G->g_mu, sizeof(double) * npt);
  if (!ok) {
    free_grad(mp);
    return SF3D_ERR_CUDA;
  }
  for (int q = 0; q < NGLLX; ++q) G->wgll[q] = (float)sqrt((double)mp->h_wxy[q + NGLLX * q]);
  G->bytes = sizeof(float) * ((size_t)G->nckpt * 3 * n3 + 2ull * G->every * G->seg_stride + 6 * n3 +
                              3ull * (mp->nrec_local > 0 ? mp->nrec_local : 1) * nstep) +
             3 * sizeof(double) * npt;
  if (device_bytes) *device_bytes = (double)G->bytes;
  return SF3D_OK;
}

int sf3d_gradient_forward(long* Mesh_pointer, realw deltat) {
  NvtxRange nvtx_range("sf3d_gradient_forward");
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!grad_ready(mp)) return SF3D_ERR_STATE;
  GradState* G = mp->grad;
  const float dt = deltat, dt2 = deltat / 2.f, dtsq2 = deltat * deltat / 2.f;
  cudaStream_t s = mp->stream;
  const size_t n3 = 3ull * mp->nglob;
  zero_state(mp, s);
  launch_set_it(mp, 1, s);
  SF3D_CUDA_RET(cudaMemsetAsync(mp->d_done, 0, sizeof(unsigned int), s), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaEventRecord(mp->ev0, s), SF3D_ERR_CUDA);
  int launches = 0;
  for (int n = 0; n < G->nstep; ++n) {
    launches += enqueue_step(mp, dt, dt2, dtsq2, n == 0, nullptr);
    const int next = n + 1;
    if (next % G->every == 0 && next < G->nstep) save_state(mp, G->ckpt + (size_t)(next / G->every - 1) * 3 * n3, s);
  }
  launch_mass_corrector(mp, dt2, s);
  SF3D_CUDA_RET(cudaEventRecord(mp->ev1, s), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaEventSynchronize(mp->ev1), SF3D_ERR_CUDA);
  if (!cuda_ok(cudaGetLastError(), "sf3d_gradient_forward")) return SF3D_ERR_CUDA;
  cudaEventElapsedTime(&mp->last_total_ms, mp->ev0, mp->ev1);
  mp->last_total_launches = launches + 1;
  if (!check_kernel_error(mp)) return SF3D_ERR_CUDA;
  // scale of the forward field for the FP32 strain products of the gradient:
  // the largest recorded displacement (a 1 N.m source gives ~1e-19 m)
  G->u_scale = 1.f;
  if (mp->nrec_local > 0) {
    float mx = 0.f;
    if (!device_maxabs(mp, mp->d_seismo_d, 3L * mp->nrec_local * mp->nlength_seismogram, &mx)) return SF3D_ERR_CUDA;
    if (mx > 0.f && mx < 3.0e38f) {
      int ex = 0;
      frexpf(mx, &ex);
      G->u_scale = ldexpf(1.f, -ex);
    }
  }
  return sf3d_last_error(nullptr, 0);
}

int sf3d_gradient_set_residual(long* Mesh_pointer, const realw* residual) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!grad_ready(mp)) return SF3D_ERR_STATE;
  if (mp->nrec_local == 0) return SF3D_OK;
  if (!residual) { set_error(SF3D_ERR_ARG, "sf3d_gradient_set_residual: null residual"); return SF3D_ERR_ARG; }
  // Waveform residuals of small sources can be far below 1 (1e-20 for a 1 N.m
  // moment tensor), which would push the adjoint field and the strain products
  // of the gradient below the FP32 normal range.  The residual is therefore
  // scaled by a power of two that brings its maximum near 1; the gradient is
  // linear in the residual and sf3d_gradient_get divides the scale out in FP64.
  const size_t n = 3ull * mp->nrec_local * mp->grad->nstep;
  float mx = 0.f;
  for (size_t q = 0; q < n; ++q) {
    const float a = fabsf(residual[q]);
    if (!(a <= 3.0e38f)) { set_error(SF3D_ERR_ARG, "sf3d_gradient_set_residual: NaN or Inf in the residual"); return SF3D_ERR_ARG; }
    mx = a > mx ? a : mx;
  }
  int ex = 0;
  if (mx > 0.f) frexpf(mx, &ex);
  const double scale = ldexp(1.0, -ex);
  std::vector<float> tmp(n);
  for (size_t q = 0; q < n; ++q) tmp[q] = (float)((double)residual[q] * scale);
  mp->grad->res_scale = scale;
  if (!copy_sync(mp->grad->residual, tmp.data(), sizeof(float) * n, cudaMemcpyHostToDevice, mp->stream))
    return SF3D_ERR_CUDA;
  return SF3D_OK;
}

int sf3d_gradient_backward(long* Mesh_pointer, realw deltat) {
  NvtxRange nvtx_range("sf3d_gradient_backward");
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!grad_ready(mp)) return SF3D_ERR_STATE;
  GradState* G = mp->grad;
  const float dt = deltat, dt2 = deltat / 2.f, dtsq2 = deltat * deltat / 2.f;
  cudaStream_t s = mp->stream;
  const size_t n3 = 3ull * mp->nglob;
  const size_t npt = (size_t)mp->nspec * NGLL3_PAD;
  SF3D_CUDA_RET(cudaMemsetAsync(G->adj_u, 0, sizeof(float) * n3, s), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaMemsetAsync(G->adj_v, 0, sizeof(float) * n3, s), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaMemsetAsync(G->adj_a, 0, sizeof(float) * n3, s), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaMemsetAsync(G->g_rho, 0, sizeof(double) * npt, s), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaMemsetAsync(G->g_kappa, 0, sizeof(double) * npt, s), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaMemsetAsync(G->g_mu, 0, sizeof(double) * npt, s), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaMemsetAsync(mp->d_done, 0, sizeof(unsigned int), s), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaEventRecord(mp->ev0, s), SF3D_ERR_CUDA);
  // p of the last step from the zero adjoint state (p = 0, accumulators cleared)
  adj_p_kernel<<<nblk((long)n3, 256), 256, 0, s>>>(G->adj_v, G->adj_a, mp->d_rmassx, mp->d_rmassy, mp->d_rmassz,
                                                   mp->nglob, dt2, G->p, G->kp, G->bp);
  const int nseg = G->nckpt + 1;
  for (int j = nseg - 1; j >= 0; --j) {
    const int n0 = j * G->every;
    const int len = (n0 + G->every <= G->nstep) ? G->every : G->nstep - n0;
    if (j == 0)
      zero_state(mp, s);
    else
      load_state(mp, G->ckpt + (size_t)(j - 1) * 3 * n3, s);
    launch_set_it(mp, n0 + 1, s);
    // each recomputed step writes its displacement and force straight into the
    // segment's buffers (and reads the previous step's from there)
    float* const base_d = mp->f.displ;
    float* const base_a = mp->f.accel;
    for (int q = 0; q < len; ++q) {
      StepIO io;
      const size_t st = G->seg_stride;
      io.d_in = q == 0 ? base_d : G->seg_u + (size_t)(q - 1) * st;
      io.d_out = G->seg_u + (size_t)q * st;
      io.a_in = q == 0 ? base_a : G->seg_a + (size_t)(q - 1) * st;
      io.a_out = G->seg_a + (size_t)q * st;
      enqueue_step(mp, dt, dt2, dtsq2, j == 0 && q == 0, nullptr, &io);
    }
    mp->f.displ = base_d;
    mp->f.accel = base_a;
    for (int q = len - 1; q >= 0; --q)
      adjoint_step(mp, n0 + q, G->seg_u + (size_t)q * G->seg_stride, G->seg_a + (size_t)q * G->seg_stride, dt, dt2,
                   dtsq2);
    if (!cuda_ok(cudaGetLastError(), "sf3d_gradient_backward")) return SF3D_ERR_CUDA;
  }
  SF3D_CUDA_RET(cudaEventRecord(mp->ev1, s), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaEventSynchronize(mp->ev1), SF3D_ERR_CUDA);
  if (!cuda_ok(cudaGetLastError(), "sf3d_gradient_backward")) return SF3D_ERR_CUDA;
  cudaEventElapsedTime(&mp->last_total_ms, mp->ev0, mp->ev1);
  if (!check_kernel_error(mp)) return SF3D_ERR_CUDA;
  return sf3d_last_error(nullptr, 0);
}

int sf3d_gradient_set_fused(long* Mesh_pointer, int fused) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!mp->grad) { set_error(SF3D_ERR_STATE, "sf3d_gradient_setup not called"); return SF3D_ERR_STATE; }
  mp->grad->fused = fused ? 1 : 0;
  return SF3D_OK;
}

int sf3d_gradient_get(long* Mesh_pointer, double* g_rho, double* g_kappa, double* g_mu) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!mp->grad) { set_error(SF3D_ERR_STATE, "sf3d_gradient_setup not called"); return SF3D_ERR_STATE; }
  const size_t npt = (size_t)mp->nspec * NGLL3_PAD;
  std::vector<double> tmp(npt);
  double* outs[3] = {g_rho, g_kappa, g_mu};
  const double* srcs[3] = {mp->grad->g_rho, mp->grad->g_kappa, mp->grad->g_mu};
  for (int q = 0; q < 3; ++q) {
    if (!outs[q]) continue;
    if (!copy_sync(tmp.data(), srcs[q], sizeof(double) * npt, cudaMemcpyDeviceToHost, mp->stream)) return SF3D_ERR_CUDA;
    const double unscale = 1.0 / (mp->grad->res_scale * (double)mp->grad->u_scale);
    for (long e = 0; e < mp->nspec; ++e)
      for (int p = 0; p < NGLL3; ++p) outs[q][e * NGLL3 + p] = tmp[e * NGLL3_PAD + p] * unscale;
  }
  return SF3D_OK;
}

int sf3d_gradient_release(long* Mesh_pointer) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  cudaStreamSynchronize(mp->stream);
  free_grad(mp);
  return SF3D_OK;
}

}  // extern "C"
