// Elastic / viscoelastic stiffness with three threads per GLL point (sm_103a).
//
// Same arithmetic as stiffness_kernel (sf3d_elastic.cu; compute_forces_viscoelastic.F90:250-860,
// compute_element_att_memory.f90:28-157), spread over a 384-thread CTA: thread
// (c, p) handles displacement component c of GLL point p.  It gathers u_c (and
// dt v_c), runs the 5-wide contractions of its component, forms the three
// derivatives of component c, owns two of the six memory-variable components
// (xx,yy | xy,xz | yz,trace) with their strains, builds row c of the stress
// terms and scatters accel_c.  The point's nine derivatives, the memory-variable
// sums and the stress terms meet in shared memory.  A CTA keeps 12 warps per
// element with about a third of the registers per thread, so an SM holds three
// times as many warps in flight as with one thread per point.
#include "sf3d_internal.h"

namespace sf3d {
namespace {

constexpr int kSplitThreads = 3 * NGLL3_PAD;

template <bool ATT, bool STRAIN, int MINB>
__global__ void __launch_bounds__(kSplitThreads, MINB) stiffness_split_kernel(const StiffnessArgs a) {
  __shared__ float s_gll[NGLL3];
  __shared__ float s_u[3][NGLL3_PAD];
  __shared__ float s_v[ATT ? 3 : 1][NGLL3_PAD];
  __shared__ float s_rs[ATT ? 6 : 1][NGLL3_PAD];     // sum over SLS of each memory-variable component
  __shared__ float s_d[9][NGLL3_PAD];                // derivative of component c along x: row 3c + x
  __shared__ float s_s[STRAIN ? 9 : 1][NGLL3_PAD];   // same for the strain field (u + dt v with attenuation)
  __shared__ float s_t[9][NGLL3_PAD];                // J sigma grad(xi): row 3d + c

  const int tid = threadIdx.x;
  const int c = tid / NGLL3_PAD, t = tid % NGLL3_PAD;  // all threads of a warp share c
  const int e = a.phase ? __ldg(a.phase + blockIdx.x) : (int)blockIdx.x;
  const bool active = t < NGLL3;
  const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
  const long eo = (long)e * NGLL3_PAD + t;
  const int ir = __ldg(a.irregular + e);
  // memory-variable components owned by this thread: 2c and 2c+1
  const int q0 = 2 * c, q1 = 2 * c + 1;

  int iglob = 0;
  float m[9];
#pragma unroll
  for (int q = 0; q < 9; ++q) m[q] = 0.f;
  float kap = 0.f, mu = 0.f, uc = 0.f, vc = 0.f;
  float R0[NSLS] = {0.f, 0.f, 0.f}, R1[NSLS] = {0.f, 0.f, 0.f}, fcs[NSLS] = {0.f, 0.f, 0.f};
  float fks[NSLS] = {0.f, 0.f, 0.f};
  float eold0 = 0.f, eold1 = 0.f;
  if (active) {
    iglob = __ldg(a.ibool + eo);
    kap = __ldg(a.kappav + eo);
    mu = __ldg(a.muv + eo);
    if (ir >= 0) {
      const long mo = (long)ir * NGLL3_PAD + t;
#pragma unroll
      for (int q = 0; q < 9; ++q) m[q] = __ldg(a.m[q] + mo);
    }
    if (ATT) {
      const long so = (long)e * (NSLS * NGLL3_PAD) + t;
#pragma unroll
      for (int s = 0; s < NSLS; ++s) {
        R0[s] = a.R[q0][so + s * NGLL3_PAD];
        R1[s] = a.R[q1][so + s * NGLL3_PAD];
        fcs[s] = __ldg(a.fc + so + s * NGLL3_PAD);
        if (c == 2) fks[s] = __ldg(a.fck + so + s * NGLL3_PAD);
      }
      eold0 = a.eps[q0][eo];
      eold1 = a.eps[q1][eo];
    }
    uc = a.displ[3L * iglob + c];
    if (ATT) vc = a.deltat * a.veloc[3L * iglob + c];
  }
  if (tid < NGLL3) s_gll[tid] = __ldg(a.gll + tid);
  s_u[c][t] = uc;
  if (ATT) {
    s_v[c][t] = vc;
    s_rs[q0][t] = R0[0] + R0[1] + R0[2];
    s_rs[q1][t] = R1[0] + R1[1] + R1[2];
  }
  __syncthreads();

  // ---- derivatives of component c ------------------------------------------------
  if (active) {
    const float* hp = s_gll;
    float t1 = 0.f, t2 = 0.f, t3 = 0.f;
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) {
      const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
      t1 = fmaf(s_u[c][p1], hp[i + NGLLX * l], t1);
      t2 = fmaf(s_u[c][p2], hp[j + NGLLX * l], t2);
      t3 = fmaf(s_u[c][p3], hp[k + NGLLX * l], t3);
    }
    float a1 = t1, a2 = t2, a3 = t3;
    if (ATT) {
#pragma unroll
      for (int l = 0; l < NGLLX; ++l) {
        const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
        a1 = fmaf(s_v[c][p1], hp[i + NGLLX * l], a1);
        a2 = fmaf(s_v[c][p2], hp[j + NGLLX * l], a2);
        a3 = fmaf(s_v[c][p3], hp[k + NGLLX * l], a3);
      }
    }
    const float xr = a.xix_regular;
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      s_d[3 * c + x][t] = ir >= 0 ? m[x] * t1 + m[3 + x] * t2 + m[6 + x] * t3 : xr * (x == 0 ? t1 : (x == 1 ? t2 : t3));
      if (STRAIN) {
        if (ATT)
          s_s[3 * c + x][t] =
              ir >= 0 ? m[x] * a1 + m[3 + x] * a2 + m[6 + x] * a3 : xr * (x == 0 ? a1 : (x == 1 ? a2 : a3));
        else
          s_s[3 * c + x][t] = s_d[3 * c + x][t];
      }
    }
  }
  __syncthreads();

  // ---- strain, stress row c, memory variables of the owned components -------------
  if (active) {
    const float dxx = s_d[0][t], dxy = s_d[1][t], dxz = s_d[2][t];
    const float dyx = s_d[3][t], dyy = s_d[4][t], dyz = s_d[5][t];
    const float dzx = s_d[6][t], dzy = s_d[7][t], dzz = s_d[8][t];
    float epsl[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (STRAIN) {
      const float sxx = s_s[0][t], sxy = s_s[1][t], sxz = s_s[2][t];
      const float syx = s_s[3][t], syy = s_s[4][t], syz = s_s[5][t];
      const float szx = s_s[6][t], szy = s_s[7][t], szz = s_s[8][t];
      const float templ = (1.f / 3.f) * (sxx + syy + szz);
      epsl[5] = sxx + syy + szz;
      epsl[0] = sxx - templ;
      epsl[1] = syy - templ;
      epsl[2] = 0.5f * (sxy + syx);
      epsl[3] = 0.5f * (szx + sxz);
      epsl[4] = 0.5f * (szy + syz);
      if (c == 0 && a.eps_trace_over_3) a.eps_trace_over_3[eo] = templ;
    }
    const float l2m = kap + (4.f / 3.f) * mu;
    const float lam = l2m - 2.f * mu;
    float sig_xx = l2m * dxx + lam * (dyy + dzz);
    float sig_yy = l2m * dyy + lam * (dxx + dzz);
    float sig_zz = l2m * dzz + lam * (dxx + dyy);
    float sig_xy = mu * (dxy + dyx);
    float sig_xz = mu * (dzx + dxz);
    float sig_yz = mu * (dzy + dyz);
    if (ATT) {
      float sR[6];
#pragma unroll
      for (int q = 0; q < 6; ++q) sR[q] = s_rs[q][t];
      sig_xx = sig_xx - sR[0] - sR[5];
      sig_yy = sig_yy - sR[1] - sR[5];
      sig_zz = sig_zz + sR[0] + sR[1] - sR[5];
      sig_xy -= sR[2];
      sig_xz -= sR[3];
      sig_yz -= sR[4];
    }
    // row c of the symmetric stress
    const float r0 = c == 0 ? sig_xx : (c == 1 ? sig_xy : sig_xz);
    const float r1 = c == 0 ? sig_xy : (c == 1 ? sig_yy : sig_yz);
    const float r2 = c == 0 ? sig_xz : (c == 1 ? sig_yz : sig_zz);
    if (ir >= 0) {
      const float jac = 1.f / (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                               m[2] * (m[3] * m[7] - m[4] * m[6]));
#pragma unroll
      for (int d = 0; d < 3; ++d) s_t[3 * d + c][t] = jac * (r0 * m[3 * d] + r1 * m[3 * d + 1] + r2 * m[3 * d + 2]);
    } else {
      const float js = a.jacobian_regular * a.xix_regular;
      s_t[c][t] = js * r0;
      s_t[3 + c][t] = js * r1;
      s_t[6 + c][t] = js * r2;
    }
    if (ATT) {
      const long so = (long)e * (NSLS * NGLL3_PAD) + t;
      const float e0 = epsl[q0], e1 = epsl[q1];
#pragma unroll
      for (int s = 0; s < NSLS; ++s) {
        const float al = a.alpha[s], be = a.beta[s], ga = a.gamma[s];
        const float fm = mu * fcs[s];
        a.R[q0][so + s * NGLL3_PAD] = al * R0[s] + fm * (be * eold0 + ga * e0);
        const float f1 = c == 2 ? kap * fks[s] : fm;
        a.R[q1][so + s * NGLL3_PAD] = al * R1[s] + f1 * (be * eold1 + ga * e1);
      }
    }
    if (STRAIN) {
      if (a.eps[q0]) a.eps[q0][eo] = epsl[q0];
      if ((ATT || q1 < 5) && a.eps[q1]) a.eps[q1][eo] = epsl[q1];
    }
  }
  __syncthreads();

  // ---- transposed contractions of component c and scatter ---------------------------
  if (active) {
    const float* hpw = s_gll + NGLL2;
    float n1 = 0.f, n2 = 0.f, n3 = 0.f;
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) {
      const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
      n1 = fmaf(s_t[c][p1], hpw[l + NGLLX * i], n1);
      n2 = fmaf(s_t[3 + c][p2], hpw[l + NGLLX * j], n2);
      n3 = fmaf(s_t[6 + c][p3], hpw[l + NGLLX * k], n3);
    }
    const float fac1 = s_gll[4 * NGLL2 + j + NGLLX * k];
    const float fac2 = s_gll[3 * NGLL2 + i + NGLLX * k];
    const float fac3 = s_gll[2 * NGLL2 + i + NGLLX * j];
    atomicAdd(a.accel + 3L * iglob + c, -(fac1 * n1 + fac2 * n2 + fac3 * n3));
  }
}

template <int MINB>
void launch_split_minb(const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s) {
  if (att)
    stiffness_split_kernel<true, true, MINB><<<a.nelem, kSplitThreads, 0, s>>>(a);
  else if (store_strain)
    stiffness_split_kernel<false, true, MINB><<<a.nelem, kSplitThreads, 0, s>>>(a);
  else
    stiffness_split_kernel<false, false, MINB><<<a.nelem, kSplitThreads, 0, s>>>(a);
}

}  // namespace

void launch_stiffness_split(const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s, int blocks_per_sm) {
  if (a.nelem <= 0) return;
  if (blocks_per_sm >= 4)
    launch_split_minb<4>(a, att, store_strain, s);
  else
    launch_split_minb<3>(a, att, store_strain, s);
}

}  // namespace sf3d
