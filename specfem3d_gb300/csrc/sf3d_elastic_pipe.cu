// Persistent, TMA-fed elastic / viscoelastic stiffness kernel (sm_103a).
//
// Same arithmetic as stiffness_kernel in sf3d_elastic.cu (which follows
// compute_forces_viscoelastic.F90:250-860 and compute_element_att_memory.f90:28-157),
// organised for HBM throughput:
//   * a persistent grid (a few CTAs per SM) walks the element list with a
//     grid stride, so consecutive CTAs work on neighbouring elements and the
//     gathered/scattered wavefield stays in L2;
//   * every per-element row (ibool, metric, kappa, mu, factor_common(_kappa),
//     memory variables, strains — 512 B each) is brought into a shared-memory
//     stage by the bulk-copy (TMA) engine (cp.async.bulk ... mbarrier::complete_tx)
//     NSTAGE-1 elements ahead, so each CTA keeps ~43 KB of reads in flight
//     while it computes;
//   * the displacement/velocity gather of element n+1 is issued before element
//     n is computed, hiding its L2 latency behind the contractions;
//   * new memory variables and strains are written back with plain coalesced
//     stores.
// Every wait on an mbarrier is bounded (2 s of %globaltimer); on timeout the
// CTA records an error word, drains its other stages with the same bound and
// returns.  The host reports the error through sf3d_last_error.
#include <stdint.h>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

constexpr int kStages = 3;
constexpr int kRowBytes = NGLL3_PAD * 4;  // 512
// row map of a stage (rows of 128 floats / ints)
constexpr int kRowIbool = 0;
constexpr int kRowMetric = 1;    // 9 rows
constexpr int kRowKappa = 10;
constexpr int kRowMu = 11;
constexpr int kRowFc = 12;       // 3 rows (sls)
constexpr int kRowFck = 15;      // 3 rows
constexpr int kRowR = 18;        // 18 rows: component c, sls s -> 18 + 3c + s
constexpr int kRowEps = 36;      // 6 rows
constexpr int kRowsAtt = 42;
constexpr int kRowsNoAtt = 12;

// Issue the bulk copies of element e into a stage; executed by warp 0.
template <bool ATT>
__device__ __forceinline__ void issue_element(const StiffnessArgs& a, int e, float* stage, uint64_t* bar, int lane) {
  const int ir = __ldg(a.irregular + e);
  const int nmetric = ir >= 0 ? 9 : 0;
  const int nrows = (ATT ? kRowsAtt : kRowsNoAtt) - (9 - nmetric);
  if (lane == 0) mbar_arrive_expect_tx(bar, (uint32_t)(nrows * kRowBytes));
  __syncwarp();
  const long eo = (long)e * NGLL3_PAD;
  const long mo = (long)(ir >= 0 ? ir : 0) * NGLL3_PAD;
  const long so = (long)e * (NSLS * NGLL3_PAD);
  // row list, one row per lane (two passes for the attenuation case)
  for (int r = lane; r < (ATT ? kRowsAtt : kRowsNoAtt); r += 32) {
    const void* src = nullptr;
    if (r == kRowIbool) src = a.ibool + eo;
    else if (r < kRowKappa) { if (nmetric) src = a.m[r - kRowMetric] + mo; }
    else if (r == kRowKappa) src = a.kappav + eo;
    else if (r == kRowMu) src = a.muv + eo;
    else if (ATT && r < kRowFck) src = a.fc + so + (r - kRowFc) * NGLL3_PAD;
    else if (ATT && r < kRowR) src = a.fck + so + (r - kRowFck) * NGLL3_PAD;
    else if (ATT && r < kRowEps) { const int c = (r - kRowR) / NSLS, s = (r - kRowR) % NSLS; src = a.R[c] + so + s * NGLL3_PAD; }
    else if (ATT) src = a.eps[r - kRowEps] + eo;
    if (src) bulk_g2s(stage + r * NGLL3_PAD, src, kRowBytes, bar);
  }
}

template <bool ATT, bool STRAIN>
__global__ void __launch_bounds__(NGLL3_PAD, ATT ? 3 : 5) stiffness_pipe_kernel(const StiffnessArgs a, int* err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  constexpr int kRows = ATT ? kRowsAtt : kRowsNoAtt;
  float* stages = reinterpret_cast<float*>(smem_raw);                       // kStages * kRows * 128
  float* s_u = stages + kStages * kRows * NGLL3_PAD;                         // 3 x 128
  float* s_v = s_u + 3 * NGLL3_PAD;                                          // 3 x 128
  float* s_t = s_v + 3 * NGLL3_PAD;                                          // 9 x 128
  float* s_gll = s_t + 9 * NGLL3_PAD;                                        // 128
  uint64_t* bars = reinterpret_cast<uint64_t*>(s_gll + NGLL3_PAD);           // kStages

  const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
  const bool active = t < NGLL3;
  const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
  const int nelem = a.nelem;
  const int first = blockIdx.x, stride = gridDim.x;

  if (t < NGLL3) s_gll[t] = __ldg(a.gll + t);
  if (t == 0) {
    for (int s = 0; s < kStages; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  auto elem_of = [&](int n) -> int {
    const int slot = first + n * stride;
    return a.phase ? __ldg(a.phase + slot) : slot;
  };
  auto exists = [&](int n) -> bool { return first + n * stride < nelem; };

  // prologue: stages for elements 0 .. kStages-1 of this CTA
  if (warp == 0)
    for (int n = 0; n < kStages; ++n)
      if (exists(n)) issue_element<ATT>(a, elem_of(n), stages + (n % kStages) * kRows * NGLL3_PAD, &bars[n % kStages], lane);

  // gather of element 0
  float ux = 0.f, uy = 0.f, uz = 0.f, vx = 0.f, vy = 0.f, vz = 0.f;
  bool ok = true;
  if (exists(0)) {
    ok = mbar_wait_bounded(&bars[0], 0);
    if (ok && active) {
      const int g = reinterpret_cast<const int*>(stages)[kRowIbool * NGLL3_PAD + t];
      ux = a.displ[3L * g]; uy = a.displ[3L * g + 1]; uz = a.displ[3L * g + 2];
      if (ATT) { vx = a.veloc[3L * g]; vy = a.veloc[3L * g + 1]; vz = a.veloc[3L * g + 2]; }
    }
  }
  if (__syncthreads_or(!ok)) {
    if (t == 0) atomicExch(err, 1);
    for (int q = 1; q < kStages; ++q)
      if (exists(q)) mbar_wait_bounded(&bars[q], 0);
    return;
  }

  for (int n = 0; exists(n); ++n) {
    const int e = elem_of(n);
    const int st = n % kStages;
    float* S = stages + st * kRows * NGLL3_PAD;
    const int* Si = reinterpret_cast<const int*>(S);
    // element n's gathered values into shared memory
    s_u[t] = ux; s_u[NGLL3_PAD + t] = uy; s_u[2 * NGLL3_PAD + t] = uz;
    if (ATT) {
      s_v[t] = a.deltat * vx; s_v[NGLL3_PAD + t] = a.deltat * vy; s_v[2 * NGLL3_PAD + t] = a.deltat * vz;
    }
    // prefetch the gather of element n+1 (its stage was issued two iterations ago)
    bool ok2 = true;
    if (exists(n + 1)) {
      const int st1 = (n + 1) % kStages;
      ok2 = mbar_wait_bounded(&bars[st1], ((n + 1) / kStages) & 1);
      if (ok2 && active) {
        const int g = reinterpret_cast<const int*>(stages + st1 * kRows * NGLL3_PAD)[kRowIbool * NGLL3_PAD + t];
        ux = a.displ[3L * g]; uy = a.displ[3L * g + 1]; uz = a.displ[3L * g + 2];
        if (ATT) { vx = a.veloc[3L * g]; vy = a.veloc[3L * g + 1]; vz = a.veloc[3L * g + 2]; }
      }
    }
    if (__syncthreads_or(!ok2)) {
      if (t == 0) atomicExch(err, 1);
      for (int q = 1; q < kStages; ++q)
        if (exists(n + q)) mbar_wait_bounded(&bars[(n + q) % kStages], ((n + q) / kStages) & 1);
      return;
    }

    const int ir = __ldg(a.irregular + e);
    const long eo = (long)e * NGLL3_PAD + t;
    float epsl[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int iglob = 0;
    if (active) {
      iglob = Si[kRowIbool * NGLL3_PAD + t];
      const float* hp = s_gll;
      float t1x = 0.f, t2x = 0.f, t3x = 0.f, t1y = 0.f, t2y = 0.f, t3y = 0.f, t1z = 0.f, t2z = 0.f, t3z = 0.f;
#pragma unroll
      for (int l = 0; l < NGLLX; ++l) {
        const float h1 = hp[i + NGLLX * l], h2 = hp[j + NGLLX * l], h3 = hp[k + NGLLX * l];
        const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
        t1x = fmaf(s_u[p1], h1, t1x); t1y = fmaf(s_u[NGLL3_PAD + p1], h1, t1y); t1z = fmaf(s_u[2 * NGLL3_PAD + p1], h1, t1z);
        t2x = fmaf(s_u[p2], h2, t2x); t2y = fmaf(s_u[NGLL3_PAD + p2], h2, t2y); t2z = fmaf(s_u[2 * NGLL3_PAD + p2], h2, t2z);
        t3x = fmaf(s_u[p3], h3, t3x); t3y = fmaf(s_u[NGLL3_PAD + p3], h3, t3y); t3z = fmaf(s_u[2 * NGLL3_PAD + p3], h3, t3z);
      }
      float a1x = t1x, a2x = t2x, a3x = t3x, a1y = t1y, a2y = t2y, a3y = t3y, a1z = t1z, a2z = t2z, a3z = t3z;
      if (ATT) {
#pragma unroll
        for (int l = 0; l < NGLLX; ++l) {
          const float h1 = hp[i + NGLLX * l], h2 = hp[j + NGLLX * l], h3 = hp[k + NGLLX * l];
          const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
          a1x = fmaf(s_v[p1], h1, a1x); a1y = fmaf(s_v[NGLL3_PAD + p1], h1, a1y); a1z = fmaf(s_v[2 * NGLL3_PAD + p1], h1, a1z);
          a2x = fmaf(s_v[p2], h2, a2x); a2y = fmaf(s_v[NGLL3_PAD + p2], h2, a2y); a2z = fmaf(s_v[2 * NGLL3_PAD + p2], h2, a2z);
          a3x = fmaf(s_v[p3], h3, a3x); a3y = fmaf(s_v[NGLL3_PAD + p3], h3, a3y); a3z = fmaf(s_v[2 * NGLL3_PAD + p3], h3, a3z);
        }
      }
      const float xr = a.xix_regular;
      float xix = 0.f, xiy = 0.f, xiz = 0.f, etax = 0.f, etay = 0.f, etaz = 0.f, gammax = 0.f, gammay = 0.f, gammaz = 0.f;
      if (ir >= 0) {
        xix = S[(kRowMetric + 0) * NGLL3_PAD + t]; xiy = S[(kRowMetric + 1) * NGLL3_PAD + t];
        xiz = S[(kRowMetric + 2) * NGLL3_PAD + t]; etax = S[(kRowMetric + 3) * NGLL3_PAD + t];
        etay = S[(kRowMetric + 4) * NGLL3_PAD + t]; etaz = S[(kRowMetric + 5) * NGLL3_PAD + t];
        gammax = S[(kRowMetric + 6) * NGLL3_PAD + t]; gammay = S[(kRowMetric + 7) * NGLL3_PAD + t];
        gammaz = S[(kRowMetric + 8) * NGLL3_PAD + t];
      }
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
      const float kap = S[kRowKappa * NGLL3_PAD + t], mu = S[kRowMu * NGLL3_PAD + t];
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
        for (int c = 0; c < 6; ++c)
          sR[c] = S[(kRowR + 3 * c) * NGLL3_PAD + t] + S[(kRowR + 3 * c + 1) * NGLL3_PAD + t] +
                  S[(kRowR + 3 * c + 2) * NGLL3_PAD + t];
        sig_xx = sig_xx - sR[0] - sR[5];
        sig_yy = sig_yy - sR[1] - sR[5];
        sig_zz = sig_zz + sR[0] + sR[1] - sR[5];
        sig_xy -= sR[2];
        sig_xz -= sR[3];
        sig_yz -= sR[4];
      }
      if (ir >= 0) {
        const float jac = 1.f / (xix * (etay * gammaz - etaz * gammay) - xiy * (etax * gammaz - etaz * gammax) +
                                 xiz * (etax * gammay - etay * gammax));
        s_t[0 * NGLL3_PAD + t] = jac * (sig_xx * xix + sig_xy * xiy + sig_xz * xiz);
        s_t[1 * NGLL3_PAD + t] = jac * (sig_xy * xix + sig_yy * xiy + sig_yz * xiz);
        s_t[2 * NGLL3_PAD + t] = jac * (sig_xz * xix + sig_yz * xiy + sig_zz * xiz);
        s_t[3 * NGLL3_PAD + t] = jac * (sig_xx * etax + sig_xy * etay + sig_xz * etaz);
        s_t[4 * NGLL3_PAD + t] = jac * (sig_xy * etax + sig_yy * etay + sig_yz * etaz);
        s_t[5 * NGLL3_PAD + t] = jac * (sig_xz * etax + sig_yz * etay + sig_zz * etaz);
        s_t[6 * NGLL3_PAD + t] = jac * (sig_xx * gammax + sig_xy * gammay + sig_xz * gammaz);
        s_t[7 * NGLL3_PAD + t] = jac * (sig_xy * gammax + sig_yy * gammay + sig_yz * gammaz);
        s_t[8 * NGLL3_PAD + t] = jac * (sig_xz * gammax + sig_yz * gammay + sig_zz * gammaz);
      } else {
        const float js = a.jacobian_regular * xr;
        s_t[0 * NGLL3_PAD + t] = js * sig_xx; s_t[1 * NGLL3_PAD + t] = js * sig_xy; s_t[2 * NGLL3_PAD + t] = js * sig_xz;
        s_t[3 * NGLL3_PAD + t] = js * sig_xy; s_t[4 * NGLL3_PAD + t] = js * sig_yy; s_t[5 * NGLL3_PAD + t] = js * sig_yz;
        s_t[6 * NGLL3_PAD + t] = js * sig_xz; s_t[7 * NGLL3_PAD + t] = js * sig_yz; s_t[8 * NGLL3_PAD + t] = js * sig_zz;
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
        n1x = fmaf(s_t[0 * NGLL3_PAD + p1], f1, n1x); n1y = fmaf(s_t[1 * NGLL3_PAD + p1], f1, n1y);
        n1z = fmaf(s_t[2 * NGLL3_PAD + p1], f1, n1z);
        n2x = fmaf(s_t[3 * NGLL3_PAD + p2], f2, n2x); n2y = fmaf(s_t[4 * NGLL3_PAD + p2], f2, n2y);
        n2z = fmaf(s_t[5 * NGLL3_PAD + p2], f2, n2z);
        n3x = fmaf(s_t[6 * NGLL3_PAD + p3], f3, n3x); n3y = fmaf(s_t[7 * NGLL3_PAD + p3], f3, n3y);
        n3z = fmaf(s_t[8 * NGLL3_PAD + p3], f3, n3z);
      }
      const float fac1 = s_gll[4 * NGLL2 + j + NGLLX * k];
      const float fac2 = s_gll[3 * NGLL2 + i + NGLLX * k];
      const float fac3 = s_gll[2 * NGLL2 + i + NGLLX * j];
      atomicAdd(a.accel + 3L * iglob, -(fac1 * n1x + fac2 * n2x + fac3 * n3x));
      atomicAdd(a.accel + 3L * iglob + 1, -(fac1 * n1y + fac2 * n2y + fac3 * n3y));
      atomicAdd(a.accel + 3L * iglob + 2, -(fac1 * n1z + fac2 * n2z + fac3 * n3z));
      if (ATT) {
        const long so = (long)e * (NSLS * NGLL3_PAD) + t;
        const float kap = S[kRowKappa * NGLL3_PAD + t], mu = S[kRowMu * NGLL3_PAD + t];
        float eold[6];
#pragma unroll
        for (int c = 0; c < 6; ++c) eold[c] = S[(kRowEps + c) * NGLL3_PAD + t];
#pragma unroll
        for (int s = 0; s < NSLS; ++s) {
          const float al = a.alpha[s], be = a.beta[s], ga = a.gamma[s];
          const float fk = kap * S[(kRowFck + s) * NGLL3_PAD + t];
          a.R[5][so + s * NGLL3_PAD] = al * S[(kRowR + 15 + s) * NGLL3_PAD + t] + fk * (be * eold[5] + ga * epsl[5]);
          const float fm = mu * S[(kRowFc + s) * NGLL3_PAD + t];
#pragma unroll
          for (int c = 0; c < 5; ++c)
            a.R[c][so + s * NGLL3_PAD] = al * S[(kRowR + 3 * c + s) * NGLL3_PAD + t] + fm * (be * eold[c] + ga * epsl[c]);
        }
      }
      if (STRAIN) {
        if (ATT) a.eps[5][eo] = epsl[5];
#pragma unroll
        for (int c = 0; c < 5; ++c)
          if (a.eps[c]) a.eps[c][eo] = epsl[c];
      }
    }
    __syncthreads();
    // stage st is free: prefetch element n + kStages into it
    if (warp == 0 && exists(n + kStages)) {
      fence_proxy_async();
      issue_element<ATT>(a, elem_of(n + kStages), S, &bars[st], lane);
    }
  }
}

template <bool ATT>
size_t pipe_smem_bytes() {
  constexpr int kRows = ATT ? kRowsAtt : kRowsNoAtt;
  return sizeof(float) * (kStages * kRows * NGLL3_PAD + (3 + 3 + 9 + 1) * NGLL3_PAD) + sizeof(uint64_t) * kStages;
}

}  // namespace

static int g_num_sms = 0;

void launch_stiffness_pipelined(const StiffnessArgs& a, bool att, bool store_strain, int* err, cudaStream_t s) {
  if (a.nelem <= 0) return;
  if (g_num_sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (g_num_sms <= 0) g_num_sms = 148;
  }
  const size_t smem = att ? pipe_smem_bytes<true>() : pipe_smem_bytes<false>();
  const int per_sm = att ? 3 : 5;
  int grid = g_num_sms * per_sm;
  if (grid > a.nelem) grid = a.nelem;
  if (att) {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(stiffness_pipe_kernel<true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr = true;
    }
    stiffness_pipe_kernel<true, true><<<grid, NGLL3_PAD, smem, s>>>(a, err);
  } else if (store_strain) {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(stiffness_pipe_kernel<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr = true;
    }
    stiffness_pipe_kernel<false, true><<<grid, NGLL3_PAD, smem, s>>>(a, err);
  } else {
    static bool attr = false;
    if (!attr) {
      cudaFuncSetAttribute(stiffness_pipe_kernel<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      attr = true;
    }
    stiffness_pipe_kernel<false, false><<<grid, NGLL3_PAD, smem, s>>>(a, err);
  }
}

}  // namespace sf3d
