// Acoustic (fluid) domain and fluid-solid coupling.
//
// Replaces prepare_fields_acoustic_device (prepare_mesh_constants_cuda.cu:434),
// compute_forces_acoustic_cuda / acoustic_enforce_free_surf_cuda
// (compute_forces_acoustic_cuda.cu:238, :334), update_displacement_ac_cuda and
// kernel_3_acoustic_cuda (update_displacement_cuda.cu:192, :448),
// compute_stacey_acoustic_cuda (compute_stacey_acoustic_cuda.cu:39),
// compute_coupling_ac_el_cuda / compute_coupling_el_ac_cuda
// (compute_coupling_cuda.cu:39, :135), compute_add_sources_ac_cuda
// (compute_add_sources_acoustic_cuda.cu:65) and the acoustic transfers.
// The physics follows the reference CPU routines cited on each kernel.
#include <vector>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

struct Metric9 {
  const float* p[9];
};

// FORWARD_OR_ADJOINT 1: the forward (adjoint, in a kernel run) potentials;
// 3: the backward / reconstructed potentials of SIMULATION_TYPE = 3
struct AcField {
  float* p;
  float* pd;
  float* pdd;
};

// every array prepare_fields_acoustic_adj_dev allocates is present
inline bool ac_adj_ready(const Mesh* mp) {
  return mp->d_b_potential && mp->d_b_potential_dot && mp->d_b_potential_dot_dot && mp->d_rho_ac_kl &&
         mp->d_kappa_ac_kl;
}

bool ac_field(Mesh* mp, const int* fa, AcField* F) {
  if (!fa || (*fa != 1 && *fa != 3)) return set_error(SF3D_ERR_ARG, "FORWARD_OR_ADJOINT must be 1 or 3 for acoustic fields");
  if (*fa == 1) {
    *F = {mp->d_potential, mp->d_potential_dot, mp->d_potential_dot_dot};
    return true;
  }
  if (!ac_adj_ready(mp)) return set_error(SF3D_ERR_STATE, "prepare_fields_acoustic_adj_dev not called");
  *F = {mp->d_b_potential, mp->d_b_potential_dot, mp->d_b_potential_dot_dot};
  return true;
}

// chi_dot_dot -= w . hprimewgll^T ( J/rho grad(xi) . grad chi )
// (compute_forces_acoustic.F90:130-340); one 128-thread CTA per element.  An
// element moves 1 KB (ibool, rho) and its gather depends on ibool, so the
// kernel is bound by that load chain: it is compiled for 16 resident CTAs per
// SM (32 registers, no spills), which took the fluid pass of the coupled
// 96x96x48 step from about 150 to 115 us against 8 CTAs/SM.
__global__ void __launch_bounds__(NGLL3_PAD, 16)
    acoustic_stiffness_kernel(int nelem, const int* __restrict__ phase, const int* __restrict__ ibool,
                              const int* __restrict__ irregular, const float* __restrict__ m0,
                              const float* __restrict__ m1, const float* __restrict__ m2, const float* __restrict__ m3,
                              const float* __restrict__ m4, const float* __restrict__ m5,
                              const float* __restrict__ m6, const float* __restrict__ m7,
                              const float* __restrict__ m8, const float* __restrict__ rhostore,
                              const float* __restrict__ gll, float xix_regular, float jacobian_regular,
                              const float* __restrict__ pot, float* __restrict__ pot_dd) {
  __shared__ float s_gll[NGLL3];
  __shared__ float s_chi[NGLL3_PAD];
  __shared__ float s_t[3][NGLL3_PAD];
  const int t = threadIdx.x;
  const int e = phase ? __ldg(phase + blockIdx.x) : (int)blockIdx.x;
  const bool active = t < NGLL3;
  const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
  const long eo = (long)e * NGLL3_PAD + t;
  const int ir = __ldg(irregular + e);
  int g = 0;
  float rho = 1.f;
  float m[9] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  if (active) {
    g = __ldg(ibool + eo);
    rho = __ldg(rhostore + eo);
    if (ir >= 0) {
      const long mo = (long)ir * NGLL3_PAD + t;
      m[0] = __ldg(m0 + mo); m[1] = __ldg(m1 + mo); m[2] = __ldg(m2 + mo);
      m[3] = __ldg(m3 + mo); m[4] = __ldg(m4 + mo); m[5] = __ldg(m5 + mo);
      m[6] = __ldg(m6 + mo); m[7] = __ldg(m7 + mo); m[8] = __ldg(m8 + mo);
    }
    s_chi[t] = pot[g];
  }
  if (t < NGLL3) s_gll[t] = __ldg(gll + t);
  __syncthreads();
  if (active) {
    float a = 0.f, b = 0.f, c = 0.f;
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) {
      a = fmaf(s_chi[l + NGLLX * j + NGLL2 * k], s_gll[i + NGLLX * l], a);
      b = fmaf(s_chi[i + NGLLX * l + NGLL2 * k], s_gll[j + NGLLX * l], b);
      c = fmaf(s_chi[i + NGLLX * j + NGLL2 * l], s_gll[k + NGLLX * l], c);
    }
    const float rho_inv = 1.f / rho;
    if (ir >= 0) {
      const float jac = 1.f / (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                               m[2] * (m[3] * m[7] - m[4] * m[6]));
      const float dx = m[0] * a + m[3] * b + m[6] * c;
      const float dy = m[1] * a + m[4] * b + m[7] * c;
      const float dz = m[2] * a + m[5] * b + m[8] * c;
      const float f = rho_inv * jac;
      s_t[0][t] = f * (m[0] * dx + m[1] * dy + m[2] * dz);
      s_t[1][t] = f * (m[3] * dx + m[4] * dy + m[5] * dz);
      s_t[2][t] = f * (m[6] * dx + m[7] * dy + m[8] * dz);
    } else {
      const float f = rho_inv * jacobian_regular * xix_regular * xix_regular;
      s_t[0][t] = f * a;
      s_t[1][t] = f * b;
      s_t[2][t] = f * c;
    }
  }
  __syncthreads();
  if (active) {
    const float* hpw = s_gll + NGLL2;
    float a = 0.f, b = 0.f, c = 0.f;
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) {
      a = fmaf(s_t[0][l + NGLLX * j + NGLL2 * k], hpw[l + NGLLX * i], a);
      b = fmaf(s_t[1][i + NGLLX * l + NGLL2 * k], hpw[l + NGLLX * j], b);
      c = fmaf(s_t[2][i + NGLLX * j + NGLL2 * l], hpw[l + NGLLX * k], c);
    }
    const float add = s_gll[4 * NGLL2 + j + NGLLX * k] * a + s_gll[3 * NGLL2 + i + NGLLX * k] * b +
                      s_gll[2 * NGLL2 + i + NGLLX * j] * c;
    atomicAdd(pot_dd + g, -add);
  }
}

// Sommerfeld condition on the faces of fluid elements
// (compute_stacey_acoustic.f90:98-125): chi_dd -= chi_dot jw / (cp rho)
__global__ void stacey_acoustic_kernel(int nfaces, const int* __restrict__ abs_ispec, const int* __restrict__ abs_pt,
                                       const float* __restrict__ jw, const int* __restrict__ is_acoustic,
                                       const int* __restrict__ ibool, const float* __restrict__ rhostore,
                                       const float* __restrict__ kappav, const float* __restrict__ pot_dot,
                                       float* __restrict__ pot_dd, float* __restrict__ record) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)nfaces * NGLL2) return;
  const int e = abs_ispec[idx / NGLL2];
  if (!is_acoustic[e]) return;
  const long q = (long)e * NGLL3_PAD + abs_pt[idx];
  const int g = ibool[q];
  const float rhol = rhostore[q];
  const float cpl = sqrtf(kappav[q] / rhol);
  const float absorbl = pot_dot[g] / rhol * jw[idx] / cpl;
  atomicAdd(pot_dd + g, -absorbl);
  // SAVE_FORWARD: b_absorb_potential(NGLL2, nfaces) of this step
  if (record) record[idx] = absorbl;
}

// replay of the boundary record on the backward potentials
// (kernels/compute_stacey_acoustic_kernel.cu, SIMULATION_TYPE = 3)
__global__ void stacey_acoustic_replay_kernel(int nfaces, const int* __restrict__ abs_ispec,
                                              const int* __restrict__ abs_pt, const int* __restrict__ is_acoustic,
                                              const int* __restrict__ ibool, const float* __restrict__ record,
                                              float* __restrict__ pot_dd) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)nfaces * NGLL2) return;
  const int e = abs_ispec[idx / NGLL2];
  if (!is_acoustic[e]) return;
  atomicAdd(pot_dd + ibool[(long)e * NGLL3_PAD + abs_pt[idx]], -record[idx]);
}

// acoustic kernels (compute_kernels.f90:257-330, kernels/compute_kernels_acoustic_kernel.cu):
// rho_ac_kl += dt grad(a) . grad(b_chi), kappa_ac_kl += dt a b_chi_dd with a = chi_adj
// (the reference) or a = chi_adj_dd (the discrete derivative of the misfit; the
// caller passes that array as pot); the 1/rho of the reference's gradient routine
// is undone there by rho, so the plain gradients are used; FP64 accumulators
__global__ void __launch_bounds__(NGLL3_PAD)
    kernels_acoustic_kernel(long nspec, const int* __restrict__ is_acoustic, const int* __restrict__ ibool,
                            const int* __restrict__ irregular, Metric9 m, const float* __restrict__ gll,
                            float xix_regular, const float* __restrict__ pot, const float* __restrict__ b_pot,
                            const float* __restrict__ b_pot_dd, double dt, double* __restrict__ rho_kl,
                            double* __restrict__ kappa_kl) {
  __shared__ float s_a[NGLL3_PAD];
  __shared__ float s_b[NGLL3_PAD];
  __shared__ float s_hp[NGLL2];
  const long e = blockIdx.x;
  const int t = threadIdx.x;
  if (e >= nspec || !is_acoustic[e]) return;
  const bool active = t < NGLL3;
  const long eo = e * NGLL3_PAD + t;
  const int g = active ? ibool[eo] : 0;
  if (t < NGLL2) s_hp[t] = gll[t];
  s_a[t] = active ? pot[g] : 0.f;
  s_b[t] = active ? b_pot[g] : 0.f;
  __syncthreads();
  if (!active) return;
  const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
  float da[3] = {0.f, 0.f, 0.f}, db[3] = {0.f, 0.f, 0.f};
#pragma unroll
  for (int l = 0; l < NGLLX; ++l) {
    const float h1 = s_hp[i + NGLLX * l], h2 = s_hp[j + NGLLX * l], h3 = s_hp[k + NGLLX * l];
    da[0] = fmaf(s_a[l + NGLLX * j + NGLL2 * k], h1, da[0]);
    da[1] = fmaf(s_a[i + NGLLX * l + NGLL2 * k], h2, da[1]);
    da[2] = fmaf(s_a[i + NGLLX * j + NGLL2 * l], h3, da[2]);
    db[0] = fmaf(s_b[l + NGLLX * j + NGLL2 * k], h1, db[0]);
    db[1] = fmaf(s_b[i + NGLLX * l + NGLL2 * k], h2, db[1]);
    db[2] = fmaf(s_b[i + NGLLX * j + NGLL2 * l], h3, db[2]);
  }
  float ga[3], gb[3];
  const int ir = irregular[e];
  if (ir >= 0) {
    const long mo = (long)ir * NGLL3_PAD + t;
    float mm[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) mm[q] = m.p[q][mo];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      ga[c] = mm[c] * da[0] + mm[3 + c] * da[1] + mm[6 + c] * da[2];
      gb[c] = mm[c] * db[0] + mm[3 + c] * db[1] + mm[6 + c] * db[2];
    }
  } else {
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      ga[c] = xix_regular * da[c];
      gb[c] = xix_regular * db[c];
    }
  }
  rho_kl[eo] += dt * ((double)ga[0] * gb[0] + (double)ga[1] * gb[1] + (double)ga[2] * gb[2]);
  kappa_kl[eo] += dt * ((double)s_a[t] * b_pot_dd[g]);
}

// chi_dd += jw (u . n)   (compute_coupling_acoustic_el.f90:70-150)
__global__ void coupling_ac_el_kernel(int nfaces, const int* __restrict__ cp_ispec, const int* __restrict__ cp_pt,
                                      const float* __restrict__ normal, const float* __restrict__ jw,
                                      const int* __restrict__ ibool, const float* __restrict__ displ, float sign,
                                      float* __restrict__ pot_dd) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)nfaces * NGLL2) return;
  const int g = ibool[(long)cp_ispec[idx / NGLL2] * NGLL3_PAD + cp_pt[idx]];
  const float dn = displ[3L * g] * normal[3 * idx] + displ[3L * g + 1] * normal[3 * idx + 1] +
                   displ[3L * g + 2] * normal[3 * idx + 2];
  atomicAdd(pot_dd + g, jw[idx] * (sign * dn));
}

// accel += jw n (-chi_dd)   (compute_coupling_viscoelastic_ac.f90:70-160)
__global__ void coupling_el_ac_kernel(int nfaces, const int* __restrict__ cp_ispec, const int* __restrict__ cp_pt,
                                      const float* __restrict__ normal, const float* __restrict__ jw,
                                      const int* __restrict__ ibool, const float* __restrict__ pot_dd, float sign,
                                      float* __restrict__ accel) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)nfaces * NGLL2) return;
  const int g = ibool[(long)cp_ispec[idx / NGLL2] * NGLL3_PAD + cp_pt[idx]];
  const float pr = sign * (-pot_dd[g]);
  const float w = jw[idx];
  atomicAdd(accel + 3L * g, w * normal[3 * idx] * pr);
  atomicAdd(accel + 3L * g + 1, w * normal[3 * idx + 1] * pr);
  atomicAdd(accel + 3L * g + 2, w * normal[3 * idx + 2] * pr);
}

// chi = chi_dot = chi_dd = 0 on the free surface of fluid elements
// (compute_forces_acoustic_calling_routine.f90:754-810)
__global__ void free_surface_kernel(int nfaces, const int* __restrict__ fs_ispec, const int* __restrict__ fs_pt,
                                    const int* __restrict__ is_acoustic, const int* __restrict__ ibool,
                                    float* __restrict__ pot, float* __restrict__ pot_dot, float* __restrict__ pot_dd) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)nfaces * NGLL2) return;
  const int e = fs_ispec[idx / NGLL2];
  if (!is_acoustic[e]) return;
  const int g = ibool[(long)e * NGLL3_PAD + fs_pt[idx]];
  pot[g] = 0.f;
  pot_dot[g] = 0.f;
  pot_dd[g] = 0.f;
}

// chi_dd -= sourcearray(1) stf / kappa for sources in fluid elements
// (compute_add_sources_acoustic.f90:100-126)
// stf from the per-call array, or from the whole-run table at the device step
// counter (stf_table != nullptr)
__global__ void sources_acoustic_kernel(int nsrc, const int* __restrict__ ispec_src, const int* __restrict__ is_acoustic,
                                        const float* __restrict__ sa, const float* __restrict__ stf,
                                        const int* __restrict__ ibool, const float* __restrict__ kappav,
                                        float* __restrict__ pot_dd, const float* __restrict__ stf_table,
                                        const int* __restrict__ d_it, int stf_nstep) {
  const int is = blockIdx.x, p = threadIdx.x;
  if (is >= nsrc || p >= NGLL3) return;
  const int e = ispec_src[is];
  if (e < 0 || !is_acoustic[e]) return;
  float f;
  if (stf_table) {
    const int it = *d_it;
    if (it < 1 || it > stf_nstep) return;
    f = stf_table[(long)(it - 1) * nsrc + is];
  } else {
    f = stf[is];
  }
  const long q = (long)e * NGLL3_PAD + p;
  atomicAdd(pot_dd + ibool[q], -(sa[((long)is * NGLL3_PAD + p) * 3] * f / kappav[q]));
}

__global__ void predictor_scalar_kernel(float* __restrict__ d, float* __restrict__ v, float* __restrict__ a, long n,
                                        float dt, float dt2, float dtsq2) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float ai = a[i], vi = v[i];
  d[i] = d[i] + dt * vi + dtsq2 * ai;
  v[i] = vi + dt2 * ai;
  a[i] = 0.f;
}

// predictor_scalar_kernel over four consecutive values per thread (16-byte
// accesses; d, v, a 16-byte aligned), thread n4 also taking the tail; n < 2^31
__global__ void predictor_scalar4_kernel(float* __restrict__ d, float* __restrict__ v, float* __restrict__ a, int n,
                                         float dt, float dt2, float dtsq2) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int n4 = n >> 2;
  if (q > n4) return;
  if (q == n4) {
    for (int i = 4 * n4; i < n; ++i) {
      const float ai = a[i], vi = v[i];
      d[i] = d[i] + dt * vi + dtsq2 * ai;
      v[i] = vi + dt2 * ai;
      a[i] = 0.f;
    }
    return;
  }
  const float4 a4 = reinterpret_cast<const float4*>(a)[q];
  float4 v4 = reinterpret_cast<const float4*>(v)[q];
  float4 d4 = reinterpret_cast<const float4*>(d)[q];
  d4.x = d4.x + dt * v4.x + dtsq2 * a4.x; v4.x = v4.x + dt2 * a4.x;
  d4.y = d4.y + dt * v4.y + dtsq2 * a4.y; v4.y = v4.y + dt2 * a4.y;
  d4.z = d4.z + dt * v4.z + dtsq2 * a4.z; v4.z = v4.z + dt2 * a4.z;
  d4.w = d4.w + dt * v4.w + dtsq2 * a4.w; v4.w = v4.w + dt2 * a4.w;
  reinterpret_cast<float4*>(d)[q] = d4;
  reinterpret_cast<float4*>(v)[q] = v4;
  reinterpret_cast<float4*>(a)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// mass_corrector_scalar_kernel over four consecutive values per thread (as above)
__global__ void mass_corrector_scalar4_kernel(float* __restrict__ v, float* __restrict__ a,
                                              const float* __restrict__ rmass, int n, float dt2) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int n4 = n >> 2;
  if (q > n4) return;
  if (q == n4) {
    for (int i = 4 * n4; i < n; ++i) {
      const float ai = a[i] * rmass[i];
      a[i] = ai;
      v[i] += dt2 * ai;
    }
    return;
  }
  float4 a4 = reinterpret_cast<const float4*>(a)[q];
  float4 v4 = reinterpret_cast<const float4*>(v)[q];
  const float4 r4 = reinterpret_cast<const float4*>(rmass)[q];
  a4.x *= r4.x; v4.x += dt2 * a4.x;
  a4.y *= r4.y; v4.y += dt2 * a4.y;
  a4.z *= r4.z; v4.z += dt2 * a4.z;
  a4.w *= r4.w; v4.w += dt2 * a4.w;
  reinterpret_cast<float4*>(a)[q] = a4;
  reinterpret_cast<float4*>(v)[q] = v4;
}

// kernel_3_acoustic: chi_dd *= rmass_acoustic; chi_dot += dt/2 chi_dd
__global__ void mass_corrector_scalar_kernel(float* __restrict__ v, float* __restrict__ a,
                                             const float* __restrict__ rmass, long n, float dt2) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float ai = a[i] * rmass[i];
  a[i] = ai;
  v[i] += dt2 * ai;
}

// acoustic Hessian kernels (compute_kernels.f90:459-510,
// kernels/compute_kernels_hess_ac_cudakernel.cu), gradients with the reference's
// 1/rho (g = grad / rho): hess_ac_kl += dt g(chi_adj_dd).g(b_chi_dd),
// hess_rho_ac_kl += dt rho |g(b_chi_dot)|^2, hess_kappa_ac_kl += dt b_chi_dot^2 / kappa;
// FP64 accumulators
__global__ void __launch_bounds__(NGLL3_PAD)
    kernels_hess_acoustic_kernel(long nspec, const int* __restrict__ is_acoustic, const int* __restrict__ ibool,
                                 const int* __restrict__ irregular, Metric9 m, const float* __restrict__ gll,
                                 float xix_regular, const float* __restrict__ rhostore,
                                 const float* __restrict__ kappav, const float* __restrict__ pot_dd,
                                 const float* __restrict__ b_pot_dot, const float* __restrict__ b_pot_dd, double dt,
                                 double* __restrict__ hess, double* __restrict__ hess_rho,
                                 double* __restrict__ hess_kappa) {
  __shared__ float s_f[3][NGLL3_PAD];
  __shared__ float s_hp[NGLL2];
  const long e = blockIdx.x;
  const int t = threadIdx.x;
  if (e >= nspec || !is_acoustic[e]) return;
  const bool active = t < NGLL3;
  const long eo = e * NGLL3_PAD + t;
  const int g = active ? ibool[eo] : 0;
  if (t < NGLL2) s_hp[t] = gll[t];
  s_f[0][t] = active ? pot_dd[g] : 0.f;
  s_f[1][t] = active ? b_pot_dd[g] : 0.f;
  s_f[2][t] = active ? b_pot_dot[g] : 0.f;
  __syncthreads();
  if (!active) return;
  const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
  const int ir = irregular[e];
  const float rinv = 1.f / rhostore[eo];
  float gr[3][3];
#pragma unroll
  for (int f = 0; f < 3; ++f) {
    float d0 = 0.f, d1 = 0.f, d2 = 0.f;
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) {
      d0 = fmaf(s_f[f][l + NGLLX * j + NGLL2 * k], s_hp[i + NGLLX * l], d0);
      d1 = fmaf(s_f[f][i + NGLLX * l + NGLL2 * k], s_hp[j + NGLLX * l], d1);
      d2 = fmaf(s_f[f][i + NGLLX * j + NGLL2 * l], s_hp[k + NGLLX * l], d2);
    }
    if (ir >= 0) {
      const long mo = (long)ir * NGLL3_PAD + t;
#pragma unroll
      for (int c = 0; c < 3; ++c) gr[f][c] = rinv * (m.p[c][mo] * d0 + m.p[3 + c][mo] * d1 + m.p[6 + c][mo] * d2);
    } else {
      gr[f][0] = rinv * xix_regular * d0;
      gr[f][1] = rinv * xix_regular * d1;
      gr[f][2] = rinv * xix_regular * d2;
    }
  }
  const double rho = (double)rhostore[eo];
  hess[eo] += dt * ((double)gr[0][0] * gr[1][0] + (double)gr[0][1] * gr[1][1] + (double)gr[0][2] * gr[1][2]);
  hess_rho[eo] += dt * rho * ((double)gr[2][0] * gr[2][0] + (double)gr[2][1] * gr[2][1] + (double)gr[2][2] * gr[2][2]);
  const double bv = (double)s_f[2][t];
  hess_kappa[eo] += dt * bv * bv / (double)kappav[eo];
}

}  // namespace

// pressure seismograms (compute_interpolated_dva.f90:280-300): p = - sum h chi_dd
__global__ void pressure_seismogram_kernel(int nrec, const int* __restrict__ ispec_rec,
                                           const int* __restrict__ rec_is_acoustic, const float* __restrict__ hx,
                                           const float* __restrict__ he, const float* __restrict__ hg,
                                           const int* __restrict__ ibool, const float* __restrict__ pot_dd,
                                           float* __restrict__ seismo_p, int slot, const int* __restrict__ d_it,
                                           int nlength) {
  __shared__ float red[4];
  const int r = blockIdx.x, t = threadIdx.x;
  float s = 0.f;
  if (r < nrec && t < NGLL3 && rec_is_acoustic[r]) {
    const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
    const float h = hx[5 * r + i] * he[5 * r + j] * hg[5 * r + k];
    s = -h * pot_dd[ibool[(long)ispec_rec[r] * NGLL3_PAD + t]];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((t & 31) == 0) red[t >> 5] = s;
  __syncthreads();
  if (t == 0 && r < nrec) {
    const int sl = d_it ? (*d_it - 1) % nlength : slot;
    seismo_p[r + (long)nrec * sl] = red[0] + red[1] + red[2] + red[3];
  }
}

void launch_pressure_seismograms(Mesh* mp, int slot) {
  if (!mp->d_seismo_p || mp->nrec_local == 0 || !mp->d_potential_dot_dot) return;
  pressure_seismogram_kernel<<<mp->nrec_local, NGLL3_PAD, 0, mp->stream>>>(
      mp->nrec_local, mp->d_ispec_rec, mp->d_rec_is_acoustic, mp->d_hxir, mp->d_hetar, mp->d_hgammar, mp->d_ibool,
      mp->d_potential_dot_dot, mp->d_seismo_p, slot, nullptr, 1);
}

// The fluid part of one fused step (compute_forces_acoustic_forward_calling,
// compute_forces_acoustic_calling_routine.f90:54-343, with the acoustic
// predictor of update_displacement_scheme.f90 in front): predictor, free
// surface, stiffness of both phases, Sommerfeld faces, coupling with the
// solid displacement, sources from the whole-run stf table at the device step
// counter, mass + corrector, free surface.  Returns the number of launches.
int enqueue_acoustic_step(Mesh* mp, float dt, float dt2, float dtsq2) {
  cudaStream_t s = mp->stream;
  int launches = 0;
  // the fluid elements' points only, when their span is known: the potentials
  // are zero at points of solid elements alone, and no kernel writes them there
  const long g0 = mp->ac_count >= 0 ? mp->ac_first : 0;
  const long n = mp->ac_count >= 0 ? mp->ac_count : mp->nglob;
  // 16-byte vectors where the span starts on a 16-byte boundary
  const bool vec = g0 % 4 == 0 && n < (1L << 31);
  if (vec)
    predictor_scalar4_kernel<<<nblk((n >> 2) + 1, 256), 256, 0, s>>>(mp->d_potential + g0, mp->d_potential_dot + g0,
                                                                      mp->d_potential_dot_dot + g0, (int)n, dt, dt2,
                                                                      dtsq2);
  else
    predictor_scalar_kernel<<<nblk(n, 256), 256, 0, s>>>(mp->d_potential + g0, mp->d_potential_dot + g0,
                                                          mp->d_potential_dot_dot + g0, n, dt, dt2, dtsq2);
  ++launches;
  const long nfs = (long)mp->num_free_surface_faces * NGLL2;
  if (nfs > 0) {
    free_surface_kernel<<<nblk(nfs, 128), 128, 0, s>>>(mp->num_free_surface_faces, mp->d_fs_ispec, mp->d_fs_pt,
                                                        mp->d_ispec_is_acoustic, mp->d_ibool, mp->d_potential,
                                                        mp->d_potential_dot, mp->d_potential_dot_dot);
    ++launches;
  }
  if (mp->nspec_outer_ac == 0 && mp->nspec_inner_ac == 0) {
    mp->nspec_outer_ac = mp->phase_valid_ac[0];
    mp->nspec_inner_ac = mp->phase_valid_ac[1];
  }
  for (int iphase = 1; iphase <= 2; ++iphase) {
    const int nel = iphase == 1 ? mp->nspec_outer_ac : mp->nspec_inner_ac;
    if (nel <= 0) continue;
    const int* ph = mp->d_phase_ispec_ac + (long)(iphase - 1) * mp->num_phase_ispec_ac;
    acoustic_stiffness_kernel<<<nel, NGLL3_PAD, 0, s>>>(
        nel, ph, mp->d_ibool, mp->d_irregular, mp->d_metric[0], mp->d_metric[1], mp->d_metric[2], mp->d_metric[3],
        mp->d_metric[4], mp->d_metric[5], mp->d_metric[6], mp->d_metric[7], mp->d_metric[8], mp->d_rhostore,
        mp->d_gll, mp->xix_regular, mp->jacobian_regular, mp->d_potential, mp->d_potential_dot_dot);
    ++launches;
  }
  if (mp->stacey && mp->num_abs_faces > 0) {
    const long nf = (long)mp->num_abs_faces * NGLL2;
    stacey_acoustic_kernel<<<nblk(nf, 128), 128, 0, s>>>(mp->num_abs_faces, mp->d_abs_ispec, mp->d_abs_pt,
                                                          mp->d_abs_jw, mp->d_ispec_is_acoustic, mp->d_ibool,
                                                          mp->d_rhostore, mp->d_kappav, mp->d_potential_dot,
                                                          mp->d_potential_dot_dot, nullptr);
    ++launches;
  }
  if (mp->num_coupling_faces > 0) {
    const long nc = (long)mp->num_coupling_faces * NGLL2;
    coupling_ac_el_kernel<<<nblk(nc, 128), 128, 0, s>>>(mp->num_coupling_faces, mp->d_cp_ispec, mp->d_cp_pt,
                                                         mp->d_cp_normal, mp->d_cp_jw, mp->d_ibool, mp->f.displ, 1.f,
                                                         mp->d_potential_dot_dot);
    ++launches;
  }
  if (mp->nsources > 0 && mp->d_stf_table) {
    sources_acoustic_kernel<<<mp->nsources, NGLL3_PAD, 0, s>>>(mp->nsources, mp->d_ispec_src, mp->d_ispec_is_acoustic,
                                                                mp->d_sourcearrays, nullptr, mp->d_ibool,
                                                                mp->d_kappav, mp->d_potential_dot_dot,
                                                                mp->d_stf_table, mp->d_it, mp->stf_nstep);
    ++launches;
  }
  if (vec)
    mass_corrector_scalar4_kernel<<<nblk((n >> 2) + 1, 256), 256, 0, s>>>(
        mp->d_potential_dot + g0, mp->d_potential_dot_dot + g0, mp->d_rmass_acoustic + g0, (int)n, dt2);
  else
    mass_corrector_scalar_kernel<<<nblk(n, 256), 256, 0, s>>>(mp->d_potential_dot + g0,
                                                              mp->d_potential_dot_dot + g0,
                                                              mp->d_rmass_acoustic + g0, n, dt2);
  ++launches;
  if (nfs > 0) {
    free_surface_kernel<<<nblk(nfs, 128), 128, 0, s>>>(mp->num_free_surface_faces, mp->d_fs_ispec, mp->d_fs_pt,
                                                        mp->d_ispec_is_acoustic, mp->d_ibool, mp->d_potential,
                                                        mp->d_potential_dot, mp->d_potential_dot_dot);
    ++launches;
  }
  return launches;
}

// the solid side of the coupling (compute_coupling_viscoelastic_ac.f90:28-140) and
// the pressure traces at the device step counter
int enqueue_coupling_el_ac(Mesh* mp) {
  if (mp->num_coupling_faces == 0) return 0;
  const long nc = (long)mp->num_coupling_faces * NGLL2;
  coupling_el_ac_kernel<<<nblk(nc, 128), 128, 0, mp->stream>>>(mp->num_coupling_faces, mp->d_cp_ispec, mp->d_cp_pt,
                                                                mp->d_cp_normal, mp->d_cp_jw, mp->d_ibool,
                                                                mp->d_potential_dot_dot, 1.f, mp->f.accel);
  return 1;
}

int enqueue_pressure_seismograms(Mesh* mp) {
  if (!mp->d_seismo_p || mp->nrec_local == 0 || !mp->d_potential_dot_dot || !mp->save_p) return 0;
  pressure_seismogram_kernel<<<mp->nrec_local, NGLL3_PAD, 0, mp->stream>>>(
      mp->nrec_local, mp->d_ispec_rec, mp->d_rec_is_acoustic, mp->d_hxir, mp->d_hetar, mp->d_hgammar, mp->d_ibool,
      mp->d_potential_dot_dot, mp->d_seismo_p, 0, mp->d_it, mp->nlength_seismogram);
  return 1;
}

bool launch_hess_acoustic(Mesh* mp, double dt) {
  if (!mp->d_hess_ac_kl[0]) return set_error(SF3D_ERR_STATE, "APPROXIMATE_HESS_KL was not prepared in fluid elements");
  Metric9 m;
  for (int q = 0; q < 9; ++q) m.p[q] = mp->d_metric[q];
  kernels_hess_acoustic_kernel<<<mp->nspec, NGLL3_PAD, 0, mp->stream>>>(
      mp->nspec, mp->d_ispec_is_acoustic, mp->d_ibool, mp->d_irregular, m, mp->d_gll, mp->xix_regular,
      mp->d_rhostore, mp->d_kappav, mp->d_potential_dot_dot, mp->d_b_potential_dot, mp->d_b_potential_dot_dot, dt,
      mp->d_hess_ac_kl[0], mp->d_hess_ac_kl[1], mp->d_hess_ac_kl[2]);
  return cuda_ok(cudaGetLastError(), "kernels_hess_acoustic_kernel");
}

}  // namespace sf3d

using namespace sf3d;

static bool copy_faces(const int* h_ispec, const int* h_ijk, int nf, long nspec, int** d_ispec, int** d_pt,
                       cudaStream_t s) {
  std::vector<int> isp(nf), pt((size_t)nf * NGLL2);
  for (int f = 0; f < nf; ++f) {
    isp[f] = h_ispec[f] - 1;
    if (isp[f] < 0 || isp[f] >= nspec) return set_error(SF3D_ERR_ARG, "face ispec out of range");
    for (int g = 0; g < NGLL2; ++g) {
      const int* ijk = h_ijk + 3 * (g + NGLL2 * f);
      for (int c = 0; c < 3; ++c)
        if (ijk[c] < 1 || ijk[c] > 5) return set_error(SF3D_ERR_ARG, "face ijk out of range");
      pt[(size_t)f * NGLL2 + g] = (ijk[0] - 1) + NGLLX * (ijk[1] - 1) + NGLL2 * (ijk[2] - 1);
    }
  }
  return alloc_zero((void**)d_ispec, sizeof(int) * nf) &&
         copy_sync(*d_ispec, isp.data(), sizeof(int) * nf, cudaMemcpyHostToDevice, s) &&
         alloc_zero((void**)d_pt, sizeof(int) * pt.size()) &&
         copy_sync(*d_pt, pt.data(), sizeof(int) * pt.size(), cudaMemcpyHostToDevice, s);
}

extern "C" {

void prepare_fields_acoustic_device_(long* Mesh_pointer, realw* rmass_acoustic, realw* rhostore, realw* kappastore,
                                     int* num_phase_ispec_acoustic, int* phase_ispec_inner_acoustic,
                                     int* NOISE_TOMOGRAPHY, int* num_free_surface_faces, int* free_surface_ispec,
                                     int* free_surface_ijk, int* b_reclen_potential, realw* b_absorb_potential,
                                     int* ELASTIC_SIMULATION, int* num_coupling_ac_el_faces,
                                     int* coupling_ac_el_ispec, int* coupling_ac_el_ijk,
                                     realw* coupling_ac_el_normal, realw* coupling_ac_el_jacobian2Dw,
                                     int* num_colors_outer_acoustic, int* num_colors_inner_acoustic,
                                     int* num_elem_colors_acoustic) {
  (void)b_reclen_potential; (void)b_absorb_potential; (void)num_colors_outer_acoustic;
  (void)num_colors_inner_acoustic; (void)num_elem_colors_acoustic;
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (NOISE_TOMOGRAPHY && *NOISE_TOMOGRAPHY) { set_error(SF3D_ERR_ARG, "noise tomography is not supported"); return; }
  if (!mp->d_ispec_is_acoustic) { set_error(SF3D_ERR_STATE, "ispec_is_acoustic not given to prepare_constants_device"); return; }
  const long nspec = mp->nspec, nglob = mp->nglob;
  cudaStream_t s = mp->stream;
  bool ok = alloc_zero((void**)&mp->d_potential, sizeof(float) * nglob) &&
            alloc_zero((void**)&mp->d_potential_dot, sizeof(float) * nglob) &&
            alloc_zero((void**)&mp->d_potential_dot_dot, sizeof(float) * nglob) &&
            alloc_zero((void**)&mp->d_rmass_acoustic, sizeof(float) * nglob) &&
            copy_sync(mp->d_rmass_acoustic, rmass_acoustic, sizeof(float) * nglob, cudaMemcpyHostToDevice, s);
  ok = ok && upload_padded(&mp->d_rhostore, rhostore, nspec, s);
  if (ok && !mp->d_kappav) ok = upload_padded(&mp->d_kappav, kappastore, nspec, s);
  mp->num_phase_ispec_ac = *num_phase_ispec_acoustic;
  if (ok && mp->num_phase_ispec_ac > 0) {
    std::vector<int> ph((size_t)2 * mp->num_phase_ispec_ac);
    for (size_t q = 0; q < ph.size() && ok; ++q) {
      ph[q] = phase_ispec_inner_acoustic[q] - 1;
      if (ph[q] >= nspec) ok = set_error(SF3D_ERR_ARG, "phase_ispec_inner_acoustic out of range");
    }
    for (int c = 0; c < 2; ++c) {
      int n = 0;
      while (n < mp->num_phase_ispec_ac && ph[(size_t)c * mp->num_phase_ispec_ac + n] >= 0) ++n;
      mp->phase_valid_ac[c] = n;
    }
    ok = ok && alloc_zero((void**)&mp->d_phase_ispec_ac, sizeof(int) * ph.size()) &&
         copy_sync(mp->d_phase_ispec_ac, ph.data(), sizeof(int) * ph.size(), cudaMemcpyHostToDevice, s);
  }
  mp->num_free_surface_faces = *num_free_surface_faces;
  if (ok && mp->num_free_surface_faces > 0)
    ok = copy_faces(free_surface_ispec, free_surface_ijk, mp->num_free_surface_faces, nspec, &mp->d_fs_ispec,
                    &mp->d_fs_pt, s);
  mp->num_coupling_faces = (ELASTIC_SIMULATION && *ELASTIC_SIMULATION) ? *num_coupling_ac_el_faces : 0;
  if (ok && mp->num_coupling_faces > 0) {
    const int nf = mp->num_coupling_faces;
    ok = copy_faces(coupling_ac_el_ispec, coupling_ac_el_ijk, nf, nspec, &mp->d_cp_ispec, &mp->d_cp_pt, s) &&
         alloc_zero((void**)&mp->d_cp_normal, sizeof(float) * 3 * NGLL2 * nf) &&
         copy_sync(mp->d_cp_normal, coupling_ac_el_normal, sizeof(float) * 3 * NGLL2 * nf, cudaMemcpyHostToDevice,
                   s) &&
         alloc_zero((void**)&mp->d_cp_jw, sizeof(float) * NGLL2 * nf) &&
         copy_sync(mp->d_cp_jw, coupling_ac_el_jacobian2Dw, sizeof(float) * NGLL2 * nf, cudaMemcpyHostToDevice, s);
  }
  mp->has_acoustic = ok ? 1 : 0;
}

void compute_forces_acoustic_cuda_(long* Mesh_pointer, int* iphase, int* nspec_outer_acoustic,
                                   int* nspec_inner_acoustic, int* FORWARD_OR_ADJOINT_f) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!mp->has_acoustic) { set_error(SF3D_ERR_STATE, "prepare_fields_acoustic_device not called"); return; }
  AcField F;
  if (!ac_field(mp, FORWARD_OR_ADJOINT_f, &F)) return;
  mp->nspec_outer_ac = *nspec_outer_acoustic;
  mp->nspec_inner_ac = *nspec_inner_acoustic;
  const int nel = *iphase == 1 ? mp->nspec_outer_ac : mp->nspec_inner_ac;
  if (*iphase != 1 && *iphase != 2) { set_error(SF3D_ERR_ARG, "iphase must be 1 or 2"); return; }
  if (nel < 0 || nel > mp->phase_valid_ac[*iphase - 1]) {
    set_error(SF3D_ERR_ARG, "nspec_outer/inner_acoustic exceeds the phase element lists");
    return;
  }
  if (nel == 0) return;
  const int* ph = mp->d_phase_ispec_ac + (long)(*iphase - 1) * mp->num_phase_ispec_ac;
  acoustic_stiffness_kernel<<<nel, NGLL3_PAD, 0, mp->stream>>>(
      nel, ph, mp->d_ibool, mp->d_irregular, mp->d_metric[0], mp->d_metric[1], mp->d_metric[2], mp->d_metric[3],
      mp->d_metric[4], mp->d_metric[5], mp->d_metric[6], mp->d_metric[7], mp->d_metric[8], mp->d_rhostore, mp->d_gll,
      mp->xix_regular, mp->jacobian_regular, F.p, F.pdd);
  cuda_ok(cudaGetLastError(), "acoustic_stiffness_kernel");
}

void acoustic_enforce_free_surf_cuda_(long* Mesh_pointer, int* ABSORB_INSTEAD_OF_FREE_SURFACE,
                                      int* FORWARD_OR_ADJOINT) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || !mp->has_acoustic) return;
  AcField F;
  if (!ac_field(mp, FORWARD_OR_ADJOINT, &F)) return;
  if (*ABSORB_INSTEAD_OF_FREE_SURFACE || mp->num_free_surface_faces == 0) return;
  const long n = (long)mp->num_free_surface_faces * NGLL2;
  free_surface_kernel<<<nblk(n, 128), 128, 0, mp->stream>>>(mp->num_free_surface_faces, mp->d_fs_ispec, mp->d_fs_pt,
                                                             mp->d_ispec_is_acoustic, mp->d_ibool, F.p, F.pd, F.pdd);
  cuda_ok(cudaGetLastError(), "free_surface_kernel");
}

void update_displacement_ac_cuda_(long* Mesh_pointer, realw* deltat_F, realw* deltatover2_F, realw* deltatsqover2_F,
                                  int* FORWARD_OR_ADJOINT) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || !mp->has_acoustic) return;
  AcField F;
  if (!ac_field(mp, FORWARD_OR_ADJOINT, &F)) return;
  const long n = mp->nglob;
  predictor_scalar_kernel<<<nblk(n, 256), 256, 0, mp->stream>>>(F.p, F.pd, F.pdd, n, *deltat_F, *deltatover2_F,
                                                                *deltatsqover2_F);
  cuda_ok(cudaGetLastError(), "predictor_scalar_kernel");
}

void kernel_3_acoustic_cuda_(long* Mesh_pointer, realw* deltatover2_F, realw* b_deltatover2_F,
                             int* FORWARD_OR_ADJOINT_f) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || !mp->has_acoustic) return;
  AcField F;
  if (!ac_field(mp, FORWARD_OR_ADJOINT_f, &F)) return;
  const float dt2 = *FORWARD_OR_ADJOINT_f == 3 ? *b_deltatover2_F : *deltatover2_F;
  const long n = mp->nglob;
  mass_corrector_scalar_kernel<<<nblk(n, 256), 256, 0, mp->stream>>>(F.pd, F.pdd, mp->d_rmass_acoustic, n, dt2);
  cuda_ok(cudaGetLastError(), "mass_corrector_scalar_kernel");
}

void compute_stacey_acoustic_cuda_(long* Mesh_pointer, int* iphasef, realw* h_b_absorb_potential,
                                   int* FORWARD_OR_ADJOINT_f) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || !mp->has_acoustic) return;
  AcField F;
  if (!ac_field(mp, FORWARD_OR_ADJOINT_f, &F)) return;
  if (*iphasef != 1 || !mp->stacey || mp->num_abs_faces == 0) return;
  const long n = (long)mp->num_abs_faces * NGLL2;
  const bool backward = *FORWARD_OR_ADJOINT_f == 3;
  if (backward && h_b_absorb_potential && mp->simulation_type == 3) {
    // replay of b_absorb_potential stored by the SAVE_FORWARD run
    if (!ensure_stage(mp, sizeof(float) * n)) return;
    SF3D_CUDA(cudaMemcpyAsync(mp->d_stage, h_b_absorb_potential, sizeof(float) * n, cudaMemcpyHostToDevice,
                              mp->stream));
    stacey_acoustic_replay_kernel<<<nblk(n, 128), 128, 0, mp->stream>>>(mp->num_abs_faces, mp->d_abs_ispec,
                                                                         mp->d_abs_pt, mp->d_ispec_is_acoustic,
                                                                         mp->d_ibool, mp->d_stage, F.pdd);
    cuda_ok(cudaGetLastError(), "stacey_acoustic_replay_kernel");
    return;
  }
  // forward, adjoint, or a recomputed backward field (undo attenuation)
  const bool store = !backward && mp->save_forward && mp->simulation_type == 1 && h_b_absorb_potential;
  if (store && !ensure_stage(mp, sizeof(float) * n)) return;
  if (store) SF3D_CUDA(cudaMemsetAsync(mp->d_stage, 0, sizeof(float) * n, mp->stream));
  stacey_acoustic_kernel<<<nblk(n, 128), 128, 0, mp->stream>>>(mp->num_abs_faces, mp->d_abs_ispec, mp->d_abs_pt,
                                                                mp->d_abs_jw, mp->d_ispec_is_acoustic, mp->d_ibool,
                                                                mp->d_rhostore, mp->d_kappav, F.pd, F.pdd,
                                                                store ? mp->d_stage : nullptr);
  if (!cuda_ok(cudaGetLastError(), "stacey_acoustic_kernel")) return;
  if (store) {
    SF3D_CUDA(cudaMemcpyAsync(h_b_absorb_potential, mp->d_stage, sizeof(float) * n, cudaMemcpyDeviceToHost,
                              mp->stream));
    SF3D_CUDA(cudaStreamSynchronize(mp->stream));
  }
}

void compute_coupling_ac_el_cuda_(long* Mesh_pointer, int* iphasef, int* num_coupling_ac_el_facesf,
                                  int* FORWARD_OR_ADJOINT) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || !mp->has_acoustic) return;
  if (*iphasef != 1 || mp->num_coupling_faces == 0) return;
  if (*num_coupling_ac_el_facesf != mp->num_coupling_faces) { set_error(SF3D_ERR_ARG, "coupling face count mismatch"); return; }
  AcField F;
  if (!ac_field(mp, FORWARD_OR_ADJOINT, &F)) return;
  const float* displ = *FORWARD_OR_ADJOINT == 3 ? mp->b.displ : mp->f.displ;
  if (!displ) { set_error(SF3D_ERR_STATE, "backward elastic field not allocated"); return; }
  const float sign = (mp->simulation_type != 1 && *FORWARD_OR_ADJOINT == 1) ? -1.f : 1.f;
  const long n = (long)mp->num_coupling_faces * NGLL2;
  coupling_ac_el_kernel<<<nblk(n, 128), 128, 0, mp->stream>>>(mp->num_coupling_faces, mp->d_cp_ispec, mp->d_cp_pt,
                                                               mp->d_cp_normal, mp->d_cp_jw, mp->d_ibool, displ,
                                                               sign, F.pdd);
  cuda_ok(cudaGetLastError(), "coupling_ac_el_kernel");
}

void compute_coupling_el_ac_cuda_(long* Mesh_pointer, int* iphasef, int* num_coupling_ac_el_facesf,
                                  int* FORWARD_OR_ADJOINT) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || !mp->has_acoustic) return;
  if (*iphasef != 1 || mp->num_coupling_faces == 0) return;
  if (*num_coupling_ac_el_facesf != mp->num_coupling_faces) { set_error(SF3D_ERR_ARG, "coupling face count mismatch"); return; }
  AcField F;
  if (!ac_field(mp, FORWARD_OR_ADJOINT, &F)) return;
  float* accel = *FORWARD_OR_ADJOINT == 3 ? mp->b.accel : mp->f.accel;
  if (!accel) { set_error(SF3D_ERR_STATE, "backward elastic field not allocated"); return; }
  const float sign = (mp->simulation_type != 1 && *FORWARD_OR_ADJOINT == 1) ? -1.f : 1.f;
  const long n = (long)mp->num_coupling_faces * NGLL2;
  coupling_el_ac_kernel<<<nblk(n, 128), 128, 0, mp->stream>>>(mp->num_coupling_faces, mp->d_cp_ispec, mp->d_cp_pt,
                                                               mp->d_cp_normal, mp->d_cp_jw, mp->d_ibool, F.pdd, sign,
                                                               accel);
  cuda_ok(cudaGetLastError(), "coupling_el_ac_kernel");
}

void compute_add_sources_ac_cuda_(long* Mesh_pointer, int* NSOURCESf, double* h_stf_pre_compute,
                                  int* run_number_of_the_source) {
  (void)run_number_of_the_source;
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || !mp->has_acoustic) return;
  if (mp->nsources_local == 0 || mp->nsources == 0) return;
  if (*NSOURCESf != mp->nsources) { set_error(SF3D_ERR_ARG, "NSOURCES mismatch"); return; }
  std::vector<float> stf(mp->nsources);
  for (int i = 0; i < mp->nsources; ++i) stf[i] = (float)h_stf_pre_compute[i];
  SF3D_CUDA(cudaMemcpyAsync(mp->d_stf_step, stf.data(), sizeof(float) * mp->nsources, cudaMemcpyHostToDevice,
                            mp->stream));
  sources_acoustic_kernel<<<mp->nsources, NGLL3_PAD, 0, mp->stream>>>(mp->nsources, mp->d_ispec_src,
                                                                      mp->d_ispec_is_acoustic, mp->d_sourcearrays,
                                                                      mp->d_stf_step, mp->d_ibool, mp->d_kappav,
                                                                      mp->d_potential_dot_dot, nullptr, nullptr, 0);
  SF3D_CUDA(cudaStreamSynchronize(mp->stream));
  cuda_ok(cudaGetLastError(), "sources_acoustic_kernel");
}

static void xfer_ac(int* size, realw* a, realw* b, realw* c, long* Mesh_pointer, bool to_device,
                    int fa = 1) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!mp->has_acoustic) { set_error(SF3D_ERR_STATE, "acoustic fields not allocated"); return; }
  if (!size || *size != mp->nglob) { set_error(SF3D_ERR_ARG, "acoustic transfer size must be NGLOB_AB"); return; }
  AcField F;
  if (!ac_field(mp, &fa, &F)) return;
  float* d[3] = {F.p, F.pd, F.pdd};
  realw* h[3] = {a, b, c};
  for (int q = 0; q < 3; ++q) {
    if (!h[q]) continue;
    if (to_device)
      SF3D_CUDA(cudaMemcpyAsync(d[q], h[q], sizeof(float) * mp->nglob, cudaMemcpyHostToDevice, mp->stream));
    else
      SF3D_CUDA(cudaMemcpyAsync(h[q], d[q], sizeof(float) * mp->nglob, cudaMemcpyDeviceToHost, mp->stream));
  }
  SF3D_CUDA(cudaStreamSynchronize(mp->stream));
}

void transfer_fields_ac_to_device_(int* size, realw* potential_acoustic, realw* potential_dot_acoustic,
                                   realw* potential_dot_dot_acoustic, long* Mesh_pointer) {
  xfer_ac(size, potential_acoustic, potential_dot_acoustic, potential_dot_dot_acoustic, Mesh_pointer, true);
}

void transfer_fields_ac_from_device_(int* size, realw* potential_acoustic, realw* potential_dot_acoustic,
                                     realw* potential_dot_dot_acoustic, long* Mesh_pointer) {
  xfer_ac(size, potential_acoustic, potential_dot_acoustic, potential_dot_dot_acoustic, Mesh_pointer, false);
}


// ---------------------------------------------------------------- SIMULATION_TYPE = 3 in fluid elements
// prepare_fields_acoustic_adj_dev (prepare_mesh_constants_cuda.cu): backward
// potentials and the rho / kappa kernel accumulators
void prepare_fields_acoustic_adj_dev_(long* Mesh_pointer, int* APPROXIMATE_HESS_KL) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!mp->has_acoustic) { set_error(SF3D_ERR_STATE, "prepare_fields_acoustic_device not called"); return; }
  const long nglob = mp->nglob, nk = (long)NGLL3_PAD * mp->nspec;
  // each array is allocated where it is still missing, so a repeated call after a
  // failed allocation completes the set instead of leaving later pointers null
  bool ok = true;
  float** pot[3] = {&mp->d_b_potential, &mp->d_b_potential_dot, &mp->d_b_potential_dot_dot};
  for (int q = 0; q < 3 && ok; ++q)
    if (!*pot[q]) ok = alloc_zero((void**)pot[q], sizeof(float) * nglob);
  double** kl[2] = {&mp->d_rho_ac_kl, &mp->d_kappa_ac_kl};
  for (int q = 0; q < 2 && ok; ++q)
    if (!*kl[q]) ok = alloc_zero((void**)kl[q], sizeof(double) * nk);
  // a repeated call may add the Hessian accumulators
  for (int q = 0; q < 3 && ok && APPROXIMATE_HESS_KL && *APPROXIMATE_HESS_KL && !mp->d_hess_ac_kl[q]; ++q)
    ok = alloc_zero((void**)&mp->d_hess_ac_kl[q], sizeof(double) * nk);
}

// transfer_kernels_hess_ac_tohost (transfer_fields_cuda.cu): (5,5,5,NSPEC) each, FP32
void transfer_kernels_hess_ac_tohost_(long* Mesh_pointer, realw* h_hess_ac_kl, realw* h_hess_rho_ac_kl,
                                      realw* h_hess_kappa_ac_kl, int* NSPEC_AB) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!NSPEC_AB || *NSPEC_AB != mp->nspec) { set_error(SF3D_ERR_ARG, "NSPEC_AB mismatch"); return; }
  if (!mp->d_hess_ac_kl[0]) { set_error(SF3D_ERR_STATE, "APPROXIMATE_HESS_KL was not prepared in fluid elements"); return; }
  const size_t nk = (size_t)NGLL3_PAD * mp->nspec;
  std::vector<double> tmp(nk);
  realw* h[3] = {h_hess_ac_kl, h_hess_rho_ac_kl, h_hess_kappa_ac_kl};
  for (int q = 0; q < 3; ++q) {
    if (!copy_sync(tmp.data(), mp->d_hess_ac_kl[q], sizeof(double) * nk, cudaMemcpyDeviceToHost, mp->stream)) return;
    for (long e = 0; e < mp->nspec; ++e)
      for (int p = 0; p < NGLL3; ++p) h[q][(size_t)NGLL3 * e + p] = (float)tmp[(size_t)NGLL3_PAD * e + p];
  }
}

// compute_add_sources_ac_s3_cuda (compute_add_sources_acoustic_cuda.cu): the
// sources on the backward potentials, stf at the caller's time
void compute_add_sources_ac_s3_cuda_(long* Mesh_pointer, int* NSOURCESf, double* h_stf_pre_compute,
                                     int* run_number_of_the_source) {
  (void)run_number_of_the_source;
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || !mp->has_acoustic) return;
  if (!ac_adj_ready(mp)) { set_error(SF3D_ERR_STATE, "prepare_fields_acoustic_adj_dev not called"); return; }
  if (mp->nsources_local == 0 || mp->nsources == 0) return;
  if (*NSOURCESf != mp->nsources) { set_error(SF3D_ERR_ARG, "NSOURCES mismatch"); return; }
  std::vector<float> stf(mp->nsources);
  for (int i = 0; i < mp->nsources; ++i) stf[i] = (float)h_stf_pre_compute[i];
  SF3D_CUDA(cudaMemcpyAsync(mp->d_stf_step, stf.data(), sizeof(float) * mp->nsources, cudaMemcpyHostToDevice,
                            mp->stream));
  sources_acoustic_kernel<<<mp->nsources, NGLL3_PAD, 0, mp->stream>>>(mp->nsources, mp->d_ispec_src,
                                                                      mp->d_ispec_is_acoustic, mp->d_sourcearrays,
                                                                      mp->d_stf_step, mp->d_ibool, mp->d_kappav,
                                                                      mp->d_b_potential_dot_dot, nullptr, nullptr, 0);
  SF3D_CUDA(cudaStreamSynchronize(mp->stream));
  cuda_ok(cudaGetLastError(), "sources_acoustic_kernel(b)");
}

// compute_kernels_acoustic_cuda (compute_kernels_cuda.cu)
void compute_kernels_acoustic_cuda_(long* Mesh_pointer, realw* deltat_f) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!ac_adj_ready(mp)) { set_error(SF3D_ERR_STATE, "prepare_fields_acoustic_adj_dev not called"); return; }
  Metric9 m;
  for (int q = 0; q < 9; ++q) m.p[q] = mp->d_metric[q];
  kernels_acoustic_kernel<<<mp->nspec, NGLL3_PAD, 0, mp->stream>>>(
      mp->nspec, mp->d_ispec_is_acoustic, mp->d_ibool, mp->d_irregular, m, mp->d_gll, mp->xix_regular,
      mp->ac_kernel_discrete ? mp->d_potential_dot_dot : mp->d_potential, mp->d_b_potential,
      mp->d_b_potential_dot_dot, (double)*deltat_f, mp->d_rho_ac_kl,
      mp->d_kappa_ac_kl);
  cuda_ok(cudaGetLastError(), "kernels_acoustic_kernel");
}

static bool ac_kernels_to_host(Mesh* mp, double* h_rho, double* h_kappa, float* f_rho, float* f_kappa) {
  if (!mp->d_rho_ac_kl || !mp->d_kappa_ac_kl) return set_error(SF3D_ERR_STATE, "acoustic kernels not allocated");
  const size_t nk = (size_t)NGLL3_PAD * mp->nspec;
  std::vector<double> tmp(nk);
  const double* d[2] = {mp->d_rho_ac_kl, mp->d_kappa_ac_kl};
  double* hd[2] = {h_rho, h_kappa};
  float* hf[2] = {f_rho, f_kappa};
  for (int q = 0; q < 2; ++q) {
    if (!copy_sync(tmp.data(), d[q], sizeof(double) * nk, cudaMemcpyDeviceToHost, mp->stream)) return false;
    for (long e = 0; e < mp->nspec; ++e)
      for (int p = 0; p < NGLL3; ++p) {
        const double v = tmp[(size_t)NGLL3_PAD * e + p];
        if (hd[q]) hd[q][(size_t)NGLL3 * e + p] = v;
        if (hf[q]) hf[q][(size_t)NGLL3 * e + p] = (float)v;
      }
  }
  return true;
}

// transfer_kernels_ac_to_host (transfer_fields_cuda.cu): rho_ac_kl, kappa_ac_kl (5,5,5,NSPEC)
void transfer_kernels_ac_to_host_(long* Mesh_pointer, realw* h_rho_ac_kl, realw* h_kappa_ac_kl, int* NSPEC_AB) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!NSPEC_AB || *NSPEC_AB != mp->nspec) { set_error(SF3D_ERR_ARG, "NSPEC_AB mismatch"); return; }
  ac_kernels_to_host(mp, nullptr, nullptr, h_rho_ac_kl, h_kappa_ac_kl);
}

// Fluid kernel pairing (library extension): 0 (default) the reference's formula
// with the adjoint potential chi_adj; 1 the adjoint chi_adj_dd, which gives the
// discrete derivative of the misfit (the reference's adjoint potential of the
// fluid is the second time integral of the discrete adjoint variable)
int sf3d_set_acoustic_kernel_pairing(long* Mesh_pointer, int discrete) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (discrete != 0 && discrete != 1) {
    set_error(SF3D_ERR_ARG, "sf3d_set_acoustic_kernel_pairing: 0 or 1");
    return SF3D_ERR_ARG;
  }
  mp->ac_kernel_discrete = discrete;
  return SF3D_OK;
}

// FP64 read-back of the acoustic accumulators (library extension)
int sf3d_get_kernels_ac_f64(long* Mesh_pointer, double* h_rho_ac_kl, double* h_kappa_ac_kl) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  return ac_kernels_to_host(mp, h_rho_ac_kl, h_kappa_ac_kl, nullptr, nullptr) ? SF3D_OK : SF3D_ERR_STATE;
}

// single-field transfers of the backward potentials (transfer_fields_cuda.cu)
void transfer_b_fields_ac_to_device_(int* size, realw* b_potential_acoustic, realw* b_potential_dot_acoustic,
                                     realw* b_potential_dot_dot_acoustic, long* Mesh_pointer) {
  xfer_ac(size, b_potential_acoustic, b_potential_dot_acoustic, b_potential_dot_dot_acoustic, Mesh_pointer, true, 3);
}
void transfer_b_fields_ac_from_device_(int* size, realw* b_potential_acoustic, realw* b_potential_dot_acoustic,
                                       realw* b_potential_dot_dot_acoustic, long* Mesh_pointer) {
  xfer_ac(size, b_potential_acoustic, b_potential_dot_acoustic, b_potential_dot_dot_acoustic, Mesh_pointer, false, 3);
}
void transfer_b_potential_ac_from_device_(int* size, realw* b_potential_acoustic, long* Mesh_pointer) {
  xfer_ac(size, b_potential_acoustic, nullptr, nullptr, Mesh_pointer, false, 3);
}
void transfer_b_potential_ac_to_device_(int* size, realw* b_potential_acoustic, long* Mesh_pointer) {
  xfer_ac(size, b_potential_acoustic, nullptr, nullptr, Mesh_pointer, true, 3);
}
void transfer_b_potential_dot_dot_ac_from_device_(int* size, realw* b_potential_dot_dot_acoustic, long* Mesh_pointer) {
  xfer_ac(size, nullptr, nullptr, b_potential_dot_dot_acoustic, Mesh_pointer, false, 3);
}
void transfer_b_potential_dot_dot_ac_to_device_(int* size, realw* b_potential_dot_dot_acoustic, long* Mesh_pointer) {
  xfer_ac(size, nullptr, nullptr, b_potential_dot_dot_acoustic, Mesh_pointer, true, 3);
}
void transfer_b_dot_dot_from_device_(int* size, realw* b_potential_dot_dot_acoustic, long* Mesh_pointer) {
  xfer_ac(size, nullptr, nullptr, b_potential_dot_dot_acoustic, Mesh_pointer, false, 3);
}

}  // extern "C"
