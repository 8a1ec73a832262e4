// C-PML absorbing layers on the device (sm_103a), forward field.
//
// The reference's GPU C-PML (src/gpu/pml_compute_accel_cuda.cu,
// kernels/pml_kernel_2_viscoelastic_impl.cu, kernels/UpdateDispVeloc_kernel.cu,
// kernels/pml_impose_boundary_condition_cuda_kernel.cu) follows the CPU solver's
// compute_forces_viscoelastic_PML (compute_forces_viscoelastic.F90:969-1400),
// pml_compute_memory_variables_elastic (pml_compute_memory_variables.f90) and
// pml_compute_accel_contribution_elastic (pml_compute_accel_contribution.f90):
//   * around the predictor, PML_displ_old / _new = u + dt/2 (1 - 2 theta) v +
//     dt^2/2 (1 - theta) a of the fields before and after it (theta = 1/8);
//   * for every CPML element, the gradients of u, PML_displ_old and _new; the
//     recursive convolution memory variables of the 21 strain terms updated with
//     the alpha / beta coefficients and combined with the strain coefficients
//     into a non-symmetric stress; the memory variables of the displacement
//     updated and combined with the A-bar coefficients into the layer's
//     acceleration term rho J w (A1 v + A2 u + A3 r_x + A4 r_y + A5 r_z); the
//     weighted transposed contractions of the non-symmetric stress and the
//     scatter-add of -(sum + acceleration term);
//   * Dirichlet condition on the layers' outer faces: u, v, a and the stored
//     predictions set to zero there, after the forces.
// The regular stiffness kernel skips the CPML elements (its phase lists are
// filtered at set-up); the backward field of SIMULATION_TYPE = 3 is not
// supported with C-PML, as in the reference's GPU code.
//
// Device layout (coalesced 512-byte rows, as the other element streams):
//   coefficients [cpml element][41][128]: alpha 0-8 (x, y, z: coef0, 1, 2), beta
//     9-17, A-bar 18-22 (A1..A5), strain 23-40 (A6..A23);
//   memory variables [cpml element][48][128]: rows 3n+q (n = 0..8) the three
//     convolutions q of dux_dxl_x, duy_dxl_y, duz_dxl_z, dux_dyl_x, duy_dyl_y,
//     duz_dyl_z, dux_dzl_x, duy_dzl_y, duz_dzl_z; rows 27-38 the single ones
//     (duz_dzl_y, duz_dyl_y, duy_dzl_z, duy_dyl_z with alpha_x; duz_dzl_x,
//     duz_dxl_x, dux_dzl_z, dux_dxl_z with alpha_y; duy_dyl_x, duy_dxl_x,
//     dux_dyl_y, dux_dxl_y with alpha_z); rows 39 + 3d + c the displacement
//     convolutions (component c, coefficient set d).
#include <string.h>

#include <vector>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

constexpr int kPmlCoefRows = 41;
constexpr int kPmlMemRows = 48;
constexpr float kTheta = 0.125f;

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

__global__ void pml_displ_kernel(const float* __restrict__ d, const float* __restrict__ v,
                                 const float* __restrict__ a, float* __restrict__ out, int ncpml,
                                 const int* __restrict__ cpml_to_spec, const int* __restrict__ ibool, float dt2,
                                 float dtsq2) {
  const int ec = blockIdx.x, t = threadIdx.x;
  if (ec >= ncpml || t >= NGLL3) return;
  const long g = ibool[(long)cpml_to_spec[ec] * NGLL3_PAD + t];
#pragma unroll
  for (int c = 0; c < 3; ++c)
    out[((long)ec * 3 + c) * NGLL3_PAD + t] =
        d[3 * g + c] + dt2 * (1.0f - 2.0f * kTheta) * v[3 * g + c] + dtsq2 * (1.0f - kTheta) * a[3 * g + c];
}

struct PmlArgs {
  int nelem;
  const int* list;               // CPML elements of the phase (0-based)
  const int* spec_to_cpml;
  const int* ibool;
  const int* irregular;
  const float* m[9];
  const float* kappav;
  const float* muv;
  const float* rho;
  const float* gll;
  const float* wgll_cube;
  float xix_regular, jacobian_regular;
  const float* displ;
  const float* veloc;
  float* accel;
  const float* pold;
  const float* pnew;
  const float* coef;
  float* rmem;
  float* eps[5];                 // epsilondev xx yy xy xz yz (COMPUTE_AND_STORE_STRAIN) or null
  int* err;                      // kernel error word (a bounded wait that timed out)
};

// gradient in the reference cube of the three components of s (3 x 128 values)
__device__ __forceinline__ void ref_grad(const float (*s)[NGLL3_PAD], const float* hp, int i, int j, int k,
                                         float T[3][3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) T[c][0] = T[c][1] = T[c][2] = 0.f;
#pragma unroll
  for (int l = 0; l < NGLLX; ++l) {
    const float h1 = hp[i + NGLLX * l], h2 = hp[j + NGLLX * l], h3 = hp[k + NGLLX * l];
    const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      T[c][0] = fmaf(s[c][p1], h1, T[c][0]);
      T[c][1] = fmaf(s[c][p2], h2, T[c][1]);
      T[c][2] = fmaf(s[c][p3], h3, T[c][2]);
    }
  }
}

// the same for two fields stored side by side (float2 .x, .y), one shared load
// per neighbour for both; each output is the FMA chain of ref_grad
__device__ __forceinline__ void ref_grad_pair(const float2 (*s)[NGLL3_PAD], const float* hp, int i, int j, int k,
                                              float T[3][3], float U[3][3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) T[c][0] = T[c][1] = T[c][2] = U[c][0] = U[c][1] = U[c][2] = 0.f;
#pragma unroll
  for (int l = 0; l < NGLLX; ++l) {
    const float h1 = hp[i + NGLLX * l], h2 = hp[j + NGLLX * l], h3 = hp[k + NGLLX * l];
    const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float2 q1 = s[c][p1], q2 = s[c][p2], q3 = s[c][p3];
      T[c][0] = fmaf(q1.x, h1, T[c][0]);
      T[c][1] = fmaf(q2.x, h2, T[c][1]);
      T[c][2] = fmaf(q3.x, h3, T[c][2]);
      U[c][0] = fmaf(q1.y, h1, U[c][0]);
      U[c][1] = fmaf(q2.y, h2, U[c][1]);
      U[c][2] = fmaf(q3.y, h3, U[c][2]);
    }
  }
}

// physical gradient D[c][x] = d u_c / d x from the reference-cube gradient
__device__ __forceinline__ void phys_grad(const float T[3][3], const float* m, int ir, float xr, float D[3][3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    if (ir >= 0) {
#pragma unroll
      for (int x = 0; x < 3; ++x) D[c][x] = m[x] * T[c][0] + m[3 + x] * T[c][1] + m[6 + x] * T[c][2];
    } else {
#pragma unroll
      for (int x = 0; x < 3; ++x) D[c][x] = xr * T[c][x];
    }
  }
}

// dynamic shared memory of pml_stiffness_kernel: the element's coefficient rows
// and convolution memory variables
constexpr size_t kPmlStageBytes = sizeof(float) * (kPmlCoefRows + kPmlMemRows) * NGLL3_PAD;

// one CTA per CPML element of the phase, thread p < 125 owns GLL point p.  The
// element's 41 coefficient rows and 48 memory-variable rows are contiguous in
// HBM ([cpml][41][128], [cpml][48][128]): thread 0 brings them into shared
// memory with two bulk copies on one mbarrier while the CTA gathers the fields,
// and every thread waits for them (bounded; error word on timeout) before the
// convolutions.  The updated memory variables go back with coalesced stores.
__global__ void __launch_bounds__(NGLL3_PAD) pml_stiffness_kernel(const PmlArgs a) {
  extern __shared__ __align__(16) float s_stage[];
  float* s_cf = s_stage;                              // [41][128]
  float* s_rm = s_stage + kPmlCoefRows * NGLL3_PAD;   // [48][128]
  __shared__ uint64_t s_bar;
  bool bulk_failed = false;
  __shared__ float s_gll[NGLL3];
  __shared__ float s_u[3][NGLL3_PAD];
  __shared__ __align__(8) float2 s_on[3][NGLL3_PAD];   // PML displacement predictions (old, new)
  __shared__ float s_t[9][NGLL3_PAD];
  const int t = threadIdx.x;
  const int e = __ldg(a.list + blockIdx.x);
  const int ec = __ldg(a.spec_to_cpml + e);
  const bool active = t < NGLL3;
  const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
  const long eo = (long)e * NGLL3_PAD + t;
  const long co = (long)ec * kPmlCoefRows * NGLL3_PAD + t;
  const long mo = (long)ec * kPmlMemRows * NGLL3_PAD + t;
  const long po = (long)ec * 3 * NGLL3_PAD + t;
  const int ir = __ldg(a.irregular + e);
  long g = 0;
  float vel[3] = {0.f, 0.f, 0.f};
  if (t == 0) {
    mbar_init(&s_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    mbar_arrive_expect_tx(&s_bar, (uint32_t)kPmlStageBytes);
    bulk_g2s(s_cf, a.coef + (long)ec * kPmlCoefRows * NGLL3_PAD, kPmlCoefRows * NGLL3_PAD * sizeof(float), &s_bar);
    bulk_g2s(s_rm, a.rmem + (long)ec * kPmlMemRows * NGLL3_PAD, kPmlMemRows * NGLL3_PAD * sizeof(float), &s_bar);
  }
  if (active) {
    s_gll[t] = __ldg(a.gll + t);
    g = __ldg(a.ibool + eo);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      s_u[c][t] = a.displ[3 * g + c];
      vel[c] = a.veloc[3 * g + c];
      s_on[c][t] = make_float2(a.pold[po + c * NGLL3_PAD], a.pnew[po + c * NGLL3_PAD]);
    }
  }
  __syncthreads();
  if (active) {
    float m[9];
    float jac = a.jacobian_regular;
#pragma unroll
    for (int q = 0; q < 9; ++q) m[q] = 0.f;
    if (ir >= 0) {
#pragma unroll
      for (int q = 0; q < 9; ++q) m[q] = __ldg(a.m[q] + (long)ir * NGLL3_PAD + t);
      jac = 1.f / (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                   m[2] * (m[3] * m[7] - m[4] * m[6]));
    }
    const float xr = a.xix_regular;
    float T[3][3], U[3][3], du[3][3], dold[3][3], dnew[3][3];
    ref_grad(s_u, s_gll, i, j, k, T);
    phys_grad(T, m, ir, xr, du);
    ref_grad_pair(s_on, s_gll, i, j, k, T, U);
    phys_grad(T, m, ir, xr, dold);
    phys_grad(U, m, ir, xr, dnew);
    if (a.eps[0]) {
      // deviatoric strain of u (kept for kernels as the reference does for PML elements)
      const float templ = (1.f / 3.f) * (du[0][0] + du[1][1] + du[2][2]);
      a.eps[0][eo] = du[0][0] - templ;
      a.eps[1][eo] = du[1][1] - templ;
      a.eps[2][eo] = 0.5f * (du[0][1] + du[1][0]);
      a.eps[3][eo] = 0.5f * (du[2][0] + du[0][2]);
      a.eps[4][eo] = 0.5f * (du[2][1] + du[1][2]);
    }
    if (!mbar_wait_bounded(&s_bar, 0)) {
      bulk_failed = true;  // this element's results are not valid; the host is told
      if (a.err) atomicExch(a.err, 1);
    }
#define CF(r) s_cf[(r) * NGLL3_PAD + t]
#define RM(r) s_rm[(r) * NGLL3_PAD + t]
    // convolution memory variables: r <- c0 r + new c1 + old c2
    auto upd = [&](int row, int set_row, float vnew, float vold) {
      float& r = RM(row);
      r = CF(set_row) * r + vnew * CF(set_row + 1) + vold * CF(set_row + 2);
    };
    // the three convolutions of the derivatives along x (sets alpha_z, alpha_y,
    // beta_x), along y (alpha_x, alpha_z, beta_y), along z (alpha_x, alpha_y, beta_z)
    const int set3[3][3] = {{6, 3, 9}, {0, 6, 12}, {0, 3, 15}};
#pragma unroll
    for (int x = 0; x < 3; ++x)
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int q = 0; q < 3; ++q) upd(3 * (3 * x + c) + q, set3[x][q], dnew[c][x], dold[c][x]);
    // single convolutions: alpha_x, alpha_y, alpha_z
    upd(27, 0, dnew[2][2], dold[2][2]);
    upd(28, 0, dnew[2][1], dold[2][1]);
    upd(29, 0, dnew[1][2], dold[1][2]);
    upd(30, 0, dnew[1][1], dold[1][1]);
    upd(31, 3, dnew[2][2], dold[2][2]);
    upd(32, 3, dnew[2][0], dold[2][0]);
    upd(33, 3, dnew[0][2], dold[0][2]);
    upd(34, 3, dnew[0][0], dold[0][0]);
    upd(35, 6, dnew[1][1], dold[1][1]);
    upd(36, 6, dnew[1][0], dold[1][0]);
    upd(37, 6, dnew[0][1], dold[0][1]);
    upd(38, 6, dnew[0][0], dold[0][0]);
    float A[18];
#pragma unroll
    for (int q = 0; q < 18; ++q) A[q] = CF(23 + q);   // A6 .. A23
    // derivative combinations: along x (A6..A9), y (A10..A13), z (A14..A17)
    auto tri = [&](int x, int c) {
      const int n = 3 * x + c;
      return A[4 * x] * du[c][x] + A[4 * x + 1] * RM(3 * n) + A[4 * x + 2] * RM(3 * n + 1) +
             A[4 * x + 3] * RM(3 * n + 2);
    };
    const float duxdxl_x = tri(0, 0), duxdyl_x = tri(1, 0), duxdzl_x = tri(2, 0);
    const float duzdzl_x = A[14] * du[2][2] + A[15] * RM(31);
    const float duzdxl_x = A[14] * du[2][0] + A[15] * RM(32);
    const float duydyl_x = A[16] * du[1][1] + A[17] * RM(35);
    const float duydxl_x = A[16] * du[1][0] + A[17] * RM(36);
    const float duydxl_y = tri(0, 1), duydyl_y = tri(1, 1), duydzl_y = tri(2, 1);
    const float duzdzl_y = A[12] * du[2][2] + A[13] * RM(27);
    const float duzdyl_y = A[12] * du[2][1] + A[13] * RM(28);
    const float duxdyl_y = A[16] * du[0][1] + A[17] * RM(37);
    const float duxdxl_y = A[16] * du[0][0] + A[17] * RM(38);
    const float duzdxl_z = tri(0, 2), duzdyl_z = tri(1, 2), duzdzl_z = tri(2, 2);
    const float duydzl_z = A[12] * du[1][2] + A[13] * RM(29);
    const float duydyl_z = A[12] * du[1][1] + A[13] * RM(30);
    const float duxdzl_z = A[14] * du[0][2] + A[15] * RM(33);
    const float duxdxl_z = A[14] * du[0][0] + A[15] * RM(34);
    const float kap = __ldg(a.kappav + eo), mu = __ldg(a.muv + eo);
    const float l2m = kap + 4.0f / 3.0f * mu;
    const float lam = l2m - 2.0f * mu;
    const float sxx = l2m * duxdxl_x + lam * duydyl_x + lam * duzdzl_x;
    const float syx = mu * duxdyl_x + mu * duydxl_x;
    const float szx = mu * duzdxl_x + mu * duxdzl_x;
    const float sxy = mu * duxdyl_y + mu * duydxl_y;
    const float syy = lam * duxdxl_y + l2m * duydyl_y + lam * duzdzl_y;
    const float szy = mu * duzdyl_y + mu * duydzl_y;
    const float sxz = mu * duzdxl_z + mu * duxdzl_z;
    const float syz = mu * duzdyl_z + mu * duydzl_z;
    const float szz = lam * duxdxl_z + lam * duydyl_z + l2m * duzdzl_z;
    // displacement convolutions and the layer's acceleration term
    float rd[3][3];
#pragma unroll
    for (int d = 0; d < 3; ++d)
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float& r = RM(39 + 3 * d + c);
        r = CF(3 * d) * r + s_on[c][t].y * CF(3 * d + 1) + s_on[c][t].x * CF(3 * d + 2);
        rd[c][d] = r;
      }
    const float wrj = __ldg(a.wgll_cube + t) * __ldg(a.rho + eo) * jac;
    const float A1 = CF(18), A2 = CF(19), A3 = CF(20), A4 = CF(21), A5 = CF(22);
    float acc[3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
      acc[c] = wrj * (A1 * vel[c] + A2 * s_u[c][t] + A3 * rd[c][0] + A4 * rd[c][1] + A5 * rd[c][2]);
    // the updated memory variables back to HBM (coalesced rows)
#pragma unroll 8
    for (int r = 0; r < kPmlMemRows; ++r) a.rmem[mo + (long)r * NGLL3_PAD] = RM(r);
#undef CF
#undef RM
    // non-symmetric stress dotted with the rows of the metric (get_dot_product)
    if (ir >= 0) {
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        const float Dx = m[3 * d], Dy = m[3 * d + 1], Dz = m[3 * d + 2];
        s_t[3 * d][t] = jac * (sxx * Dx + syx * Dy + szx * Dz);
        s_t[3 * d + 1][t] = jac * (sxy * Dx + syy * Dy + szy * Dz);
        s_t[3 * d + 2][t] = jac * (sxz * Dx + syz * Dy + szz * Dz);
      }
    } else {
      const float jr = a.jacobian_regular;
      s_t[0][t] = jr * (sxx * xr); s_t[1][t] = jr * (sxy * xr); s_t[2][t] = jr * (sxz * xr);
      s_t[3][t] = jr * (syx * xr); s_t[4][t] = jr * (syy * xr); s_t[5][t] = jr * (syz * xr);
      s_t[6][t] = jr * (szx * xr); s_t[7][t] = jr * (szy * xr); s_t[8][t] = jr * (szz * xr);
    }
    vel[0] = acc[0];
    vel[1] = acc[1];
    vel[2] = acc[2];
  }
  __syncthreads();
  if (active) {
    const float* hpw = s_gll + NGLL2;
    float n[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c) n[c][0] = n[c][1] = n[c][2] = 0.f;
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) {
      const float f1 = hpw[l + NGLLX * i], f2 = hpw[l + NGLLX * j], f3 = hpw[l + NGLLX * k];
      const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        n[c][0] = fmaf(s_t[c][p1], f1, n[c][0]);
        n[c][1] = fmaf(s_t[3 + c][p2], f2, n[c][1]);
        n[c][2] = fmaf(s_t[6 + c][p3], f3, n[c][2]);
      }
    }
    const float fac1 = s_gll[4 * NGLL2 + j + NGLLX * k];
    const float fac2 = s_gll[3 * NGLL2 + i + NGLLX * k];
    const float fac3 = s_gll[2 * NGLL2 + i + NGLLX * j];
#pragma unroll
    for (int c = 0; c < 3; ++c)
      atomicAdd(a.accel + 3 * g + c, -(fac1 * n[c][0] + fac2 * n[c][1] + fac3 * n[c][2] + vel[c]));
  }
  // a bulk copy still in flight must land before the CTA's shared memory is
  // released: wait once more, with the same bound
  if (bulk_failed) mbar_wait_bounded(&s_bar, 0);
}

__global__ void pml_boundary_kernel(int nfaces, const int* __restrict__ abs_ispec, const int* __restrict__ abs_pt,
                                    const int* __restrict__ ibool, const int* __restrict__ is_acoustic,
                                    const int* __restrict__ is_cpml, const int* __restrict__ spec_to_cpml,
                                    float* __restrict__ d, float* __restrict__ v, float* __restrict__ a,
                                    float* __restrict__ pold, float* __restrict__ pnew) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)nfaces * NGLL2) return;
  const int f = (int)(idx / NGLL2);
  const int e = abs_ispec[f];
  if ((is_acoustic && is_acoustic[e]) || !is_cpml[e]) return;
  const int p = abs_pt[idx];
  const long g = ibool[(long)e * NGLL3_PAD + p];
  const long po = (long)spec_to_cpml[e] * 3 * NGLL3_PAD + p;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    d[3 * g + c] = 0.f;
    v[3 * g + c] = 0.f;
    a[3 * g + c] = 0.f;
    pold[po + c * NGLL3_PAD] = 0.f;
    pnew[po + c * NGLL3_PAD] = 0.f;
  }
}

}  // namespace

void launch_pml_displ(Mesh* mp, bool after_predictor, float dt2, float dtsq2, cudaStream_t s) {
  if (!mp->pml || mp->nspec_cpml == 0) return;
  pml_displ_kernel<<<mp->nspec_cpml, NGLL3_PAD, 0, s>>>(mp->f.displ, mp->f.veloc, mp->f.accel,
                                                         after_predictor ? mp->d_pml_displ_new : mp->d_pml_displ_old,
                                                         mp->nspec_cpml, mp->d_cpml_to_spec, mp->d_ibool, dt2, dtsq2);
}

int launch_pml_stiffness(Mesh* mp, int iphase, bool strain, cudaStream_t s) {
  if (!mp->pml || mp->nspec_cpml == 0) return 0;
  PmlArgs a;
  memset(&a, 0, sizeof(a));
  a.nelem = mp->phase_pml_n[iphase - 1];
  if (a.nelem <= 0) return 0;
  a.list = mp->d_phase_pml + (long)(iphase - 1) * mp->num_phase_ispec;
  a.spec_to_cpml = mp->d_spec_to_cpml;
  a.ibool = mp->d_ibool;
  a.irregular = mp->d_irregular;
  for (int q = 0; q < 9; ++q) a.m[q] = mp->d_metric[q];
  a.kappav = mp->d_kappav;
  a.muv = mp->d_muv;
  a.rho = mp->d_rhostore;
  a.gll = mp->d_gll;
  a.wgll_cube = mp->d_wgll_cube;
  a.xix_regular = mp->xix_regular;
  a.jacobian_regular = mp->jacobian_regular;
  a.displ = mp->f.displ;
  a.veloc = mp->f.veloc;
  a.accel = mp->f.accel;
  a.pold = mp->d_pml_displ_old;
  a.pnew = mp->d_pml_displ_new;
  a.coef = mp->d_pml_coef;
  a.rmem = mp->d_pml_rmem;
  a.err = mp->d_kerr;
  if (strain)
    for (int c = 0; c < 5; ++c) a.eps[c] = mp->f.eps[c];
  static bool configured = false;  // opt in to > 48 KB of shared memory once
  if (!configured) {
    if (!cuda_ok(cudaFuncSetAttribute(pml_stiffness_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)kPmlStageBytes),
                 "cudaFuncSetAttribute(pml_stiffness_kernel)"))
      return 0;
    configured = true;
  }
  pml_stiffness_kernel<<<a.nelem, NGLL3_PAD, kPmlStageBytes, s>>>(a);
  return 1;
}

void launch_pml_boundary(Mesh* mp, cudaStream_t s) {
  if (!mp->pml || mp->nspec_cpml == 0 || mp->num_abs_faces == 0) return;
  const long n = (long)mp->num_abs_faces * NGLL2;
  pml_boundary_kernel<<<nblk(n, 128), 128, 0, s>>>(mp->num_abs_faces, mp->d_abs_ispec, mp->d_abs_pt, mp->d_ibool,
                                                   mp->d_ispec_is_acoustic, mp->d_is_cpml, mp->d_spec_to_cpml,
                                                   mp->f.displ, mp->f.veloc, mp->f.accel, mp->d_pml_displ_old,
                                                   mp->d_pml_displ_new);
}

void free_pml(Mesh* mp) {
  cudaFree(mp->d_is_cpml); cudaFree(mp->d_spec_to_cpml); cudaFree(mp->d_cpml_to_spec);
  cudaFree(mp->d_pml_coef); cudaFree(mp->d_pml_rmem); cudaFree(mp->d_pml_displ_old); cudaFree(mp->d_pml_displ_new);
  cudaFree(mp->d_wgll_cube); cudaFree(mp->d_phase_nopml); cudaFree(mp->d_phase_pml);
  mp->d_is_cpml = mp->d_spec_to_cpml = mp->d_cpml_to_spec = nullptr;
  mp->d_pml_coef = mp->d_pml_rmem = mp->d_pml_displ_old = mp->d_pml_displ_new = mp->d_wgll_cube = nullptr;
  mp->d_phase_nopml = mp->d_phase_pml = nullptr;
  mp->pml = 0;
  mp->nspec_cpml = 0;
}

}  // namespace sf3d

using namespace sf3d;

extern "C" {

// prepare_fields_elastic_pml (prepare_mesh_constants_cuda.cu; arguments as the
// reference's stub list): is_CPML (NSPEC) logical, CPML_to_spec (NSPEC_CPML)
// 1-based, spec_to_CPML (NSPEC) 1-based, pml_convolution_coef_alpha / _beta
// (9,5,5,5,NSPEC_CPML), _abar (5,...), _strain (18,...), wgll_cube (5,5,5),
// rhostore (5,5,5,NSPEC).
void prepare_fields_elastic_pml_(long* Mesh_pointer, int* NSPEC_CPML, int* is_CPML, int* CPML_to_spec,
                                 int* spec_to_CPML, realw* pml_convolution_coef_alpha, realw* pml_convolution_coef_beta,
                                 realw* pml_convolution_coef_abar, realw* pml_convolution_coef_strain,
                                 realw* h_wgll_cube, realw* rhostore) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!NSPEC_CPML || *NSPEC_CPML < 0 || (*NSPEC_CPML > 0 && (!is_CPML || !CPML_to_spec || !spec_to_CPML ||
                                                            !pml_convolution_coef_alpha || !pml_convolution_coef_beta ||
                                                            !pml_convolution_coef_abar || !pml_convolution_coef_strain ||
                                                            !h_wgll_cube || !rhostore))) {
    set_error(SF3D_ERR_ARG, "prepare_fields_elastic_pml: invalid arguments");
    return;
  }
  if (!mp->f.displ || !mp->d_phase_ispec) {
    set_error(SF3D_ERR_STATE, "prepare_fields_elastic_pml: prepare_fields_elastic_device not called");
    return;
  }
  if (mp->simulation_type == 3 || mp->use_mesh_coloring || mp->anisotropy || mp->attenuation) {
    // the reference's GPU C-PML covers the isotropic elastic forward field only
    set_error(SF3D_ERR_UNSUPPORTED, "prepare_fields_elastic_pml: C-PML on the GPU supports isotropic elastic "
                                    "forward runs without attenuation or mesh colouring");
    return;
  }
  free_pml(mp);
  const int ncpml = *NSPEC_CPML;
  const long nspec = mp->nspec;
  mp->nspec_cpml = ncpml;
  if (ncpml == 0) return;
  std::vector<int> isc(nspec), s2c(nspec, -1), c2s(ncpml);
  for (long e = 0; e < nspec; ++e) isc[e] = is_CPML[e] ? 1 : 0;
  for (int q = 0; q < ncpml; ++q) {
    const int e = CPML_to_spec[q] - 1;
    if (e < 0 || e >= nspec || !isc[e] || spec_to_CPML[e] != q + 1) {
      set_error(SF3D_ERR_ARG, "prepare_fields_elastic_pml: CPML_to_spec / spec_to_CPML / is_CPML disagree");
      return;
    }
    c2s[q] = e;
    s2c[e] = q;
  }
  // coefficient rows [cpml][41][128] from the Fortran (n,5,5,5,NSPEC_CPML) arrays
  std::vector<float> coef((size_t)ncpml * kPmlCoefRows * NGLL3_PAD, 0.f);
  const realw* src[4] = {pml_convolution_coef_alpha, pml_convolution_coef_beta, pml_convolution_coef_abar,
                         pml_convolution_coef_strain};
  const int nrow[4] = {9, 9, 5, 18}, row0[4] = {0, 9, 18, 23};
  for (int s = 0; s < 4; ++s)
    for (long ec = 0; ec < ncpml; ++ec)
      for (int p = 0; p < NGLL3; ++p)
        for (int r = 0; r < nrow[s]; ++r)
          coef[((size_t)ec * kPmlCoefRows + row0[s] + r) * NGLL3_PAD + p] =
              src[s][r + (size_t)nrow[s] * (p + (size_t)NGLL3 * ec)];
  // phase lists split into the regular and the CPML elements
  const int nph = mp->num_phase_ispec;
  std::vector<int> ph((size_t)2 * nph), nop((size_t)2 * nph, 0), pml((size_t)2 * nph, 0);
  float wc[NGLL3_PAD] = {};
  for (int p = 0; p < NGLL3; ++p) wc[p] = h_wgll_cube[p];
  bool ok = copy_sync(ph.data(), mp->d_phase_ispec, sizeof(int) * 2 * nph, cudaMemcpyDeviceToHost, mp->stream);
  for (int c = 0; ok && c < 2; ++c) {
    int a = 0, b = 0;
    for (int q = 0; q < mp->phase_valid[c]; ++q) {
      const int e = ph[(size_t)c * nph + q];
      if (isc[e]) pml[(size_t)c * nph + b++] = e;
      else nop[(size_t)c * nph + a++] = e;
    }
    mp->phase_nopml_n[c] = a;
    mp->phase_pml_n[c] = b;
  }
  ok = ok && alloc_zero((void**)&mp->d_is_cpml, sizeof(int) * nspec) &&
       alloc_zero((void**)&mp->d_spec_to_cpml, sizeof(int) * nspec) &&
       alloc_zero((void**)&mp->d_cpml_to_spec, sizeof(int) * ncpml) &&
       alloc_zero((void**)&mp->d_pml_coef, sizeof(float) * coef.size()) &&
       alloc_zero((void**)&mp->d_pml_rmem, sizeof(float) * (size_t)ncpml * kPmlMemRows * NGLL3_PAD) &&
       alloc_zero((void**)&mp->d_pml_displ_old, sizeof(float) * (size_t)ncpml * 3 * NGLL3_PAD) &&
       alloc_zero((void**)&mp->d_pml_displ_new, sizeof(float) * (size_t)ncpml * 3 * NGLL3_PAD) &&
       alloc_zero((void**)&mp->d_wgll_cube, sizeof(float) * NGLL3_PAD) &&
       alloc_zero((void**)&mp->d_phase_nopml, sizeof(int) * 2 * nph) &&
       alloc_zero((void**)&mp->d_phase_pml, sizeof(int) * 2 * nph);
  ok = ok && copy_sync(mp->d_is_cpml, isc.data(), sizeof(int) * nspec, cudaMemcpyHostToDevice, mp->stream) &&
       copy_sync(mp->d_spec_to_cpml, s2c.data(), sizeof(int) * nspec, cudaMemcpyHostToDevice, mp->stream) &&
       copy_sync(mp->d_cpml_to_spec, c2s.data(), sizeof(int) * ncpml, cudaMemcpyHostToDevice, mp->stream) &&
       copy_sync(mp->d_pml_coef, coef.data(), sizeof(float) * coef.size(), cudaMemcpyHostToDevice, mp->stream) &&
       copy_sync(mp->d_wgll_cube, wc, sizeof(wc), cudaMemcpyHostToDevice, mp->stream) &&
       copy_sync(mp->d_phase_nopml, nop.data(), sizeof(int) * 2 * nph, cudaMemcpyHostToDevice, mp->stream) &&
       copy_sync(mp->d_phase_pml, pml.data(), sizeof(int) * 2 * nph, cudaMemcpyHostToDevice, mp->stream);
  if (ok && !mp->d_rhostore) ok = upload_padded(&mp->d_rhostore, rhostore, nspec, mp->stream);
  if (!ok) {
    free_pml(mp);
    return;
  }
  mp->pml = 1;
}

// pml_impose_boundary_condition_elastic_cuda (pml_compute_accel_cuda.cu:245):
// zero u, v, a and the stored predictions on the outer faces of the layers
void pml_impose_boundary_condition_elastic_cuda_(long* Mesh_pointer) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  launch_pml_boundary(mp, mp->stream);
  cuda_ok(cudaGetLastError(), "pml_boundary_kernel");
}

static void xfer_pml(int* size, realw* old_h, realw* new_h, long* Mesh_pointer, bool to_device) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!mp->pml) { set_error(SF3D_ERR_STATE, "prepare_fields_elastic_pml not called"); return; }
  const long n = 3L * NGLL3 * mp->nspec_cpml;
  if (!size || *size != n || !old_h || !new_h) {
    set_error(SF3D_ERR_ARG, "transfer_pml_displ: size must be 3*125*NSPEC_CPML");
    return;
  }
  // host (3,5,5,5,NSPEC_CPML) <-> device [cpml][3][128]
  std::vector<float> tmp((size_t)mp->nspec_cpml * 3 * NGLL3_PAD, 0.f);
  realw* h[2] = {old_h, new_h};
  float* d[2] = {mp->d_pml_displ_old, mp->d_pml_displ_new};
  for (int q = 0; q < 2; ++q) {
    if (to_device) {
      for (long ec = 0; ec < mp->nspec_cpml; ++ec)
        for (int p = 0; p < NGLL3; ++p)
          for (int c = 0; c < 3; ++c) tmp[((size_t)ec * 3 + c) * NGLL3_PAD + p] = h[q][c + 3 * (p + (size_t)NGLL3 * ec)];
      if (!copy_sync(d[q], tmp.data(), sizeof(float) * tmp.size(), cudaMemcpyHostToDevice, mp->stream)) return;
    } else {
      if (!copy_sync(tmp.data(), d[q], sizeof(float) * tmp.size(), cudaMemcpyDeviceToHost, mp->stream)) return;
      for (long ec = 0; ec < mp->nspec_cpml; ++ec)
        for (int p = 0; p < NGLL3; ++p)
          for (int c = 0; c < 3; ++c) h[q][c + 3 * (p + (size_t)NGLL3 * ec)] = tmp[((size_t)ec * 3 + c) * NGLL3_PAD + p];
    }
  }
}

void transfer_pml_displ_from_device_(int* size, realw* PML_displ_old, realw* PML_displ_new, long* Mesh_pointer) {
  xfer_pml(size, PML_displ_old, PML_displ_new, Mesh_pointer, false);
}

void transfer_pml_displ_to_device_(int* size, realw* PML_displ_old, realw* PML_displ_new, long* Mesh_pointer) {
  xfer_pml(size, PML_displ_old, PML_displ_new, Mesh_pointer, true);
}

}  // extern "C"
