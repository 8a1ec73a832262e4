// Adjoint (SIMULATION_TYPE = 3) building blocks: backward-field preparation,
// adjoint sources at the receivers, element strain of a field, and the
// rho / mu / kappa sensitivity-kernel accumulation.
//
// Replaces prepare_fields_elastic_adj_dev / prepare_sim2_or_3_const_device
// (prepare_mesh_constants_cuda.cu:999, :1306), add_sources_el_sim_type_2_or_3
// (compute_add_sources_viscoelastic_cuda.cu:224), compute_strain_cuda
// (compute_strain_cuda.cu) and compute_kernels_elastic_cuda
// (compute_kernels_cuda.cu:39).  The kernels are accumulated in FP64 (the
// reference accumulates in CUSTOM_REAL); transfer_kernels_el_to_host rounds them
// to the reference's single-precision arrays.
#include <vector>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

struct Ptrs10 {
  const float* p[10];
};

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

// accel += source_adjoint(:, irec, it_index) * h_xi h_eta h_gamma
// (kernels/add_sources_el_SIM_TYPE_2_OR_3_kernel.cu:31-70)
__global__ void adjoint_sources_kernel(int nadj, const int* __restrict__ ispec, const float* __restrict__ hx,
                                       const float* __restrict__ he, const float* __restrict__ hg,
                                       const float* __restrict__ src, int it_index, const int* __restrict__ ibool,
                                       const int* __restrict__ is_acoustic, float* __restrict__ accel) {
  const int r = blockIdx.x, t = threadIdx.x;
  if (r >= nadj || t >= NGLL3) return;
  if (is_acoustic && is_acoustic[ispec[r]]) return;  // elastic receivers only
  const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
  const float h = hx[5 * r + i] * he[5 * r + j] * hg[5 * r + k];
  const int g = ibool[(long)ispec[r] * NGLL3_PAD + t];
  const float* s = src + 3L * (r + (long)nadj * it_index);
  atomicAdd(accel + 3L * g, s[0] * h);
  atomicAdd(accel + 3L * g + 1, s[1] * h);
  atomicAdd(accel + 3L * g + 2, s[2] * h);
}

// adjoint sources of receivers in fluid elements: the first component into
// potential_dot_dot (kernels/add_sources_ac_SIM_TYPE_2_OR_3_kernel.cu:31-85)
__global__ void adjoint_sources_ac_kernel(int nadj, const int* __restrict__ ispec, const float* __restrict__ hx,
                                          const float* __restrict__ he, const float* __restrict__ hg,
                                          const float* __restrict__ src, int it_index, const int* __restrict__ ibool,
                                          const int* __restrict__ is_acoustic, float* __restrict__ pot_dd) {
  const int r = blockIdx.x, t = threadIdx.x;
  if (r >= nadj || t >= NGLL3 || !is_acoustic[ispec[r]]) return;
  const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
  const float h = hx[5 * r + i] * he[5 * r + j] * hg[5 * r + k];
  atomicAdd(pot_dd + ibool[(long)ispec[r] * NGLL3_PAD + t], src[3L * (r + (long)nadj * it_index)] * h);
}

// deviatoric strain and trace/3 of a displacement field per element
// (compute_forces_viscoelastic.F90:495-568 without attenuation;
// kernels/compute_element_strain_cudakernel.cu)
__global__ void element_strain_kernel(const int* __restrict__ ibool, const int* __restrict__ irregular,
                                      const Ptrs10 m, const float* __restrict__ gll,
                                      float xix_regular, const float* __restrict__ displ, float* eps0, float* eps1,
                                      float* eps2, float* eps3, float* eps4, float* trace_over_3,
                                      float* trace) {
  __shared__ float s_u[3][NGLL3_PAD];
  __shared__ float s_hp[NGLL2];
  const int e = blockIdx.x, t = threadIdx.x;
  const bool active = t < NGLL3;
  const long eo = (long)e * NGLL3_PAD + t;
  if (t < NGLL2) s_hp[t] = gll[t];
  int g = active ? ibool[eo] : 0;
  s_u[0][t] = active ? displ[3L * g] : 0.f;
  s_u[1][t] = active ? displ[3L * g + 1] : 0.f;
  s_u[2][t] = active ? displ[3L * g + 2] : 0.f;
  __syncthreads();
  if (!active) return;
  const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
  float d[3][3];
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    float t1 = 0.f, t2 = 0.f, t3 = 0.f;
#pragma unroll
    for (int l = 0; l < NGLLX; ++l) {
      t1 = fmaf(s_u[c][l + NGLLX * j + NGLL2 * k], s_hp[i + NGLLX * l], t1);
      t2 = fmaf(s_u[c][i + NGLLX * l + NGLL2 * k], s_hp[j + NGLLX * l], t2);
      t3 = fmaf(s_u[c][i + NGLLX * j + NGLL2 * l], s_hp[k + NGLLX * l], t3);
    }
    const int ir = irregular[e];
    if (ir >= 0) {
      const long mo = (long)ir * NGLL3_PAD + t;
      d[c][0] = m.p[0][mo] * t1 + m.p[3][mo] * t2 + m.p[6][mo] * t3;
      d[c][1] = m.p[1][mo] * t1 + m.p[4][mo] * t2 + m.p[7][mo] * t3;
      d[c][2] = m.p[2][mo] * t1 + m.p[5][mo] * t2 + m.p[8][mo] * t3;
    } else {
      d[c][0] = xix_regular * t1;
      d[c][1] = xix_regular * t2;
      d[c][2] = xix_regular * t3;
    }
  }
  const float tr = d[0][0] + d[1][1] + d[2][2];
  const float templ = (1.f / 3.f) * tr;
  trace_over_3[eo] = templ;
  if (trace) trace[eo] = tr;  // epsilondev_trace of the memory-variable update
  eps0[eo] = d[0][0] - templ;
  eps1[eo] = d[1][1] - templ;
  eps2[eo] = 0.5f * (d[0][1] + d[1][0]);
  eps3[eo] = 0.5f * (d[2][0] + d[0][2]);
  eps4[eo] = 0.5f * (d[2][1] + d[1][2]);
}

// rho/mu/kappa accumulation (compute_kernels.f90:151-186,
// kernels/compute_kernels_cudakernel.cu:31-86), FP64 accumulators
__global__ void kernels_accum_kernel(long nspec, const int* __restrict__ ibool, const float* __restrict__ accel,
                                     const float* __restrict__ b_displ, const Ptrs10 E, const float* __restrict__ tr,
                                     const float* __restrict__ btr, double dt, double* __restrict__ rho_kl,
                                     double* __restrict__ mu_kl, double* __restrict__ kappa_kl) {
  const long e = blockIdx.x;
  const int t = threadIdx.x;
  if (e >= nspec || t >= NGLL3) return;
  const long eo = e * NGLL3_PAD + t;
  const int g = ibool[eo];
  const double r = (double)accel[3L * g] * b_displ[3L * g] + (double)accel[3L * g + 1] * b_displ[3L * g + 1] +
                   (double)accel[3L * g + 2] * b_displ[3L * g + 2];
  rho_kl[eo] += dt * r;
  const double e0 = E.p[0][eo], e1 = E.p[1][eo], e2 = E.p[2][eo], e3 = E.p[3][eo], e4 = E.p[4][eo];
  const double b0 = E.p[5][eo], b1 = E.p[6][eo], b2 = E.p[7][eo], b3 = E.p[8][eo], b4 = E.p[9][eo];
  mu_kl[eo] += dt * (e0 * b0 + e1 * b1 + (e0 + e1) * (b0 + b1) + 2.0 * (e2 * b2 + e3 * b3 + e4 * b4));
  kappa_kl[eo] += dt * (9.0 * (double)tr[eo] * (double)btr[eo]);
}

// ANISOTROPIC_KL: the 21 strain products of compute_strain_product
// (compute_kernels.f90:566-618; kernels/compute_kernels_ani_cudakernel.cu), FP64
__global__ void kernels_aniso_kernel(long nspec, const Ptrs10 E, const float* __restrict__ tr,
                                     const float* __restrict__ btr, double dt, double* __restrict__ cijkl) {
  const long e = blockIdx.x;
  const int t = threadIdx.x;
  if (e >= nspec || t >= NGLL3) return;
  const long eo = e * NGLL3_PAD + t;
  // Voigt strains: 11, 22, 33, 23, 13, 12 from the deviatoric parts and the trace
  double a[6], b[6];
  const double ta = tr[eo], tb = btr[eo];
  a[0] = E.p[0][eo] + ta; a[1] = E.p[1][eo] + ta; a[2] = -(a[0] + a[1]) + 3.0 * ta;
  a[3] = E.p[4][eo]; a[4] = E.p[3][eo]; a[5] = E.p[2][eo];
  b[0] = E.p[5][eo] + tb; b[1] = E.p[6][eo] + tb; b[2] = -(b[0] + b[1]) + 3.0 * tb;
  b[3] = E.p[9][eo]; b[4] = E.p[8][eo]; b[5] = E.p[7][eo];
  double* out = cijkl + eo * 21;
  int p = 0;
#pragma unroll
  for (int i = 0; i < 6; ++i)
#pragma unroll
    for (int j = i; j < 6; ++j) {
      double v = a[i] * b[j];
      if (j > i) {
        v += a[j] * b[i];
        if (j > 2 && i < 3) v *= 2.0;
      }
      if (i > 2) v *= 4.0;
      out[p] += dt * v;
      ++p;
    }
}

// APPROXIMATE_HESS_KL (compute_kernels.f90:513-545;
// kernels/compute_kernels_hess_el_cudakernel.cu), FP64
__global__ void kernels_hess_kernel(long nspec, const int* __restrict__ ibool, const int* __restrict__ is_acoustic,
                                    const float* __restrict__ accel, const float* __restrict__ b_accel,
                                    const float* __restrict__ b_veloc, const Ptrs10 E, const float* __restrict__ btr,
                                    double dt, double* __restrict__ h0, double* __restrict__ h_rho,
                                    double* __restrict__ h_kappa, double* __restrict__ h_mu) {
  const long e = blockIdx.x;
  const int t = threadIdx.x;
  if (e >= nspec || t >= NGLL3) return;
  if (is_acoustic && is_acoustic[e]) return;
  const long eo = e * NGLL3_PAD + t;
  const long g = ibool[eo];
  double aa = 0.0, vv = 0.0;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    aa += (double)accel[3 * g + c] * b_accel[3 * g + c];
    vv += (double)b_veloc[3 * g + c] * b_veloc[3 * g + c];
  }
  h0[eo] += dt * aa;
  h_rho[eo] += dt * vv;
  const double b0 = E.p[5][eo], b1 = E.p[6][eo], b2 = E.p[7][eo], b3 = E.p[8][eo], b4 = E.p[9][eo];
  h_mu[eo] += dt * (b0 * b0 + b1 * b1 + (b0 + b1) * (b0 + b1) + 2.0 * (b2 * b2 + b3 * b3 + b4 * b4));
  h_kappa[eo] += dt * (9.0 * (double)btr[eo] * (double)btr[eo]);
}

__global__ void kl_to_float_kernel(float* __restrict__ dst, const double* __restrict__ src, long nspec) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= nspec * NGLL3) return;
  dst[idx] = (float)src[(idx / NGLL3) * NGLL3_PAD + idx % NGLL3];
}

}  // namespace

static bool alloc_field_set(Mesh* mp, Fields& F) {
  const size_t n3 = 3 * (size_t)mp->nglob;
  bool ok = true;
  if (!F.displ) ok = ok && alloc_zero((void**)&F.displ, sizeof(float) * n3);
  if (!F.veloc) ok = ok && alloc_zero((void**)&F.veloc, sizeof(float) * n3);
  if (!F.accel) ok = ok && alloc_zero((void**)&F.accel, sizeof(float) * n3);
  for (int c = 0; c < 5 && ok; ++c)
    if (!F.eps[c]) ok = alloc_zero((void**)&F.eps[c], sizeof(float) * NGLL3_PAD * (size_t)mp->nspec);
  if (ok && !F.eps_trace_over_3)
    ok = alloc_zero((void**)&F.eps_trace_over_3, sizeof(float) * NGLL3_PAD * (size_t)mp->nspec);
  return ok;
}

}  // namespace sf3d

using namespace sf3d;

extern "C" {

void prepare_fields_elastic_adj_dev_(long* Mesh_pointer, int* size_f, realw* epsilon_trace_over_3,
                                     realw* b_epsilondev_xx, realw* b_epsilondev_yy, realw* b_epsilondev_xy,
                                     realw* b_epsilondev_xz, realw* b_epsilondev_yz, realw* b_epsilon_trace_over_3,
                                     int* R_size, realw* b_R_xx, realw* b_R_yy, realw* b_R_xy, realw* b_R_xz,
                                     realw* b_R_yz, realw* b_R_trace, realw* b_epsilondev_trace, realw* b_alphaval,
                                     realw* b_betaval, realw* b_gammaval, int* ANISOTROPIC_KL,
                                     int* APPROXIMATE_HESS_KL) {
  (void)R_size; (void)epsilon_trace_over_3; (void)b_epsilon_trace_over_3; (void)b_epsilondev_xx;
  (void)b_epsilondev_yy; (void)b_epsilondev_xy; (void)b_epsilondev_xz; (void)b_epsilondev_yz;
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  mp->anisotropic_kl = (ANISOTROPIC_KL && *ANISOTROPIC_KL) ? 1 : 0;
  mp->hess_kl = (APPROXIMATE_HESS_KL && *APPROXIMATE_HESS_KL) ? 1 : 0;
  if (!size_f || *size_f != 3 * mp->nglob) { set_error(SF3D_ERR_ARG, "size_f must be NDIM*NGLOB_AB"); return; }
  bool ok = alloc_field_set(mp, mp->f) && alloc_field_set(mp, mp->b);
  const size_t nk = NGLL3_PAD * (size_t)mp->nspec;
  ok = ok && alloc_zero((void**)&mp->d_rho_kl, sizeof(double) * nk);
  ok = ok && alloc_zero((void**)&mp->d_mu_kl, sizeof(double) * nk);
  ok = ok && alloc_zero((void**)&mp->d_kappa_kl, sizeof(double) * nk);
  if (mp->anisotropic_kl) ok = ok && alloc_zero((void**)&mp->d_cijkl_kl, sizeof(double) * 21 * nk);
  for (int q = 0; q < 4 && mp->hess_kl; ++q) ok = ok && alloc_zero((void**)&mp->d_hess_kl[q], sizeof(double) * nk);
  if (ok && mp->attenuation) {
    realw* hr[6] = {b_R_xx, b_R_yy, b_R_xy, b_R_xz, b_R_yz, b_R_trace};
    for (int c = 0; c < 6 && ok; ++c) ok = upload_sls_padded(&mp->b.R[c], hr[c], mp->nspec, mp->stream);
    ok = ok && upload_padded(&mp->b.eps[5], b_epsilondev_trace, mp->nspec, mp->stream);
    for (int q = 0; q < NSLS; ++q) {
      mp->b_alphaval[q] = b_alphaval[q];
      mp->b_betaval[q] = b_betaval[q];
      mp->b_gammaval[q] = b_gammaval[q];
    }
  }
}

void prepare_sim2_or_3_const_device_(long* Mesh_pointer, int* nadj_rec_local, int* NTSTEP_BETWEEN_READ_ADJSRC,
                                     realw* hxir_adjstore, realw* hetar_adjstore, realw* hgammar_adjstore, int* nrec,
                                     int* h_islice_selected_rec, int* h_ispec_selected_rec) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  mp->nadj_rec_local = *nadj_rec_local;
  mp->ntstep_between_read_adjsrc = *NTSTEP_BETWEEN_READ_ADJSRC;
  if (mp->nadj_rec_local <= 0) return;
  std::vector<int> isp;
  for (int r = 0; r < *nrec; ++r) {
    if (h_islice_selected_rec && h_islice_selected_rec[r] != 0) continue;
    isp.push_back(h_ispec_selected_rec[r] - 1);
  }
  if ((int)isp.size() != mp->nadj_rec_local) { set_error(SF3D_ERR_ARG, "nadj_rec_local mismatch"); return; }
  for (int v : isp)
    if (v < 0 || v >= mp->nspec) { set_error(SF3D_ERR_ARG, "ispec_selected_rec out of range"); return; }
  const size_t nl = (size_t)mp->nadj_rec_local;
  bool ok = alloc_zero((void**)&mp->d_ispec_adj, sizeof(int) * nl) &&
            copy_sync(mp->d_ispec_adj, isp.data(), sizeof(int) * nl, cudaMemcpyHostToDevice, mp->stream);
  float** dst[3] = {&mp->d_hxir_adj, &mp->d_hetar_adj, &mp->d_hgammar_adj};
  realw* src[3] = {hxir_adjstore, hetar_adjstore, hgammar_adjstore};
  for (int q = 0; q < 3 && ok; ++q)
    ok = alloc_zero((void**)dst[q], sizeof(float) * 5 * nl) &&
         copy_sync(*dst[q], src[q], sizeof(float) * 5 * nl, cudaMemcpyHostToDevice, mp->stream);
  ok = ok && alloc_zero((void**)&mp->d_source_adjoint, sizeof(float) * 3 * nl * mp->ntstep_between_read_adjsrc);
}

void add_sources_el_sim_type_2_or_3_(long* Mesh_pointer, realw* h_source_adjoint, int* nrec, int* nadj_rec_local,
                                     int* NTSTEP_BETWEEN_READ_ADJSRC, int* it) {
  (void)nrec;
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (*nadj_rec_local != mp->nadj_rec_local) { set_error(SF3D_ERR_ARG, "nadj_rec_local not equal"); return; }
  if (mp->nadj_rec_local == 0) return;
  const int nt = *NTSTEP_BETWEEN_READ_ADJSRC;
  if (nt != mp->ntstep_between_read_adjsrc || nt <= 0) { set_error(SF3D_ERR_ARG, "NTSTEP_BETWEEN_READ_ADJSRC mismatch"); return; }
  // time-reversed index inside the current block of adjoint-source samples
  const int it_index = nt - (*it - 1) % nt - 1;
  if ((*it - 1) % nt == 0)
    SF3D_CUDA(cudaMemcpyAsync(mp->d_source_adjoint, h_source_adjoint, sizeof(float) * 3 * (size_t)mp->nadj_rec_local * nt,
                              cudaMemcpyHostToDevice, mp->stream));
  adjoint_sources_kernel<<<mp->nadj_rec_local, NGLL3_PAD, 0, mp->stream>>>(
      mp->nadj_rec_local, mp->d_ispec_adj, mp->d_hxir_adj, mp->d_hetar_adj, mp->d_hgammar_adj, mp->d_source_adjoint,
      it_index, mp->d_ibool, mp->d_ispec_is_acoustic, mp->f.accel);
  SF3D_CUDA(cudaStreamSynchronize(mp->stream));
  cuda_ok(cudaGetLastError(), "adjoint_sources_kernel");
}

// add_sources_ac_sim_2_or_3_cuda (compute_add_sources_acoustic_cuda.cu): the same
// time-reversed block of adjoint traces, receivers in fluid elements
void add_sources_ac_sim_2_or_3_cuda_(long* Mesh_pointer, realw* h_source_adjoint, int* nrec, int* nadj_rec_local,
                                     int* NTSTEP_BETWEEN_READ_ADJSRC, int* it) {
  (void)nrec;
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!mp->d_potential_dot_dot) { set_error(SF3D_ERR_STATE, "acoustic fields not prepared"); return; }
  if (*nadj_rec_local != mp->nadj_rec_local) { set_error(SF3D_ERR_ARG, "nadj_rec_local not equal"); return; }
  if (mp->nadj_rec_local == 0) return;
  const int nt = *NTSTEP_BETWEEN_READ_ADJSRC;
  if (nt != mp->ntstep_between_read_adjsrc || nt <= 0) { set_error(SF3D_ERR_ARG, "NTSTEP_BETWEEN_READ_ADJSRC mismatch"); return; }
  const int it_index = nt - (*it - 1) % nt - 1;
  if ((*it - 1) % nt == 0)
    SF3D_CUDA(cudaMemcpyAsync(mp->d_source_adjoint, h_source_adjoint, sizeof(float) * 3 * (size_t)mp->nadj_rec_local * nt,
                              cudaMemcpyHostToDevice, mp->stream));
  adjoint_sources_ac_kernel<<<mp->nadj_rec_local, NGLL3_PAD, 0, mp->stream>>>(
      mp->nadj_rec_local, mp->d_ispec_adj, mp->d_hxir_adj, mp->d_hetar_adj, mp->d_hgammar_adj, mp->d_source_adjoint,
      it_index, mp->d_ibool, mp->d_ispec_is_acoustic, mp->d_potential_dot_dot);
  SF3D_CUDA(cudaStreamSynchronize(mp->stream));
  cuda_ok(cudaGetLastError(), "adjoint_sources_ac_kernel");
}

namespace {
// strain of a field from its displacement (compute_strain_cuda.cu,
// kernels/compute_element_strain_cudakernel.cu)
bool field_strain(Mesh* mp, Fields& F) {
  if (!F.displ || !F.eps[0] || !F.eps_trace_over_3) { set_error(SF3D_ERR_STATE, "strain arrays not allocated"); return false; }
  Ptrs10 m = {};
  for (int q = 0; q < 9; ++q) m.p[q] = mp->d_metric[q];
  element_strain_kernel<<<mp->nspec, NGLL3_PAD, 0, mp->stream>>>(mp->d_ibool, mp->d_irregular, m, mp->d_gll,
                                                                 mp->xix_regular, F.displ, F.eps[0], F.eps[1],
                                                                 F.eps[2], F.eps[3], F.eps[4], F.eps_trace_over_3,
                                                                 F.eps[5]);
  return cuda_ok(cudaGetLastError(), "element_strain_kernel");
}
}  // namespace

void compute_strain_cuda_(long* Mesh_pointer, int* FORWARD_OR_ADJOINT) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!FORWARD_OR_ADJOINT || (*FORWARD_OR_ADJOINT != 1 && *FORWARD_OR_ADJOINT != 3)) {
    set_error(SF3D_ERR_ARG, "compute_strain_cuda: FORWARD_OR_ADJOINT must be 1 or 3");
    return;
  }
  field_strain(mp, (*FORWARD_OR_ADJOINT == 3) ? mp->b : mp->f);
}

void compute_kernels_elastic_cuda_(long* Mesh_pointer, realw* deltat_f) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!mp->d_rho_kl || !mp->b.displ) { set_error(SF3D_ERR_STATE, "prepare_fields_elastic_adj_dev not called"); return; }
  // undo attenuation: b_displ was restored from the recomputed history; its
  // strain is recomputed here
  if (mp->undo_attenuation && !field_strain(mp, mp->b)) return;
  const Ptrs10 E = {{mp->f.eps[0], mp->f.eps[1], mp->f.eps[2], mp->f.eps[3], mp->f.eps[4],
                     mp->b.eps[0], mp->b.eps[1], mp->b.eps[2], mp->b.eps[3], mp->b.eps[4]}};
  kernels_accum_kernel<<<mp->nspec, NGLL3_PAD, 0, mp->stream>>>(
      mp->nspec, mp->d_ibool, mp->f.accel, mp->b.displ, E, mp->f.eps_trace_over_3, mp->b.eps_trace_over_3,
      (double)*deltat_f, mp->d_rho_kl, mp->d_mu_kl, mp->d_kappa_kl);
  if (mp->anisotropic_kl)
    // with ANISOTROPIC_KL the reference accumulates cijkl_kl in place of mu/kappa;
    // both are kept here (mu_kl, kappa_kl stay available)
    kernels_aniso_kernel<<<mp->nspec, NGLL3_PAD, 0, mp->stream>>>(
        mp->nspec, E, mp->f.eps_trace_over_3, mp->b.eps_trace_over_3, (double)*deltat_f, mp->d_cijkl_kl);
  SF3D_CUDA(cudaStreamSynchronize(mp->stream));
  cuda_ok(cudaGetLastError(), "kernels_accum_kernel");
}

void transfer_kernels_el_to_host_(long* Mesh_pointer, realw* h_rho_kl, realw* h_mu_kl, realw* h_kappa_kl,
                                  realw* h_cijkl_kl, int* NSPEC_AB) {
  (void)h_cijkl_kl;
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (*NSPEC_AB != mp->nspec || !mp->d_rho_kl) { set_error(SF3D_ERR_ARG, "kernels not allocated / NSPEC mismatch"); return; }
  const long n = (long)mp->nspec * NGLL3;
  if (!ensure_stage(mp, sizeof(float) * n)) return;
  realw* h[3] = {h_rho_kl, h_mu_kl, h_kappa_kl};
  double* d[3] = {mp->d_rho_kl, mp->d_mu_kl, mp->d_kappa_kl};
  for (int q = 0; q < 3; ++q) {
    kl_to_float_kernel<<<nblk(n, 256), 256, 0, mp->stream>>>(mp->d_stage, d[q], mp->nspec);
    SF3D_CUDA(cudaMemcpyAsync(h[q], mp->d_stage, sizeof(float) * n, cudaMemcpyDeviceToHost, mp->stream));
    SF3D_CUDA(cudaStreamSynchronize(mp->stream));
  }
  if (mp->anisotropic_kl && h_cijkl_kl) {
    // cijkl_kl(21,5,5,5,NSPEC)
    std::vector<double> tmp(21 * NGLL3_PAD * (size_t)mp->nspec);
    if (!copy_sync(tmp.data(), mp->d_cijkl_kl, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost, mp->stream)) return;
    for (long e = 0; e < mp->nspec; ++e)
      for (int p = 0; p < NGLL3; ++p)
        for (int c = 0; c < 21; ++c)
          h_cijkl_kl[c + 21 * (p + NGLL3 * e)] = (float)tmp[c + 21 * (p + (size_t)NGLL3_PAD * e)];
  }
}

void compute_kernels_hess_cuda_(long* Mesh_pointer, realw* deltat_f, int* ELASTIC_SIMULATION,
                                int* ACOUSTIC_SIMULATION) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (ACOUSTIC_SIMULATION && *ACOUSTIC_SIMULATION && mp->has_acoustic &&
      !launch_hess_acoustic(mp, (double)*deltat_f))
    return;
  if (ELASTIC_SIMULATION && !*ELASTIC_SIMULATION) return;
  if (!mp->hess_kl || !mp->d_hess_kl[0]) { set_error(SF3D_ERR_STATE, "APPROXIMATE_HESS_KL was not prepared"); return; }
  const Ptrs10 E = {{mp->f.eps[0], mp->f.eps[1], mp->f.eps[2], mp->f.eps[3], mp->f.eps[4],
                     mp->b.eps[0], mp->b.eps[1], mp->b.eps[2], mp->b.eps[3], mp->b.eps[4]}};
  kernels_hess_kernel<<<mp->nspec, NGLL3_PAD, 0, mp->stream>>>(
      mp->nspec, mp->d_ibool, mp->d_ispec_is_acoustic, mp->f.accel, mp->b.accel, mp->b.veloc, E,
      mp->b.eps_trace_over_3, (double)*deltat_f, mp->d_hess_kl[0], mp->d_hess_kl[1], mp->d_hess_kl[2],
      mp->d_hess_kl[3]);
  cuda_ok(cudaGetLastError(), "kernels_hess_kernel");
}

void transfer_kernels_hess_el_tohost_(long* Mesh_pointer, realw* h_hess_kl, realw* h_hess_rho_kl,
                                      realw* h_hess_kappa_kl, realw* h_hess_mu_kl, int* NSPEC_AB) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (*NSPEC_AB != mp->nspec || !mp->d_hess_kl[0]) { set_error(SF3D_ERR_ARG, "Hessian kernels not allocated / NSPEC mismatch"); return; }
  const long n = (long)mp->nspec * NGLL3;
  if (!ensure_stage(mp, sizeof(float) * n)) return;
  realw* h[4] = {h_hess_kl, h_hess_rho_kl, h_hess_kappa_kl, h_hess_mu_kl};
  for (int q = 0; q < 4; ++q) {
    kl_to_float_kernel<<<nblk(n, 256), 256, 0, mp->stream>>>(mp->d_stage, mp->d_hess_kl[q], mp->nspec);
    SF3D_CUDA(cudaMemcpyAsync(h[q], mp->d_stage, sizeof(float) * n, cudaMemcpyDeviceToHost, mp->stream));
    SF3D_CUDA(cudaStreamSynchronize(mp->stream));
  }
}

// FP64 anisotropic (21 per point) and Hessian (4 per point) accumulators, either may be NULL
int sf3d_get_extra_kernels_f64(long* Mesh_pointer, double* h_cijkl_kl, double* h_hess) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  const size_t np = NGLL3_PAD * (size_t)mp->nspec;
  if (h_cijkl_kl) {
    if (!mp->d_cijkl_kl) { set_error(SF3D_ERR_STATE, "ANISOTROPIC_KL was not prepared"); return SF3D_ERR_STATE; }
    std::vector<double> tmp(21 * np);
    if (!copy_sync(tmp.data(), mp->d_cijkl_kl, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost, mp->stream))
      return SF3D_ERR_CUDA;
    for (long e = 0; e < mp->nspec; ++e)
      for (int p = 0; p < NGLL3; ++p)
        for (int c = 0; c < 21; ++c) h_cijkl_kl[c + 21 * (p + NGLL3 * e)] = tmp[c + 21 * (p + (size_t)NGLL3_PAD * e)];
  }
  if (h_hess) {
    if (!mp->d_hess_kl[0]) { set_error(SF3D_ERR_STATE, "APPROXIMATE_HESS_KL was not prepared"); return SF3D_ERR_STATE; }
    std::vector<double> tmp(np);
    for (int q = 0; q < 4; ++q) {
      if (!copy_sync(tmp.data(), mp->d_hess_kl[q], sizeof(double) * np, cudaMemcpyDeviceToHost, mp->stream))
        return SF3D_ERR_CUDA;
      for (long e = 0; e < mp->nspec; ++e)
        for (int p = 0; p < NGLL3; ++p) h_hess[(size_t)q * NGLL3 * mp->nspec + p + NGLL3 * e] = tmp[p + (size_t)NGLL3_PAD * e];
    }
  }
  return SF3D_OK;
}

// FP64 kernels straight from the device accumulators, (5,5,5,NSPEC) each
int sf3d_get_kernels_f64(long* Mesh_pointer, double* h_rho_kl, double* h_mu_kl, double* h_kappa_kl) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!mp->d_rho_kl) { set_error(SF3D_ERR_STATE, "kernels not allocated"); return SF3D_ERR_STATE; }
  std::vector<double> tmp(NGLL3_PAD * (size_t)mp->nspec);
  double* h[3] = {h_rho_kl, h_mu_kl, h_kappa_kl};
  double* d[3] = {mp->d_rho_kl, mp->d_mu_kl, mp->d_kappa_kl};
  for (int q = 0; q < 3; ++q) {
    if (!copy_sync(tmp.data(), d[q], sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost, mp->stream)) return SF3D_ERR_CUDA;
    for (long e = 0; e < mp->nspec; ++e)
      for (int p = 0; p < NGLL3; ++p) h[q][e * NGLL3 + p] = tmp[e * NGLL3_PAD + p];
  }
  return SF3D_OK;
}

}  // extern "C"
