// The remaining FC_FUNC_ entry points of the reference's GPU layer, so that the
// library links into xspecfem3D in place of src/gpu (every symbol of
// specfem3D_gpu_cuda_method_stubs.c exists here):
//
// * debugging and norm checks (check_fields_cuda.cu): check_max_norm_*,
//   check_error_vectors, get_max_accel, get_norm_*_from_device,
//   get/output_free_device_memory, make_displ_rand, pause_for_debug,
//   register/unregister_host_array;
// * single-field transfers (transfer_fields_cuda.cu) of the backward elastic
//   fields, the acoustic potentials, strains, memory variables and kernels;
// * acoustic MPI interface pack / assembly (transfer_boun_pot_from_device,
//   transfer_asmbl_pot_to_device);
// * Stacey of a recomputed backward field (*_undoatt_cuda);
// * features this library does not provide (noise tomography, faults,
//   gravity, ocean load): the call records
//   SF3D_ERR_UNSUPPORTED (sf3d_last_error) and does nothing else.
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>

#include <cmath>
#include <vector>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

void unsupported(const char* what) {
  char msg[200];
  snprintf(msg, sizeof msg, "%s is not supported by this library", what);
  set_error(SF3D_ERR_UNSUPPORTED, msg);
}

// the reference's diagnostics print on stdout; flushed so that they interleave
// with the caller's own output
void report(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vprintf(fmt, ap);
  va_end(ap);
  fflush(stdout);
}

float host_max_abs(const float* v, long n) {
  float m = 0.f;
  for (long i = 0; i < n; ++i) {
    const float a = fabsf(v[i]);
    if (a > m || std::isnan(a)) m = a;
  }
  return m;
}

// copy a device field of n floats to the host
bool to_host(Mesh* mp, float* h, const float* d, long n) {
  if (!d) { set_error(SF3D_ERR_STATE, "field not allocated"); return false; }
  return copy_sync(h, d, sizeof(float) * n, cudaMemcpyDeviceToHost, mp->stream);
}

bool to_device(Mesh* mp, float* d, const float* h, long n) {
  if (!d) { set_error(SF3D_ERR_STATE, "field not allocated"); return false; }
  return copy_sync(d, h, sizeof(float) * n, cudaMemcpyHostToDevice, mp->stream);
}

// (5,5,5,NSPEC) host layout <-> [nspec][128] device layout
bool padded_to_host(Mesh* mp, float* h, const float* d) {
  if (!d) { set_error(SF3D_ERR_STATE, "array not allocated"); return false; }
  std::vector<float> tmp((size_t)NGLL3_PAD * mp->nspec);
  if (!copy_sync(tmp.data(), d, sizeof(float) * tmp.size(), cudaMemcpyDeviceToHost, mp->stream)) return false;
  for (long e = 0; e < mp->nspec; ++e)
    for (int p = 0; p < NGLL3; ++p) h[p + NGLL3 * e] = tmp[p + (size_t)NGLL3_PAD * e];
  return true;
}

bool padded_to_device(Mesh* mp, float* d, const float* h) {
  if (!d) { set_error(SF3D_ERR_STATE, "array not allocated"); return false; }
  std::vector<float> tmp((size_t)NGLL3_PAD * mp->nspec, 0.f);
  for (long e = 0; e < mp->nspec; ++e)
    for (int p = 0; p < NGLL3; ++p) tmp[p + (size_t)NGLL3_PAD * e] = h[p + NGLL3 * e];
  return copy_sync(d, tmp.data(), sizeof(float) * tmp.size(), cudaMemcpyHostToDevice, mp->stream);
}

// memory variables: host (N_SLS,5,5,5,NSPEC) -> device [nspec][N_SLS][128]
bool sls_to_device(Mesh* mp, float* d, const float* h) {
  if (!d) { set_error(SF3D_ERR_STATE, "array not allocated"); return false; }
  std::vector<float> tmp((size_t)NGLL3_PAD * NSLS * mp->nspec, 0.f);
  for (long e = 0; e < mp->nspec; ++e)
    for (int s = 0; s < NSLS; ++s)
      for (int p = 0; p < NGLL3; ++p) tmp[p + NGLL3_PAD * (s + (size_t)NSLS * e)] = h[s + NSLS * (p + NGLL3 * e)];
  return copy_sync(d, tmp.data(), sizeof(float) * tmp.size(), cudaMemcpyHostToDevice, mp->stream);
}

bool kernel_to_host(Mesh* mp, float* h, const double* d) {
  if (!d) { set_error(SF3D_ERR_STATE, "kernels not allocated"); return false; }
  std::vector<double> tmp((size_t)NGLL3_PAD * mp->nspec);
  if (!copy_sync(tmp.data(), d, sizeof(double) * tmp.size(), cudaMemcpyDeviceToHost, mp->stream)) return false;
  for (long e = 0; e < mp->nspec; ++e)
    for (int p = 0; p < NGLL3; ++p) h[p + NGLL3 * e] = (float)tmp[p + (size_t)NGLL3_PAD * e];
  return true;
}

// scalar (acoustic) interface buffers, (max_nibool, num_interfaces)
__global__ void pack_scalar_kernel(const float* __restrict__ f, float* __restrict__ buf, int nif, int mxn,
                                   const int* __restrict__ nibool, const int* __restrict__ ibool_if) {
  const long id = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (long)nif * mxn) return;
  const int i = (int)(id / mxn);
  if ((int)(id - (long)i * mxn) >= nibool[i]) return;
  buf[id] = f[ibool_if[id]];
}

__global__ void add_scalar_kernel(float* __restrict__ f, const float* __restrict__ buf, int nif, int mxn,
                                  const int* __restrict__ nibool, const int* __restrict__ ibool_if) {
  const long id = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (long)nif * mxn) return;
  const int i = (int)(id / mxn);
  if ((int)(id - (long)i * mxn) >= nibool[i]) return;
  atomicAdd(f + ibool_if[id], buf[id]);
}

}  // namespace
}  // namespace sf3d

using namespace sf3d;

extern "C" {

// ---------------------------------------------------------------- norms, checks
void check_max_norm_vector_(int* size, realw* vector1, int* announceID) {
  report("%d: maximum norm of vector = %e\n", announceID ? *announceID : 0, host_max_abs(vector1, *size));
}
void check_max_norm_displ_(int* size, realw* displ, int* announceID) {
  report("%d: maximum displacement = %e\n", announceID ? *announceID : 0, host_max_abs(displ, *size));
}
void check_max_norm_b_displ_(int* size, realw* b_displ, int* announceID) {
  report("%d: maximum backward displacement = %e\n", announceID ? *announceID : 0, host_max_abs(b_displ, *size));
}
void check_max_norm_b_accel_(int* size, realw* b_accel, int* announceID) {
  report("%d: maximum backward acceleration = %e\n", announceID ? *announceID : 0, host_max_abs(b_accel, *size));
}
void check_error_vectors_(int* sizef, realw* vector1, realw* vector2) {
  float m = 0.f;
  for (long i = 0; i < *sizef; ++i) m = fmaxf(m, fabsf(vector1[i] - vector2[i]));
  report("maximum difference between the vectors = %e\n", m);
}
static void norm_gpu(int* size, realw* h, long* Mesh_pointer, int* announceID, bool backward, int which,
                     const char* label) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!size || *size != 3 * mp->nglob) { set_error(SF3D_ERR_ARG, "size must be NDIM*NGLOB_AB"); return; }
  Fields& F = backward ? mp->b : mp->f;
  const float* d = which == 0 ? F.displ : (which == 1 ? F.veloc : F.accel);
  if (!to_host(mp, h, d, *size)) return;
  report("%d: maximum %s = %e\n", announceID ? *announceID : 0, label, host_max_abs(h, *size));
}
void check_max_norm_displ_gpu_(int* size, realw* displ, long* Mesh_pointer, int* announceID) {
  norm_gpu(size, displ, Mesh_pointer, announceID, false, 0, "displacement");
}
void check_max_norm_b_displ_gpu_(int* size, realw* b_displ, long* Mesh_pointer, int* announceID) {
  norm_gpu(size, b_displ, Mesh_pointer, announceID, true, 0, "backward displacement");
}
void check_max_norm_b_veloc_gpu_(int* size, realw* b_veloc, long* Mesh_pointer, int* announceID) {
  norm_gpu(size, b_veloc, Mesh_pointer, announceID, true, 1, "backward velocity");
}
void check_max_norm_b_accel_gpu_(int* size, realw* b_accel, long* Mesh_pointer, int* announceID) {
  norm_gpu(size, b_accel, Mesh_pointer, announceID, true, 2, "backward acceleration");
}
void get_max_accel_(int* itf, int* sizef, long* Mesh_pointer) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  std::vector<float> h((size_t)3 * mp->nglob);
  if (!to_host(mp, h.data(), mp->f.accel, (long)h.size())) return;
  (void)sizef;
  report("%d/%d: maximum acceleration = %e\n", itf ? *itf : 0, mp->nglob, host_max_abs(h.data(), (long)h.size()));
}
// max |displ| (type 1) or |b_displ| (type 3), the norm check_stability uses
void get_norm_elastic_from_device_(realw* norm, long* Mesh_pointer, int* type) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  const float* d = (type && *type == 3) ? mp->b.displ : mp->f.displ;
  float m = 0.f;
  if (!d) { set_error(SF3D_ERR_STATE, "field not allocated"); return; }
  if (!device_maxabs(mp, d, 3L * mp->nglob, &m)) return;
  *norm = m;
}
void get_norm_acoustic_from_device_(realw* norm, long* Mesh_pointer, int* sim_type) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  const float* d = (sim_type && *sim_type == 3) ? mp->d_b_potential_dot_dot : mp->d_potential_dot_dot;
  float m = 0.f;
  if (!d) { set_error(SF3D_ERR_STATE, "acoustic fields not prepared"); return; }
  if (!device_maxabs(mp, d, (long)mp->nglob, &m)) return;
  *norm = m;
}
void get_free_device_memory_(realw* free_mb, realw* used_mb, realw* total_mb) {
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { set_error(SF3D_ERR_CUDA, "cudaMemGetInfo failed"); return; }
  *free_mb = (realw)(fr / 1048576.0);
  *total_mb = (realw)(tot / 1048576.0);
  *used_mb = *total_mb - *free_mb;
}
void output_free_device_memory_(int* myrank) {
  realw f = 0, u = 0, t = 0;
  get_free_device_memory_(&f, &u, &t);
  report("%d: GPU memory used %.1f MB of %.1f MB (%.1f MB free)\n", myrank ? *myrank : 0, u, t, f);
}
// fills displ with pseudo-random values (debugging aid of the reference), on host and device
void make_displ_rand_(long* Mesh_pointer, realw* h_displ) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  unsigned s = 12345u;
  for (long i = 0; i < 3L * mp->nglob; ++i) {
    s = s * 1664525u + 1013904223u;
    h_displ[i] = (realw)((s >> 8) * (1.0 / 16777216.0));
  }
  to_device(mp, mp->f.displ, h_displ, 3L * mp->nglob);
}
void pause_for_debug_() {}
void register_host_array_(int* size, realw* h_array) {
  if (!size || *size <= 0 || !h_array) return;
  if (cudaHostRegister(h_array, sizeof(realw) * (size_t)*size, cudaHostRegisterDefault) != cudaSuccess) {
    cudaGetLastError();
    set_error(SF3D_ERR_CUDA, "register_host_array: cudaHostRegister failed");
  }
}
void unregister_host_array_(realw* h_array) {
  if (h_array && cudaHostUnregister(h_array) != cudaSuccess) cudaGetLastError();
}

// ---------------------------------------------------------------- transfers
static bool size3(Mesh* mp, int* size) {
  if (!size || *size != 3 * mp->nglob) { set_error(SF3D_ERR_ARG, "transfer size must be NDIM*NGLOB_AB"); return false; }
  return true;
}
void transfer_b_accel_from_device_(int* size, realw* b_accel, long* Mesh_pointer) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (mp && size3(mp, size)) to_host(mp, b_accel, mp->b.accel, *size);
}
void transfer_b_accel_to_device_(int* size, realw* b_accel, long* Mesh_pointer) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (mp && size3(mp, size)) to_device(mp, mp->b.accel, b_accel, *size);
}
void transfer_b_veloc_from_device_(int* size, realw* b_veloc, long* Mesh_pointer) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (mp && size3(mp, size)) to_host(mp, b_veloc, mp->b.veloc, *size);
}
void transfer_b_veloc_to_device_(int* size, realw* b_veloc, long* Mesh_pointer) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (mp && size3(mp, size)) to_device(mp, mp->b.veloc, b_veloc, *size);
}
static bool size1(Mesh* mp, int* size) {
  if (!size || *size != mp->nglob) { set_error(SF3D_ERR_ARG, "transfer size must be NGLOB_AB"); return false; }
  if (!mp->d_potential) { set_error(SF3D_ERR_STATE, "acoustic fields not prepared"); return false; }
  return true;
}
void transfer_potential_ac_from_device_(int* size, realw* potential_acoustic, long* Mesh_pointer) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (mp && size1(mp, size)) to_host(mp, potential_acoustic, mp->d_potential, *size);
}
void transfer_dot_dot_from_device_(int* size, realw* potential_dot_dot_acoustic, long* Mesh_pointer) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (mp && size1(mp, size)) to_host(mp, potential_dot_dot_acoustic, mp->d_potential_dot_dot, *size);
}
void transfer_dot_dot_to_device_(int* size, realw* potential_dot_dot_acoustic, long* Mesh_pointer) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (mp && size1(mp, size)) to_device(mp, mp->d_potential_dot_dot, potential_dot_dot_acoustic, *size);
}
// backward strains and memory variables of an undo-attenuation restart
// (transfer_fields_cuda.cu: transfer_b_strain_to_device, transfer_b_rmemory_to_device)
void transfer_b_strain_to_device_(long* Mesh_pointer, realw* b_epsilondev_xx, realw* b_epsilondev_yy,
                                  realw* b_epsilondev_xy, realw* b_epsilondev_xz, realw* b_epsilondev_yz,
                                  realw* b_epsilondev_trace, int* size_epsilondev) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!size_epsilondev || *size_epsilondev != NGLL3 * mp->nspec) {
    set_error(SF3D_ERR_ARG, "size_epsilondev must be NGLL3*NSPEC_AB");
    return;
  }
  realw* h[6] = {b_epsilondev_xx, b_epsilondev_yy, b_epsilondev_xy, b_epsilondev_xz, b_epsilondev_yz,
                 b_epsilondev_trace};
  for (int c = 0; c < 6; ++c)
    if (h[c] && mp->b.eps[c] && !padded_to_device(mp, mp->b.eps[c], h[c])) return;
}
void transfer_b_rmemory_to_device_(long* Mesh_pointer, realw* b_R_xx, realw* b_R_yy, realw* b_R_xy, realw* b_R_xz,
                                   realw* b_R_yz, realw* b_R_trace, int* size_R) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!size_R || *size_R != NSLS * NGLL3 * mp->nspec) {
    set_error(SF3D_ERR_ARG, "size_R must be N_SLS*NGLL3*NSPEC_AB");
    return;
  }
  realw* h[6] = {b_R_xx, b_R_yy, b_R_xy, b_R_xz, b_R_yz, b_R_trace};
  for (int c = 0; c < 6; ++c) {
    if (!mp->b.R[c]) { set_error(SF3D_ERR_STATE, "backward memory variables not allocated"); return; }
    if (!sls_to_device(mp, mp->b.R[c], h[c])) return;
  }
}
// debugging read-backs of the kernel computation (transfer_fields_cuda.cu)
void transfer_compute_kernel_answers_from_device_(long* Mesh_pointer, realw* rho_kl, int* size_rho, realw* mu_kl,
                                                  int* size_mu, realw* kappa_kl, int* size_kappa) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  (void)size_rho; (void)size_mu; (void)size_kappa;
  kernel_to_host(mp, rho_kl, mp->d_rho_kl) && kernel_to_host(mp, mu_kl, mp->d_mu_kl) &&
      kernel_to_host(mp, kappa_kl, mp->d_kappa_kl);
}
void transfer_compute_kernel_fields_from_device_(
    long* Mesh_pointer, realw* accel, int* size_accel, realw* b_displ, int* size_b_displ, realw* epsilondev_xx,
    realw* epsilondev_yy, realw* epsilondev_xy, realw* epsilondev_xz, realw* epsilondev_yz, int* size_epsilondev,
    realw* b_epsilondev_xx, realw* b_epsilondev_yy, realw* b_epsilondev_xy, realw* b_epsilondev_xz,
    realw* b_epsilondev_yz, int* size_b_epsilondev, realw* rho_kl, int* size_rho, realw* mu_kl, int* size_mu,
    realw* kappa_kl, int* size_kappa, realw* epsilon_trace_over_3, realw* b_epsilon_trace_over_3,
    int* size_epsilon_trace_over_3) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  (void)size_epsilondev; (void)size_b_epsilondev; (void)size_epsilon_trace_over_3;
  if (size_accel && *size_accel == 3 * mp->nglob && !to_host(mp, accel, mp->f.accel, *size_accel)) return;
  if (size_b_displ && *size_b_displ == 3 * mp->nglob && !to_host(mp, b_displ, mp->b.displ, *size_b_displ)) return;
  realw* he[5] = {epsilondev_xx, epsilondev_yy, epsilondev_xy, epsilondev_xz, epsilondev_yz};
  realw* hb[5] = {b_epsilondev_xx, b_epsilondev_yy, b_epsilondev_xy, b_epsilondev_xz, b_epsilondev_yz};
  for (int c = 0; c < 5; ++c) {
    if (mp->f.eps[c] && !padded_to_host(mp, he[c], mp->f.eps[c])) return;
    if (mp->b.eps[c] && !padded_to_host(mp, hb[c], mp->b.eps[c])) return;
  }
  if (mp->f.eps_trace_over_3 && !padded_to_host(mp, epsilon_trace_over_3, mp->f.eps_trace_over_3)) return;
  if (mp->b.eps_trace_over_3 && !padded_to_host(mp, b_epsilon_trace_over_3, mp->b.eps_trace_over_3)) return;
  transfer_compute_kernel_answers_from_device_(Mesh_pointer, rho_kl, size_rho, mu_kl, size_mu, kappa_kl, size_kappa);
}

// ---------------------------------------------------------------- acoustic MPI interfaces
// transfer_boun_pot_from_device / transfer_asmbl_pot_to_device
// (assemble_MPI_scalar_cuda.cu): potential_dot_dot at the interface points of
// this slice into the (max_nibool, num_interfaces) buffer, and the neighbours'
// contributions added back
void transfer_boun_pot_from_device_(long* Mesh_pointer, realw* send_potential_dot_dot_buffer,
                                    const int* FORWARD_OR_ADJOINT) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  float* pdd = (FORWARD_OR_ADJOINT && *FORWARD_OR_ADJOINT == 3) ? mp->d_b_potential_dot_dot : mp->d_potential_dot_dot;
  const long n = (long)mp->num_interfaces * mp->max_nibool_interfaces;
  if (n == 0) return;
  if (!pdd) { set_error(SF3D_ERR_STATE, "acoustic fields not prepared"); return; }
  if (!ensure_stage(mp, sizeof(float) * n)) return;
  pack_scalar_kernel<<<nblk(n, 128), 128, 0, mp->stream>>>(pdd, mp->d_stage, mp->num_interfaces,
                                                           mp->max_nibool_interfaces, mp->d_nibool_interfaces,
                                                           mp->d_ibool_interfaces);
  if (!cuda_ok(cudaGetLastError(), "pack_scalar_kernel")) return;
  copy_sync(send_potential_dot_dot_buffer, mp->d_stage, sizeof(float) * n, cudaMemcpyDeviceToHost, mp->stream);
}
void transfer_asmbl_pot_to_device_(long* Mesh_pointer, realw* buffer_recv_scalar_ext_mesh,
                                   const int* FORWARD_OR_ADJOINT) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  float* pdd = (FORWARD_OR_ADJOINT && *FORWARD_OR_ADJOINT == 3) ? mp->d_b_potential_dot_dot : mp->d_potential_dot_dot;
  const long n = (long)mp->num_interfaces * mp->max_nibool_interfaces;
  if (n == 0) return;
  if (!pdd) { set_error(SF3D_ERR_STATE, "acoustic fields not prepared"); return; }
  if (!ensure_stage(mp, sizeof(float) * n)) return;
  if (!copy_sync(mp->d_stage, buffer_recv_scalar_ext_mesh, sizeof(float) * n, cudaMemcpyHostToDevice, mp->stream)) return;
  add_scalar_kernel<<<nblk(n, 128), 128, 0, mp->stream>>>(pdd, mp->d_stage, mp->num_interfaces,
                                                          mp->max_nibool_interfaces, mp->d_nibool_interfaces,
                                                          mp->d_ibool_interfaces);
  cuda_ok(cudaGetLastError(), "add_scalar_kernel");
}

// ---------------------------------------------------------------- undo-attenuation Stacey
// the backward field is recomputed (not replayed): Stacey from b_veloc
void compute_stacey_viscoelastic_undoatt_cuda_(long* Mesh_pointer, int* iphasef, int* FORWARD_OR_ADJOINT_f) {
  compute_stacey_viscoelastic_cuda_(Mesh_pointer, iphasef, nullptr, FORWARD_OR_ADJOINT_f);
}
void compute_stacey_acoustic_undoatt_cuda_(long* Mesh_pointer, int* iphasef, int* FORWARD_OR_ADJOINT_f) {
  compute_stacey_acoustic_cuda_(Mesh_pointer, iphasef, nullptr, FORWARD_OR_ADJOINT_f);
}

// ---------------------------------------------------------------- not provided
// noise tomography
void prepare_fields_noise_device_(long* Mesh_pointer, int* NSPEC_AB, int* NGLOB_AB, int* free_surface_ispec,
                                  int* free_surface_ijk, int* num_free_surface_faces, int* NOISE_TOMOGRAPHY,
                                  int* NSTEP, realw* noise_sourcearray, realw* normal_x_noise, realw* normal_y_noise,
                                  realw* normal_z_noise, realw* mask_noise, realw* free_surface_jacobian2Dw) {
  (void)Mesh_pointer; (void)NSPEC_AB; (void)NGLOB_AB; (void)free_surface_ispec; (void)free_surface_ijk;
  (void)num_free_surface_faces; (void)NOISE_TOMOGRAPHY; (void)NSTEP; (void)noise_sourcearray;
  (void)normal_x_noise; (void)normal_y_noise; (void)normal_z_noise; (void)mask_noise; (void)free_surface_jacobian2Dw;
  unsupported("noise tomography (prepare_fields_noise_device)");
}
void add_source_main_rec_noise_cu_(long* Mesh_pointer, int* it_f, int* irec_main_noise_f, int* islice_selected_rec) {
  (void)Mesh_pointer; (void)it_f; (void)irec_main_noise_f; (void)islice_selected_rec;
  unsupported("noise tomography (add_source_main_rec_noise_cu)");
}
void noise_read_add_surface_movie_cu_(long* Mesh_pointer, realw* h_noise_surface_movie, int* NOISE_TOMOGRAPHYf) {
  (void)Mesh_pointer; (void)h_noise_surface_movie; (void)NOISE_TOMOGRAPHYf;
  unsupported("noise tomography (noise_read_add_surface_movie_cu)");
}
void compute_kernels_strgth_noise_cu_(long* Mesh_pointer, realw* h_noise_surface_movie, realw* deltat) {
  (void)Mesh_pointer; (void)h_noise_surface_movie; (void)deltat;
  unsupported("noise tomography (compute_kernels_strgth_noise_cu)");
}
void transfer_kernels_noise_to_host_(long* Mesh_pointer, realw* h_sigma_kl, int* NSPEC_AB) {
  (void)Mesh_pointer; (void)h_sigma_kl; (void)NSPEC_AB;
  unsupported("noise tomography (transfer_kernels_noise_to_host)");
}
void transfer_sigma_from_device_(int* size, realw* sigma_kl, long* Mesh_pointer) {
  (void)size; (void)sigma_kl; (void)Mesh_pointer;
  unsupported("noise tomography (transfer_sigma_from_device)");
}
void transfer_surface_to_host_(long* Mesh_pointer, realw* h_noise_surface_movie) {
  (void)Mesh_pointer; (void)h_noise_surface_movie;
  unsupported("noise tomography (transfer_surface_to_host)");
}

// gravity, ocean load (C-PML: sf3d_pml.cu)
void prepare_fields_gravity_device_(long* Mesh_pointer, int* GRAVITY, realw* minus_deriv_gravity, realw* minus_g,
                                    realw* h_wgll_cube, realw* rhostore) {
  (void)Mesh_pointer; (void)minus_deriv_gravity; (void)minus_g; (void)h_wgll_cube; (void)rhostore;
  if (GRAVITY && *GRAVITY) unsupported("gravity (prepare_fields_gravity_device)");
}
void compute_coupling_ocean_cuda_(long* Mesh_pointer, int* FORWARD_OR_ADJOINT) {
  (void)Mesh_pointer; (void)FORWARD_OR_ADJOINT;
  unsupported("the ocean load (compute_coupling_ocean_cuda)");
}

// dynamic faults (kinematic / rate-and-state / slip-weakening)
void prepare_fault_device_(long* Mesh_pointer, int* KELVIN_VOIGT_DAMPING, realw* Kelvin_Voigt_eta) {
  (void)Mesh_pointer; (void)Kelvin_Voigt_eta;
  if (KELVIN_VOIGT_DAMPING && *KELVIN_VOIGT_DAMPING) unsupported("Kelvin-Voigt damping (prepare_fault_device)");
}
void initialize_fault_solver_gpu_(long* Fault_solver, int* num_of_faults, realw* v_healing, realw* v_rupt,
                                  int* RATE_AND_STATE) {
  (void)Fault_solver; (void)num_of_faults; (void)v_healing; (void)v_rupt; (void)RATE_AND_STATE;
  unsupported("fault simulations (initialize_fault_solver_gpu)");
}
void initialize_fault_data_gpu_(long* Fault_solver, int* fault_index, int* iglob, int* num_of_records, int* ndat,
                                int* NT_RECORD_LENGTH) {
  (void)Fault_solver; (void)fault_index; (void)iglob; (void)num_of_records; (void)ndat; (void)NT_RECORD_LENGTH;
  unsupported("fault simulations (initialize_fault_data_gpu)");
}
void fault_solver_gpu_(long* Mesh_pointer, long* Fault_pointer, realw* dt, int* it) {
  (void)Mesh_pointer; (void)Fault_pointer; (void)dt; (void)it;
  unsupported("fault simulations (fault_solver_gpu)");
}
void transfer_fault_data_to_device_(long* Fault_pointer, int* fault_index, int* NSPEC_FLT, int* NGLOB_FLT, realw* D,
                                    realw* T0, realw* T, realw* B, realw* R, realw* V0, realw* Z, realw* invM1,
                                    realw* invM2, int* ibulk1, int* ibulk2, int* allow_opening) {
  (void)Fault_pointer; (void)fault_index; (void)NSPEC_FLT; (void)NGLOB_FLT; (void)D; (void)T0; (void)T; (void)B;
  (void)R; (void)V0; (void)Z; (void)invM1; (void)invM2; (void)ibulk1; (void)ibulk2; (void)allow_opening;
  unsupported("fault simulations (transfer_fault_data_to_device)");
}
void transfer_fault_data_to_host_(long* Fault_pointer, int* fault_index, int* NSPEC_FLT, int* NGLOB_FLT, realw* D,
                                  realw* V, realw* T) {
  (void)Fault_pointer; (void)fault_index; (void)NSPEC_FLT; (void)NGLOB_FLT; (void)D; (void)V; (void)T;
  unsupported("fault simulations (transfer_fault_data_to_host)");
}
void transfer_datat_to_host_(long* Fault_pointer, int* fault_index, realw* h_dataT, int* it_in) {
  (void)Fault_pointer; (void)fault_index; (void)h_dataT; (void)it_in;
  unsupported("fault simulations (transfer_datat_to_host)");
}
void transfer_rsf_data_todevice_(long* Fault_pointer, int* fault_index, int* NGLOB_FLT, realw* Fload, realw* V0,
                                 realw* f0, realw* V_init, realw* a, realw* b, realw* L, realw* theta, realw* T,
                                 realw* C, realw* fw, realw* Vw, int* StateLaw) {
  (void)Fault_pointer; (void)fault_index; (void)NGLOB_FLT; (void)Fload; (void)V0; (void)f0; (void)V_init; (void)a;
  (void)b; (void)L; (void)theta; (void)T; (void)C; (void)fw; (void)Vw; (void)StateLaw;
  unsupported("fault simulations (transfer_rsf_data_todevice)");
}
void transfer_rsf_data_tohost_(long* Fault_pointer, int* fault_index, int* NGLOB_FLT, realw* V0, realw* f0,
                               realw* V_init, realw* a, realw* b, realw* L, realw* theta, realw* T, realw* C,
                               realw* fw, realw* Vw) {
  (void)Fault_pointer; (void)fault_index; (void)NGLOB_FLT; (void)V0; (void)f0; (void)V_init; (void)a; (void)b;
  (void)L; (void)theta; (void)T; (void)C; (void)fw; (void)Vw;
  unsupported("fault simulations (transfer_rsf_data_tohost)");
}
void transfer_swf_data_todevice_(long* Fault_pointer, int* fault_index, int* NGLOB_FLT, realw* Dc, realw* mus,
                                 realw* mud, realw* T, realw* C, realw* theta) {
  (void)Fault_pointer; (void)fault_index; (void)NGLOB_FLT; (void)Dc; (void)mus; (void)mud; (void)T; (void)C;
  (void)theta;
  unsupported("fault simulations (transfer_swf_data_todevice)");
}
void transfer_swf_data_tohost_(long* Fault_pointer, int* fault_index, int* NGLOB_FLT, realw* Dc, realw* mus,
                               realw* mud, realw* T, realw* C, realw* theta) {
  (void)Fault_pointer; (void)fault_index; (void)NGLOB_FLT; (void)Dc; (void)mus; (void)mud; (void)T; (void)C;
  (void)theta;
  unsupported("fault simulations (transfer_swf_data_tohost)");
}

}  // extern "C"
