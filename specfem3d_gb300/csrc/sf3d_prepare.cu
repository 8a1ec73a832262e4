// Handle set-up, layout conversion, transfers and error reporting.
//
// Replaces src/gpu/prepare_mesh_constants_cuda.cu, transfer_fields_cuda.cu,
// initialize_gpu.cu and helper_functions.cu of the reference: same entry points
// and argument meaning, but host arrays are converted on the device into the
// element-major 128-stride layout described in sf3d_internal.h, and errors are
// recorded (sf3d_last_error) instead of aborting the process.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <mutex>

#include "sf3d_internal.h"

namespace sf3d {

static std::mutex g_err_mu;
static int g_err = SF3D_OK;
static std::string g_err_msg;

bool set_error(int code, const std::string& msg) {
  {
    std::lock_guard<std::mutex> lk(g_err_mu);
    if (g_err == SF3D_OK) {
      g_err = code;
      g_err_msg = msg;
    }
  }
  const char* ab = getenv("SF3D_ABORT_ON_ERROR");
  if (ab && ab[0] == '1') {
    fprintf(stderr, "specfem3d_gb300 error %d: %s\n", code, msg.c_str());
    exit(1);
  }
  return false;
}

bool cuda_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  return set_error(SF3D_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// Allocates and zeroes device memory.  The memset runs on the legacy default
// stream, which does not order with the library's non-blocking stream, so the
// device is synchronised before anything can be queued behind it.
bool alloc_zero(void** d, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (!cuda_ok(cudaMalloc(d, bytes), "cudaMalloc")) return false;
  if (!cuda_ok(cudaMemset(*d, 0, bytes), "cudaMemset")) return false;
  return cuda_ok(cudaDeviceSynchronize(), "cudaDeviceSynchronize");
}

bool ensure_stage(Mesh* mp, size_t bytes) {
  if (mp->stage_bytes >= bytes) return true;
  if (mp->d_stage) cudaFree(mp->d_stage);
  mp->d_stage = nullptr;
  mp->stage_bytes = 0;
  if (!cuda_ok(cudaMalloc((void**)&mp->d_stage, bytes), "cudaMalloc(stage)")) return false;
  mp->stage_bytes = bytes;
  return true;
}

namespace {

// (5,5,5,n) -> [n][128]
__global__ void pad_kernel(float* __restrict__ dst, const float* __restrict__ src, long n) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * NGLL3_PAD) return;
  long e = idx / NGLL3_PAD;
  int p = (int)(idx % NGLL3_PAD);
  dst[idx] = p < NGLL3 ? src[e * NGLL3 + p] : 0.f;
}
__global__ void unpad_kernel(float* __restrict__ dst, const float* __restrict__ src, long n) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * NGLL3) return;
  long e = idx / NGLL3;
  int p = (int)(idx % NGLL3);
  dst[idx] = src[e * NGLL3_PAD + p];
}
// 1-based index array (5,5,5,n) -> 0-based [n][128] (pad entries repeat point 0)
__global__ void pad_int_kernel(int* __restrict__ dst, const int* __restrict__ src, long n) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * NGLL3_PAD) return;
  long e = idx / NGLL3_PAD;
  int p = (int)(idx % NGLL3_PAD);
  dst[idx] = (p < NGLL3 ? src[e * NGLL3 + p] : src[e * NGLL3]) - 1;
}
// (N_SLS,5,5,5,n) -> [n][N_SLS][128]
__global__ void sls_pad_kernel(float* __restrict__ dst, const float* __restrict__ src, long n) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * NSLS * NGLL3_PAD) return;
  long e = idx / (NSLS * NGLL3_PAD);
  int r = (int)(idx % (NSLS * NGLL3_PAD));
  int s = r / NGLL3_PAD, p = r % NGLL3_PAD;
  dst[idx] = p < NGLL3 ? src[(e * NGLL3 + p) * NSLS + s] : 0.f;
}
__global__ void sls_unpad_kernel(float* __restrict__ dst, const float* __restrict__ src, long n) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= n * NGLL3 * NSLS) return;
  int s = (int)(idx % NSLS);
  long q = idx / NSLS;  // e*125 + p
  long e = q / NGLL3;
  int p = (int)(q % NGLL3);
  dst[idx] = src[(e * NSLS + s) * NGLL3_PAD + p];
}

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

}  // namespace

bool upload_padded(float** d, const float* h, long n, cudaStream_t s) {
  if (!alloc_zero((void**)d, sizeof(float) * n * NGLL3_PAD)) return false;
  if (n == 0 || !h) return true;
  float* tmp = nullptr;
  if (!cuda_ok(cudaMalloc((void**)&tmp, sizeof(float) * n * NGLL3), "cudaMalloc(tmp)")) return false;
  bool ok = cuda_ok(cudaMemcpyAsync(tmp, h, sizeof(float) * n * NGLL3, cudaMemcpyHostToDevice, s), "upload");
  if (ok) {
    pad_kernel<<<nblk(n * NGLL3_PAD, 256), 256, 0, s>>>(*d, tmp, n);
    ok = cuda_ok(cudaGetLastError(), "pad_kernel") && cuda_ok(cudaStreamSynchronize(s), "sync");
  }
  cudaFree(tmp);
  return ok;
}

bool upload_padded_int_minus1(int** d, const int* h, long n, cudaStream_t s) {
  if (!alloc_zero((void**)d, sizeof(int) * n * NGLL3_PAD)) return false;
  if (n == 0 || !h) return true;
  int* tmp = nullptr;
  if (!cuda_ok(cudaMalloc((void**)&tmp, sizeof(int) * n * NGLL3), "cudaMalloc(tmp)")) return false;
  bool ok = cuda_ok(cudaMemcpyAsync(tmp, h, sizeof(int) * n * NGLL3, cudaMemcpyHostToDevice, s), "upload");
  if (ok) {
    pad_int_kernel<<<nblk(n * NGLL3_PAD, 256), 256, 0, s>>>(*d, tmp, n);
    ok = cuda_ok(cudaGetLastError(), "pad_int_kernel") && cuda_ok(cudaStreamSynchronize(s), "sync");
  }
  cudaFree(tmp);
  return ok;
}

bool upload_sls_padded(float** d, const float* h, long n, cudaStream_t s) {
  if (!alloc_zero((void**)d, sizeof(float) * n * NSLS * NGLL3_PAD)) return false;
  if (n == 0 || !h) return true;
  float* tmp = nullptr;
  if (!cuda_ok(cudaMalloc((void**)&tmp, sizeof(float) * n * NSLS * NGLL3), "cudaMalloc(tmp)")) return false;
  bool ok = cuda_ok(cudaMemcpyAsync(tmp, h, sizeof(float) * n * NSLS * NGLL3, cudaMemcpyHostToDevice, s), "upload");
  if (ok) {
    sls_pad_kernel<<<nblk(n * NSLS * NGLL3_PAD, 256), 256, 0, s>>>(*d, tmp, n);
    ok = cuda_ok(cudaGetLastError(), "sls_pad_kernel") && cuda_ok(cudaStreamSynchronize(s), "sync");
  }
  cudaFree(tmp);
  return ok;
}

bool download_padded(float* h, const float* d, long n, Mesh* mp) {
  if (!d || !h || n == 0) return true;
  if (!ensure_stage(mp, sizeof(float) * n * NGLL3)) return false;
  unpad_kernel<<<nblk(n * NGLL3, 256), 256, 0, mp->stream>>>(mp->d_stage, d, n);
  if (!cuda_ok(cudaGetLastError(), "unpad_kernel")) return false;
  if (!cuda_ok(cudaMemcpyAsync(h, mp->d_stage, sizeof(float) * n * NGLL3, cudaMemcpyDeviceToHost, mp->stream),
               "download"))
    return false;
  return cuda_ok(cudaStreamSynchronize(mp->stream), "sync");
}

bool download_sls_padded(float* h, const float* d, long n, Mesh* mp) {
  if (!d || !h || n == 0) return true;
  if (!ensure_stage(mp, sizeof(float) * n * NSLS * NGLL3)) return false;
  sls_unpad_kernel<<<nblk(n * NSLS * NGLL3, 256), 256, 0, mp->stream>>>(mp->d_stage, d, n);
  if (!cuda_ok(cudaGetLastError(), "sls_unpad_kernel")) return false;
  if (!cuda_ok(cudaMemcpyAsync(h, mp->d_stage, sizeof(float) * n * NSLS * NGLL3, cudaMemcpyDeviceToHost,
                               mp->stream),
               "download"))
    return false;
  return cuda_ok(cudaStreamSynchronize(mp->stream), "sync");
}

static bool copy_in(void** d, const void* h, size_t bytes, cudaStream_t s) {
  if (!alloc_zero(d, bytes)) return false;
  if (!h || bytes == 0) return true;
  return cuda_ok(cudaMemcpyAsync(*d, h, bytes, cudaMemcpyHostToDevice, s), "cudaMemcpyAsync") &&
         cuda_ok(cudaStreamSynchronize(s), "sync");
}

static void free_fields(Fields& f) {
  cudaFree(f.displ); cudaFree(f.veloc); cudaFree(f.accel);
  for (int c = 0; c < 6; ++c) { cudaFree(f.R[c]); cudaFree(f.eps[c]); }
  cudaFree(f.eps_trace_over_3);
  f = Fields();
}

}  // namespace sf3d

using namespace sf3d;

extern "C" {

int sf3d_last_error(char* msg, int msg_len) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  if (msg && msg_len > 0) {
    strncpy(msg, g_err_msg.c_str(), (size_t)msg_len - 1);
    msg[msg_len - 1] = 0;
  }
  return g_err;
}

void sf3d_clear_error(void) {
  std::lock_guard<std::mutex> lk(g_err_mu);
  g_err = SF3D_OK;
  g_err_msg.clear();
}

int sf3d_version(void) { return 10000; }

void initialize_gpu_device_(int* myrank_f, int* ncuda_devices) {
  int n = 0;
  if (!cuda_ok(cudaGetDeviceCount(&n), "cudaGetDeviceCount")) { if (ncuda_devices) *ncuda_devices = 0; return; }
  if (ncuda_devices) *ncuda_devices = n;
  if (n <= 0) { set_error(SF3D_ERR_CUDA, "no CUDA device visible"); return; }
  int dev = (myrank_f ? *myrank_f : 0) % n;
  cuda_ok(cudaSetDevice(dev), "cudaSetDevice");
}

void prepare_constants_device_(long* Mesh_pointer, int* h_NGLLX, int* NSPEC_AB, int* NGLOB_AB,
                               int* NSPEC_IRREGULAR, int* h_irregular_element_number, realw* h_xix,
                               realw* h_xiy, realw* h_xiz, realw* h_etax, realw* h_etay, realw* h_etaz,
                               realw* h_gammax, realw* h_gammay, realw* h_gammaz, realw* xix_regular,
                               realw* jacobian_regular, int* h_ibool, int* num_interfaces_ext_mesh,
                               int* max_nibool_interfaces_ext_mesh, int* h_nibool_interfaces_ext_mesh,
                               int* h_ibool_interfaces_ext_mesh, realw* h_hprime_xx, realw* h_hprimewgll_xx,
                               realw* h_wgllwgll_xy, realw* h_wgllwgll_xz, realw* h_wgllwgll_yz,
                               int* STACEY_ABSORBING_CONDITIONS, int* h_abs_boundary_ispec,
                               int* h_abs_boundary_ijk, realw* h_abs_boundary_normal,
                               realw* h_abs_boundary_jacobian2Dw, int* h_num_abs_boundary_faces,
                               int* h_ispec_is_inner, int* NSOURCES, int* nsources_local_f,
                               realw* h_sourcearrays, int* h_islice_selected_source,
                               int* h_ispec_selected_source, int* h_ispec_selected_rec, int* nrec,
                               int* nrec_local, int* SIMULATION_TYPE, int* USE_MESH_COLORING_GPU_f,
                               int* nspec_acoustic, int* nspec_elastic, int* ispec_is_acoustic,
                               int* ispec_is_elastic, int* h_myrank, int* SAVE_FORWARD, realw* h_xir,
                               realw* h_etar, realw* h_gammar, double* nu_rec, double* nu_source,
                               int* h_islice_selected_rec, int* nlength_seismogram,
                               int* SAVE_SEISMOGRAMS_DISPLACEMENT, int* SAVE_SEISMOGRAMS_VELOCITY,
                               int* SAVE_SEISMOGRAMS_ACCELERATION, int* SAVE_SEISMOGRAMS_PRESSURE,
                               int* h_NB_RUNS_ACOUSTIC_GPU, int* FAULT_SIMULATION,
                               int* UNDO_ATTENUATION_AND_OR_PML, int* PML_CONDITIONS) {
  (void)h_ispec_is_inner;
  (void)nspec_elastic; (void)ispec_is_elastic;
  (void)FAULT_SIMULATION; (void)nu_source;
  if (!Mesh_pointer) { set_error(SF3D_ERR_ARG, "Mesh_pointer is NULL"); return; }
  *Mesh_pointer = 0;
  if (*h_NGLLX != NGLLX) { set_error(SF3D_ERR_ARG, "NGLLX must be 5"); return; }
  if (h_NB_RUNS_ACOUSTIC_GPU && *h_NB_RUNS_ACOUSTIC_GPU != 1) {
    set_error(SF3D_ERR_ARG, "NB_RUNS_ACOUSTIC_GPU must be 1");
    return;
  }
  if (PML_CONDITIONS && *PML_CONDITIONS) { set_error(SF3D_ERR_ARG, "C-PML is not supported"); return; }
  if (*NSPEC_AB <= 0 || *NGLOB_AB <= 0 || *NSPEC_IRREGULAR < 0 || *NSPEC_IRREGULAR > *NSPEC_AB) {
    set_error(SF3D_ERR_ARG, "invalid NSPEC_AB / NGLOB_AB / NSPEC_IRREGULAR");
    return;
  }
  Mesh* mp = new Mesh();
  mp->use_mesh_coloring = USE_MESH_COLORING_GPU_f ? *USE_MESH_COLORING_GPU_f : 0;
  const long nspec = *NSPEC_AB;
  mp->nspec = (int)nspec;
  mp->nglob = *NGLOB_AB;
  mp->nspec_irregular = *NSPEC_IRREGULAR;
  mp->xix_regular = *xix_regular;
  mp->jacobian_regular = *jacobian_regular;
  mp->simulation_type = *SIMULATION_TYPE;
  mp->undo_attenuation = (UNDO_ATTENUATION_AND_OR_PML && *UNDO_ATTENUATION_AND_OR_PML) ? 1 : 0;
  mp->save_forward = SAVE_FORWARD ? *SAVE_FORWARD : 0;
  bool ok = cuda_ok(cudaStreamCreateWithFlags(&mp->stream, cudaStreamNonBlocking), "cudaStreamCreate") &&
            cuda_ok(cudaEventCreate(&mp->ev0), "event") && cuda_ok(cudaEventCreate(&mp->ev1), "event");
  cudaStream_t s = mp->stream;

  // validate ibool before anything reads through it
  if (ok) {
    const long n = nspec * NGLL3;
    for (long q = 0; q < n; ++q)
      if (h_ibool[q] < 1 || h_ibool[q] > mp->nglob) {
        ok = set_error(SF3D_ERR_ARG, "ibool entry out of range [1, NGLOB_AB]");
        break;
      }
    for (long e = 0; ok && e < nspec; ++e)
      if (h_irregular_element_number[e] < 0 || h_irregular_element_number[e] > mp->nspec_irregular)
        ok = set_error(SF3D_ERR_ARG, "irregular_element_number out of range");
  }
  if (ok) {
    std::vector<int> irr(nspec);
    for (long e = 0; e < nspec; ++e) irr[e] = h_irregular_element_number[e] - 1;
    ok = copy_in((void**)&mp->d_irregular, irr.data(), sizeof(int) * nspec, s);
  }
  if (ok) ok = upload_padded_int_minus1(&mp->d_ibool, h_ibool, nspec, s);
  if (ok && num_interfaces_ext_mesh && *num_interfaces_ext_mesh > 0)
    ok = prepare_interfaces(mp, *num_interfaces_ext_mesh, *max_nibool_interfaces_ext_mesh,
                            h_nibool_interfaces_ext_mesh, h_ibool_interfaces_ext_mesh);
  realw* hm[9] = {h_xix, h_xiy, h_xiz, h_etax, h_etay, h_etaz, h_gammax, h_gammay, h_gammaz};
  for (int q = 0; ok && q < 9; ++q) ok = upload_padded(&mp->d_metric[q], hm[q], mp->nspec_irregular, s);
  if (ok) {
    float gll[5 * 25];
    memcpy(gll, h_hprime_xx, sizeof(float) * 25);
    memcpy(gll + 25, h_hprimewgll_xx, sizeof(float) * 25);
    memcpy(gll + 50, h_wgllwgll_xy, sizeof(float) * 25);
    memcpy(mp->h_hprime, h_hprime_xx, sizeof(float) * 25);
    memcpy(mp->h_hprimewgll, h_hprimewgll_xx, sizeof(float) * 25);
    memcpy(mp->h_wxy, h_wgllwgll_xy, sizeof(float) * 25);
    memcpy(mp->h_wxz, h_wgllwgll_xz, sizeof(float) * 25);
    memcpy(mp->h_wyz, h_wgllwgll_yz, sizeof(float) * 25);
    memcpy(gll + 75, h_wgllwgll_xz, sizeof(float) * 25);
    memcpy(gll + 100, h_wgllwgll_yz, sizeof(float) * 25);
    ok = copy_in((void**)&mp->d_gll, gll, sizeof(gll), s);
  }

  // absorbing faces
  mp->stacey = *STACEY_ABSORBING_CONDITIONS;
  mp->num_abs_faces = *h_num_abs_boundary_faces;
  if (ok && mp->num_abs_faces > 0) {
    const int nf = mp->num_abs_faces;
    std::vector<int> isp(nf), pt((size_t)nf * NGLL2);
    for (int f = 0; f < nf && ok; ++f) {
      isp[f] = h_abs_boundary_ispec[f] - 1;
      if (isp[f] < 0 || isp[f] >= nspec) ok = set_error(SF3D_ERR_ARG, "abs_boundary_ispec out of range");
      for (int g = 0; g < NGLL2 && ok; ++g) {
        const int* ijk = h_abs_boundary_ijk + 3 * (g + NGLL2 * f);
        if (ijk[0] < 1 || ijk[0] > 5 || ijk[1] < 1 || ijk[1] > 5 || ijk[2] < 1 || ijk[2] > 5)
          ok = set_error(SF3D_ERR_ARG, "abs_boundary_ijk out of range");
        pt[(size_t)f * NGLL2 + g] = (ijk[0] - 1) + NGLLX * (ijk[1] - 1) + NGLL2 * (ijk[2] - 1);
      }
    }
    if (ok) ok = copy_in((void**)&mp->d_abs_ispec, isp.data(), sizeof(int) * nf, s);
    if (ok) ok = copy_in((void**)&mp->d_abs_pt, pt.data(), sizeof(int) * pt.size(), s);
    if (ok) ok = copy_in((void**)&mp->d_abs_normal, h_abs_boundary_normal, sizeof(float) * 3 * NGLL2 * nf, s);
    if (ok) ok = copy_in((void**)&mp->d_abs_jw, h_abs_boundary_jacobian2Dw, sizeof(float) * NGLL2 * nf, s);
  }

  // sources (this single-process library owns every source of the slice)
  const int myrank = h_myrank ? *h_myrank : 0;
  mp->nsources = *NSOURCES;
  mp->nsources_local = nsources_local_f ? *nsources_local_f : mp->nsources;
  if (ok && mp->nsources > 0) {
    const int ns = mp->nsources;
    std::vector<float> sa((size_t)ns * NGLL3_PAD * 3, 0.f);
    std::vector<int> isp(ns);
    for (int is = 0; is < ns && ok; ++is) {
      bool here = !h_islice_selected_source || h_islice_selected_source[is] == myrank;
      isp[is] = here ? h_ispec_selected_source[is] - 1 : -1;
      if (here && (isp[is] < 0 || isp[is] >= nspec)) ok = set_error(SF3D_ERR_ARG, "ispec_selected_source out of range");
      if (h_sourcearrays && (mp->simulation_type == 1 || mp->simulation_type == 3))
        for (int p = 0; p < NGLL3; ++p)
          for (int c = 0; c < 3; ++c)
            sa[((size_t)is * NGLL3_PAD + p) * 3 + c] = h_sourcearrays[is + (size_t)ns * (c + 3 * p)];
    }
    if (ok) ok = copy_in((void**)&mp->d_sourcearrays, sa.data(), sizeof(float) * sa.size(), s);
    if (ok) ok = copy_in((void**)&mp->d_ispec_src, isp.data(), sizeof(int) * ns, s);
    if (ok) ok = alloc_zero((void**)&mp->d_stf_step, sizeof(float) * ns);
  }

  // receivers
  mp->nrec = *nrec;
  mp->nrec_local = *nrec_local;
  mp->nlength_seismogram = *nlength_seismogram;
  mp->save_d = *SAVE_SEISMOGRAMS_DISPLACEMENT;
  mp->save_v = *SAVE_SEISMOGRAMS_VELOCITY;
  mp->save_a = *SAVE_SEISMOGRAMS_ACCELERATION;
  mp->save_p = *SAVE_SEISMOGRAMS_PRESSURE;
  if (ok && mp->nrec_local > 0) {
    const int nl = mp->nrec_local;
    std::vector<int> isp;
    std::vector<float> nu;
    for (int r = 0; r < mp->nrec; ++r) {
      if (h_islice_selected_rec && h_islice_selected_rec[r] != myrank) continue;
      isp.push_back(h_ispec_selected_rec[r] - 1);
      for (int q = 0; q < 9; ++q) nu.push_back(nu_rec ? (float)nu_rec[q + 9 * r] : (q % 4 == 0 ? 1.f : 0.f));
    }
    if ((int)isp.size() != nl) ok = set_error(SF3D_ERR_ARG, "nrec_local does not match islice_selected_rec");
    for (size_t r = 0; ok && r < isp.size(); ++r)
      if (isp[r] < 0 || isp[r] >= nspec) ok = set_error(SF3D_ERR_ARG, "ispec_selected_rec out of range");
    if (ok) ok = copy_in((void**)&mp->d_ispec_rec, isp.data(), sizeof(int) * nl, s);
    if (ok) ok = copy_in((void**)&mp->d_nu_rec, nu.data(), sizeof(float) * 9 * nl, s);
    if (ok) ok = copy_in((void**)&mp->d_hxir, h_xir, sizeof(float) * NGLLX * nl, s);
    if (ok) ok = copy_in((void**)&mp->d_hetar, h_etar, sizeof(float) * NGLLX * nl, s);
    if (ok) ok = copy_in((void**)&mp->d_hgammar, h_gammar, sizeof(float) * NGLLX * nl, s);
    const size_t sz = sizeof(float) * 3 * (size_t)nl * (size_t)mp->nlength_seismogram;
    if (ok && mp->save_d) ok = alloc_zero((void**)&mp->d_seismo_d, sz);
    if (ok && mp->save_v) ok = alloc_zero((void**)&mp->d_seismo_v, sz);
    if (ok && mp->save_a) ok = alloc_zero((void**)&mp->d_seismo_a, sz);
  }
  // fluid elements (always kept: the seismogram and source routines need them)
  if (ok) {
    std::vector<int> isac(nspec, 0);
    if (ispec_is_acoustic && nspec_acoustic && *nspec_acoustic > 0)
      for (long e = 0; e < nspec; ++e) isac[e] = ispec_is_acoustic[e] ? 1 : 0;
    ok = copy_in((void**)&mp->d_ispec_is_acoustic, isac.data(), sizeof(int) * nspec, s);
    if (ok && mp->nrec_local > 0) {
      std::vector<int> racs;
      for (int r = 0; r < mp->nrec; ++r) {
        if (h_islice_selected_rec && h_islice_selected_rec[r] != myrank) continue;
        racs.push_back(isac[h_ispec_selected_rec[r] - 1]);
      }
      ok = copy_in((void**)&mp->d_rec_is_acoustic, racs.data(), sizeof(int) * racs.size(), s);
      if (ok && mp->save_p)
        ok = alloc_zero((void**)&mp->d_seismo_p, sizeof(float) * (size_t)mp->nrec_local * mp->nlength_seismogram);
    }
  }
  if (ok) ok = alloc_zero((void**)&mp->d_it, sizeof(int) * 4);
  if (ok) ok = alloc_zero((void**)&mp->d_done, sizeof(unsigned int) * 4);
  if (ok) ok = alloc_zero((void**)&mp->d_scratch, sizeof(float) * 4096);
  if (ok) ok = alloc_zero((void**)&mp->d_kerr, sizeof(int) * 4);
  if (!ok) {
    long tmp = (long)mp;
    prepare_cleanup_device_(&tmp, nullptr, nullptr, nullptr);
    return;
  }
  *Mesh_pointer = (long)mp;
}

void prepare_fields_elastic_device_(long* Mesh_pointer, realw* rmassx, realw* rmassy, realw* rmassz,
                                    realw* rho_vp, realw* rho_vs, realw* h_kappav, realw* h_muv,
                                    int* num_phase_ispec_elastic, int* phase_ispec_inner_elastic,
                                    realw* b_absorb_field, int* b_reclen_field, int* COMPUTE_AND_STORE_STRAIN,
                                    realw* epsilondev_xx, realw* epsilondev_yy, realw* epsilondev_xy,
                                    realw* epsilondev_xz, realw* epsilondev_yz, int* ATTENUATION, int* R_size,
                                    realw* R_xx, realw* R_yy, realw* R_xy, realw* R_xz, realw* R_yz,
                                    realw* factor_common, realw* R_trace, realw* epsilondev_trace,
                                    realw* factor_common_kappa, realw* alphaval, realw* betaval,
                                    realw* gammaval, int* APPROXIMATE_OCEAN_LOAD, realw* rmass_ocean_load,
                                    int* NOISE_TOMOGRAPHY, realw* free_surface_normal, int* free_surface_ispec,
                                    int* free_surface_ijk, int* num_free_surface_faces,
                                    int* ACOUSTIC_SIMULATION, int* num_colors_outer_elastic,
                                    int* num_colors_inner_elastic, int* num_elem_colors_elastic,
                                    int* ANISOTROPY, realw* c11store, realw* c12store, realw* c13store,
                                    realw* c14store, realw* c15store, realw* c16store, realw* c22store,
                                    realw* c23store, realw* c24store, realw* c25store, realw* c26store,
                                    realw* c33store, realw* c34store, realw* c35store, realw* c36store,
                                    realw* c44store, realw* c45store, realw* c46store, realw* c55store,
                                    realw* c56store, realw* c66store) {
  (void)b_absorb_field; (void)b_reclen_field; (void)R_size; (void)rmass_ocean_load; (void)free_surface_normal;
  (void)free_surface_ispec; (void)free_surface_ijk; (void)num_free_surface_faces; (void)ACOUSTIC_SIMULATION;
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (APPROXIMATE_OCEAN_LOAD && *APPROXIMATE_OCEAN_LOAD) { set_error(SF3D_ERR_ARG, "ocean load is not supported"); return; }
  if (NOISE_TOMOGRAPHY && *NOISE_TOMOGRAPHY) { set_error(SF3D_ERR_ARG, "noise tomography is not supported"); return; }
  const long nspec = mp->nspec, nglob = mp->nglob;
  cudaStream_t s = mp->stream;
  bool ok = true;
  ok = ok && alloc_zero((void**)&mp->f.displ, sizeof(float) * 3 * nglob);
  ok = ok && alloc_zero((void**)&mp->f.veloc, sizeof(float) * 3 * nglob);
  ok = ok && alloc_zero((void**)&mp->f.accel, sizeof(float) * 3 * nglob);
  ok = ok && copy_in((void**)&mp->d_rmassx, rmassx, sizeof(float) * nglob, s);
  ok = ok && copy_in((void**)&mp->d_rmassy, rmassy, sizeof(float) * nglob, s);
  ok = ok && copy_in((void**)&mp->d_rmassz, rmassz, sizeof(float) * nglob, s);
  if (mp->d_kappav) { cudaFree(mp->d_kappav); mp->d_kappav = nullptr; }
  ok = ok && upload_padded(&mp->d_kappav, h_kappav, nspec, s);
  ok = ok && upload_padded(&mp->d_muv, h_muv, nspec, s);
  mp->anisotropy = (ANISOTROPY && *ANISOTROPY) ? 1 : 0;
  if (ok && mp->anisotropy) {
    // c11..c66 (5,5,5,NSPEC) each, padded to 128 per element like kappav
    realw* hc[21] = {c11store, c12store, c13store, c14store, c15store, c16store, c22store,
                     c23store, c24store, c25store, c26store, c33store, c34store, c35store,
                     c36store, c44store, c45store, c46store, c55store, c56store, c66store};
    for (int q = 0; q < 21 && ok; ++q) {
      if (!hc[q]) ok = set_error(SF3D_ERR_ARG, "ANISOTROPY needs all 21 c_ij arrays");
      else ok = upload_padded(&mp->d_cstore[q], hc[q], nspec, s);
    }
  }
  if (mp->stacey && mp->num_abs_faces > 0) {
    ok = ok && upload_padded(&mp->d_rho_vp, rho_vp, nspec, s);
    ok = ok && upload_padded(&mp->d_rho_vs, rho_vs, nspec, s);
  }
  // phase element lists (Fortran phase_ispec_inner_elastic(num_phase_ispec,2))
  mp->num_phase_ispec = *num_phase_ispec_elastic;
  if (ok && mp->num_phase_ispec > 0) {
    std::vector<int> ph((size_t)2 * mp->num_phase_ispec);
    for (size_t q = 0; q < ph.size() && ok; ++q) {
      ph[q] = phase_ispec_inner_elastic[q] - 1;
      // entries past nspec_outer/nspec_inner are unused padding; only range-check set ones
      if (ph[q] >= nspec) ok = set_error(SF3D_ERR_ARG, "phase_ispec_inner_elastic out of range");
    }
    // the element counts used later may not reach into padding
    for (int c = 0; c < 2; ++c) {
      int n = 0;
      while (n < mp->num_phase_ispec && ph[(size_t)c * mp->num_phase_ispec + n] >= 0) ++n;
      mp->phase_valid[c] = n;
    }
    if (ok) ok = copy_in((void**)&mp->d_phase_ispec, ph.data(), sizeof(int) * ph.size(), s);
  }
  // colours: num_elem_colors_elastic(num_colors_outer + num_colors_inner), the
  // phase lists ordered colour by colour (outer colours for phase 1, inner for phase 2)
  if (ok && mp->use_mesh_coloring) {
    const int nco = num_colors_outer_elastic ? *num_colors_outer_elastic : 0;
    const int nci = num_colors_inner_elastic ? *num_colors_inner_elastic : 0;
    if (nco < 0 || nci < 0 || (nco + nci > 0 && !num_elem_colors_elastic)) {
      ok = set_error(SF3D_ERR_ARG, "invalid mesh colouring arguments");
    } else {
      long so = 0, si = 0;
      for (int c = 0; c < nco + nci; ++c) {
        if (num_elem_colors_elastic[c] < 0) ok = set_error(SF3D_ERR_ARG, "negative colour size");
        (c < nco ? so : si) += num_elem_colors_elastic[c];
      }
      if (ok && (so > mp->phase_valid[0] || si > mp->phase_valid[1]))
        ok = set_error(SF3D_ERR_ARG, "colour sizes exceed the phase element lists");
      if (ok) {
        mp->num_colors_outer = nco;
        mp->num_colors_inner = nci;
        mp->elem_colors.assign(num_elem_colors_elastic, num_elem_colors_elastic + nco + nci);
      }
    }
  }
  mp->compute_and_store_strain = *COMPUTE_AND_STORE_STRAIN;
  mp->attenuation = *ATTENUATION;
  if (ok && mp->compute_and_store_strain) {
    realw* he[5] = {epsilondev_xx, epsilondev_yy, epsilondev_xy, epsilondev_xz, epsilondev_yz};
    for (int c = 0; c < 5 && ok; ++c) ok = upload_padded(&mp->f.eps[c], he[c], nspec, s);
  }
  if (ok && mp->attenuation) {
    realw* hr[6] = {R_xx, R_yy, R_xy, R_xz, R_yz, R_trace};
    for (int c = 0; c < 6 && ok; ++c) ok = upload_sls_padded(&mp->f.R[c], hr[c], nspec, s);
    ok = ok && upload_padded(&mp->f.eps[5], epsilondev_trace, nspec, s);
    ok = ok && upload_sls_padded(&mp->d_factor_common, factor_common, nspec, s);
    ok = ok && upload_sls_padded(&mp->d_factor_common_kappa, factor_common_kappa, nspec, s);
    for (int q = 0; q < NSLS; ++q) {
      mp->alphaval[q] = alphaval[q];
      mp->betaval[q] = betaval[q];
      mp->gammaval[q] = gammaval[q];
    }
  }
}

void prepare_cleanup_device_(long* Mesh_pointer, int* ACOUSTIC_SIMULATION, int* ELASTIC_SIMULATION,
                             int* NOISE_TOMOGRAPHY) {
  (void)ACOUSTIC_SIMULATION; (void)ELASTIC_SIMULATION; (void)NOISE_TOMOGRAPHY;
  if (!Mesh_pointer || *Mesh_pointer == 0) return;
  Mesh* mp = reinterpret_cast<Mesh*>(*Mesh_pointer);
  if (mp->stream) cudaStreamSynchronize(mp->stream);
  cudaFree(mp->d_ibool); cudaFree(mp->d_irregular);
  for (int q = 0; q < 9; ++q) cudaFree(mp->d_metric[q]);
  cudaFree(mp->d_kappav); cudaFree(mp->d_muv); cudaFree(mp->d_rho_vp); cudaFree(mp->d_rho_vs);
  cudaFree(mp->d_rmassx); cudaFree(mp->d_rmassy); cudaFree(mp->d_rmassz); cudaFree(mp->d_gll);
  cudaFree(mp->d_phase_ispec);
  cudaFree(mp->d_abs_ispec); cudaFree(mp->d_abs_pt); cudaFree(mp->d_abs_normal); cudaFree(mp->d_abs_jw);
  cudaFree(mp->d_sourcearrays); cudaFree(mp->d_ispec_src); cudaFree(mp->d_stf_step); cudaFree(mp->d_stf_table);
  cudaFree(mp->d_ispec_rec); cudaFree(mp->d_hxir); cudaFree(mp->d_hetar); cudaFree(mp->d_hgammar);
  for (int q = 0; q < 21; ++q) cudaFree(mp->d_cstore[q]);
  cudaFree(mp->d_nu_rec); cudaFree(mp->d_seismo_d); cudaFree(mp->d_seismo_v); cudaFree(mp->d_seismo_a);
  cudaFree(mp->d_factor_common); cudaFree(mp->d_factor_common_kappa);
  free_fields(mp->f);
  free_fields(mp->b);
  cudaFree(mp->d_rho_kl); cudaFree(mp->d_mu_kl); cudaFree(mp->d_kappa_kl); cudaFree(mp->d_cijkl_kl);
  for (int q = 0; q < 4; ++q) cudaFree(mp->d_hess_kl[q]);
  cudaFree(mp->d_ispec_adj); cudaFree(mp->d_hxir_adj); cudaFree(mp->d_hetar_adj); cudaFree(mp->d_hgammar_adj);
  cudaFree(mp->d_source_adjoint);
  cudaFree(mp->d_ispec_is_acoustic); cudaFree(mp->d_rhostore); cudaFree(mp->d_potential);
  cudaFree(mp->d_potential_dot); cudaFree(mp->d_potential_dot_dot); cudaFree(mp->d_rmass_acoustic);
  cudaFree(mp->d_b_potential); cudaFree(mp->d_b_potential_dot); cudaFree(mp->d_b_potential_dot_dot);
  cudaFree(mp->d_rho_ac_kl); cudaFree(mp->d_kappa_ac_kl);
  for (int q = 0; q < 3; ++q) cudaFree(mp->d_hess_ac_kl[q]);
  cudaFree(mp->d_phase_ispec_ac); cudaFree(mp->d_fs_ispec); cudaFree(mp->d_fs_pt); cudaFree(mp->d_cp_ispec);
  cudaFree(mp->d_cp_pt); cudaFree(mp->d_cp_normal); cudaFree(mp->d_cp_jw); cudaFree(mp->d_seismo_p);
  cudaFree(mp->d_rec_is_acoustic);
  free_grad(mp);
  free_batch(mp);
  free_geometry_pack(mp);
  free_pml(mp);
  free_interfaces(mp);
  cudaFree(mp->d_it); cudaFree(mp->d_done); cudaFree(mp->d_scratch); cudaFree(mp->d_kerr); cudaFree(mp->d_stage);
  if (mp->ev0) cudaEventDestroy(mp->ev0);
  if (mp->ev1) cudaEventDestroy(mp->ev1);
  for (cudaEvent_t e : mp->tev) cudaEventDestroy(e);
  if (mp->stream) cudaStreamDestroy(mp->stream);
  delete mp;
  *Mesh_pointer = 0;
}

// ---------------------------------------------------------------------------
// field transfers (transfer_fields_cuda.cu)
// ---------------------------------------------------------------------------

static void xfer(long* Mesh_pointer, int* size, realw* h, bool backward, int which, bool to_device) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!size || *size != 3 * mp->nglob) { set_error(SF3D_ERR_ARG, "transfer size must be NDIM*NGLOB_AB"); return; }
  Fields& F = backward ? mp->b : mp->f;
  float* d = which == 0 ? F.displ : (which == 1 ? F.veloc : F.accel);
  if (!d) { set_error(SF3D_ERR_STATE, "field not allocated"); return; }
  size_t bytes = sizeof(float) * (size_t)(*size);
  if (to_device)
    SF3D_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, mp->stream));
  else
    SF3D_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, mp->stream));
  SF3D_CUDA(cudaStreamSynchronize(mp->stream));
}

void transfer_fields_el_to_device_(int* size, realw* displ, realw* veloc, realw* accel, long* Mesh_pointer) {
  xfer(Mesh_pointer, size, displ, false, 0, true);
  xfer(Mesh_pointer, size, veloc, false, 1, true);
  xfer(Mesh_pointer, size, accel, false, 2, true);
}
void transfer_fields_el_from_device_(int* size, realw* displ, realw* veloc, realw* accel, long* Mesh_pointer) {
  xfer(Mesh_pointer, size, displ, false, 0, false);
  xfer(Mesh_pointer, size, veloc, false, 1, false);
  xfer(Mesh_pointer, size, accel, false, 2, false);
}
void transfer_b_fields_to_device_(int* size, realw* d, realw* v, realw* a, long* Mesh_pointer) {
  xfer(Mesh_pointer, size, d, true, 0, true);
  xfer(Mesh_pointer, size, v, true, 1, true);
  xfer(Mesh_pointer, size, a, true, 2, true);
}
void transfer_b_fields_from_device_(int* size, realw* d, realw* v, realw* a, long* Mesh_pointer) {
  xfer(Mesh_pointer, size, d, true, 0, false);
  xfer(Mesh_pointer, size, v, true, 1, false);
  xfer(Mesh_pointer, size, a, true, 2, false);
}
void transfer_displ_from_device_(int* size, realw* d, long* Mesh_pointer) { xfer(Mesh_pointer, size, d, false, 0, false); }
void transfer_displ_to_device_(int* size, realw* d, long* Mesh_pointer) { xfer(Mesh_pointer, size, d, false, 0, true); }
void transfer_veloc_from_device_(int* size, realw* v, long* Mesh_pointer) { xfer(Mesh_pointer, size, v, false, 1, false); }
void transfer_veloc_to_device_(int* size, realw* v, long* Mesh_pointer) { xfer(Mesh_pointer, size, v, false, 1, true); }
void transfer_accel_from_device_(int* size, realw* a, long* Mesh_pointer) { xfer(Mesh_pointer, size, a, false, 2, false); }
void transfer_accel_to_device_(int* size, realw* a, long* Mesh_pointer) { xfer(Mesh_pointer, size, a, false, 2, true); }
void transfer_b_displ_from_device_(int* size, realw* d, long* Mesh_pointer) { xfer(Mesh_pointer, size, d, true, 0, false); }
void transfer_b_displ_to_device_(int* size, realw* d, long* Mesh_pointer) { xfer(Mesh_pointer, size, d, true, 0, true); }

void transfer_rmemory_from_device_(long* Mesh_pointer, realw* R_xx, realw* R_yy, realw* R_xy, realw* R_xz,
                                   realw* R_yz, realw* R_trace, int* size_R) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!mp->attenuation) { set_error(SF3D_ERR_STATE, "attenuation arrays not allocated"); return; }
  if (!size_R || *size_R != NSLS * NGLL3 * mp->nspec) { set_error(SF3D_ERR_ARG, "size_R must be N_SLS*NGLL3*NSPEC"); return; }
  realw* h[6] = {R_xx, R_yy, R_xy, R_xz, R_yz, R_trace};
  for (int c = 0; c < 6; ++c)
    if (!download_sls_padded(h[c], mp->f.R[c], mp->nspec, mp)) return;
}

void transfer_strain_from_device_(long* Mesh_pointer, realw* exx, realw* eyy, realw* exy, realw* exz, realw* eyz,
                                  realw* etr, int* size_epsilondev) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (!size_epsilondev || *size_epsilondev != NGLL3 * mp->nspec) {
    set_error(SF3D_ERR_ARG, "size_epsilondev must be NGLL3*NSPEC");
    return;
  }
  realw* h[6] = {exx, eyy, exy, exz, eyz, etr};
  for (int c = 0; c < 6; ++c)
    if (mp->f.eps[c] && !download_padded(h[c], mp->f.eps[c], mp->nspec, mp)) return;
}

void* sf3d_device_ptr(long* Mesh_pointer, const char* name) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp || !name) return nullptr;
  std::string n(name);
  if (n == "displ") return mp->f.displ;
  if (n == "veloc") return mp->f.veloc;
  if (n == "accel") return mp->f.accel;
  if (n == "b_displ") return mp->b.displ;
  if (n == "b_veloc") return mp->b.veloc;
  if (n == "b_accel") return mp->b.accel;
  if (n == "seismograms_d") return mp->d_seismo_d;
  if (n == "rho_kl") return mp->d_rho_kl;
  if (n == "mu_kl") return mp->d_mu_kl;
  if (n == "kappa_kl") return mp->d_kappa_kl;
  return nullptr;
}

int sf3d_synchronize(long* Mesh_pointer) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (cuda_ok(cudaStreamSynchronize(mp->stream), "cudaStreamSynchronize")) check_kernel_error(mp);
  return sf3d_last_error(nullptr, 0);
}

}  // extern "C"
