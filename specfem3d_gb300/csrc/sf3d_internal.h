// Internal definitions of the GB300 spectral-element library.
//
// Device layout (chosen for coalesced, 16-byte-aligned element streams on HBM):
//   * per-element arrays are stored element-major with a 128-point stride
//     (125 GLL points + 3 pad), so each element's array is one aligned 512-byte
//     row: ibool[e*128 + p] (0-based global index), kappa/mu[e*128 + p],
//     metric m[e_irr*128 + p] for irregular elements only;
//   * attenuation memory variables are [e][sls][128] (three 512-byte rows per
//     element and component), epsilondev [e][128];
//   * wavefields keep the reference's interleaved (3, NGLOB) layout so the
//     host transfers of the Fortran arrays are plain copies.
#pragma once

#include <nvtx3/nvToolsExt.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/specfem3d_gb300.h"

#define NGLLX 5
#define NGLL2 25
#define NGLL3 125
#define NGLL3_PAD 128
#define NSLS 3

namespace sf3d {

// Records the first error; returns false on failure so callers can bail out.
bool set_error(int code, const std::string& msg);

// NVTX range over one library call (header-only NVTX v3: inactive unless a
// profiler is attached), so timelines show the step blocks, sweeps and passes
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};
// acoustic Hessian kernels of one step (sf3d_acoustic.cu)
struct Mesh;
bool launch_hess_acoustic(Mesh* mp, double dt);
bool cuda_ok(cudaError_t e, const char* what);
#define SF3D_CUDA(call)                           \
  do {                                            \
    if (!::sf3d::cuda_ok((call), #call)) return;  \
  } while (0)
#define SF3D_CUDA_RET(call, ret)                      \
  do {                                                \
    if (!::sf3d::cuda_ok((call), #call)) return ret;  \
  } while (0)

// Static per-element streams of the stiffness kernel in packed form.  Stream q:
// 0-8 the metric (xix xiy xiz etax etay etaz gammax gammay gammaz; irregular
// elements), 9 kappa, 10 mu, 11-13 factor_common, 14-16 factor_common_kappa.
// value(q, p) = so[q].x                                  if bit q of vary is clear
//             = so[q].x + so[q].y * pool[row(q)][p]      otherwise, with
// row(q) = base + popcount(vary & ((1 << q) - 1)): only the streams that vary
// inside the element carry a 128-value payload row.
constexpr int kPackStreams = 17;
enum GeomFormat { kGeomFP32 = 0, kGeomPackF16 = 1, kGeomPackBF16 = 2, kGeomPackF32 = 3 };
struct __align__(16) ElemPack {
  float2 so[kPackStreams];  // (offset, scale)
  unsigned vary;            // bit q: stream q has a payload row
  int base;                 // first payload row of this element
  int pad[4];
};
static_assert(sizeof(ElemPack) == 160, "ElemPack is five 32-byte sectors");

// payload value i of a packed pool in the format GEOM
template <int GEOM>
__device__ __forceinline__ float pool_value(const void* pool, long i) {
  if (GEOM == kGeomPackF16)
    return __half2float(__ushort_as_half(__ldg(static_cast<const unsigned short*>(pool) + i)));
  if (GEOM == kGeomPackBF16)
    return __bfloat162float(__ushort_as_bfloat16(__ldg(static_cast<const unsigned short*>(pool) + i)));
  return __ldg(static_cast<const float*>(pool) + i);
}

// mbarrier and bulk-copy (TMA, non-tensor) helpers.  Every wait is bounded:
// mbar_wait_bounded gives up after ~2 s of %globaltimer and returns false, and
// the caller records an error word instead of spinning on.
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// bounded wait: true when the phase completed, false after limit_ns (2 s unless
// a caller asks for another bound)
constexpr uint64_t kWaitLimitNs = 2000000000ull;
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint64_t limit_ns = kWaitLimitNs) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

__device__ __forceinline__ void bulk_g2s(void* dst_smem, const void* src_gmem, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst_smem)),
      "l"(reinterpret_cast<uint64_t>(src_gmem)), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 4-byte asynchronous global -> shared copy (cp.async; completes at
// cp.async.wait_all of the issuing thread)
__device__ __forceinline__ void cp_async4(void* smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(static_cast<unsigned>(__cvta_generic_to_shared(smem))),
               "l"(gmem)
               : "memory");
}

// value of stream q at point t of the element whose record is pk (vary, base: its
// varying-stream mask and first payload row, read once per element)
template <int GEOM>
__device__ __forceinline__ float pack_value(const ElemPack* pk, const void* pool, unsigned vary, int base, int q,
                                            int t) {
  const float2 so = __ldg(&pk->so[q]);
  if (!((vary >> q) & 1u)) return so.x;
  const long row = (long)base + __popc(vary & ((1u << q) - 1u));
  return fmaf(so.y, pool_value<GEOM>(pool, row * NGLL3_PAD + t), so.x);
}

struct Fields {
  float* displ = nullptr;
  float* veloc = nullptr;
  float* accel = nullptr;
  // attenuation memory variables [e][sls][128] and strains [e][128]
  float* R[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // xx yy xy xz yz trace
  float* eps[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};  // xx yy xy xz yz trace
  float* eps_trace_over_3 = nullptr;                                      // [e][128]
};

// Checkpointed discrete-adjoint gradient state (sf3d_gradient_*).
struct GradState {
  int nstep = 0, every = 0, nckpt = 0;
  float* ckpt = nullptr;       // [nckpt][3][3*nglob]: displ, veloc, accel at segment starts
  // [every][seg_stride]: displacement / force (before the mass matrix) after each step
  // of a segment; seg_stride = 3*nglob rounded up to a multiple of 4, so that every
  // step's slice starts on a 16-byte boundary (the step kernels use 16-byte accesses)
  float* seg_u = nullptr;
  float* seg_a = nullptr;
  size_t seg_stride = 0;
  float* adj_u = nullptr;      // adjoint of displacement, velocity, acceleration [3*nglob]
  float* adj_v = nullptr;
  float* adj_a = nullptr;
  float* p = nullptr;          // -M^-1 (adjoint of the new acceleration) [3*nglob]
  float* kp = nullptr;         // -K p   [3*nglob]
  float* bp = nullptr;         // -B p   [3*nglob]
  float* residual = nullptr;   // (3, nrec, nstep): dJ/d(seismogram sample)
  double* g_rho = nullptr;     // [nspec][128] dJ/d(rho), dJ/d(kappa), dJ/d(mu) per GLL point
  double* g_kappa = nullptr;
  double* g_mu = nullptr;
  float wgll[NGLLX] = {};
  double res_scale = 1.0;      // power of two applied to the residual (undone in sf3d_gradient_get)
  float u_scale = 1.f;         // power of two applied to the forward field in the strain products
  int fused = 1;               // 1: K p and the gradient terms in one kernel per element
  size_t bytes = 0;
};

// Many shots on one mesh (sf3d_batch_*): wavefields stacked shot-innermost,
// index (3 * iglob + component) * nshots + shot.
struct BatchState {
  int nshots = 0, nstep = 0, nlength = 0;
  int shots_per_block = 8, elements_per_block = 1;
  int shots_per_thread = 1;     // 4: vector kernel (shots_per_block 4 or 8)
  int pencil_lanes = 0;         // > 0: register-blocked pencil kernel, shots per CTA (8, 16, 32)
  float* displ = nullptr;
  float* veloc = nullptr;
  float* accel = nullptr;
  int* d_ispec_src = nullptr;   // [nshots] 0-based element of each shot's source
  float* d_sa = nullptr;        // [nshots][128][3] source arrays
  float* d_stf = nullptr;       // [nstep][nshots]
  float* d_seismo = nullptr;    // [nlength][nshots][nrec_local][3]
  int* d_it = nullptr;          // device step counters (1-based), one per shot half
  size_t bytes = 0;
  float last_ms = 0.f;
  int last_launches = 0;
  // 2: the two shot halves advance as two independent chains on two streams
  // (shots never interact), the correctors launched at the higher priority so
  // that one half's HBM-bound corrector runs beside the other half's stiffness
  // (pencil kernel only)
  int halves = 1;
  int prio_hi = 0;              // greatest stream priority of the device
  cudaStream_t side = nullptr;
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

struct Mesh {
  int nspec = 0, nglob = 0, nspec_irregular = 0;
  float xix_regular = 0.f, jacobian_regular = 0.f;
  int simulation_type = 1;
  int save_forward = 0;

  // geometry / material (element-major, 128 stride)
  int* d_ibool = nullptr;                // [nspec][128] 0-based
  int* d_irregular = nullptr;            // [nspec] 0-based irregular index, -1 if regular
  float* d_metric[9] = {};               // [nspec_irr][128] xix xiy xiz etax etay etaz gammax gammay gammaz
  float* d_kappav = nullptr;             // [nspec][128]
  float* d_muv = nullptr;                // [nspec][128]
  float* d_rho_vp = nullptr;             // [nspec][128]
  float* d_rho_vs = nullptr;             // [nspec][128]
  int anisotropy = 0;
  float* d_cstore[21] = {};              // ANISOTROPY c11..c66, each [nspec][128]
  float* d_rmassx = nullptr;             // [nglob]
  float* d_rmassy = nullptr;
  float* d_rmassz = nullptr;
  float h_hprime[25] = {}, h_hprimewgll[25] = {}, h_wxy[25] = {}, h_wxz[25] = {}, h_wyz[25] = {};
  float* d_gll = nullptr;                // [5*25]: hprime, hprimewgll, wxy, wxz, wyz

  // phases: [2][num_phase_ispec] 0-based element lists
  int num_phase_ispec = 0;
  int phase_valid[2] = {0, 0};           // leading in-range entries of each phase column
  // mesh colouring (USE_MESH_COLORING_GPU): phase lists ordered by colour, no two
  // elements of a colour share a point, so a colour's scatter needs no atomics
  int use_mesh_coloring = 0;
  int num_colors_outer = 0, num_colors_inner = 0;
  std::vector<int> elem_colors;          // elements per colour, outer colours first
  int nspec_outer = 0, nspec_inner = 0;
  int* d_phase_ispec = nullptr;

  // Stacey
  int stacey = 0;
  int num_abs_faces = 0;
  int* d_abs_ispec = nullptr;            // [nf] 0-based
  int* d_abs_pt = nullptr;               // [nf][25] element-local point index p = i+5j+25k
  float* d_abs_normal = nullptr;         // [nf][25][3]
  float* d_abs_jw = nullptr;             // [nf][25]

  // sources
  int nsources = 0, nsources_local = 0;
  float* d_sourcearrays = nullptr;       // [nsrc][128][3] (point-major, xyz innermost)
  int* d_ispec_src = nullptr;            // [nsrc] 0-based
  int* h_ispec_src = nullptr;
  float* d_stf_step = nullptr;           // [nsrc] stf of the current ABI call
  float* d_stf_table = nullptr;          // [nstep][nsrc]
  int stf_nstep = 0;

  // receivers
  int nrec = 0, nrec_local = 0;
  int nlength_seismogram = 0;
  int save_d = 0, save_v = 0, save_a = 0, save_p = 0;
  int* d_ispec_rec = nullptr;            // [nrec_local] 0-based
  float* d_hxir = nullptr;               // [nrec_local][5] each
  float* d_hetar = nullptr;
  float* d_hgammar = nullptr;
  float* d_nu_rec = nullptr;             // [nrec_local][9]
  float* d_seismo_d = nullptr;           // (3, nrec_local, nlength)
  float* d_seismo_v = nullptr;
  float* d_seismo_a = nullptr;

  // attenuation
  int attenuation = 0;
  int compute_and_store_strain = 0;
  // UNDO_ATTENUATION_AND_OR_PML: the backward field is recomputed forward in time
  // from snapshots and its strain is recomputed from b_displ before each kernel
  // accumulation (compute_kernels_cuda.cu:57)
  int undo_attenuation = 0;
  float alphaval[NSLS] = {}, betaval[NSLS] = {}, gammaval[NSLS] = {};
  float b_alphaval[NSLS] = {}, b_betaval[NSLS] = {}, b_gammaval[NSLS] = {};
  float* d_factor_common = nullptr;      // [nspec][3][128]
  float* d_factor_common_kappa = nullptr;

  Fields f;   // forward (or adjoint) field
  Fields b;   // backward / reconstructed field (SIMULATION_TYPE == 3)

  // adjoint kernels (SIMULATION_TYPE == 3): [nspec][128], FP64 accumulation
  double* d_rho_kl = nullptr;
  double* d_mu_kl = nullptr;
  double* d_kappa_kl = nullptr;
  int anisotropic_kl = 0, hess_kl = 0;
  double* d_cijkl_kl = nullptr;          // ANISOTROPIC_KL: [nspec][128][21]
  double* d_hess_kl[4] = {};             // APPROXIMATE_HESS_KL: hess, hess_rho, hess_kappa, hess_mu
  int nadj_rec_local = 0;
  int ntstep_between_read_adjsrc = 0;
  int* d_ispec_adj = nullptr;             // [nadj_rec_local] 0-based
  float* d_hxir_adj = nullptr;            // [nadj][5]
  float* d_hetar_adj = nullptr;
  float* d_hgammar_adj = nullptr;
  float* d_source_adjoint = nullptr;      // (3, nadj, NTSTEP_BETWEEN_READ_ADJSRC)

  // acoustic domain and fluid-solid coupling
  int* d_ispec_is_acoustic = nullptr;     // [nspec] 0/1
  int has_acoustic = 0;
  float* d_rhostore = nullptr;            // [nspec][128]
  float* d_potential = nullptr;
  float* d_potential_dot = nullptr;
  float* d_potential_dot_dot = nullptr;
  // SIMULATION_TYPE = 3 in fluid elements: backward potentials and the FP64
  // rho / kappa kernel accumulators [nspec][128] (prepare_fields_acoustic_adj_dev)
  float* d_b_potential = nullptr;
  float* d_b_potential_dot = nullptr;
  float* d_b_potential_dot_dot = nullptr;
  double* d_rho_ac_kl = nullptr;
  double* d_kappa_ac_kl = nullptr;
  // 1: fluid kernels pair the adjoint chi_dd (the discrete adjoint variable of the
  // fluid) instead of chi (the reference's formula); sf3d_set_acoustic_kernel_pairing
  int ac_kernel_discrete = 0;
  // APPROXIMATE_HESS_KL in fluid elements: hess_ac_kl, hess_rho_ac_kl, hess_kappa_ac_kl
  double* d_hess_ac_kl[3] = {nullptr, nullptr, nullptr};
  float* d_rmass_acoustic = nullptr;
  int num_phase_ispec_ac = 0, nspec_outer_ac = 0, nspec_inner_ac = 0;
  int phase_valid_ac[2] = {0, 0};
  int* d_phase_ispec_ac = nullptr;        // [2][num_phase_ispec_ac] 0-based
  int num_free_surface_faces = 0;
  int* d_fs_ispec = nullptr;              // [nf] 0-based
  int* d_fs_pt = nullptr;                 // [nf][25]
  int num_coupling_faces = 0;
  int* d_cp_ispec = nullptr;
  int* d_cp_pt = nullptr;
  float* d_cp_normal = nullptr;           // [nf][25][3]
  float* d_cp_jw = nullptr;               // [nf][25]
  float* d_seismo_p = nullptr;            // (nrec_local, nlength)
  int* d_rec_is_acoustic = nullptr;       // [nrec_local]

  // device step counter for graph-captured time loops, and completion counter
  int* d_it = nullptr;
  unsigned int* d_done = nullptr;
  // fluid-solid meshes: the global points (0-based, first and count) spanned by
  // the solid and by the fluid elements; the fused time loop runs the solid and
  // fluid predictor/corrector passes over these spans only (count -1: not
  // computed, the passes cover every point)
  long el_first = 0, el_count = -1, ac_first = 0, ac_count = -1;
  float* d_scratch = nullptr;             // reduction scratch
  int* d_kerr = nullptr;                  // kernel error word (bounded waits that timed out)
  GradState* grad = nullptr;              // checkpointed adjoint gradient (optional)
  BatchState* batch = nullptr;            // batched shots (optional)

  // MPI interfaces of this slice (inter-slice assembly of accel)
  int num_interfaces = 0, max_nibool_interfaces = 0;
  long size_mpi_buffer = 0;               // NDIM * max_nibool * num_interfaces
  int* d_nibool_interfaces = nullptr;     // [num_interfaces]
  int* d_ibool_interfaces = nullptr;      // [num_interfaces][max_nibool] 0-based
  float* d_send_accel_buffer = nullptr;   // (3, max_nibool, num_interfaces)
  float* d_b_send_accel_buffer = nullptr;
  float* h_send_accel_buffer = nullptr;   // pinned staging
  float* h_recv_accel_buffer = nullptr;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_pack = nullptr;          // packing done on the compute stream
  int stiffness_variant = 3;              // see variant_blocks_per_sm; 1: persistent bulk-copy pipeline
  // packed static element streams of the stiffness kernel (sf3d_set_geometry_format):
  // one ElemPack record per element, payload rows only for streams that vary
  int geom_format = 0;                    // kGeomFP32 (plain arrays) ... kGeomPackF32
  ElemPack* d_pack = nullptr;             // [nspec]
  void* d_pack_pool = nullptr;            // [pack_rows][128] FP16 / BF16 / FP32 values
  long pack_rows = 0;

  // C-PML layers (prepare_fields_elastic_pml): forward field only
  int pml = 0, nspec_cpml = 0;
  int* d_is_cpml = nullptr;               // [nspec] 0/1
  int* d_spec_to_cpml = nullptr;          // [nspec] 0-based CPML index, -1 outside the layers
  int* d_cpml_to_spec = nullptr;          // [nspec_cpml] 0-based
  float* d_pml_coef = nullptr;            // [nspec_cpml][41][128]: alpha 9, beta 9, A-bar 5, strain 18
  float* d_pml_rmem = nullptr;            // [nspec_cpml][48][128] convolution memory variables
  float* d_pml_displ_old = nullptr;       // [nspec_cpml][3][128]
  float* d_pml_displ_new = nullptr;
  float* d_wgll_cube = nullptr;           // [128]
  int* d_phase_nopml = nullptr;           // [2][num_phase_ispec] phase lists without the CPML elements
  int* d_phase_pml = nullptr;             // [2][num_phase_ispec] the CPML elements of each phase
  int phase_nopml_n[2] = {0, 0}, phase_pml_n[2] = {0, 0};

  cudaStream_t stream = nullptr;
  // deferred mass + corrector of the forward [0] and backward [1] field, and its dt/2
  int pend_corrector[2] = {0, 0};
  float pend_dt2[2] = {0.f, 0.f};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<cudaEvent_t> tev;           // timing mode: start/end event per stiffness step
  float last_stiff_ms = 0.f, last_total_ms = 0.f;
  int last_stiff_launches = 0, last_total_launches = 0;

  // staging buffer for layout conversions
  float* d_stage = nullptr;
  size_t stage_bytes = 0;
};

// Applies deferred mass/corrector passes (kernel_3_a_cuda leaves its work for the
// next update_displacement_cuda, which fuses it with the predictor).
void flush_correctors(Mesh* mp);

// Every entry point fetches its Mesh here; by default any deferred corrector is
// applied first, so entry points that read or write veloc / accel see the state
// the reference would leave.
inline Mesh* get_mesh(long* p, bool flush = true) {
  if (!p || *p == 0) {
    set_error(SF3D_ERR_STATE, "Mesh_pointer is not prepared");
    return nullptr;
  }
  Mesh* mp = reinterpret_cast<Mesh*>(*p);
  if (flush && (mp->pend_corrector[0] || mp->pend_corrector[1])) flush_correctors(mp);
  return mp;
}

// element-major upload of a (5,5,5,n) host array into [n][128]
bool upload_padded(float** d, const float* h, long n, cudaStream_t s);
bool upload_padded_int_minus1(int** d, const int* h, long n, cudaStream_t s);
bool upload_sls_padded(float** d, const float* h, long n, cudaStream_t s);
bool download_padded(float* h, const float* d, long n, Mesh* mp);
bool download_sls_padded(float* h, const float* d, long n, Mesh* mp);
bool alloc_zero(void** d, size_t bytes);
// stream-ordered copy that returns when the copy has completed
inline bool copy_sync(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
  return cuda_ok(cudaMemcpyAsync(dst, src, bytes, kind, s), "cudaMemcpyAsync") &&
         cuda_ok(cudaStreamSynchronize(s), "cudaStreamSynchronize");
}
bool ensure_stage(Mesh* mp, size_t bytes);

// kernels launched from several translation units
struct StiffnessArgs {
  int nelem;
  const int* phase;             // element list (0-based) or nullptr (identity)
  const int* ibool;
  const int* irregular;
  const float* m[9];
  const float* kappav;
  const float* muv;
  const float* gll;             // hprime, hprimewgll, wxy, wxz, wyz
  float xix_regular;
  float jacobian_regular;
  float deltat;
  const float* displ;
  const float* veloc;
  float* accel;
  float* R[6];
  float* eps[6];
  float* eps_trace_over_3;
  const float* fc;
  const float* fck;
  float alpha[NSLS], beta[NSLS], gamma[NSLS];
  // packed static streams (sf3d_set_geometry_format); nullptr: the FP32 arrays above
  const ElemPack* pack;         // [nspec]
  const void* pool;             // payload rows
  int nonatomic;                // 1: the elements of this launch share no point (one colour)
  int* err;                     // kernel error word (a bounded wait that timed out), or nullptr
  // ANISOTROPY: c11 c12 c13 c14 c15 c16 c22 c23 c24 c25 c26 c33 c34 c35 c36 c44
  // c45 c46 c55 c56 c66, each [nspec][128]; nullptr for isotropic meshes
  const float* c[21];
};

void launch_stiffness(const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s, int blocks_per_sm,
                      int geom_format = kGeomFP32, bool staged = false, bool streaming = false, bool bulk = false);
// one wavefield without attenuation, register-blocked pencils (sf3d_elastic_pencil.cu):
// five elements per CTA, a thread per (element, z-line), 8 or 7 CTAs/SM
struct ElemPencilArgs {
  int nelem;
  const int* phase;             // element list (0-based) or nullptr (identity)
  const int* ibool;
  const int* irregular;
  const float* m[9];
  const float* kappav;
  const float* muv;
  const float* gll;             // hprime, hprimewgll, wxy, wxz, wyz
  float xix_regular;
  float jacobian_regular;
  const float* displ;
  float* accel;
  float hp[NGLL2];              // hprime, hprimewgll by value (parameter bank)
  float hpw[NGLL2];
  float ek[12];                 // their even / odd coefficients (eo5)
  float ekw[12];
};
bool launch_elem_pencil(const ElemPencilArgs& a, int blocks_per_sm, cudaStream_t s);
struct Mesh;
void run_elem_pencil(Mesh* mp, const StiffnessArgs& a, int blocks_per_sm, cudaStream_t s);
// batched-shots stiffness with register-blocked pencils (sf3d_batch_pencil.cu):
// elements of a phase list x shots [shot_offset, shot_offset + shot_tiles * lanes)
// of fields stacked shot-innermost with nshots shots per point
struct PencilArgs {
  int nelem;
  int nshots;                   // stride of the stacked fields
  int shot_offset;              // first shot of this launch
  int shot_tiles;               // CTAs per element (shots of this launch / lanes)
  const int* phase;
  const int* ibool;
  const int* irregular;
  const float* m[9];
  const float* kappav;
  const float* muv;
  const ElemPack* pack;         // packed static streams, or nullptr
  const void* pool;
  const float* gll;
  float xix_regular;
  float jacobian_regular;
  const float* displ;
  float* accel;
  // hprime and hprimewgll by value: the pencil loops index them with
  // compile-time constants, so every FMA reads its coefficient from the
  // kernel's parameter bank instead of shared memory
  float hp[NGLL2];
  float hpw[NGLL2];
  // even / odd coefficients of hprime (ek: out_o = sum_l hprime(o, l) v_l) and of
  // hprimewgll transposed (ekw: out_o = sum_l hprimewgll(l, o) v_l), see eo5
  float ek[12];
  float ekw[12];
};
// even / odd coefficients of a centro-antisymmetric 5x5 matrix M[o][l] = m[o * so + l * sl]
void even_odd_coefficients(const float* m, int so, int sl, float k[12]);
// out[o] = sum_l M[o][l] v[l] for the 5x5 GLL derivative matrices, which are
// centro-antisymmetric (M[4-o][4-l] = -M[o][l], the GLL points being symmetric):
// from the even and odd parts e_l = v_l + v_{4-l}, d_l = v_l - v_{4-l},
//   out_o, out_{4-o} = S_o +- A_o,  S_o = a_o0 d_0 + a_o1 d_1,
//   A_o = b_o0 e_0 + b_o1 e_1 + c_o v_2   (o = 0, 1),   out_2 = m_20 d_0 + m_21 d_1,
// 20 operations instead of 25 FMAs (k: a00 a01 b00 b01 c0 a10 a11 b10 b11 c1 m20 m21)
__device__ __forceinline__ void eo5(const float v[NGLLX], const float* k, float out[NGLLX]) {
  const float e0 = v[0] + v[4], e1 = v[1] + v[3], d0 = v[0] - v[4], d1 = v[1] - v[3];
  const float v2 = v[2];
#pragma unroll
  for (int o = 0; o < 2; ++o) {
    const float* q = k + 5 * o;
    const float S = fmaf(q[1], d1, q[0] * d0);
    const float A = fmaf(q[4], v2, fmaf(q[3], e1, q[2] * e0));
    out[o] = S + A;
    out[4 - o] = S - A;
  }
  out[2] = fmaf(k[11], d1, k[10] * d0);
}

bool launch_batch_pencil(const PencilArgs& a, int lanes, int geom_format, cudaStream_t s);

void launch_stiffness_pipelined(const StiffnessArgs& a, bool att, bool store_strain, int* err, cudaStream_t s);
// stiffness kernel variants (sf3d_set_stiffness_variant / sf3d_autotune_stiffness)
//   0, 2, 3, 4: one CTA per element at 4, 5, 6, 7 CTAs/SM; 1: persistent bulk-copy pipeline;
//   5, 6, 7: one CTA per element with cp.async-staged memory variables at 6, 7, 8 CTAs/SM;
//   8, 9: one CTA per element, evict-first hints on the element streams, 6 and 7 CTAs/SM;
//   10, 11: three threads per point (384-thread CTAs), 3 and 4 CTAs/SM;
//   12, 13, 14: one CTA per element with the memory variables, strains and
//   attenuation factors brought into shared memory by 14 bulk copies (one
//   thread, one mbarrier) at 8, 9, 10 CTAs/SM (without attenuation: the plain
//   build at 8, 10, 12 CTAs/SM)
// Under a packed geometry format (sf3d_set_geometry_format) 4 selects the packed
// build at 7 CTAs/SM, 5, 6, 7 the packed builds with cp.async-staged memory
// variables at 8, 9, 10 CTAs/SM, 12, 13, 14 the packed builds with bulk-copied
// ones at 8, 9, 10, and every other variant the packed build at 6.
constexpr int kNumStiffnessVariants = 17;
inline int variant_blocks_per_sm(int v) {
  // 15, 16: the register-blocked pencil kernel without attenuation (five
  // elements a CTA, 8 and 7 CTAs/SM); the other builds (attenuation, strain,
  // packed or anisotropic streams) run the default 6-CTA build under these numbers
  const int t[kNumStiffnessVariants] = {4, 0, 5, 6, 7, 6, 7, 8, 6, 7, 3, 4, 8, 9, 10, 6, 6};
  return (v >= 0 && v < kNumStiffnessVariants) ? t[v] : 4;
}
inline bool variant_pencil(int v) { return v == 15 || v == 16; }
inline bool variant_staged(int v) { return v >= 5 && v <= 7; }
inline bool variant_bulk(int v) { return v >= 12 && v <= 14; }
inline bool variant_streaming(int v) { return v == 8 || v == 9; }
inline bool variant_split(int v) { return v == 10 || v == 11; }
void launch_stiffness_split(const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s, int blocks_per_sm);
void free_grad(Mesh* mp);
void free_batch(Mesh* mp);
void free_geometry_pack(Mesh* mp);
// max |x| over n values on the compute stream (NaN if any value is NaN); synchronises
bool device_maxabs(Mesh* mp, const float* x, long n, float* out);
// inter-slice assembly buffers (sf3d_assemble.cu)
bool prepare_interfaces(Mesh* mp, int num_interfaces, int max_nibool, const int* nibool, const int* ibool_interfaces);
void free_interfaces(Mesh* mp);
// default element counts of the two elastic phases for the fused drivers
inline void default_phase_counts(Mesh* mp) {
  if (mp->nspec_outer == 0 && mp->nspec_inner == 0) {
    mp->nspec_outer = mp->phase_valid[0];
    mp->nspec_inner = mp->phase_valid[1];
  }
}
// reads and clears the kernel error word; false (and a stored error) if set
bool check_kernel_error(Mesh* mp);
// dispatch on Mesh::stiffness_variant
void launch_stiffness_colored(const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s);
inline void run_stiffness(Mesh* mp, const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s);
void launch_stiffness_aniso(const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s, int blocks_per_sm);
// iphase's elements colour by colour with plain read-modify-write assembly
inline bool run_stiffness_by_color(Mesh* mp, const StiffnessArgs& a, int iphase, bool att, bool store_strain,
                                   cudaStream_t s) {
  if (!mp->use_mesh_coloring || mp->elem_colors.empty() || !a.phase) return false;
  const int c0 = iphase == 1 ? 0 : mp->num_colors_outer;
  const int c1 = iphase == 1 ? mp->num_colors_outer : mp->num_colors_outer + mp->num_colors_inner;
  int off = 0;
  for (int c = c0; c < c1 && off < a.nelem; ++c) {
    StiffnessArgs b = a;
    b.phase = a.phase + off;
    b.nelem = mp->elem_colors[c] < a.nelem - off ? mp->elem_colors[c] : a.nelem - off;
    launch_stiffness_colored(b, att, store_strain, s);
    off += mp->elem_colors[c];
  }
  return true;
}
inline void run_stiffness(Mesh* mp, const StiffnessArgs& a, bool att, bool store_strain, cudaStream_t s) {
  if (a.c[0]) {
    // anisotropic stress: its own build of the one-CTA-per-element kernel
    // (atomic assembly, which is correct with or without a colouring)
    // the 21 extra moduli take registers: one CTA/SM fewer than the isotropic
    // build of the same variant (the default, 6, becomes the measured best, 5)
    // the bulk-copy variants (12-14) map to the measured best anisotropic build (5):
    // with the 21 c_ij rows bulk-copied as well, 34 KB of shared memory a CTA
    // held it to 6 CTAs/SM and 9.5-9.7 ms against 8.96 ms on the main workload
    const int v = mp->stiffness_variant;
    const int bps = variant_bulk(v) ? 5 : variant_blocks_per_sm(v) - 1;
    launch_stiffness_aniso(a, att, store_strain, s, bps < 4 ? 4 : bps);
    return;
  }
  if (mp->use_mesh_coloring && !mp->geom_format && a.phase && mp->d_phase_ispec) {
    const int iphase = a.phase == mp->d_phase_ispec ? 1 : 2;
    if (run_stiffness_by_color(mp, a, iphase, att, store_strain, s)) return;
  }
  if (mp->geom_format) {
    // packed static streams: the one-CTA-per-element kernel at 6 or 7 CTAs/SM
    // (variant 4: 7), or with cp.async-staged memory variables at 8, 9 or 10
    // (variants 5, 6, 7), or with bulk-copied ones at 8, 9 or 10 (12, 13, 14)
    StiffnessArgs h = a;
    h.pack = mp->d_pack;
    h.pool = mp->d_pack_pool;
    const int v = mp->stiffness_variant;
    if (variant_staged(v))
      launch_stiffness(h, att, store_strain, s, v + 3, mp->geom_format, true);
    else if (variant_bulk(v))
      launch_stiffness(h, att, store_strain, s, v - 4, mp->geom_format, true, false, true);
    else
      launch_stiffness(h, att, store_strain, s, v == 4 ? 7 : 6, mp->geom_format);
  } else if (variant_pencil(mp->stiffness_variant) && !att && !store_strain) {
    run_elem_pencil(mp, a, mp->stiffness_variant == 15 ? 8 : 7, s);
  } else if (mp->stiffness_variant == 1 && mp->d_kerr) {
    launch_stiffness_pipelined(a, att, store_strain, mp->d_kerr, s);
  } else if (variant_split(mp->stiffness_variant)) {
    launch_stiffness_split(a, att, store_strain, s, variant_blocks_per_sm(mp->stiffness_variant));
  } else {
    launch_stiffness(a, att, store_strain, s, variant_blocks_per_sm(mp->stiffness_variant), false,
                     variant_staged(mp->stiffness_variant), variant_streaming(mp->stiffness_variant),
                     variant_bulk(mp->stiffness_variant));
  }
}
void launch_pressure_seismograms(Mesh* mp, int slot);
// fused-loop pieces of a coupled fluid/solid step (sf3d_acoustic.cu)
int enqueue_acoustic_step(Mesh* mp, float dt, float dt2, float dtsq2);
int enqueue_coupling_el_ac(Mesh* mp);
int enqueue_pressure_seismograms(Mesh* mp);
// one fused forward elastic step of sf3d_iterate_time (predictor fused with the
// previous corrector unless first_step); returns the number of launches
// out-of-place displacement / force buffers of one step (the gradient's reverse sweep)
struct StepIO {
  const float* d_in;
  float* d_out;
  const float* a_in;
  float* a_out;
};
int enqueue_step(Mesh* mp, float dt, float dt2, float dtsq2, bool first_step, cudaEvent_t* ev,
                 const StepIO* io = nullptr);
// fills Mesh::el_first/el_count/ac_first/ac_count from ibool (synchronises the stream)
bool compute_point_spans(Mesh* mp);
// accel += sign * (Stacey traction of veloc) on the absorbing faces (sign -1:
// the force of the absorbing boundary)
void launch_stacey(Mesh* mp, const float* veloc, float* accel, cudaStream_t s, float sign = -1.f);
void launch_set_it(Mesh* mp, int it, cudaStream_t s);
void launch_mass_corrector(Mesh* mp, float dt2, cudaStream_t s);
StiffnessArgs stiffness_args(Mesh* mp, Fields& F, int iphase, float deltat, bool att, bool strain, bool backward);
// C-PML (sf3d_pml.cu): PML_displ_old / _new around the predictor of the forward
// field (before: from the fields about to be predicted; after: from the predicted
// ones), the CPML elements' stiffness of one phase, the Dirichlet condition on
// the layers' outer faces
void launch_pml_displ(Mesh* mp, bool after_predictor, float dt2, float dtsq2, cudaStream_t s);
int launch_pml_stiffness(Mesh* mp, int iphase, bool strain, cudaStream_t s);
void launch_pml_boundary(Mesh* mp, cudaStream_t s);
void free_pml(Mesh* mp);

}  // namespace sf3d
