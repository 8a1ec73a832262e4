// Time scheme, boundary terms, sources, receivers and the graph-captured
// forward time loop.
//
// Per-call entry points keep the semantics of the reference's
// update_displacement_cuda.cu, compute_forces_viscoelastic_cuda.cu,
// compute_stacey_viscoelastic_cuda.cu, compute_add_sources_viscoelastic_cuda.cu
// and write_seismograms_cuda.cu.  sf3d_iterate_time replaces the Fortran
// time loop (iterate_time.F90:219-330) for forward runs (elastic, viscoelastic,
// and coupled fluid/solid meshes): it fuses the corrector of step n-1 with the
// predictor of step n into one streaming pass, reads the step index from device
// memory, and captures blocks of steps into CUDA graphs, so a step costs a few
// graph nodes and no host round trip.
#include <limits.h>
#include <stdint.h>
#include <math.h>
#include <string.h>

#include <utility>
#include <vector>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

// Newmark predictor (update_displacement_scheme.f90:359-410,
// kernels/UpdateDispVeloc_kernel.cu): u += dt v + dt^2/2 a; v += dt/2 a; a = 0.
__global__ void predictor_kernel(float* __restrict__ d, float* __restrict__ v, float* __restrict__ a, long n,
                                 float dt, float dt2, float dtsq2) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float ai = a[i], vi = v[i];
  d[i] = d[i] + dt * vi + dtsq2 * ai;
  v[i] = vi + dt2 * ai;
  a[i] = 0.f;
}

// The predictor (first step) and the corrector/predictor with the displacement
// written to a buffer of its own and the force left in place: the reverse sweep
// of the checkpointed gradient keeps every step's displacement and force of a
// segment, and these forms let the step write them where they are kept instead
// of copying them there afterwards.  Same arithmetic as predictor_kernel and
// corrector_predictor_kernel.
__global__ void predictor_oop_kernel(const float* __restrict__ d_in, float* __restrict__ d_out,
                                     float* __restrict__ v, const float* __restrict__ a, long n, float dt, float dt2,
                                     float dtsq2) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float ai = a[i], vi = v[i];
  d_out[i] = d_in[i] + dt * vi + dtsq2 * ai;
  v[i] = vi + dt2 * ai;
}
// four consecutive values per thread (16-byte accesses; all buffers 16-byte
// aligned), thread n4 also taking the tail; n = 3 * nglob < 2^31
__global__ void corrector_predictor_oop_kernel(const float* __restrict__ d_in, float* __restrict__ d_out,
                                               float* __restrict__ v, const float* __restrict__ a,
                                               const float* __restrict__ rmx, const float* __restrict__ rmy,
                                               const float* __restrict__ rmz, int n, float dt, float dt2,
                                               float dtsq2) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int n4 = n >> 2;
  if (q > n4) return;
  auto rm_of = [&](int i) {
    const int g = i / 3;
    const int c = i - 3 * g;
    return c == 0 ? __ldg(rmx + g) : (c == 1 ? __ldg(rmy + g) : __ldg(rmz + g));
  };
  auto one = [&](float ai, float vi, float di, float rm, float& dn, float& vn) {
    const float ac = ai * rm;
    const float vh = vi + dt2 * ac;
    dn = di + dt * vh + dtsq2 * ac;
    vn = vh + dt2 * ac;
  };
  if (q == n4) {
    for (int i = 4 * n4; i < n; ++i) one(a[i], v[i], d_in[i], rm_of(i), d_out[i], v[i]);
    return;
  }
  const int i0 = 4 * q;
  const float4 a4 = reinterpret_cast<const float4*>(a)[q];
  const float4 v4 = reinterpret_cast<const float4*>(v)[q];
  const float4 d4 = reinterpret_cast<const float4*>(d_in)[q];
  float4 dn, vn;
  one(a4.x, v4.x, d4.x, rm_of(i0), dn.x, vn.x);
  one(a4.y, v4.y, d4.y, rm_of(i0 + 1), dn.y, vn.y);
  one(a4.z, v4.z, d4.z, rm_of(i0 + 2), dn.z, vn.z);
  one(a4.w, v4.w, d4.w, rm_of(i0 + 3), dn.w, vn.w);
  reinterpret_cast<float4*>(d_out)[q] = dn;
  reinterpret_cast<float4*>(v)[q] = vn;
}

// Mass matrix + corrector (kernels/kernel_3_cuda_device.cu,
// compute_forces_viscoelastic_calling_routine.F90:369-416), unit-stride over (3, NGLOB).
__global__ void mass_corrector_kernel(float* __restrict__ v, float* __restrict__ a, const float* __restrict__ rmx,
                                      const float* __restrict__ rmy, const float* __restrict__ rmz, long nglob,
                                      float dt2) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * nglob) return;
  const long g = i / 3;
  const int c = (int)(i - 3 * g);
  const float rm = c == 0 ? __ldg(rmx + g) : (c == 1 ? __ldg(rmy + g) : __ldg(rmz + g));
  const float ac = a[i] * rm;
  a[i] = ac;
  v[i] += dt2 * ac;
}

__global__ void corrector_kernel(float* __restrict__ v, const float* __restrict__ a, long n, float dt2) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  v[i] += dt2 * a[i];
}

// Corrector of step n-1 fused with the predictor of step n: one read and one
// write of u, v, a per point instead of two passes.  Arithmetic per value is
// identical to mass_corrector_kernel followed by predictor_kernel.  Threads walk
// the interleaved (3, NGLOB) arrays with unit stride so every access is
// coalesced; the mass value comes from the component's rmass array.
__global__ void corrector_predictor_kernel(float* __restrict__ d, float* __restrict__ v, float* __restrict__ a,
                                           const float* __restrict__ rmx, const float* __restrict__ rmy,
                                           const float* __restrict__ rmz, long nglob, float dt, float dt2,
                                           float dtsq2) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 3 * nglob) return;
  const long g = i / 3;
  const int c = (int)(i - 3 * g);
  const float rm = c == 0 ? __ldg(rmx + g) : (c == 1 ? __ldg(rmy + g) : __ldg(rmz + g));
  const float ac = a[i] * rm;
  const float vh = v[i] + dt2 * ac;
  d[i] = d[i] + dt * vh + dtsq2 * ac;
  v[i] = vh + dt2 * ac;
  a[i] = 0.f;
}

// lowest and highest global point (0-based) of the solid elements (out[0],
// out[1]) and of the fluid elements (out[2], out[3])
__global__ void point_span_kernel(const int* __restrict__ ibool, const int* __restrict__ is_ac, int* out) {
  const int t = threadIdx.x;
  if (t >= NGLL3) return;
  const int g = __ldg(ibool + (long)blockIdx.x * NGLL3_PAD + t);
  const int k = (is_ac && __ldg(is_ac + blockIdx.x)) ? 2 : 0;
  atomicMin(out + k, g);
  atomicMax(out + k + 1, g);
}

// corrector_predictor_kernel over four consecutive values of the (3, NGLOB) arrays
// per thread (16-byte loads and stores; the mass of each value by its own point
// and component); thread n4 also takes the n - 4 n4 values of the tail.  d, v, a
// 16-byte aligned; n = 3 * nglob < 2^31.
__global__ void corrector_predictor4_kernel(float* __restrict__ d, float* __restrict__ v, float* __restrict__ a,
                                            const float* __restrict__ rmx, const float* __restrict__ rmy,
                                            const float* __restrict__ rmz, int n, float dt, float dt2,
                                            float dtsq2) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int n4 = n >> 2;
  if (q > n4) return;
  auto rm_of = [&](int i) {
    const int g = i / 3;
    const int c = i - 3 * g;
    return c == 0 ? __ldg(rmx + g) : (c == 1 ? __ldg(rmy + g) : __ldg(rmz + g));
  };
  if (q == n4) {
    for (int i = 4 * n4; i < n; ++i) {
      const float ac = a[i] * rm_of(i);
      const float vh = v[i] + dt2 * ac;
      d[i] = d[i] + dt * vh + dtsq2 * ac;
      v[i] = vh + dt2 * ac;
      a[i] = 0.f;
    }
    return;
  }
  const int i0 = 4 * q;
  const float4 a4 = reinterpret_cast<const float4*>(a)[q];
  float4 v4 = reinterpret_cast<const float4*>(v)[q];
  float4 d4 = reinterpret_cast<const float4*>(d)[q];
#define SF3D_NEWMARK(x, k)                   \
  {                                          \
    const float ac = a4.x * rm_of(i0 + k);   \
    const float vh = v4.x + dt2 * ac;        \
    d4.x = d4.x + dt * vh + dtsq2 * ac;      \
    v4.x = vh + dt2 * ac;                    \
  }
  SF3D_NEWMARK(x, 0) SF3D_NEWMARK(y, 1) SF3D_NEWMARK(z, 2) SF3D_NEWMARK(w, 3)
#undef SF3D_NEWMARK
  reinterpret_cast<float4*>(d)[q] = d4;
  reinterpret_cast<float4*>(v)[q] = v4;
  reinterpret_cast<float4*>(a)[q] = make_float4(0.f, 0.f, 0.f, 0.f);
}

// corrector/predictor over (3, nglob) arrays: the 16-byte vector kernel where the
// arrays start on 16-byte boundaries, else one value per thread
void launch_corrector_predictor(float* d, float* v, float* a, const float* rmx, const float* rmy, const float* rmz,
                                long nglob, float dt, float dt2, float dtsq2, cudaStream_t s) {
  const bool aligned = ((reinterpret_cast<uintptr_t>(d) | reinterpret_cast<uintptr_t>(v) |
                         reinterpret_cast<uintptr_t>(a)) & 15) == 0;
  if (aligned && 3 * nglob < (1L << 31)) {
    const int n = (int)(3 * nglob);
    corrector_predictor4_kernel<<<nblk((n >> 2) + 1, 256), 256, 0, s>>>(d, v, a, rmx, rmy, rmz, n, dt, dt2, dtsq2);
  } else {
    corrector_predictor_kernel<<<nblk(3 * nglob, 256), 256, 0, s>>>(d, v, a, rmx, rmy, rmz, nglob, dt, dt2, dtsq2);
  }
}

// Stacey absorbing traction (compute_stacey_viscoelastic.F90:90-130,
// kernels/compute_stacey_elastic_kernel.cu): one thread per face GLL point.
__global__ void stacey_kernel(int nfaces, const int* __restrict__ abs_ispec, const int* __restrict__ abs_pt,
                              const float* __restrict__ normal, const float* __restrict__ jw,
                              const int* __restrict__ ibool, const float* __restrict__ rho_vp,
                              const float* __restrict__ rho_vs, const float* __restrict__ veloc,
                              float* __restrict__ accel, float* __restrict__ record,
                              const int* __restrict__ is_acoustic, float sign = -1.f) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)nfaces * NGLL2) return;
  const int f = (int)(idx / NGLL2);
  const int e = abs_ispec[f];
  if (is_acoustic[e]) return;
  const long q = (long)e * NGLL3_PAD + abs_pt[idx];
  const int g = ibool[q];
  const float vx = veloc[3L * g], vy = veloc[3L * g + 1], vz = veloc[3L * g + 2];
  const float nx = normal[3 * idx], ny = normal[3 * idx + 1], nz = normal[3 * idx + 2];
  const float vn = vx * nx + vy * ny + vz * nz;
  const float rvp = rho_vp[q], rvs = rho_vs[q];
  const float tx = rvp * vn * nx + rvs * (vx - vn * nx);
  const float ty = rvp * vn * ny + rvs * (vy - vn * ny);
  const float tz = rvp * vn * nz + rvs * (vz - vn * nz);
  const float w = jw[idx];
  atomicAdd(accel + 3L * g, sign * tx * w);
  atomicAdd(accel + 3L * g + 1, sign * ty * w);
  atomicAdd(accel + 3L * g + 2, sign * tz * w);
  if (record) {
    record[3 * idx] = tx * w;
    record[3 * idx + 1] = ty * w;
    record[3 * idx + 2] = tz * w;
  }
}

// Replay of a stored boundary record on the backward field
// (kernels/compute_stacey_elastic_kernel.cu:111-147).
__global__ void stacey_replay_kernel(int nfaces, const int* __restrict__ abs_ispec, const int* __restrict__ abs_pt,
                                     const int* __restrict__ ibool, const float* __restrict__ record,
                                     const int* __restrict__ is_acoustic, float* __restrict__ accel) {
  long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)nfaces * NGLL2) return;
  const int f = (int)(idx / NGLL2);
  if (is_acoustic && is_acoustic[abs_ispec[f]]) return;  // faces of fluid elements carry no elastic record
  const int g = ibool[(long)abs_ispec[f] * NGLL3_PAD + abs_pt[idx]];
  atomicAdd(accel + 3L * g, -record[3 * idx]);
  atomicAdd(accel + 3L * g + 1, -record[3 * idx + 1]);
  atomicAdd(accel + 3L * g + 2, -record[3 * idx + 2]);
}

// Point sources (compute_add_sources_viscoelastic.F90:100-140,
// kernels/compute_add_sources_kernel.cu): block = source, thread = GLL point.
// The stf comes either from a per-call array or from the whole-run table at
// the device step counter (*d_it, 1-based).
__global__ void sources_kernel(int nsrc, const int* __restrict__ ispec_src, const float* __restrict__ sa,
                               const float* __restrict__ stf_step, const float* __restrict__ stf_table,
                               const int* __restrict__ d_it, int stf_nstep, const int* __restrict__ ibool,
                               float* __restrict__ accel, const int* __restrict__ is_acoustic) {
  const int is = blockIdx.x, p = threadIdx.x;
  if (is >= nsrc || p >= NGLL3) return;
  const int e = ispec_src[is];
  if (e < 0 || is_acoustic[e]) return;
  float stf;
  if (stf_table) {
    const int it = *d_it;
    if (it < 1 || it > stf_nstep) return;
    stf = stf_table[(long)(it - 1) * nsrc + is];
  } else {
    stf = stf_step[is];
  }
  const int g = ibool[(long)e * NGLL3_PAD + p];
  const float* s = sa + ((long)is * NGLL3_PAD + p) * 3;
  atomicAdd(accel + 3L * g, s[0] * stf);
  atomicAdd(accel + 3L * g + 1, s[1] * stf);
  atomicAdd(accel + 3L * g + 2, s[2] * stf);
}

// Fluid receivers of vector seismograms: the field is (1/rho) grad of a potential
// (chi, chi_dot, chi_dot_dot for displacement, velocity, acceleration) evaluated
// at the element's GLL points (compute_gradient_in_acoustic.f90:28-200) before
// the interpolation.  scalar == nullptr: no fluid receivers.
struct AcousticSeismo {
  const float* scalar = nullptr;
  const int* rec_is_acoustic = nullptr;
  const int* irregular = nullptr;
  const float* m[9] = {};
  const float* rhostore = nullptr;
  const float* gll = nullptr;          // hprime first
  float xix_regular = 0.f;
};

// Receiver interpolation (compute_interpolated_dva.f90:28-110,
// kernels/compute_elastic_seismogram_kernel.cu): block = receiver; warp-shuffle
// tree sum of h_xi h_eta h_gamma u over the 125 points, then rotation by nu.
// With advance != 0 the last block to finish increments the device step
// counter (threadfence completion pattern, no spinning).
__global__ void seismogram_kernel(int nrec, const int* __restrict__ ispec_rec, const float* __restrict__ hx,
                                  const float* __restrict__ he, const float* __restrict__ hg,
                                  const float* __restrict__ nu, const int* __restrict__ ibool,
                                  const float* __restrict__ field, float* __restrict__ seismo, int nlength,
                                  int slot, const int* __restrict__ d_it_slot, int* d_it, unsigned int* d_done,
                                  int advance, AcousticSeismo ac) {
  __shared__ float red[3][4];
  __shared__ float s_chi[NGLL3_PAD];
  __shared__ float s_hp[NGLL2];
  const int r = blockIdx.x, t = threadIdx.x;
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  // block-uniform: the whole block takes one branch
  const bool fluid = ac.scalar != nullptr && r < nrec && ac.rec_is_acoustic[r] != 0;
  if (fluid) {
    const int e = ispec_rec[r];
    const long eo = (long)e * NGLL3_PAD + t;
    if (t < NGLL3) s_chi[t] = ac.scalar[ibool[eo]];
    if (t < NGLL2) s_hp[t] = ac.gll[t];
    __syncthreads();
    if (t < NGLL3) {
      const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
      float a = 0.f, b = 0.f, c = 0.f;
#pragma unroll
      for (int l = 0; l < NGLLX; ++l) {
        a = fmaf(s_chi[l + NGLLX * j + NGLL2 * k], s_hp[i + NGLLX * l], a);
        b = fmaf(s_chi[i + NGLLX * l + NGLL2 * k], s_hp[j + NGLLX * l], b);
        c = fmaf(s_chi[i + NGLLX * j + NGLL2 * l], s_hp[k + NGLLX * l], c);
      }
      const float rho_inv = 1.f / ac.rhostore[eo];
      const int ir = ac.irregular[e];
      float gx, gy, gz;
      if (ir >= 0) {
        const long mo = (long)ir * NGLL3_PAD + t;
        gx = ac.m[0][mo] * a + ac.m[3][mo] * b + ac.m[6][mo] * c;
        gy = ac.m[1][mo] * a + ac.m[4][mo] * b + ac.m[7][mo] * c;
        gz = ac.m[2][mo] * a + ac.m[5][mo] * b + ac.m[8][mo] * c;
      } else {
        gx = ac.xix_regular * a;
        gy = ac.xix_regular * b;
        gz = ac.xix_regular * c;
      }
      const float h = hx[5 * r + i] * he[5 * r + j] * hg[5 * r + k];
      s0 = h * (rho_inv * gx);
      s1 = h * (rho_inv * gy);
      s2 = h * (rho_inv * gz);
    }
  } else if (r < nrec && t < NGLL3) {
    const int e = ispec_rec[r];
    const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
    const float h = hx[5 * r + i] * he[5 * r + j] * hg[5 * r + k];
    const int g = ibool[(long)e * NGLL3_PAD + t];
    s0 = h * field[3L * g];
    s1 = h * field[3L * g + 1];
    s2 = h * field[3L * g + 2];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    s0 += __shfl_down_sync(0xffffffffu, s0, o);
    s1 += __shfl_down_sync(0xffffffffu, s1, o);
    s2 += __shfl_down_sync(0xffffffffu, s2, o);
  }
  if ((t & 31) == 0) {
    red[0][t >> 5] = s0;
    red[1][t >> 5] = s1;
    red[2][t >> 5] = s2;
  }
  __syncthreads();
  if (t == 0 && r < nrec) {
    const float u0 = red[0][0] + red[0][1] + red[0][2] + red[0][3];
    const float u1 = red[1][0] + red[1][1] + red[1][2] + red[1][3];
    const float u2 = red[2][0] + red[2][1] + red[2][2] + red[2][3];
    const float* n = nu + 9 * r;  // nu(3,3) column-major
    int sl = d_it_slot ? ((*d_it_slot - 1) % nlength) : slot;
    float* o = seismo + 3L * (r + (long)nrec * sl);
    o[0] = n[0] * u0 + n[3] * u1 + n[6] * u2;
    o[1] = n[1] * u0 + n[4] * u1 + n[7] * u2;
    o[2] = n[2] * u0 + n[5] * u1 + n[8] * u2;
  }
  if (advance && t == 0) {
    __threadfence();
    unsigned prev = atomicAdd(d_done, 1u);
    if (prev == gridDim.x - 1) {
      *d_it += 1;
      *d_done = 0u;
      __threadfence();
    }
  }
}

__global__ void advance_it_kernel(int* d_it) { *d_it += 1; }

// fluid-receiver arguments for a potential field (nullptr: none)
AcousticSeismo acoustic_seismo(const Mesh* mp, const float* potential) {
  AcousticSeismo ac;
  if (!mp->has_acoustic || !mp->d_rec_is_acoustic || !potential) return ac;
  ac.scalar = potential;
  ac.rec_is_acoustic = mp->d_rec_is_acoustic;
  ac.irregular = mp->d_irregular;
  for (int q = 0; q < 9; ++q) ac.m[q] = mp->d_metric[q];
  ac.rhostore = mp->d_rhostore;
  ac.gll = mp->d_gll;
  ac.xix_regular = mp->xix_regular;
  return ac;
}
__global__ void set_it_kernel(int* d_it, int v) { *d_it = v; }

// max |u| over the field (check_stability.f90:408), NaN-propagating
__global__ void maxabs_kernel(const float* __restrict__ x, long n, float* __restrict__ out) {
  float m = 0.f;
  bool nan = false;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const float v = fabsf(x[i]);
    if (v != v)
      nan = true;
    else
      m = fmaxf(m, v);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, o));
  nan = __any_sync(0xffffffffu, nan);
  if ((threadIdx.x & 31) == 0) {
    unsigned int* ui = reinterpret_cast<unsigned int*>(out);
    if (nan) atomicExch(ui + 1, 1u);
    atomicMax(ui, __float_as_uint(m));  // non-negative floats order like their bits
  }
}

Fields* pick(Mesh* mp, int fwd_or_adj) { return fwd_or_adj == 3 ? &mp->b : &mp->f; }

}  // namespace

StiffnessArgs stiffness_args(Mesh* mp, Fields& F, int iphase, float deltat, bool att, bool strain, bool backward) {
  StiffnessArgs a;
  memset(&a, 0, sizeof(a));
  a.nelem = iphase == 1 ? mp->nspec_outer : mp->nspec_inner;
  a.phase = mp->d_phase_ispec ? mp->d_phase_ispec + (long)(iphase - 1) * mp->num_phase_ispec : nullptr;
  if (mp->pml && !backward) {
    // C-PML: the CPML elements of the phase run launch_pml_stiffness instead
    a.nelem = mp->phase_nopml_n[iphase - 1];
    a.phase = mp->d_phase_nopml + (long)(iphase - 1) * mp->num_phase_ispec;
  }
  a.ibool = mp->d_ibool;
  a.irregular = mp->d_irregular;
  for (int q = 0; q < 9; ++q) a.m[q] = mp->d_metric[q];
  a.kappav = mp->d_kappav;
  a.muv = mp->d_muv;
  a.gll = mp->d_gll;
  a.xix_regular = mp->xix_regular;
  a.jacobian_regular = mp->jacobian_regular;
  a.deltat = deltat;
  a.displ = F.displ;
  a.veloc = F.veloc;
  a.accel = F.accel;
  for (int c = 0; c < 6; ++c) { a.R[c] = F.R[c]; a.eps[c] = F.eps[c]; }
  a.eps_trace_over_3 = (mp->simulation_type == 3) ? F.eps_trace_over_3 : nullptr;
  a.fc = mp->d_factor_common;
  a.fck = mp->d_factor_common_kappa;
  a.err = mp->d_kerr;
  for (int s = 0; s < NSLS; ++s) {
    a.alpha[s] = backward ? mp->b_alphaval[s] : mp->alphaval[s];
    a.beta[s] = backward ? mp->b_betaval[s] : mp->betaval[s];
    a.gamma[s] = backward ? mp->b_gammaval[s] : mp->gammaval[s];
  }
  if (mp->anisotropy)
    for (int q = 0; q < 21; ++q) a.c[q] = mp->d_cstore[q];
  (void)att; (void)strain;
  return a;
}


// Reads and clears the kernel error word (set by a bounded wait that timed out).
bool check_kernel_error(Mesh* mp) {
  if (!mp->d_kerr) return true;
  int h = 0;
  if (!copy_sync(&h, mp->d_kerr, sizeof(int), cudaMemcpyDeviceToHost, mp->stream)) return false;
  if (h != 0) {
    cudaMemsetAsync(mp->d_kerr, 0, sizeof(int), mp->stream);
    set_error(SF3D_ERR_CUDA, "stiffness pipeline: a bulk-copy wait timed out; the step result is invalid");
    return false;
  }
  return true;
}

// One fused forward step on the compute stream; the predictor of this step is
// fused with the corrector of the previous one unless first_step.
// ev (optional): events recorded on the compute stream around the stiffness
// launches of the step.  io (optional, elastic meshes without C-PML): the step
// reads the displacement from io->d_in and the previous step's force from
// io->a_in, leaves the force there, writes the new displacement to io->d_out and
// scatters this step's force into io->a_out (cleared first); Mesh::f.displ and
// f.accel are pointed at d_out and a_out for the rest of the step.
int enqueue_step(Mesh* mp, float dt, float dt2, float dtsq2, bool first_step, cudaEvent_t* ev, const StepIO* io) {
  Fields& F = mp->f;
  cudaStream_t s = mp->stream;
  int launches = 0;
  if (io) {
    const long n = 3L * mp->nglob;
    cudaMemsetAsync(io->a_out, 0, sizeof(float) * n, s);
    if (first_step)
      predictor_oop_kernel<<<nblk(n, 256), 256, 0, s>>>(io->d_in, io->d_out, F.veloc, io->a_in, n, dt, dt2, dtsq2);
    else
      corrector_predictor_oop_kernel<<<nblk((n >> 2) + 1, 256), 256, 0, s>>>(
          io->d_in, io->d_out, F.veloc, io->a_in, mp->d_rmassx, mp->d_rmassy, mp->d_rmassz, (int)n, dt, dt2, dtsq2);
    F.displ = io->d_out;
    F.accel = io->a_out;
  } else if (mp->pml) {
    // C-PML stores predictions of the field before and after the predictor, so
    // the corrector of the previous step runs on its own
    const long n = 3L * mp->nglob;
    if (!first_step) {
      mass_corrector_kernel<<<nblk(n, 256), 256, 0, s>>>(F.veloc, F.accel, mp->d_rmassx, mp->d_rmassy, mp->d_rmassz,
                                                         mp->nglob, dt2);
      ++launches;
    }
    launch_pml_displ(mp, false, dt2, dtsq2, s);
    predictor_kernel<<<nblk(n, 256), 256, 0, s>>>(F.displ, F.veloc, F.accel, n, dt, dt2, dtsq2);
    launch_pml_displ(mp, true, dt2, dtsq2, s);
    launches += 2;
  } else {
    // the solid's points only, when the fluid elements' span is known: the
    // solid fields are zero at points of fluid elements alone, and no kernel
    // writes them there
    const long g0 = mp->el_count >= 0 ? mp->el_first : 0;
    const long ng = mp->el_count >= 0 ? mp->el_count : mp->nglob;
    if (ng == 0) {
      --launches;   // no solid element: nothing to advance
    } else if (first_step) {
      predictor_kernel<<<nblk(3 * ng, 256), 256, 0, s>>>(F.displ + 3 * g0, F.veloc + 3 * g0, F.accel + 3 * g0,
                                                          3 * ng, dt, dt2, dtsq2);
    } else {
      launch_corrector_predictor(F.displ + 3 * g0, F.veloc + 3 * g0, F.accel + 3 * g0, mp->d_rmassx + g0,
                                 mp->d_rmassy + g0, mp->d_rmassz + g0, ng, dt, dt2, dtsq2, s);
    }
  }
  ++launches;
  // fluid domain: its whole step (it reads the solid displacement just predicted)
  if (mp->has_acoustic) launches += enqueue_acoustic_step(mp, dt, dt2, dtsq2);
  if (mp->stacey && mp->num_abs_faces > 0) {
    const long n = (long)mp->num_abs_faces * NGLL2;
    stacey_kernel<<<nblk(n, 128), 128, 0, s>>>(mp->num_abs_faces, mp->d_abs_ispec, mp->d_abs_pt, mp->d_abs_normal,
                                                mp->d_abs_jw, mp->d_ibool, mp->d_rho_vp, mp->d_rho_vs, F.veloc,
                                                F.accel, nullptr, mp->d_ispec_is_acoustic);
    ++launches;
  }
  if (mp->has_acoustic) launches += enqueue_coupling_el_ac(mp);
  if (mp->nsources > 0 && mp->d_stf_table) {
    sources_kernel<<<mp->nsources, NGLL3_PAD, 0, s>>>(mp->nsources, mp->d_ispec_src, mp->d_sourcearrays, nullptr,
                                                      mp->d_stf_table, mp->d_it, mp->stf_nstep, mp->d_ibool, F.accel,
                                                      mp->d_ispec_is_acoustic);
    ++launches;
  }
  const bool att = mp->attenuation != 0;
  const bool strain = mp->compute_and_store_strain != 0;
  if (ev) cudaEventRecord(ev[0], s);
  for (int iphase = 1; iphase <= 2; ++iphase) {
    StiffnessArgs a = stiffness_args(mp, F, iphase, dt, att, strain, false);
    if (a.nelem <= 0) continue;
    run_stiffness(mp, a, att, strain, s);
    ++launches;
  }
  if (mp->pml) {
    for (int iphase = 1; iphase <= 2; ++iphase) launches += launch_pml_stiffness(mp, iphase, strain, s);
    launch_pml_boundary(mp, s);
    ++launches;
  }
  if (ev) cudaEventRecord(ev[1], s);
  if (mp->has_acoustic) launches += enqueue_pressure_seismograms(mp);
  if (mp->nrec_local > 0 && mp->save_d) {
    seismogram_kernel<<<mp->nrec_local, NGLL3_PAD, 0, s>>>(mp->nrec_local, mp->d_ispec_rec, mp->d_hxir, mp->d_hetar,
                                                           mp->d_hgammar, mp->d_nu_rec, mp->d_ibool, F.displ,
                                                           mp->d_seismo_d, mp->nlength_seismogram, 0, mp->d_it,
                                                           mp->d_it, mp->d_done, 1,
                                                           acoustic_seismo(mp, mp->d_potential));
  } else {
    advance_it_kernel<<<1, 1, 0, s>>>(mp->d_it);
  }
  ++launches;
  return launches;
}

bool compute_point_spans(Mesh* mp) {
  int* d = nullptr;
  const int init[4] = {INT_MAX, -1, INT_MAX, -1};
  int h[4];
  bool ok = cuda_ok(cudaMalloc(&d, sizeof(init)), "cudaMalloc") &&
            copy_sync(d, init, sizeof(init), cudaMemcpyHostToDevice, mp->stream);
  if (ok) {
    point_span_kernel<<<(unsigned)mp->nspec, NGLL3_PAD, 0, mp->stream>>>(mp->d_ibool, mp->d_ispec_is_acoustic, d);
    ok = copy_sync(h, d, sizeof(h), cudaMemcpyDeviceToHost, mp->stream);
  }
  cudaFree(d);
  if (!ok) return false;
  mp->el_first = h[1] >= 0 ? h[0] : 0;
  mp->el_count = h[1] >= 0 ? h[1] - h[0] + 1 : 0;
  mp->ac_first = h[3] >= 0 ? h[2] : 0;
  mp->ac_count = h[3] >= 0 ? h[3] - h[2] + 1 : 0;
  return true;
}

// Stacey traction of a velocity-like field into an acceleration-like buffer.
void launch_stacey(Mesh* mp, const float* veloc, float* accel, cudaStream_t s, float sign) {
  if (!mp->stacey || mp->num_abs_faces == 0) return;
  const long n = (long)mp->num_abs_faces * NGLL2;
  stacey_kernel<<<nblk(n, 128), 128, 0, s>>>(mp->num_abs_faces, mp->d_abs_ispec, mp->d_abs_pt, mp->d_abs_normal,
                                              mp->d_abs_jw, mp->d_ibool, mp->d_rho_vp, mp->d_rho_vs, veloc, accel,
                                              nullptr, mp->d_ispec_is_acoustic, sign);
}

void launch_set_it(Mesh* mp, int it, cudaStream_t s) { set_it_kernel<<<1, 1, 0, s>>>(mp->d_it, it); }

void launch_mass_corrector(Mesh* mp, float dt2, cudaStream_t s) {
  mass_corrector_kernel<<<nblk(3L * mp->nglob, 256), 256, 0, s>>>(mp->f.veloc, mp->f.accel, mp->d_rmassx,
                                                                  mp->d_rmassy, mp->d_rmassz, mp->nglob, dt2);
}

bool device_maxabs(Mesh* mp, const float* x, long n, float* out) {
  if (!cuda_ok(cudaMemsetAsync(mp->d_scratch, 0, sizeof(float) * 2, mp->stream), "cudaMemsetAsync")) return false;
  maxabs_kernel<<<4 * 152, 256, 0, mp->stream>>>(x, n, mp->d_scratch);
  float h[2];
  if (!copy_sync(h, mp->d_scratch, sizeof(h), cudaMemcpyDeviceToHost, mp->stream)) return false;
  unsigned nanflag;
  memcpy(&nanflag, &h[1], 4);
  *out = nanflag ? NAN : h[0];
  return true;
}

void flush_correctors(Mesh* mp) {
  for (int idx = 0; idx < 2; ++idx) {
    if (!mp->pend_corrector[idx]) continue;
    mp->pend_corrector[idx] = 0;
    Fields* F = idx == 0 ? &mp->f : &mp->b;
    if (!F->veloc) continue;
    mass_corrector_kernel<<<nblk(3L * mp->nglob, 256), 256, 0, mp->stream>>>(F->veloc, F->accel, mp->d_rmassx,
                                                                            mp->d_rmassy, mp->d_rmassz, mp->nglob,
                                                                            mp->pend_dt2[idx]);
    cuda_ok(cudaGetLastError(), "mass_corrector_kernel");
  }
}

}  // namespace sf3d

using namespace sf3d;

extern "C" {

void update_displacement_cuda_(long* Mesh_pointer, realw* deltat_F, realw* deltatover2_F, realw* deltatsqover2_F,
                               int* FORWARD_OR_ADJOINT) {
  Mesh* mp = get_mesh(Mesh_pointer, false);
  if (!mp) return;
  const int idx = *FORWARD_OR_ADJOINT == 1 ? 0 : 1;
  Fields* F = pick(mp, idx == 0 ? 1 : 3);
  if (!F->displ) { set_error(SF3D_ERR_STATE, "update_displacement_cuda: field not allocated"); return; }
  const long n = 3L * mp->nglob;
  if (mp->pml && idx == 0) {
    // C-PML: PML_displ_old / _new around an unfused predictor
    // (update_displacement_cuda.cu:95-160)
    flush_correctors(mp);
    launch_pml_displ(mp, false, *deltatover2_F, *deltatsqover2_F, mp->stream);
    predictor_kernel<<<nblk(n, 256), 256, 0, mp->stream>>>(F->displ, F->veloc, F->accel, n, *deltat_F,
                                                           *deltatover2_F, *deltatsqover2_F);
    launch_pml_displ(mp, true, *deltatover2_F, *deltatsqover2_F, mp->stream);
    cuda_ok(cudaGetLastError(), "predictor_kernel (C-PML)");
    return;
  }
  if (mp->pend_corrector[idx] && mp->pend_dt2[idx] == *deltatover2_F) {
    // the deferred corrector of the previous step fused with this predictor
    mp->pend_corrector[idx] = 0;
    launch_corrector_predictor(F->displ, F->veloc, F->accel, mp->d_rmassx, mp->d_rmassy, mp->d_rmassz, mp->nglob,
                               *deltat_F, *deltatover2_F, *deltatsqover2_F, mp->stream);
    cuda_ok(cudaGetLastError(), "corrector_predictor_kernel");
    return;
  }
  if (mp->pend_corrector[idx]) flush_correctors(mp);
  predictor_kernel<<<nblk(n, 256), 256, 0, mp->stream>>>(F->displ, F->veloc, F->accel, n, *deltat_F,
                                                          *deltatover2_F, *deltatsqover2_F);
  cuda_ok(cudaGetLastError(), "predictor_kernel");
}

void compute_forces_viscoelastic_cuda_(long* Mesh_pointer, int* iphase, realw* deltat, int* nspec_outer_elastic,
                                       int* nspec_inner_elastic, int* COMPUTE_AND_STORE_STRAIN, int* ATTENUATION,
                                       int* FORWARD_OR_ADJOINT_f) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  const int fa = *FORWARD_OR_ADJOINT_f;
  if (fa != 0 && fa != 1 && fa != 3) { set_error(SF3D_ERR_ARG, "invalid FORWARD_OR_ADJOINT"); return; }
  if (*iphase != 1 && *iphase != 2) { set_error(SF3D_ERR_ARG, "iphase must be 1 or 2"); return; }
  mp->nspec_outer = *nspec_outer_elastic;
  mp->nspec_inner = *nspec_inner_elastic;
  const int nel = *iphase == 1 ? mp->nspec_outer : mp->nspec_inner;
  if (nel < 0 || nel > mp->phase_valid[*iphase - 1]) {
    set_error(SF3D_ERR_ARG, "nspec_outer/inner_elastic exceeds the phase element lists");
    return;
  }
  const bool att = *ATTENUATION && mp->attenuation;
  const bool strain = *COMPUTE_AND_STORE_STRAIN && mp->compute_and_store_strain;
  if (fa == 1 || fa == 0) {
    StiffnessArgs a = stiffness_args(mp, mp->f, *iphase, *deltat, att, strain, false);
    run_stiffness(mp, a, att, strain, mp->stream);
    launch_pml_stiffness(mp, *iphase, strain, mp->stream);
  }
  if ((fa == 3 || fa == 0) && mp->b.displ) {
    StiffnessArgs a = stiffness_args(mp, mp->b, *iphase, *deltat, att, strain, true);
    run_stiffness(mp, a, att && mp->b.R[0] != nullptr, strain && mp->b.eps[0] != nullptr, mp->stream);
  }
  cuda_ok(cudaGetLastError(), "stiffness_kernel");
}

void compute_stacey_viscoelastic_cuda_(long* Mesh_pointer, int* iphasef, realw* b_absorb_field,
                                       int* FORWARD_OR_ADJOINT_f) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (*iphasef != 1 || !mp->stacey || mp->num_abs_faces == 0) return;
  const int fa = *FORWARD_OR_ADJOINT_f;
  const long n = (long)mp->num_abs_faces * NGLL2;
  const bool store = (fa == 1) && mp->save_forward && mp->simulation_type == 1 && b_absorb_field;
  if (store && !ensure_stage(mp, sizeof(float) * 3 * n)) return;
  // faces of fluid elements are skipped by the kernel: their record entries are zero
  if (store) SF3D_CUDA(cudaMemsetAsync(mp->d_stage, 0, sizeof(float) * 3 * n, mp->stream));
  if (fa == 1 || fa == 0) {
    stacey_kernel<<<nblk(n, 128), 128, 0, mp->stream>>>(mp->num_abs_faces, mp->d_abs_ispec, mp->d_abs_pt,
                                                        mp->d_abs_normal, mp->d_abs_jw, mp->d_ibool, mp->d_rho_vp,
                                                        mp->d_rho_vs, mp->f.veloc, mp->f.accel,
                                                        store ? mp->d_stage : nullptr, mp->d_ispec_is_acoustic);
    if (!cuda_ok(cudaGetLastError(), "stacey_kernel")) return;
    if (store) {
      SF3D_CUDA(cudaMemcpyAsync(b_absorb_field, mp->d_stage, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost,
                                mp->stream));
      SF3D_CUDA(cudaStreamSynchronize(mp->stream));
    }
  }
  if ((fa == 3 || fa == 0) && mp->b.displ) {
    if (b_absorb_field && mp->simulation_type == 3) {
      // replay of the boundary record stored by the forward run
      if (!ensure_stage(mp, sizeof(float) * 3 * n)) return;
      SF3D_CUDA(cudaMemcpyAsync(mp->d_stage, b_absorb_field, sizeof(float) * 3 * n, cudaMemcpyHostToDevice,
                                mp->stream));
      stacey_replay_kernel<<<nblk(n, 128), 128, 0, mp->stream>>>(mp->num_abs_faces, mp->d_abs_ispec, mp->d_abs_pt,
                                                                 mp->d_ibool, mp->d_stage, mp->d_ispec_is_acoustic,
                                                                 mp->b.accel);
    } else {
      // recomputed (checkpointed) backward field: same traction from b_veloc
      stacey_kernel<<<nblk(n, 128), 128, 0, mp->stream>>>(mp->num_abs_faces, mp->d_abs_ispec, mp->d_abs_pt,
                                                          mp->d_abs_normal, mp->d_abs_jw, mp->d_ibool, mp->d_rho_vp,
                                                          mp->d_rho_vs, mp->b.veloc, mp->b.accel, nullptr,
                                                          mp->d_ispec_is_acoustic);
    }
    cuda_ok(cudaGetLastError(), "stacey_kernel(b)");
  }
}

static void add_sources(long* Mesh_pointer, double* h_stf, int* h_NSOURCES, bool backward) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  if (*h_NSOURCES != mp->nsources) { set_error(SF3D_ERR_ARG, "NSOURCES does not match prepare_constants_device"); return; }
  if (mp->nsources == 0 || mp->nsources_local == 0) return;
  Fields* F = backward ? &mp->b : &mp->f;
  if (!F->accel) { set_error(SF3D_ERR_STATE, "field not allocated"); return; }
  std::vector<float> stf(mp->nsources);
  for (int i = 0; i < mp->nsources; ++i) stf[i] = (float)h_stf[i];
  SF3D_CUDA(cudaMemcpyAsync(mp->d_stf_step, stf.data(), sizeof(float) * mp->nsources, cudaMemcpyHostToDevice,
                            mp->stream));
  sources_kernel<<<mp->nsources, NGLL3_PAD, 0, mp->stream>>>(mp->nsources, mp->d_ispec_src, mp->d_sourcearrays,
                                                             mp->d_stf_step, nullptr, nullptr, 0, mp->d_ibool,
                                                             F->accel, mp->d_ispec_is_acoustic);
  // the host stf buffer is reused by the caller on the next step
  SF3D_CUDA(cudaStreamSynchronize(mp->stream));
  cuda_ok(cudaGetLastError(), "sources_kernel");
}

void compute_add_sources_el_cuda_(long* Mesh_pointer, double* h_stf_pre_compute, int* h_NSOURCES) {
  add_sources(Mesh_pointer, h_stf_pre_compute, h_NSOURCES, false);
}
void compute_add_sources_el_s3_cuda_(long* Mesh_pointer, double* h_stf_pre_compute, int* h_NSOURCES) {
  add_sources(Mesh_pointer, h_stf_pre_compute, h_NSOURCES, true);
}

// Deferred: the mass matrix and corrector run at the next update_displacement_cuda
// of the same field (fused with its predictor), or before any other entry point
// (get_mesh) -- the reference's call sequence sees the same fields.
void kernel_3_a_cuda_(long* Mesh_pointer, realw* deltatover2_F, realw* b_deltatover2_F, int* APPROXIMATE_OCEAN_LOAD,
                      int* FORWARD_OR_ADJOINT) {
  Mesh* mp = get_mesh(Mesh_pointer, false);
  if (!mp) return;
  if (*FORWARD_OR_ADJOINT != 1 && *FORWARD_OR_ADJOINT != 3) { set_error(SF3D_ERR_ARG, "invalid FORWARD_OR_ADJOINT"); return; }
  if (*APPROXIMATE_OCEAN_LOAD) { set_error(SF3D_ERR_ARG, "ocean load is not supported"); return; }
  const int idx = *FORWARD_OR_ADJOINT == 1 ? 0 : 1;
  if (!pick(mp, *FORWARD_OR_ADJOINT)->veloc) { set_error(SF3D_ERR_STATE, "kernel_3_a_cuda: field not allocated"); return; }
  if (mp->pend_corrector[idx]) flush_correctors(mp);
  mp->pend_corrector[idx] = 1;
  mp->pend_dt2[idx] = *FORWARD_OR_ADJOINT == 1 ? *deltatover2_F : *b_deltatover2_F;
}

void kernel_3_b_cuda_(long* Mesh_pointer, realw* deltatover2_F, realw* b_deltatover2_F, int* FORWARD_OR_ADJOINT) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return;
  Fields* F = pick(mp, *FORWARD_OR_ADJOINT);
  const float dt2 = *FORWARD_OR_ADJOINT == 1 ? *deltatover2_F : *b_deltatover2_F;
  const long n = 3L * mp->nglob;
  corrector_kernel<<<nblk(n, 256), 256, 0, mp->stream>>>(F->veloc, F->accel, n, dt2);
  cuda_ok(cudaGetLastError(), "corrector_kernel");
}

void compute_seismograms_cuda_(long* Mesh_pointer_f, realw* seismograms_d, realw* seismograms_v,
                               realw* seismograms_a, realw* seismograms_p, int* seismo_currentf,
                               int* nlength_seismogramf, int* itf, int* it_endf, int* ACOUSTIC_SIMULATION,
                               int* ELASTIC_SIMULATION, int* USE_TRICK_FOR_BETTER_PRESSURE) {
  (void)seismograms_p; (void)ACOUSTIC_SIMULATION; (void)ELASTIC_SIMULATION;
  Mesh* mp = get_mesh(Mesh_pointer_f, false);
  if (!mp) return;
  // displacement and pressure traces do not depend on a deferred corrector
  if ((mp->save_v || mp->save_a) && (mp->pend_corrector[0] || mp->pend_corrector[1])) flush_correctors(mp);
  if (mp->nrec_local == 0) return;
  const int cur = *seismo_currentf - 1;
  const int nlen = *nlength_seismogramf;
  if (nlen != mp->nlength_seismogram || cur < 0 || cur >= nlen) {
    set_error(SF3D_ERR_ARG, "seismo_current / nlength_seismogram out of range");
    return;
  }
  // kernel simulations record the reconstructed forward field
  Fields* F = mp->simulation_type == 3 ? &mp->b : &mp->f;
  const bool fwd = mp->simulation_type != 3;
  struct { int on; float* field; float* dst; const float* pot; } kinds[3] = {
      {mp->save_d, F->displ, mp->d_seismo_d, fwd ? mp->d_potential : nullptr},
      {mp->save_v, F->veloc, mp->d_seismo_v, fwd ? mp->d_potential_dot : nullptr},
      {mp->save_a, F->accel, mp->d_seismo_a, fwd ? mp->d_potential_dot_dot : nullptr}};
  for (auto& kd : kinds) {
    if (!kd.on || !kd.field) continue;
    seismogram_kernel<<<mp->nrec_local, NGLL3_PAD, 0, mp->stream>>>(
        mp->nrec_local, mp->d_ispec_rec, mp->d_hxir, mp->d_hetar, mp->d_hgammar, mp->d_nu_rec, mp->d_ibool, kd.field,
        kd.dst, nlen, cur, nullptr, nullptr, nullptr, 0, acoustic_seismo(mp, kd.pot));
  }
  if (mp->save_p) launch_pressure_seismograms(mp, cur);
  if (!cuda_ok(cudaGetLastError(), "seismogram_kernel")) return;
  if (cur == nlen - 1 || *itf == *it_endf) {
    const size_t bytes = sizeof(float) * 3 * (size_t)mp->nrec_local * nlen;
    const bool trick = USE_TRICK_FOR_BETTER_PRESSURE && *USE_TRICK_FOR_BETTER_PRESSURE;
    if (mp->save_d && !trick && seismograms_d)
      SF3D_CUDA(cudaMemcpyAsync(seismograms_d, mp->d_seismo_d, bytes, cudaMemcpyDeviceToHost, mp->stream));
    if (mp->save_v && !trick && seismograms_v)
      SF3D_CUDA(cudaMemcpyAsync(seismograms_v, mp->d_seismo_v, bytes, cudaMemcpyDeviceToHost, mp->stream));
    if (mp->save_a && !trick && seismograms_a)
      SF3D_CUDA(cudaMemcpyAsync(seismograms_a, mp->d_seismo_a, bytes, cudaMemcpyDeviceToHost, mp->stream));
    std::vector<float> pbuf;
    if (mp->save_p && mp->d_seismo_p && seismograms_p) {
      pbuf.resize((size_t)mp->nrec_local * nlen);
      SF3D_CUDA(cudaMemcpyAsync(pbuf.data(), mp->d_seismo_p, sizeof(float) * pbuf.size(), cudaMemcpyDeviceToHost,
                                mp->stream));
    }
    SF3D_CUDA(cudaStreamSynchronize(mp->stream));
    // pressure goes to component 1 of the (NDIM, nrec_local, nlength) host array
    for (int jt = 0; jt < (int)(pbuf.empty() ? 0 : nlen); ++jt)
      for (int r = 0; r < mp->nrec_local; ++r) {
        float* o = seismograms_p + 3L * (r + (long)mp->nrec_local * jt);
        o[0] = pbuf[r + (size_t)mp->nrec_local * jt];
        o[1] = 0.f;
        o[2] = 0.f;
      }
  }
}

int sf3d_set_stf_table(long* Mesh_pointer, const double* h_stf, int nsources, int nstep) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (nsources != mp->nsources || nstep <= 0 || (nsources > 0 && !h_stf)) {
    set_error(SF3D_ERR_ARG, "sf3d_set_stf_table: size mismatch");
    return SF3D_ERR_ARG;
  }
  std::vector<float> tab((size_t)nstep * nsources);
  for (int it = 0; it < nstep; ++it)
    for (int is = 0; is < nsources; ++is) tab[(size_t)it * nsources + is] = (float)h_stf[is + (size_t)nsources * it];
  cudaFree(mp->d_stf_table);
  mp->d_stf_table = nullptr;
  if (!alloc_zero((void**)&mp->d_stf_table, sizeof(float) * tab.size())) return SF3D_ERR_CUDA;
  if (!copy_sync(mp->d_stf_table, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice, mp->stream)) return SF3D_ERR_CUDA;
  mp->stf_nstep = nstep;
  return SF3D_OK;
}

int sf3d_set_sources(long* Mesh_pointer, int nsources, const int* ispec_selected_source, const realw* sourcearrays,
                     const double* h_stf, int nstep) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (nsources < 1 || nstep < 1 || !ispec_selected_source || !sourcearrays || !h_stf) {
    set_error(SF3D_ERR_ARG, "sf3d_set_sources: invalid arguments");
    return SF3D_ERR_ARG;
  }
  std::vector<float> sa((size_t)nsources * NGLL3_PAD * 3, 0.f);
  std::vector<int> isp(nsources);
  for (int is = 0; is < nsources; ++is) {
    isp[is] = ispec_selected_source[is] - 1;
    if (isp[is] < 0 || isp[is] >= mp->nspec) {
      set_error(SF3D_ERR_ARG, "sf3d_set_sources: ispec_selected_source out of range");
      return SF3D_ERR_ARG;
    }
    for (int p = 0; p < NGLL3; ++p)
      for (int c = 0; c < 3; ++c)
        sa[((size_t)is * NGLL3_PAD + p) * 3 + c] = sourcearrays[is + (size_t)nsources * (c + 3 * p)];
  }
  SF3D_CUDA_RET(cudaStreamSynchronize(mp->stream), SF3D_ERR_CUDA);
  if (nsources != mp->nsources) {
    cudaFree(mp->d_sourcearrays); cudaFree(mp->d_ispec_src); cudaFree(mp->d_stf_step);
    mp->d_sourcearrays = nullptr; mp->d_ispec_src = nullptr; mp->d_stf_step = nullptr;
    if (!alloc_zero((void**)&mp->d_sourcearrays, sizeof(float) * sa.size()) ||
        !alloc_zero((void**)&mp->d_ispec_src, sizeof(int) * nsources) ||
        !alloc_zero((void**)&mp->d_stf_step, sizeof(float) * nsources)) {
      mp->nsources = 0;
      return SF3D_ERR_CUDA;
    }
    mp->nsources = mp->nsources_local = nsources;
  }
  if (!copy_sync(mp->d_sourcearrays, sa.data(), sizeof(float) * sa.size(), cudaMemcpyHostToDevice, mp->stream) ||
      !copy_sync(mp->d_ispec_src, isp.data(), sizeof(int) * nsources, cudaMemcpyHostToDevice, mp->stream))
    return SF3D_ERR_CUDA;
  return sf3d_set_stf_table(Mesh_pointer, h_stf, nsources, nstep);
}

int sf3d_iterate_time(long* Mesh_pointer, int it_begin, int it_end, realw deltat, int steps_per_graph, int flags) {
  NvtxRange nvtx_range("sf3d_iterate_time");
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!mp->f.displ) { set_error(SF3D_ERR_STATE, "prepare_fields_elastic_device not called"); return SF3D_ERR_STATE; }
  if (it_begin < 1 || it_end < it_begin) { set_error(SF3D_ERR_ARG, "invalid it range"); return SF3D_ERR_ARG; }
  if (mp->nsources > 0 && (!mp->d_stf_table || it_end > mp->stf_nstep)) {
    set_error(SF3D_ERR_STATE, "sf3d_set_stf_table must cover it_end");
    return SF3D_ERR_STATE;
  }
  if (mp->num_phase_ispec <= 0) { set_error(SF3D_ERR_STATE, "phase element lists not prepared"); return SF3D_ERR_STATE; }
  default_phase_counts(mp);
  const float dt = deltat, dt2 = deltat / 2.f, dtsq2 = deltat * deltat / 2.f;
  const bool timing = (flags & 1) != 0;
  const int nsteps = it_end - it_begin + 1;
  if (timing) {
    while (mp->tev.size() < 2 * (size_t)nsteps) {
      cudaEvent_t e;
      SF3D_CUDA_RET(cudaEventCreate(&e), SF3D_ERR_CUDA);
      mp->tev.push_back(e);
    }
  }
  cudaStream_t s = mp->stream;
  if (mp->has_acoustic && mp->el_count < 0 && !mp->pml && !compute_point_spans(mp)) return SF3D_ERR_CUDA;
  set_it_kernel<<<1, 1, 0, s>>>(mp->d_it, it_begin);
  SF3D_CUDA_RET(cudaMemsetAsync(mp->d_done, 0, sizeof(unsigned int), s), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaEventRecord(mp->ev0, s), SF3D_ERR_CUDA);
  int launches = 0, done = 0;
  auto step = [&](bool first) {
    launches += enqueue_step(mp, dt, dt2, dtsq2, first, timing ? &mp->tev[2 * (size_t)done] : nullptr);
    ++done;
  };
  step(true);
  int remaining = nsteps - 1;
  // timing mode brackets every stiffness launch with its own events, so it
  // launches the steps one by one instead of through a graph
  const int K = (steps_per_graph > 0 && !timing) ? steps_per_graph : 0;
  if (K > 0 && remaining >= K) {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int per_block = 0;
    SF3D_CUDA_RET(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), SF3D_ERR_CUDA);
    for (int q = 0; q < K; ++q) per_block += enqueue_step(mp, dt, dt2, dtsq2, false, nullptr);
    SF3D_CUDA_RET(cudaStreamEndCapture(s, &graph), SF3D_ERR_CUDA);
    SF3D_CUDA_RET(cudaGraphInstantiate(&exec, graph, 0), SF3D_ERR_CUDA);
    while (remaining >= K) {
      if (!cuda_ok(cudaGraphLaunch(exec, s), "cudaGraphLaunch")) break;
      launches += per_block;
      remaining -= K;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
  }
  while (remaining > 0) { step(false); --remaining; }
  {
    const long g0 = mp->el_count >= 0 ? mp->el_first : 0;
    const long ng = mp->el_count >= 0 ? mp->el_count : mp->nglob;
    if (ng > 0)
      mass_corrector_kernel<<<nblk(3 * ng, 256), 256, 0, s>>>(mp->f.veloc + 3 * g0, mp->f.accel + 3 * g0,
                                                              mp->d_rmassx + g0, mp->d_rmassy + g0,
                                                              mp->d_rmassz + g0, ng, dt2);
    else
      --launches;
  }
  ++launches;
  SF3D_CUDA_RET(cudaEventRecord(mp->ev1, s), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaEventSynchronize(mp->ev1), SF3D_ERR_CUDA);
  if (!cuda_ok(cudaGetLastError(), "sf3d_iterate_time")) return SF3D_ERR_CUDA;
  cudaEventElapsedTime(&mp->last_total_ms, mp->ev0, mp->ev1);
  mp->last_total_launches = launches;
  mp->last_stiff_launches = 0;
  mp->last_stiff_ms = 0.f;
  if (timing) {
    double ms = 0;
    for (int q = 0; q < nsteps; ++q) {
      float d = 0.f;
      if (cudaEventElapsedTime(&d, mp->tev[2 * q], mp->tev[2 * q + 1]) == cudaSuccess && d > 0.f) {
        ms += d;
        ++mp->last_stiff_launches;
      }
    }
    mp->last_stiff_ms = (float)ms;
  }
  if (!check_kernel_error(mp)) return SF3D_ERR_CUDA;
  return sf3d_last_error(nullptr, 0);
}

int sf3d_set_stiffness_variant(long* Mesh_pointer, int variant) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (variant < 0 || variant >= kNumStiffnessVariants) {
    set_error(SF3D_ERR_ARG, "unknown stiffness variant");
    return SF3D_ERR_ARG;
  }
  mp->stiffness_variant = variant;
  return SF3D_OK;
}

int sf3d_autotune_stiffness(long* Mesh_pointer, int reps, float* ms_per_variant, int* best_variant) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!mp->f.displ || mp->num_phase_ispec <= 0) {
    set_error(SF3D_ERR_STATE, "sf3d_autotune_stiffness: fields and phase lists not prepared");
    return SF3D_ERR_STATE;
  }
  if (reps < 1) reps = 1;
  default_phase_counts(mp);
  // timing the kernels on a wavefield at rest leaves every array unchanged
  // (zero strain keeps zero memory variables and adds zero force)
  const bool att = mp->attenuation != 0;
  std::vector<std::pair<const float*, long>> check = {{mp->f.displ, 3L * mp->nglob}, {mp->f.veloc, 3L * mp->nglob}};
  if (att)
    for (int c = 0; c < 6; ++c)
      if (mp->f.R[c]) check.push_back({mp->f.R[c], (long)mp->nspec * NSLS * NGLL3_PAD});
  for (auto& q : check) {
    float m = 0.f;
    if (!device_maxabs(mp, q.first, q.second, &m)) return SF3D_ERR_CUDA;
    if (!(m == 0.f)) {
      set_error(SF3D_ERR_STATE, "sf3d_autotune_stiffness must run on a wavefield at rest (before the first step)");
      return SF3D_ERR_STATE;
    }
  }
  const bool strain = mp->compute_and_store_strain != 0;
  const int keep = mp->stiffness_variant;
  auto pass = [&]() {
    for (int iphase = 1; iphase <= 2; ++iphase) {
      StiffnessArgs a = stiffness_args(mp, mp->f, iphase, 0.f, att, strain, false);
      if (a.nelem > 0) run_stiffness(mp, a, att, strain, mp->stream);
    }
  };
  int best = -1;
  float best_ms = 0.f;
  for (int v = 0; v < kNumStiffnessVariants; ++v) {
    mp->stiffness_variant = v;
    pass();
    SF3D_CUDA_RET(cudaEventRecord(mp->ev0, mp->stream), SF3D_ERR_CUDA);
    for (int r = 0; r < reps; ++r) pass();
    SF3D_CUDA_RET(cudaEventRecord(mp->ev1, mp->stream), SF3D_ERR_CUDA);
    SF3D_CUDA_RET(cudaEventSynchronize(mp->ev1), SF3D_ERR_CUDA);
    if (!cuda_ok(cudaGetLastError(), "sf3d_autotune_stiffness")) { mp->stiffness_variant = keep; return SF3D_ERR_CUDA; }
    if (!check_kernel_error(mp)) { mp->stiffness_variant = keep; return SF3D_ERR_CUDA; }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, mp->ev0, mp->ev1);
    ms /= (float)reps;
    if (ms_per_variant) ms_per_variant[v] = ms;
    if (best < 0 || ms < best_ms) { best = v; best_ms = ms; }
  }
  mp->stiffness_variant = best;
  if (best_variant) *best_variant = best;
  return SF3D_OK;
}

int sf3d_last_timing(long* Mesh_pointer, float* stiffness_ms, int* stiffness_launches, float* total_ms,
                     int* total_launches) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (stiffness_ms) *stiffness_ms = mp->last_stiff_ms;
  if (stiffness_launches) *stiffness_launches = mp->last_stiff_launches;
  if (total_ms) *total_ms = mp->last_total_ms;
  if (total_launches) *total_launches = mp->last_total_launches;
  return SF3D_OK;
}

int sf3d_get_seismograms(long* Mesh_pointer, realw* h) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (mp->nrec_local == 0) return SF3D_OK;
  if (!mp->save_d && mp->save_p && mp->d_seismo_p) {
    // pressure runs: pressure in component 0, as compute_seismograms_cuda returns it
    const size_t n = (size_t)mp->nrec_local * mp->nlength_seismogram;
    std::vector<float> p(n);
    if (!copy_sync(p.data(), mp->d_seismo_p, sizeof(float) * n, cudaMemcpyDeviceToHost, mp->stream))
      return SF3D_ERR_CUDA;
    for (size_t q = 0; q < n; ++q) {
      h[3 * q] = p[q];
      h[3 * q + 1] = 0.f;
      h[3 * q + 2] = 0.f;
    }
    return SF3D_OK;
  }
  if (!mp->d_seismo_d) return SF3D_OK;
  const size_t bytes = sizeof(float) * 3 * (size_t)mp->nrec_local * mp->nlength_seismogram;
  SF3D_CUDA_RET(cudaMemcpyAsync(h, mp->d_seismo_d, bytes, cudaMemcpyDeviceToHost, mp->stream), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaStreamSynchronize(mp->stream), SF3D_ERR_CUDA);
  return SF3D_OK;
}

int sf3d_get_seismograms_kind(long* Mesh_pointer, int kind, realw* h) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (kind < 0 || kind > 3) {
    set_error(SF3D_ERR_ARG, "sf3d_get_seismograms_kind: kind must be 0..3");
    return SF3D_ERR_ARG;
  }
  if (mp->nrec_local == 0) return SF3D_OK;
  const size_t n = (size_t)mp->nrec_local * mp->nlength_seismogram;
  if (kind == 3) {
    if (!mp->d_seismo_p) {
      set_error(SF3D_ERR_STATE, "pressure seismograms were not enabled");
      return SF3D_ERR_STATE;
    }
    std::vector<float> p(n);
    if (!copy_sync(p.data(), mp->d_seismo_p, sizeof(float) * n, cudaMemcpyDeviceToHost, mp->stream))
      return SF3D_ERR_CUDA;
    for (size_t q = 0; q < n; ++q) {
      h[3 * q] = p[q];
      h[3 * q + 1] = 0.f;
      h[3 * q + 2] = 0.f;
    }
    return SF3D_OK;
  }
  const float* src = kind == 0 ? mp->d_seismo_d : (kind == 1 ? mp->d_seismo_v : mp->d_seismo_a);
  if (!src) {
    set_error(SF3D_ERR_STATE, "this seismogram kind was not enabled");
    return SF3D_ERR_STATE;
  }
  if (!copy_sync(h, src, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, mp->stream)) return SF3D_ERR_CUDA;
  return SF3D_OK;
}

int sf3d_check_stability(long* Mesh_pointer, realw threshold, realw* max_norm) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!mp->f.displ) return SF3D_ERR_STATE;
  SF3D_CUDA_RET(cudaMemsetAsync(mp->d_scratch, 0, sizeof(float) * 2, mp->stream), SF3D_ERR_CUDA);
  maxabs_kernel<<<4 * 152, 256, 0, mp->stream>>>(mp->f.displ, 3L * mp->nglob, mp->d_scratch);
  float h[2];
  SF3D_CUDA_RET(cudaMemcpyAsync(h, mp->d_scratch, sizeof(h), cudaMemcpyDeviceToHost, mp->stream), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaStreamSynchronize(mp->stream), SF3D_ERR_CUDA);
  if (!check_kernel_error(mp)) return SF3D_ERR_CUDA;
  unsigned nanflag;
  memcpy(&nanflag, &h[1], 4);
  if (max_norm) *max_norm = nanflag ? NAN : h[0];
  if (nanflag || !(h[0] < threshold) || isinf(h[0])) {
    set_error(SF3D_ERR_UNSTABLE, "wavefield is unstable (NaN/Inf or above threshold)");
    return SF3D_ERR_UNSTABLE;
  }
  return SF3D_OK;
}

}  // extern "C"
