// Many shots on one mesh in one pass over the elements (sm_103a).
//
// The reference runs independent shots as separate simulations
// (NUMBER_OF_SIMULTANEOUS_RUNS, src/shared/parallel.f90:2171-2260), each
// re-reading the mesh every step.  Here S shots share one Mesh: the
// wavefields are stacked shot-innermost, index (3 * iglob + c) * S + shot,
// and the stiffness kernel gives each CTA one element (or a few) and a tile of
// SB shots, so ibool, the metric and the moduli are read once per element and
// tile while the SB lanes of a point gather and scatter SB consecutive floats.
// The elastic arithmetic per shot is that of stiffness_kernel<ATT=0>
// (compute_forces_viscoelastic.F90:250-860); the time scheme, Stacey faces,
// sources and receivers are those of sf3d_step.cu applied per shot.  Each step
// is six launches, captured in CUDA graphs in blocks of steps; the stiffness
// kernel (per-point kernels with their (shots-per-block, elements-per-block)
// tilings, or the register-blocked pencil kernel of sf3d_batch_pencil.cu with
// 8, 16 or 32 shots per CTA) is chosen by timing (sf3d_batch_autotune).
#include <math.h>
#include <string.h>

#include <vector>

#include "sf3d_internal.h"

namespace sf3d {
namespace {

inline unsigned nblk(long n, int b) { return (unsigned)((n + b - 1) / b); }

struct BatchStiffArgs {
  int nelem;
  int nshots;
  const int* phase;
  const int* ibool;
  const int* irregular;
  const float* m[9];
  const float* kappav;
  const float* muv;
  const float* gll;
  float xix_regular;
  float jacobian_regular;
  const float* displ;
  float* accel;
};

// CTA: EB elements (one after the other) x SB shots; thread = (GLL point p, shot lane s), s fastest.
template <int SB, int EB>
__global__ void __launch_bounds__(NGLL3_PAD * SB, 8 / SB) batch_stiffness_kernel(const BatchStiffArgs a) {
  __shared__ float s_gll[NGLL3];
  __shared__ float s_buf[9 * NGLL3_PAD * SB];  // displacement (3 comps), then J sigma grad(xi) (9)
  const int tid = threadIdx.x;
  const int sl = tid % SB, p = tid / SB;
  // shot tiles vary fastest over consecutive CTAs: the tiles of one element run
  // together and read the same 128-byte lines of the stacked fields from L2
  const int ntiles = a.nshots / SB;
  const int tile = blockIdx.x % ntiles;
  const int egroup = blockIdx.x / ntiles;
  const int shot = tile * SB + sl;
  const bool active = p < NGLL3;
  const int k = p / NGLL2, j = (p / NGLLX) % NGLLX, i = p % NGLLX;
  const long S = a.nshots;
  for (int q = tid; q < NGLL3; q += NGLL3_PAD * SB) s_gll[q] = __ldg(a.gll + q);
  auto U = [&](int c, int pt) -> float& { return s_buf[(c * NGLL3_PAD + pt) * SB + sl]; };
#pragma unroll 1
  for (int eb = 0; eb < EB; ++eb) {
    const int slot = egroup * EB + eb;
    if (slot >= a.nelem) break;
    const int e = a.phase ? __ldg(a.phase + slot) : slot;
    const int ir = __ldg(a.irregular + e);
    const long eo = (long)e * NGLL3_PAD + p;
    int g = 0;
    float kap = 0.f, mu = 0.f, m[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) m[c] = 0.f;
    float ux = 0.f, uy = 0.f, uz = 0.f;
    if (active) {
      g = __ldg(a.ibool + eo);
      kap = __ldg(a.kappav + eo);
      mu = __ldg(a.muv + eo);
      if (ir >= 0) {
        const long mo = (long)ir * NGLL3_PAD + p;
#pragma unroll
        for (int c = 0; c < 9; ++c) m[c] = __ldg(a.m[c] + mo);
      }
      ux = a.displ[(3L * g) * S + shot];
      uy = a.displ[(3L * g + 1) * S + shot];
      uz = a.displ[(3L * g + 2) * S + shot];
    }
    U(0, p) = ux;
    U(1, p) = uy;
    U(2, p) = uz;
    __syncthreads();
    float t1x = 0.f, t2x = 0.f, t3x = 0.f, t1y = 0.f, t2y = 0.f, t3y = 0.f, t1z = 0.f, t2z = 0.f, t3z = 0.f;
    if (active) {
      const float* hp = s_gll;
#pragma unroll
      for (int l = 0; l < NGLLX; ++l) {
        const float h1 = hp[i + NGLLX * l], h2 = hp[j + NGLLX * l], h3 = hp[k + NGLLX * l];
        const int p1 = l + NGLLX * j + NGLL2 * k, p2 = i + NGLLX * l + NGLL2 * k, p3 = i + NGLLX * j + NGLL2 * l;
        t1x = fmaf(U(0, p1), h1, t1x); t1y = fmaf(U(1, p1), h1, t1y); t1z = fmaf(U(2, p1), h1, t1z);
        t2x = fmaf(U(0, p2), h2, t2x); t2y = fmaf(U(1, p2), h2, t2y); t2z = fmaf(U(2, p2), h2, t2z);
        t3x = fmaf(U(0, p3), h3, t3x); t3y = fmaf(U(1, p3), h3, t3y); t3z = fmaf(U(2, p3), h3, t3z);
      }
    }
    __syncthreads();  // displacement reads done before the stress terms overwrite the buffer
    if (active) {
      const float xr = a.xix_regular;
      const float xix = m[0], xiy = m[1], xiz = m[2], etax = m[3], etay = m[4], etaz = m[5];
      const float gammax = m[6], gammay = m[7], gammaz = m[8];
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
      const float l2m = kap + (4.f / 3.f) * mu;
      const float lam = l2m - 2.f * mu;
      const float sig_xx = l2m * dxx + lam * (dyy + dzz);
      const float sig_yy = l2m * dyy + lam * (dxx + dzz);
      const float sig_zz = l2m * dzz + lam * (dxx + dyy);
      const float sig_xy = mu * (dxy + dyx);
      const float sig_xz = mu * (dzx + dxz);
      const float sig_yz = mu * (dzy + dyz);
      if (ir >= 0) {
        const float jac = 1.f / (xix * (etay * gammaz - etaz * gammay) - xiy * (etax * gammaz - etaz * gammax) +
                                 xiz * (etax * gammay - etay * gammax));
        U(0, p) = jac * (sig_xx * xix + sig_xy * xiy + sig_xz * xiz);
        U(1, p) = jac * (sig_xy * xix + sig_yy * xiy + sig_yz * xiz);
        U(2, p) = jac * (sig_xz * xix + sig_yz * xiy + sig_zz * xiz);
        U(3, p) = jac * (sig_xx * etax + sig_xy * etay + sig_xz * etaz);
        U(4, p) = jac * (sig_xy * etax + sig_yy * etay + sig_yz * etaz);
        U(5, p) = jac * (sig_xz * etax + sig_yz * etay + sig_zz * etaz);
        U(6, p) = jac * (sig_xx * gammax + sig_xy * gammay + sig_xz * gammaz);
        U(7, p) = jac * (sig_xy * gammax + sig_yy * gammay + sig_yz * gammaz);
        U(8, p) = jac * (sig_xz * gammax + sig_yz * gammay + sig_zz * gammaz);
      } else {
        const float js = a.jacobian_regular * xr;
        U(0, p) = js * sig_xx; U(1, p) = js * sig_xy; U(2, p) = js * sig_xz;
        U(3, p) = js * sig_xy; U(4, p) = js * sig_yy; U(5, p) = js * sig_yz;
        U(6, p) = js * sig_xz; U(7, p) = js * sig_yz; U(8, p) = js * sig_zz;
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
        n1x = fmaf(U(0, p1), f1, n1x); n1y = fmaf(U(1, p1), f1, n1y); n1z = fmaf(U(2, p1), f1, n1z);
        n2x = fmaf(U(3, p2), f2, n2x); n2y = fmaf(U(4, p2), f2, n2y); n2z = fmaf(U(5, p2), f2, n2z);
        n3x = fmaf(U(6, p3), f3, n3x); n3y = fmaf(U(7, p3), f3, n3y); n3z = fmaf(U(8, p3), f3, n3z);
      }
      const float fac1 = s_gll[4 * NGLL2 + j + NGLLX * k];
      const float fac2 = s_gll[3 * NGLL2 + i + NGLLX * k];
      const float fac3 = s_gll[2 * NGLL2 + i + NGLLX * j];
      atomicAdd(a.accel + (3L * g) * S + shot, -(fac1 * n1x + fac2 * n2x + fac3 * n3x));
      atomicAdd(a.accel + (3L * g + 1) * S + shot, -(fac1 * n1y + fac2 * n2y + fac3 * n3y));
      atomicAdd(a.accel + (3L * g + 2) * S + shot, -(fac1 * n1z + fac2 * n2z + fac3 * n3z));
    }
    __syncthreads();  // stress reads done before the next element's displacement
  }
}

// Newmark predictor of the first step (update_displacement_scheme.f90:359-410) on stacked fields.
__global__ void batch_predictor_kernel(float* __restrict__ d, float* __restrict__ v, float* __restrict__ a, long n,
                                       float dt, float dt2, float dtsq2) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float ai = a[i], vi = v[i];
  d[i] = d[i] + dt * vi + dtsq2 * ai;
  v[i] = vi + dt2 * ai;
  a[i] = 0.f;
}

__device__ __forceinline__ float rmass_of(long i, long S, const float* __restrict__ rmx,
                                          const float* __restrict__ rmy, const float* __restrict__ rmz) {
  const long gc = i / S;  // 3 * iglob + c
  const long g = gc / 3;
  const int c = (int)(gc - 3 * g);
  return c == 0 ? __ldg(rmx + g) : (c == 1 ? __ldg(rmy + g) : __ldg(rmz + g));
}

// corrector of step n-1 fused with the predictor of step n (same arithmetic as
// corrector_predictor_kernel of sf3d_step.cu, per shot)
__global__ void batch_corrector_predictor_kernel(float* __restrict__ d, float* __restrict__ v, float* __restrict__ a,
                                                 const float* __restrict__ rmx, const float* __restrict__ rmy,
                                                 const float* __restrict__ rmz, long n, long S, float dt, float dt2,
                                                 float dtsq2, int soff = 0, int scnt = 0) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (scnt > 0) {
    // shots [soff, soff + scnt) of every (point, component): n counts those values
    if (i >= n) return;
    i = (i / scnt) * S + soff + i % scnt;
  } else if (i >= n) {
    return;
  }
  const float ac = a[i] * rmass_of(i, S, rmx, rmy, rmz);
  const float vh = v[i] + dt2 * ac;
  d[i] = d[i] + dt * vh + dtsq2 * ac;
  v[i] = vh + dt2 * ac;
  a[i] = 0.f;
}

// The same on four consecutive shots of one (point, component) per thread
// (float4; S, soff and scnt multiples of 4): one mass lookup per vector.
__global__ void batch_corrector_predictor4_kernel(float4* __restrict__ d, float4* __restrict__ v,
                                                  float4* __restrict__ a, const float* __restrict__ rmx,
                                                  const float* __restrict__ rmy, const float* __restrict__ rmz,
                                                  long n4, int S4, int soff4, int scnt4, float dt, float dt2,
                                                  float dtsq2) {
  const long q = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n4) return;
  const long gc = q / scnt4;                 // 3 * iglob + c
  const long i = gc * S4 + soff4 + (q - gc * scnt4);
  const long g = gc / 3;
  const int c = (int)(gc - 3 * g);
  const float rm = c == 0 ? __ldg(rmx + g) : (c == 1 ? __ldg(rmy + g) : __ldg(rmz + g));
  const float4 a4 = a[i];
  float4 v4 = v[i], d4 = d[i];
#define SF3D_NEWMARK(x)                        \
  {                                            \
    const float ac = a4.x * rm;                \
    const float vh = v4.x + dt2 * ac;          \
    d4.x = d4.x + dt * vh + dtsq2 * ac;        \
    v4.x = vh + dt2 * ac;                      \
  }
  SF3D_NEWMARK(x) SF3D_NEWMARK(y) SF3D_NEWMARK(z) SF3D_NEWMARK(w)
#undef SF3D_NEWMARK
  d[i] = d4;
  v[i] = v4;
  a[i] = make_float4(0.f, 0.f, 0.f, 0.f);
}

__global__ void batch_mass_corrector_kernel(float* __restrict__ v, float* __restrict__ a,
                                            const float* __restrict__ rmx, const float* __restrict__ rmy,
                                            const float* __restrict__ rmz, long n, long S, float dt2) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float ac = a[i] * rmass_of(i, S, rmx, rmy, rmz);
  a[i] = ac;
  v[i] += dt2 * ac;
}

// Stacey traction (compute_stacey_viscoelastic.F90:90-130) per face point and shot.
__global__ void batch_stacey_kernel(int nfaces, int S, const int* __restrict__ abs_ispec,
                                    const int* __restrict__ abs_pt, const float* __restrict__ normal,
                                    const float* __restrict__ jw, const int* __restrict__ ibool,
                                    const float* __restrict__ rho_vp, const float* __restrict__ rho_vs,
                                    const float* __restrict__ veloc, float* __restrict__ accel,
                                    const int* __restrict__ is_acoustic, int soff, int scnt) {
  const long idx = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long)nfaces * NGLL2 * scnt) return;
  const long fp = idx / scnt;
  const int s = soff + (int)(idx - fp * scnt);
  const int f = (int)(fp / NGLL2);
  const int e = abs_ispec[f];
  if (is_acoustic[e]) return;
  const long q = (long)e * NGLL3_PAD + abs_pt[fp];
  const long g = ibool[q];
  const float vx = veloc[(3 * g) * S + s], vy = veloc[(3 * g + 1) * S + s], vz = veloc[(3 * g + 2) * S + s];
  const float nx = normal[3 * fp], ny = normal[3 * fp + 1], nz = normal[3 * fp + 2];
  const float vn = vx * nx + vy * ny + vz * nz;
  const float rvp = rho_vp[q], rvs = rho_vs[q];
  const float tx = rvp * vn * nx + rvs * (vx - vn * nx);
  const float ty = rvp * vn * ny + rvs * (vy - vn * ny);
  const float tz = rvp * vn * nz + rvs * (vz - vn * nz);
  const float w = jw[fp];
  atomicAdd(accel + (3 * g) * S + s, -tx * w);
  atomicAdd(accel + (3 * g + 1) * S + s, -ty * w);
  atomicAdd(accel + (3 * g + 2) * S + s, -tz * w);
}

// One point source per shot (compute_add_sources_viscoelastic.F90:100-140): block = shot.
__global__ void batch_sources_kernel(int S, const int* __restrict__ ispec_src, const float* __restrict__ sa,
                                     const float* __restrict__ stf, const int* __restrict__ d_it, int nstep,
                                     const int* __restrict__ ibool, float* __restrict__ accel,
                                     const int* __restrict__ is_acoustic, int soff) {
  const int s = soff + blockIdx.x, p = threadIdx.x;
  if (s >= S || p >= NGLL3) return;
  const int e = ispec_src[s];
  if (e < 0 || is_acoustic[e]) return;
  const int it = *d_it;
  if (it < 1 || it > nstep) return;
  const float f = stf[(long)(it - 1) * S + s];
  const long g = ibool[(long)e * NGLL3_PAD + p];
  const float* w = sa + ((long)s * NGLL3_PAD + p) * 3;
  atomicAdd(accel + (3 * g) * S + s, w[0] * f);
  atomicAdd(accel + (3 * g + 1) * S + s, w[1] * f);
  atomicAdd(accel + (3 * g + 2) * S + s, w[2] * f);
}

// Receivers shared by all shots (compute_interpolated_dva.f90:28-110): block = (receiver, shot).
__global__ void batch_seismogram_kernel(int nrec, int S, const int* __restrict__ ispec_rec,
                                        const float* __restrict__ hx, const float* __restrict__ he,
                                        const float* __restrict__ hg, const float* __restrict__ nu,
                                        const int* __restrict__ ibool, const float* __restrict__ field,
                                        float* __restrict__ seismo, int nlength, const int* __restrict__ d_it,
                                        int soff) {
  __shared__ float red[3][4];
  const int r = blockIdx.x, s = soff + blockIdx.y, t = threadIdx.x;
  float s0 = 0.f, s1 = 0.f, s2 = 0.f;
  if (t < NGLL3) {
    const int e = ispec_rec[r];
    const int k = t / NGLL2, j = (t / NGLLX) % NGLLX, i = t % NGLLX;
    const float h = hx[5 * r + i] * he[5 * r + j] * hg[5 * r + k];
    const long g = ibool[(long)e * NGLL3_PAD + t];
    s0 = h * field[(3 * g) * S + s];
    s1 = h * field[(3 * g + 1) * S + s];
    s2 = h * field[(3 * g + 2) * S + s];
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
  if (t == 0) {
    const float u0 = red[0][0] + red[0][1] + red[0][2] + red[0][3];
    const float u1 = red[1][0] + red[1][1] + red[1][2] + red[1][3];
    const float u2 = red[2][0] + red[2][1] + red[2][2] + red[2][3];
    const float* n = nu + 9 * r;
    const int slot = (*d_it - 1) % nlength;
    float* o = seismo + 3L * (r + (long)nrec * (s + (long)S * slot));
    o[0] = n[0] * u0 + n[3] * u1 + n[6] * u2;
    o[1] = n[1] * u0 + n[4] * u1 + n[7] * u2;
    o[2] = n[2] * u0 + n[5] * u1 + n[8] * u2;
  }
}

__global__ void batch_advance_kernel(int* d_it) { *d_it += 1; }
__global__ void batch_set_it_kernel(int* d_it, int v) {
  d_it[0] = v;
  d_it[1] = v;
}

bool alloc_f(float** d, size_t n) { return alloc_zero((void**)d, sizeof(float) * n); }

// the pencil kernel indexes the stacked fields with 32-bit unsigned offsets
bool pencil_fits_index32(const Mesh* mp, long nshots) { return 3.0 * (double)mp->nglob * nshots < 4294967296.0; }

// Four shots per thread: thread = (GLL point p, shot group gi of 4 consecutive
// shots), gi fastest.  The four shots of a point are one 16-byte vector in the
// stacked fields, in shared memory (float4 rows) and in the scatter
// (atomicAdd on float4: one vector reduction instead of four), and the
// hprime/metric/moduli values of the point serve all four shots.
template <int GB, int EB>
__global__ void __launch_bounds__(NGLL3_PAD * GB, 4 / GB) batch_stiffness4_kernel(const BatchStiffArgs a) {
  __shared__ float s_gll[NGLL3];
  __shared__ float4 s_buf[GB][9][NGLL3_PAD];
  const int tid = threadIdx.x;
  const int gi = tid % GB, p = tid / GB;
  const long S = a.nshots;
  const int ntiles = a.nshots / (4 * GB);
  const int tile = blockIdx.x % ntiles;
  const int egroup = blockIdx.x / ntiles;
  const long shot0 = 4L * (tile * GB + gi);
  const bool active = p < NGLL3;
  const int k = p / NGLL2, j = (p / NGLLX) % NGLLX, i = p % NGLLX;
  for (int q = tid; q < NGLL3; q += NGLL3_PAD * GB) s_gll[q] = __ldg(a.gll + q);
  float4(*B)[NGLL3_PAD] = s_buf[gi];
#pragma unroll 1
  for (int eb = 0; eb < EB; ++eb) {
    const int slot = egroup * EB + eb;
    if (slot >= a.nelem) break;
    const int e = a.phase ? __ldg(a.phase + slot) : slot;
    const int ir = __ldg(a.irregular + e);
    const long eo = (long)e * NGLL3_PAD + p;
    long g = 0;
    float kap = 0.f, mu = 0.f, m[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) m[c] = 0.f;
    float4 u[3] = {make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f), make_float4(0.f, 0.f, 0.f, 0.f)};
    if (active) {
      g = __ldg(a.ibool + eo);
      kap = __ldg(a.kappav + eo);
      mu = __ldg(a.muv + eo);
      if (ir >= 0) {
        const long mo = (long)ir * NGLL3_PAD + p;
#pragma unroll
        for (int c = 0; c < 9; ++c) m[c] = __ldg(a.m[c] + mo);
      }
#pragma unroll
      for (int c = 0; c < 3; ++c) u[c] = *reinterpret_cast<const float4*>(a.displ + (3 * g + c) * S + shot0);
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) B[c][p] = u[c];
    __syncthreads();
    // T[c][d][w]: derivative of component c along reference direction d, shot w
    float T[3][3][4];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int w = 0; w < 4; ++w) T[c][d][w] = 0.f;
    if (active) {
      const float* hp = s_gll;
#pragma unroll
      for (int l = 0; l < NGLLX; ++l) {
        const float h[3] = {hp[i + NGLLX * l], hp[j + NGLLX * l], hp[k + NGLLX * l]};
        const int pp[3] = {l + NGLLX * j + NGLL2 * k, i + NGLLX * l + NGLL2 * k, i + NGLLX * j + NGLL2 * l};
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            const float4 v = B[c][pp[d]];
            T[c][d][0] = fmaf(v.x, h[d], T[c][d][0]);
            T[c][d][1] = fmaf(v.y, h[d], T[c][d][1]);
            T[c][d][2] = fmaf(v.z, h[d], T[c][d][2]);
            T[c][d][3] = fmaf(v.w, h[d], T[c][d][3]);
          }
      }
    }
    __syncthreads();  // displacement reads done before the stress terms overwrite the buffer
    if (active) {
      const float xr = a.xix_regular;
      const float l2m = kap + (4.f / 3.f) * mu;
      const float lam = l2m - 2.f * mu;
      float jac = 0.f;
      if (ir >= 0)
        jac = 1.f / (m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
                     m[2] * (m[3] * m[7] - m[4] * m[6]));
      float F[9][4];
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        // D[c][x]: derivative of component c along x, y, z
        float D[3][3];
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int x = 0; x < 3; ++x)
            D[c][x] = ir >= 0 ? m[x] * T[c][0][w] + m[3 + x] * T[c][1][w] + m[6 + x] * T[c][2][w] : xr * T[c][x][w];
        const float sxx = l2m * D[0][0] + lam * (D[1][1] + D[2][2]);
        const float syy = l2m * D[1][1] + lam * (D[0][0] + D[2][2]);
        const float szz = l2m * D[2][2] + lam * (D[0][0] + D[1][1]);
        const float sxy = mu * (D[0][1] + D[1][0]);
        const float sxz = mu * (D[2][0] + D[0][2]);
        const float syz = mu * (D[2][1] + D[1][2]);
        if (ir >= 0) {
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            const float gx = m[3 * d], gy = m[3 * d + 1], gz = m[3 * d + 2];
            F[3 * d + 0][w] = jac * (sxx * gx + sxy * gy + sxz * gz);
            F[3 * d + 1][w] = jac * (sxy * gx + syy * gy + syz * gz);
            F[3 * d + 2][w] = jac * (sxz * gx + syz * gy + szz * gz);
          }
        } else {
          const float js = a.jacobian_regular * xr;
          F[0][w] = js * sxx; F[1][w] = js * sxy; F[2][w] = js * sxz;
          F[3][w] = js * sxy; F[4][w] = js * syy; F[5][w] = js * syz;
          F[6][w] = js * sxz; F[7][w] = js * syz; F[8][w] = js * szz;
        }
      }
#pragma unroll
      for (int q = 0; q < 9; ++q) B[q][p] = make_float4(F[q][0], F[q][1], F[q][2], F[q][3]);
    }
    __syncthreads();
    if (active) {
      const float* hpw = s_gll + NGLL2;
      float N[3][3][4];
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
          for (int w = 0; w < 4; ++w) N[c][d][w] = 0.f;
#pragma unroll
      for (int l = 0; l < NGLLX; ++l) {
        const float f[3] = {hpw[l + NGLLX * i], hpw[l + NGLLX * j], hpw[l + NGLLX * k]};
        const int pp[3] = {l + NGLLX * j + NGLL2 * k, i + NGLLX * l + NGLL2 * k, i + NGLLX * j + NGLL2 * l};
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            const float4 v = B[3 * d + c][pp[d]];
            N[c][d][0] = fmaf(v.x, f[d], N[c][d][0]);
            N[c][d][1] = fmaf(v.y, f[d], N[c][d][1]);
            N[c][d][2] = fmaf(v.z, f[d], N[c][d][2]);
            N[c][d][3] = fmaf(v.w, f[d], N[c][d][3]);
          }
      }
      const float fac1 = s_gll[4 * NGLL2 + j + NGLLX * k];
      const float fac2 = s_gll[3 * NGLL2 + i + NGLLX * k];
      const float fac3 = s_gll[2 * NGLL2 + i + NGLLX * j];
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float4 r;
        r.x = -(fac1 * N[c][0][0] + fac2 * N[c][1][0] + fac3 * N[c][2][0]);
        r.y = -(fac1 * N[c][0][1] + fac2 * N[c][1][1] + fac3 * N[c][2][1]);
        r.z = -(fac1 * N[c][0][2] + fac2 * N[c][1][2] + fac3 * N[c][2][2]);
        r.w = -(fac1 * N[c][0][3] + fac2 * N[c][1][3] + fac3 * N[c][2][3]);
        atomicAdd(reinterpret_cast<float4*>(a.accel + (3 * g + c) * S + shot0), r);
      }
    }
    __syncthreads();  // stress reads done before the next element's displacement
  }
}

// Meshes whose elements are all regular (cubes: xix = etay = gammaz = xix_regular,
// no metric arrays): the float4 kernel without the metric path.  The stress of
// a regular element is symmetric, so J sigma grad(xi) needs 6 shared rows, not 9,
// and the transposed contraction runs one displacement component at a time (12
// live accumulators instead of 36).  Fewer registers give more resident CTAs,
// which is what this shared-memory-latency-bound kernel is short of.
template <int EB, int MINB>
__global__ void __launch_bounds__(NGLL3_PAD, MINB) batch_stiffness4_regular_kernel(const BatchStiffArgs a) {
  __shared__ float s_gll[NGLL3];
  __shared__ float4 B[6][NGLL3_PAD];   // displacement (rows 0-2), then sxx syy szz sxy sxz syz
  const int p = threadIdx.x;
  const long S = a.nshots;
  const int ntiles = a.nshots / 4;
  const int tile = blockIdx.x % ntiles;
  const int egroup = blockIdx.x / ntiles;
  const long shot0 = 4L * tile;
  const bool active = p < NGLL3;
  const int k = p / NGLL2, j = (p / NGLLX) % NGLLX, i = p % NGLLX;
  if (p < NGLL3) s_gll[p] = __ldg(a.gll + p);
  const float xr = a.xix_regular;
  const float js = a.jacobian_regular * xr;
  // row of sigma[d][c] in B
  constexpr int sym[3][3] = {{0, 3, 4}, {3, 1, 5}, {4, 5, 2}};
#pragma unroll 1
  for (int eb = 0; eb < EB; ++eb) {
    const int slot = egroup * EB + eb;
    if (slot >= a.nelem) break;
    const int e = a.phase ? __ldg(a.phase + slot) : slot;
    const long eo = (long)e * NGLL3_PAD + p;
    long g = 0;
    float kap = 0.f, mu = 0.f;
    if (active) {
      g = __ldg(a.ibool + eo);
      kap = __ldg(a.kappav + eo);
      mu = __ldg(a.muv + eo);
#pragma unroll
      for (int c = 0; c < 3; ++c) B[c][p] = *reinterpret_cast<const float4*>(a.displ + (3 * g + c) * S + shot0);
    }
    __syncthreads();
    float T[3][3][4];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int d = 0; d < 3; ++d)
#pragma unroll
        for (int w = 0; w < 4; ++w) T[c][d][w] = 0.f;
    if (active) {
#pragma unroll
      for (int l = 0; l < NGLLX; ++l) {
        const float h[3] = {s_gll[i + NGLLX * l], s_gll[j + NGLLX * l], s_gll[k + NGLLX * l]};
        const int pp[3] = {l + NGLLX * j + NGLL2 * k, i + NGLLX * l + NGLL2 * k, i + NGLLX * j + NGLL2 * l};
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            const float4 v = B[c][pp[d]];
            T[c][d][0] = fmaf(v.x, h[d], T[c][d][0]);
            T[c][d][1] = fmaf(v.y, h[d], T[c][d][1]);
            T[c][d][2] = fmaf(v.z, h[d], T[c][d][2]);
            T[c][d][3] = fmaf(v.w, h[d], T[c][d][3]);
          }
      }
    }
    __syncthreads();  // displacement reads done before the stress overwrites rows 0-2
    if (active) {
      const float l2m = kap + (4.f / 3.f) * mu;
      const float lam = l2m - 2.f * mu;
      float sg[6][4];
#pragma unroll
      for (int w = 0; w < 4; ++w) {
        const float d00 = xr * T[0][0][w], d11 = xr * T[1][1][w], d22 = xr * T[2][2][w];
        sg[0][w] = js * (l2m * d00 + lam * (d11 + d22));
        sg[1][w] = js * (l2m * d11 + lam * (d00 + d22));
        sg[2][w] = js * (l2m * d22 + lam * (d00 + d11));
        sg[3][w] = js * (mu * (xr * T[0][1][w] + xr * T[1][0][w]));
        sg[4][w] = js * (mu * (xr * T[2][0][w] + xr * T[0][2][w]));
        sg[5][w] = js * (mu * (xr * T[2][1][w] + xr * T[1][2][w]));
      }
#pragma unroll
      for (int q = 0; q < 6; ++q) B[q][p] = make_float4(sg[q][0], sg[q][1], sg[q][2], sg[q][3]);
    }
    __syncthreads();
    if (active) {
      const float* hpw = s_gll + NGLL2;
      const float fac[3] = {s_gll[4 * NGLL2 + j + NGLLX * k], s_gll[3 * NGLL2 + i + NGLLX * k],
                            s_gll[2 * NGLL2 + i + NGLLX * j]};
#pragma unroll
      for (int c = 0; c < 3; ++c) {
        float N[3][4];
#pragma unroll
        for (int d = 0; d < 3; ++d)
#pragma unroll
          for (int w = 0; w < 4; ++w) N[d][w] = 0.f;
#pragma unroll
        for (int l = 0; l < NGLLX; ++l) {
          const float f[3] = {hpw[l + NGLLX * i], hpw[l + NGLLX * j], hpw[l + NGLLX * k]};
          const int pp[3] = {l + NGLLX * j + NGLL2 * k, i + NGLLX * l + NGLL2 * k, i + NGLLX * j + NGLL2 * l};
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            const float4 v = B[sym[d][c]][pp[d]];
            N[d][0] = fmaf(v.x, f[d], N[d][0]);
            N[d][1] = fmaf(v.y, f[d], N[d][1]);
            N[d][2] = fmaf(v.z, f[d], N[d][2]);
            N[d][3] = fmaf(v.w, f[d], N[d][3]);
          }
        }
        float4 r;
        r.x = -(fac[0] * N[0][0] + fac[1] * N[1][0] + fac[2] * N[2][0]);
        r.y = -(fac[0] * N[0][1] + fac[1] * N[1][1] + fac[2] * N[2][1]);
        r.z = -(fac[0] * N[0][2] + fac[1] * N[1][2] + fac[2] * N[2][2]);
        r.w = -(fac[0] * N[0][3] + fac[1] * N[1][3] + fac[2] * N[2][3]);
        atomicAdd(reinterpret_cast<float4*>(a.accel + (3 * g + c) * S + shot0), r);
      }
    }
    __syncthreads();  // stress reads done before the next element's displacement
  }
}

template <int EB>
void launch_tile4_regular(const BatchStiffArgs& a, cudaStream_t s) {
  const long nblocks = (long)((a.nelem + EB - 1) / EB) * (a.nshots / 4);
  batch_stiffness4_regular_kernel<EB, 7><<<(unsigned)nblocks, NGLL3_PAD, 0, s>>>(a);
}

template <int GB, int EB>
void launch_tile4(const BatchStiffArgs& a, cudaStream_t s) {
  const long nblocks = (long)((a.nelem + EB - 1) / EB) * (a.nshots / (4 * GB));
  batch_stiffness4_kernel<GB, EB><<<(unsigned)nblocks, NGLL3_PAD * GB, 0, s>>>(a);
}

template <int GB>
void launch_gb4(const BatchStiffArgs& a, int eb, cudaStream_t s) {
  if (eb == 4)
    launch_tile4<GB, 4>(a, s);
  else if (eb == 2)
    launch_tile4<GB, 2>(a, s);
  else
    launch_tile4<GB, 1>(a, s);
}

template <int SB, int EB>
void launch_tile(const BatchStiffArgs& a, cudaStream_t s) {
  const long nblocks = (long)((a.nelem + EB - 1) / EB) * (a.nshots / SB);
  batch_stiffness_kernel<SB, EB><<<(unsigned)nblocks, NGLL3_PAD * SB, 0, s>>>(a);
}

template <int SB>
void launch_sb(const BatchStiffArgs& a, int eb, cudaStream_t s) {
  if (eb == 4)
    launch_tile<SB, 4>(a, s);
  else if (eb == 2)
    launch_tile<SB, 2>(a, s);
  else
    launch_tile<SB, 1>(a, s);
}

void launch_batch_stiffness(Mesh* mp, int iphase, cudaStream_t s, int soff = 0, int scnt = 0) {
  BatchState* B = mp->batch;
  if (B->pencil_lanes > 0) {
    PencilArgs q;
    memset(&q, 0, sizeof(q));
    q.nelem = iphase == 1 ? mp->nspec_outer : mp->nspec_inner;
    if (q.nelem <= 0) return;
    q.nshots = B->nshots;
    q.shot_offset = soff;
    q.shot_tiles = (scnt > 0 ? scnt : B->nshots) / B->pencil_lanes;
    q.phase = mp->d_phase_ispec + (long)(iphase - 1) * mp->num_phase_ispec;
    q.ibool = mp->d_ibool;
    q.irregular = mp->d_irregular;
    for (int c = 0; c < 9; ++c) q.m[c] = mp->d_metric[c];
    q.kappav = mp->d_kappav;
    q.muv = mp->d_muv;
    q.pack = mp->d_pack;
    q.pool = mp->d_pack_pool;
    q.gll = mp->d_gll;
    q.xix_regular = mp->xix_regular;
    q.jacobian_regular = mp->jacobian_regular;
    q.displ = B->displ;
    q.accel = B->accel;
    memcpy(q.hp, mp->h_hprime, sizeof(q.hp));
    memcpy(q.hpw, mp->h_hprimewgll, sizeof(q.hpw));
    // hp[i2 + 5 i1] = hprime(i2, i1): M[o][l] = hp[o + 5 l]; the transposed
    // contraction takes M[o][l] = hprimewgll(l, o) = hpw[l + 5 o]
    even_odd_coefficients(mp->h_hprime, 1, NGLLX, q.ek);
    even_odd_coefficients(mp->h_hprimewgll, NGLLX, 1, q.ekw);
    launch_batch_pencil(q, B->pencil_lanes, mp->geom_format, s);
    return;
  }
  BatchStiffArgs a;
  memset(&a, 0, sizeof(a));
  a.nelem = iphase == 1 ? mp->nspec_outer : mp->nspec_inner;
  if (a.nelem <= 0) return;
  a.nshots = B->nshots;
  a.phase = mp->d_phase_ispec + (long)(iphase - 1) * mp->num_phase_ispec;
  a.ibool = mp->d_ibool;
  a.irregular = mp->d_irregular;
  for (int q = 0; q < 9; ++q) a.m[q] = mp->d_metric[q];
  a.kappav = mp->d_kappav;
  a.muv = mp->d_muv;
  a.gll = mp->d_gll;
  a.xix_regular = mp->xix_regular;
  a.jacobian_regular = mp->jacobian_regular;
  a.displ = B->displ;
  a.accel = B->accel;
  if (B->shots_per_thread == 4) {
    if (B->shots_per_block == 8) {
      launch_gb4<2>(a, B->elements_per_block, s);
    } else if (mp->nspec_irregular == 0) {
      // every element regular: the metric-free float4 kernel
      if (B->elements_per_block == 4)
        launch_tile4_regular<4>(a, s);
      else if (B->elements_per_block == 2)
        launch_tile4_regular<2>(a, s);
      else
        launch_tile4_regular<1>(a, s);
    } else {
      launch_gb4<1>(a, B->elements_per_block, s);
    }
    return;
  }
  switch (B->shots_per_block) {
    case 1: launch_sb<1>(a, B->elements_per_block, s); break;
    case 2: launch_sb<2>(a, B->elements_per_block, s); break;
    case 4: launch_sb<4>(a, B->elements_per_block, s); break;
    default: launch_sb<8>(a, B->elements_per_block, s); break;
  }
}

// The kernels of one batched step for shots [soff, soff + scnt) on stream s (the
// whole batch: soff 0, scnt nshots); d_it: the counter of those shots.  The
// predictor is fused with the previous corrector unless first.
int enqueue_batch_part(Mesh* mp, float dt, float dt2, float dtsq2, bool first, int soff, int scnt, int* d_it,
                       cudaStream_t s, bool predictor) {
  BatchState* B = mp->batch;
  const long S = B->nshots;
  const bool whole = soff == 0 && scnt == S;
  int launches = 0;
  if (predictor) {
    const long n = 3L * mp->nglob * scnt;
    if (first) {
      batch_predictor_kernel<<<nblk(3L * mp->nglob * S, 256), 256, 0, s>>>(B->displ, B->veloc, B->accel,
                                                                          3L * mp->nglob * S, dt, dt2, dtsq2);
    } else if (S % 4 == 0 && soff % 4 == 0 && scnt % 4 == 0) {
      const long n4 = n / 4;
      cudaLaunchConfig_t cfg = {};
      cudaLaunchAttribute attr[1];
      cfg.gridDim = dim3((unsigned)nblk(n4, 256));
      cfg.blockDim = dim3(256);
      cfg.stream = s;
      if (B->halves == 2) {
        attr[0].id = cudaLaunchAttributePriority;
        attr[0].val.priority = B->prio_hi;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
      }
      cudaLaunchKernelEx(&cfg, batch_corrector_predictor4_kernel, (float4*)B->displ, (float4*)B->veloc,
                         (float4*)B->accel, (const float*)mp->d_rmassx, (const float*)mp->d_rmassy,
                         (const float*)mp->d_rmassz, n4, (int)(S / 4), soff / 4, scnt / 4, dt, dt2, dtsq2);
    } else {
      batch_corrector_predictor_kernel<<<nblk(n, 256), 256, 0, s>>>(B->displ, B->veloc, B->accel, mp->d_rmassx,
                                                                    mp->d_rmassy, mp->d_rmassz, n, S, dt, dt2, dtsq2,
                                                                    whole ? 0 : soff, whole ? 0 : scnt);
    }
    ++launches;
    return launches;
  }
  if (mp->stacey && mp->num_abs_faces > 0) {
    const long nf = (long)mp->num_abs_faces * NGLL2 * scnt;
    batch_stacey_kernel<<<nblk(nf, 256), 256, 0, s>>>(mp->num_abs_faces, (int)S, mp->d_abs_ispec, mp->d_abs_pt,
                                                       mp->d_abs_normal, mp->d_abs_jw, mp->d_ibool, mp->d_rho_vp,
                                                       mp->d_rho_vs, B->veloc, B->accel, mp->d_ispec_is_acoustic, soff,
                                                       scnt);
    ++launches;
  }
  batch_sources_kernel<<<(unsigned)scnt, NGLL3_PAD, 0, s>>>((int)S, B->d_ispec_src, B->d_sa, B->d_stf, d_it,
                                                            B->nstep, mp->d_ibool, B->accel, mp->d_ispec_is_acoustic,
                                                            soff);
  ++launches;
  for (int iphase = 1; iphase <= 2; ++iphase) {
    if ((iphase == 1 ? mp->nspec_outer : mp->nspec_inner) <= 0) continue;
    launch_batch_stiffness(mp, iphase, s, soff, whole ? 0 : scnt);
    ++launches;
  }
  if (mp->nrec_local > 0) {
    dim3 grid((unsigned)mp->nrec_local, (unsigned)scnt);
    batch_seismogram_kernel<<<grid, NGLL3_PAD, 0, s>>>(mp->nrec_local, (int)S, mp->d_ispec_rec, mp->d_hxir,
                                                      mp->d_hetar, mp->d_hgammar, mp->d_nu_rec, mp->d_ibool,
                                                      B->displ, B->d_seismo, B->nlength, d_it, soff);
    ++launches;
  }
  batch_advance_kernel<<<1, 1, 0, s>>>(d_it);
  ++launches;
  return launches;
}

// One batched step of every shot on the compute stream (the first step: the
// predictor of every shot, then the rest of the step per counter).
int enqueue_batch_step(Mesh* mp, float dt, float dt2, float dtsq2, bool first) {
  BatchState* B = mp->batch;
  cudaStream_t s = mp->stream;
  const int S = B->nshots;
  int launches = 0;
  if (B->halves == 2 && first) {
    launches += enqueue_batch_part(mp, dt, dt2, dtsq2, true, 0, S, B->d_it, s, true);
    launches += enqueue_batch_part(mp, dt, dt2, dtsq2, false, 0, S / 2, B->d_it, s, false);
    launches += enqueue_batch_part(mp, dt, dt2, dtsq2, false, S / 2, S / 2, B->d_it + 1, s, false);
    return launches;
  }
  launches += enqueue_batch_part(mp, dt, dt2, dtsq2, first, 0, S, B->d_it, s, true);
  launches += enqueue_batch_part(mp, dt, dt2, dtsq2, first, 0, S, B->d_it, s, false);
  return launches;
}

// nsteps batched steps (not the first).  With two halves the shot halves run as
// two independent chains, the first on the compute stream and the second on the
// side stream, forked from and joined back into the compute stream around the
// whole segment: with no edge between the chains, one half's corrector (launched
// at the higher priority) is dispatched while the other half's stiffness runs.
int enqueue_batch_steps(Mesh* mp, float dt, float dt2, float dtsq2, int nsteps) {
  BatchState* B = mp->batch;
  int launches = 0;
  if (B->halves != 2) {
    for (int q = 0; q < nsteps; ++q) launches += enqueue_batch_step(mp, dt, dt2, dtsq2, false);
    return launches;
  }
  cudaStream_t s = mp->stream;
  const int h = B->nshots / 2;
  cudaEventRecord(B->ev_fork, s);
  cudaStreamWaitEvent(B->side, B->ev_fork, 0);
  for (int q = 0; q < nsteps; ++q) {
    launches += enqueue_batch_part(mp, dt, dt2, dtsq2, false, 0, h, B->d_it, s, true);
    launches += enqueue_batch_part(mp, dt, dt2, dtsq2, false, 0, h, B->d_it, s, false);
    launches += enqueue_batch_part(mp, dt, dt2, dtsq2, false, h, h, B->d_it + 1, B->side, true);
    launches += enqueue_batch_part(mp, dt, dt2, dtsq2, false, h, h, B->d_it + 1, B->side, false);
  }
  cudaEventRecord(B->ev_join, B->side);
  cudaStreamWaitEvent(s, B->ev_join, 0);
  return launches;
}

bool batch_ready(Mesh* mp) {
  if (!mp->batch) return set_error(SF3D_ERR_STATE, "sf3d_batch_prepare not called");
  default_phase_counts(mp);
  return true;
}

}  // namespace

void free_batch(Mesh* mp) {
  BatchState* B = mp->batch;
  if (!B) return;
  cudaFree(B->displ); cudaFree(B->veloc); cudaFree(B->accel);
  cudaFree(B->d_ispec_src); cudaFree(B->d_sa); cudaFree(B->d_stf); cudaFree(B->d_seismo); cudaFree(B->d_it);
  if (B->side) cudaStreamDestroy(B->side);
  if (B->ev_fork) cudaEventDestroy(B->ev_fork);
  if (B->ev_join) cudaEventDestroy(B->ev_join);
  delete B;
  mp->batch = nullptr;
}

}  // namespace sf3d

using namespace sf3d;

extern "C" {

int sf3d_batch_prepare(long* Mesh_pointer, int nshots, const int* ispec_selected_source,
                       const realw* sourcearrays, const double* stf, int nstep, int nlength, double* device_bytes) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (mp->anisotropy) {
    set_error(SF3D_ERR_ARG, "sf3d_batch_prepare: the batched kernels are isotropic");
    return SF3D_ERR_ARG;
  }
  if (!mp->f.displ || mp->num_phase_ispec <= 0) {
    set_error(SF3D_ERR_STATE, "sf3d_batch_prepare: prepare_fields_elastic_device not called");
    return SF3D_ERR_STATE;
  }
  if (mp->attenuation || mp->has_acoustic || mp->pml) {
    set_error(SF3D_ERR_ARG, "sf3d_batch_prepare: batched shots support elastic meshes without attenuation or C-PML");
    return SF3D_ERR_ARG;
  }
  if (nshots < 1 || nstep < 1 || nlength < 1 || !ispec_selected_source || !sourcearrays || !stf) {
    set_error(SF3D_ERR_ARG, "sf3d_batch_prepare: invalid arguments");
    return SF3D_ERR_ARG;
  }
  std::vector<int> isp(nshots);
  for (int s = 0; s < nshots; ++s) {
    if (ispec_selected_source[s] < 1 || ispec_selected_source[s] > mp->nspec) {
      set_error(SF3D_ERR_ARG, "sf3d_batch_prepare: ispec_selected_source out of range");
      return SF3D_ERR_ARG;
    }
    isp[s] = ispec_selected_source[s] - 1;
  }
  free_batch(mp);
  BatchState* B = new BatchState();
  mp->batch = B;
  B->nshots = nshots;
  B->nstep = nstep;
  B->nlength = nlength;
  B->shots_per_block = nshots % 8 == 0 ? 8 : (nshots % 4 == 0 ? 4 : (nshots % 2 == 0 ? 2 : 1));
  B->shots_per_thread = nshots % 4 == 0 ? 4 : 1;
  B->pencil_lanes = !pencil_fits_index32(mp, nshots) ? 0 : (nshots % 16 == 0 ? 16 : (nshots % 8 == 0 ? 8 : 0));
  const size_t n = 3ull * mp->nglob * nshots;
  std::vector<float> sa((size_t)nshots * NGLL3_PAD * 3, 0.f), tab((size_t)nstep * nshots);
  for (int s = 0; s < nshots; ++s)
    for (int p = 0; p < NGLL3; ++p)
      for (int c = 0; c < 3; ++c) sa[((size_t)s * NGLL3_PAD + p) * 3 + c] = sourcearrays[s + (size_t)nshots * (c + 3 * p)];
  for (int it = 0; it < nstep; ++it)
    for (int s = 0; s < nshots; ++s) tab[(size_t)it * nshots + s] = (float)stf[s + (size_t)nshots * it];
  const size_t nseis = 3ull * (mp->nrec_local > 0 ? mp->nrec_local : 1) * nshots * nlength;
  bool ok = alloc_f(&B->displ, n) && alloc_f(&B->veloc, n) && alloc_f(&B->accel, n) &&
            alloc_zero((void**)&B->d_ispec_src, sizeof(int) * nshots) && alloc_f(&B->d_sa, sa.size()) &&
            alloc_f(&B->d_stf, tab.size()) && alloc_f(&B->d_seismo, nseis) &&
            alloc_zero((void**)&B->d_it, 2 * sizeof(int)) &&
            cuda_ok(cudaStreamCreateWithFlags(&B->side, cudaStreamNonBlocking), "cudaStreamCreate") &&
            cuda_ok(cudaEventCreateWithFlags(&B->ev_fork, cudaEventDisableTiming), "cudaEventCreate") &&
            cuda_ok(cudaEventCreateWithFlags(&B->ev_join, cudaEventDisableTiming), "cudaEventCreate");
  int prio_lo = 0;
  ok = ok && cuda_ok(cudaDeviceGetStreamPriorityRange(&prio_lo, &B->prio_hi), "cudaDeviceGetStreamPriorityRange");
  ok = ok && copy_sync(B->d_ispec_src, isp.data(), sizeof(int) * nshots, cudaMemcpyHostToDevice, mp->stream) &&
       copy_sync(B->d_sa, sa.data(), sizeof(float) * sa.size(), cudaMemcpyHostToDevice, mp->stream) &&
       copy_sync(B->d_stf, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice, mp->stream);
  if (!ok) {
    free_batch(mp);
    return SF3D_ERR_CUDA;
  }
  B->bytes = sizeof(float) * (3 * n + sa.size() + tab.size() + nseis);
  if (device_bytes) *device_bytes = (double)B->bytes;
  return SF3D_OK;
}

int sf3d_batch_set_tiling(long* Mesh_pointer, int shots_per_block, int elements_per_block, int shots_per_thread) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!mp->batch) { set_error(SF3D_ERR_STATE, "sf3d_batch_prepare not called"); return SF3D_ERR_STATE; }
  const int sb = shots_per_block, eb = elements_per_block, spt = shots_per_thread;
  if (spt == 0) {
    // register-blocked pencils: sb shots per CTA, one element per CTA
    if ((sb != 8 && sb != 16 && sb != 32) || mp->batch->nshots % sb != 0 || eb != 1) {
      set_error(SF3D_ERR_ARG, "sf3d_batch_set_tiling: the pencil kernel takes 8, 16 or 32 shots per CTA "
                              "dividing nshots and one element per CTA");
      return SF3D_ERR_ARG;
    }
    if (!pencil_fits_index32(mp, mp->batch->nshots)) {
      set_error(SF3D_ERR_ARG, "sf3d_batch_set_tiling: the pencil kernel indexes the stacked fields in 32 bits "
                              "(3 nglob nshots < 2^32); use a per-point tiling");
      return SF3D_ERR_ARG;
    }
    mp->batch->pencil_lanes = sb;
    if (mp->batch->nshots % (2 * sb) != 0) mp->batch->halves = 1;
    return SF3D_OK;
  }
  const bool ok_sb = (sb == 1 || sb == 2 || sb == 4 || sb == 8) && mp->batch->nshots % sb == 0;
  const bool ok_spt = spt == 1 || (spt == 4 && (sb == 4 || sb == 8));
  if (!ok_sb || !ok_spt || (eb != 1 && eb != 2 && eb != 4)) {
    set_error(SF3D_ERR_ARG, "sf3d_batch_set_tiling: shots_per_block in {1,2,4,8} dividing nshots, "
                            "elements_per_block in {1,2,4}, shots_per_thread 1 or 4 (4 with 4 or 8 shots per block)");
    return SF3D_ERR_ARG;
  }
  mp->batch->pencil_lanes = 0;
  mp->batch->halves = 1;
  mp->batch->shots_per_block = sb;
  mp->batch->elements_per_block = eb;
  mp->batch->shots_per_thread = spt;
  return SF3D_OK;
}

int sf3d_batch_set_halves(long* Mesh_pointer, int halves) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!mp->batch) { set_error(SF3D_ERR_STATE, "sf3d_batch_prepare not called"); return SF3D_ERR_STATE; }
  BatchState* B = mp->batch;
  if (halves != 1 && halves != 2) {
    set_error(SF3D_ERR_ARG, "sf3d_batch_set_halves: halves must be 1 or 2");
    return SF3D_ERR_ARG;
  }
  if (halves == 2 && (B->pencil_lanes <= 0 || B->nshots % (2 * B->pencil_lanes) != 0)) {
    set_error(SF3D_ERR_ARG, "sf3d_batch_set_halves: two halves need the pencil kernel and a half of the shots "
                            "divisible by its shots per CTA");
    return SF3D_ERR_ARG;
  }
  B->halves = halves;
  return SF3D_OK;
}

int sf3d_batch_autotune(long* Mesh_pointer, int reps, float* ms_table, int* best_shots_per_block,
                        int* best_elements_per_block, int* best_shots_per_thread) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!batch_ready(mp)) return SF3D_ERR_STATE;
  BatchState* B = mp->batch;
  float mx = 0.f;
  if (!device_maxabs(mp, B->displ, 3L * mp->nglob * B->nshots, &mx)) return SF3D_ERR_CUDA;
  if (!(mx == 0.f)) {
    set_error(SF3D_ERR_STATE, "sf3d_batch_autotune must run on wavefields at rest (before the first step)");
    return SF3D_ERR_STATE;
  }
  if (reps < 1) reps = 1;
  const int sbs[4] = {1, 2, 4, 8}, ebs[3] = {1, 2, 4}, spts[2] = {1, 4}, lanes[3] = {8, 16, 32};
  int bsb = -1, beb = -1, bspt = -1;
  float best = 0.f;
  auto pass = [&]() {
    for (int iphase = 1; iphase <= 2; ++iphase) launch_batch_stiffness(mp, iphase, mp->stream);
  };
  auto time_it = [&](float* ms) -> bool {
    pass();
    if (!cuda_ok(cudaEventRecord(mp->ev0, mp->stream), "cudaEventRecord")) return false;
    for (int r = 0; r < reps; ++r) pass();
    if (!cuda_ok(cudaEventRecord(mp->ev1, mp->stream), "cudaEventRecord") ||
        !cuda_ok(cudaEventSynchronize(mp->ev1), "cudaEventSynchronize") ||
        !cuda_ok(cudaGetLastError(), "sf3d_batch_autotune"))
      return false;
    cudaEventElapsedTime(ms, mp->ev0, mp->ev1);
    *ms /= (float)reps;
    return true;
  };
  // table entries 0-23: per-point kernels [shots per thread 1,4] x [shots per CTA
  // 1,2,4,8] x [elements 1,2,4]; 24-26: pencil kernel with 8, 16, 32 shots per CTA
  B->pencil_lanes = 0;
  for (int v = 0; v < 2; ++v)
    for (int a = 0; a < 4; ++a)
      for (int b = 0; b < 3; ++b) {
        const int idx = (v * 4 + a) * 3 + b;
        if (ms_table) ms_table[idx] = -1.f;
        if (B->nshots % sbs[a] != 0) continue;
        if (spts[v] == 4 && sbs[a] < 4) continue;
        B->shots_per_block = sbs[a];
        B->elements_per_block = ebs[b];
        B->shots_per_thread = spts[v];
        float ms = 0.f;
        if (!time_it(&ms)) return SF3D_ERR_CUDA;
        if (ms_table) ms_table[idx] = ms;
        if (bsb < 0 || ms < best) { best = ms; bsb = sbs[a]; beb = ebs[b]; bspt = spts[v]; }
      }
  int blanes = 0;
  for (int q = 0; q < 3; ++q) {
    if (ms_table) ms_table[24 + q] = -1.f;
    if (B->nshots % lanes[q] != 0 || !pencil_fits_index32(mp, B->nshots)) continue;
    B->pencil_lanes = lanes[q];
    float ms = 0.f;
    if (!time_it(&ms)) return SF3D_ERR_CUDA;
    if (ms_table) ms_table[24 + q] = ms;
    if (bsb < 0 || ms < best) { best = ms; blanes = lanes[q]; }
  }
  B->pencil_lanes = blanes;
  if (blanes == 0 || B->nshots % (2 * blanes) != 0) B->halves = 1;
  if (blanes > 0) {
    bsb = blanes;
    beb = 1;
    bspt = 0;
  } else {
    B->shots_per_block = bsb;
    B->elements_per_block = beb;
    B->shots_per_thread = bspt;
  }
  if (best_shots_per_block) *best_shots_per_block = bsb;
  if (best_elements_per_block) *best_elements_per_block = beb;
  if (best_shots_per_thread) *best_shots_per_thread = bspt;
  return SF3D_OK;
}

int sf3d_batch_iterate(long* Mesh_pointer, int it_begin, int it_end, realw deltat, int steps_per_graph) {
  NvtxRange nvtx_range("sf3d_batch_iterate");
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!batch_ready(mp)) return SF3D_ERR_STATE;
  BatchState* B = mp->batch;
  if (it_begin < 1 || it_end < it_begin || it_end > B->nstep) {
    set_error(SF3D_ERR_ARG, "sf3d_batch_iterate: it range outside [1, nstep]");
    return SF3D_ERR_ARG;
  }
  const float dt = deltat, dt2 = deltat / 2.f, dtsq2 = deltat * deltat / 2.f;
  cudaStream_t s = mp->stream;
  batch_set_it_kernel<<<1, 1, 0, s>>>(B->d_it, it_begin);
  SF3D_CUDA_RET(cudaEventRecord(mp->ev0, s), SF3D_ERR_CUDA);
  int launches = 1 + enqueue_batch_step(mp, dt, dt2, dtsq2, true);
  int remaining = it_end - it_begin;
  const int K = steps_per_graph > 0 ? steps_per_graph : 0;
  if (K > 0 && remaining >= K) {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int per_block = 0;
    SF3D_CUDA_RET(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), SF3D_ERR_CUDA);
    per_block = enqueue_batch_steps(mp, dt, dt2, dtsq2, K);
    SF3D_CUDA_RET(cudaStreamEndCapture(s, &graph), SF3D_ERR_CUDA);
    SF3D_CUDA_RET(cudaGraphInstantiateWithFlags(&exec, graph, cudaGraphInstantiateFlagUseNodePriority),
                  SF3D_ERR_CUDA);
    while (remaining >= K) {
      if (!cuda_ok(cudaGraphLaunch(exec, s), "cudaGraphLaunch")) break;
      launches += per_block;
      remaining -= K;
    }
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
  }
  if (remaining > 0) launches += enqueue_batch_steps(mp, dt, dt2, dtsq2, remaining);
  const long n = 3L * mp->nglob * B->nshots;
  batch_mass_corrector_kernel<<<nblk(n, 256), 256, 0, s>>>(B->veloc, B->accel, mp->d_rmassx, mp->d_rmassy,
                                                          mp->d_rmassz, n, B->nshots, dt2);
  ++launches;
  SF3D_CUDA_RET(cudaEventRecord(mp->ev1, s), SF3D_ERR_CUDA);
  SF3D_CUDA_RET(cudaEventSynchronize(mp->ev1), SF3D_ERR_CUDA);
  if (!cuda_ok(cudaGetLastError(), "sf3d_batch_iterate")) return SF3D_ERR_CUDA;
  cudaEventElapsedTime(&B->last_ms, mp->ev0, mp->ev1);
  B->last_launches = launches;
  return sf3d_last_error(nullptr, 0);
}

int sf3d_batch_timing(long* Mesh_pointer, float* total_ms, int* launches) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!mp->batch) { set_error(SF3D_ERR_STATE, "sf3d_batch_prepare not called"); return SF3D_ERR_STATE; }
  if (total_ms) *total_ms = mp->batch->last_ms;
  if (launches) *launches = mp->batch->last_launches;
  return SF3D_OK;
}

int sf3d_batch_get_seismograms(long* Mesh_pointer, realw* h) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!mp->batch) { set_error(SF3D_ERR_STATE, "sf3d_batch_prepare not called"); return SF3D_ERR_STATE; }
  if (mp->nrec_local == 0) return SF3D_OK;
  BatchState* B = mp->batch;
  const size_t bytes = sizeof(float) * 3ull * mp->nrec_local * B->nshots * B->nlength;
  if (!copy_sync(h, B->d_seismo, bytes, cudaMemcpyDeviceToHost, mp->stream)) return SF3D_ERR_CUDA;
  return SF3D_OK;
}

int sf3d_batch_get_displ(long* Mesh_pointer, realw* h) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  if (!mp->batch) { set_error(SF3D_ERR_STATE, "sf3d_batch_prepare not called"); return SF3D_ERR_STATE; }
  const size_t bytes = sizeof(float) * 3ull * mp->nglob * mp->batch->nshots;
  if (!copy_sync(h, mp->batch->displ, bytes, cudaMemcpyDeviceToHost, mp->stream)) return SF3D_ERR_CUDA;
  return SF3D_OK;
}

int sf3d_batch_release(long* Mesh_pointer) {
  Mesh* mp = get_mesh(Mesh_pointer);
  if (!mp) return SF3D_ERR_STATE;
  cudaStreamSynchronize(mp->stream);
  free_batch(mp);
  return SF3D_OK;
}

}  // extern "C"
