/*
 * CPU oracle for the SPECFEM3D Cartesian spectral-element time step.
 *
 * TEST INFRASTRUCTURE ONLY: the reference against which the GB300 CUDA path is
 * tested.  sem_oracle.h gives the layout conventions.  Every routine below restates the
 * reference's CPU algorithm; the citation is the reference file:line it follows
 * (paths relative to the SPECFEM3D source tree).
 */
#include "sem_oracle.h"

#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define IJK(i, j, k) ((i) + NGLL * (j) + NGLL2 * (k))

/* ------------------------------------------------------------------------- */
/* named field table: lets the Python side hand over numpy buffers by name    */
/* ------------------------------------------------------------------------- */

typedef struct { const char *name; size_t off; } orc_field;
#define F(x) {#x, offsetof(orc_sim, x)}
static const orc_field k_ptr_fields[] = {
  F(ibool), F(irregular_element_number), F(xix), F(xiy), F(xiz), F(etax), F(etay), F(etaz),
  F(gammax), F(gammay), F(gammaz), F(jacobian), F(kappastore), F(mustore), F(rho_vp), F(rho_vs),
  F(rhostore), F(rmassx), F(rmassy), F(rmassz), F(hprime_xx), F(hprimewgll_xx), F(wgllwgll_xy),
  F(wgllwgll_xz), F(wgllwgll_yz), F(abs_boundary_ispec), F(abs_boundary_ijk),
  F(abs_boundary_normal), F(abs_boundary_jacobian2Dw), F(alphaval), F(betaval), F(gammaval),
  F(factor_common), F(factor_common_kappa), F(R_xx), F(R_yy), F(R_xy), F(R_xz), F(R_yz),
  F(R_trace), F(epsilondev_xx), F(epsilondev_yy), F(epsilondev_xy), F(epsilondev_xz),
  F(epsilondev_yz), F(epsilondev_trace), F(epsilon_trace_over_3), F(sourcearrays),
  F(ispec_selected_source), F(stf), F(ispec_selected_rec), F(hxir), F(hetar), F(hgammar),
  F(nu_rec), F(seismograms), F(displ), F(veloc), F(accel), F(b_displ), F(b_veloc), F(b_accel),
  F(b_epsilondev_xx), F(b_epsilondev_yy), F(b_epsilondev_xy), F(b_epsilondev_xz),
  F(b_epsilondev_yz), F(b_epsilon_trace_over_3), F(rho_kl), F(mu_kl), F(kappa_kl),
  F(source_adjoint), F(hxir_adj), F(hetar_adj), F(hgammar_adj), F(elastic_list), F(acoustic_list),
  F(ispec_is_acoustic), F(potential), F(potential_dot), F(potential_dot_dot), F(rmass_acoustic),
  F(coupling_ispec), F(coupling_ijk), F(coupling_normal), F(coupling_jacobian2Dw), F(free_surface_ispec),
  F(free_surface_ijk), F(rec_is_acoustic), F(cstore), F(is_cpml), F(cpml_to_spec), F(spec_to_cpml),
  F(pml_coef_alpha), F(pml_coef_beta), F(pml_coef_abar), F(pml_coef_strain), F(wgll_cube), F(pml_displ_old),
  F(pml_displ_new), F(pml_rmem),
};
static const orc_field k_int_fields[] = {
  F(nspec), F(nglob), F(nspec_irregular), F(nsources), F(nrec), F(nstep), F(it),
  F(attenuation), F(stacey), F(compute_and_store_strain), F(simulation_type), F(nthreads),
  F(record_what), F(num_abs_boundary_faces), F(n_elastic), F(n_acoustic), F(num_coupling_faces),
  F(num_free_surface_faces), F(fluid_vector), F(nspec_cpml),
};
static const orc_field k_real_fields[] = {
  F(xix_regular), F(jacobian_regular), F(deltat), F(deltatover2), F(deltatsqover2),
  F(b_deltat), F(b_deltatover2), F(b_deltatsqover2),
};
#undef F
#define NFIELDS(t) (sizeof(t) / sizeof((t)[0]))

int orc_realw_size(void) { return (int)sizeof(realw); }

orc_sim *orc_sim_new(void) {
  orc_sim *s = (orc_sim *)calloc(1, sizeof(orc_sim));
  if (s) { s->nthreads = 1; s->record_what = 1; s->simulation_type = 1; s->it = 1; s->n_elastic = -1; }
  return s;
}
void orc_sim_free(orc_sim *s) { free(s); }

int orc_set_ptr(orc_sim *s, const char *name, void *p) {
  for (size_t i = 0; i < NFIELDS(k_ptr_fields); ++i)
    if (!strcmp(k_ptr_fields[i].name, name)) { *(void **)((char *)s + k_ptr_fields[i].off) = p; return 0; }
  return -1;
}
int orc_set_int(orc_sim *s, const char *name, int v) {
  for (size_t i = 0; i < NFIELDS(k_int_fields); ++i)
    if (!strcmp(k_int_fields[i].name, name)) { *(int *)((char *)s + k_int_fields[i].off) = v; return 0; }
  return -1;
}
int orc_get_int(orc_sim *s, const char *name, int *v) {
  for (size_t i = 0; i < NFIELDS(k_int_fields); ++i)
    if (!strcmp(k_int_fields[i].name, name)) { *v = *(int *)((char *)s + k_int_fields[i].off); return 0; }
  return -1;
}
int orc_set_real(orc_sim *s, const char *name, double v) {
  for (size_t i = 0; i < NFIELDS(k_real_fields); ++i)
    if (!strcmp(k_real_fields[i].name, name)) { *(realw *)((char *)s + k_real_fields[i].off) = (realw)v; return 0; }
  return -1;
}

/* ------------------------------------------------------------------------- */
/* GLL quadrature and derivation matrices                                     */
/* ------------------------------------------------------------------------- */

/* Legendre polynomial P_n and derivative (gll_library.f90 pnleg/pndleg). */
static double pnleg(double z, int n) {
  double p1 = 1.0, p2 = z, p3 = 0.0;
  if (n == 0) return 1.0;
  for (int k = 1; k < n; ++k) { p3 = ((2.0 * k + 1.0) * z * p2 - k * p1) / (k + 1.0); p1 = p2; p2 = p3; }
  return p2;
}
static double pndleg(double z, int n) {
  double p1 = 1.0, p2 = z, p1d = 0.0, p2d = 1.0, p3, p3d;
  if (n == 0) return 0.0;
  for (int k = 1; k < n; ++k) {
    p3 = ((2.0 * k + 1.0) * z * p2 - k * p1) / (k + 1.0);
    p3d = ((2.0 * k + 1.0) * p2 + (2.0 * k + 1.0) * z * p2d - k * p1d) / (k + 1.0);
    p1 = p2; p2 = p3; p1d = p2d; p2d = p3d;
  }
  return p2d;
}

/* GLL points/weights for NGLL=5 (zwgljd, gll_library.f90:521-593, alpha=beta=0):
 * the roots of (1-x^2) P'_4(x), weights 2/(N(N+1) P_N(x)^2). */
void orc_gll(double *xigll, double *wgll) {
  const int N = NGLL - 1;
  xigll[0] = -1.0; xigll[1] = -sqrt(3.0 / 7.0); xigll[2] = 0.0; xigll[3] = sqrt(3.0 / 7.0); xigll[4] = 1.0;
  for (int i = 0; i < NGLL; ++i) {
    double p = pnleg(xigll[i], N);
    wgll[i] = 2.0 / (N * (N + 1.0) * p * p);
  }
}

/* lagrange_deriv_GLL (gll_library.f90:208-242): derivative of the i-th Lagrange
 * polynomial at GLL point j. */
static double lagrange_deriv_gll(int i, int j, const double *z) {
  const int d = NGLL - 1;
  if (i == 0 && j == 0) return -(double)d * (d + 1.0) / 4.0;
  if (i == d && j == d) return (double)d * (d + 1.0) / 4.0;
  if (i == j) return 0.0;
  return pnleg(z[j], d) / (pnleg(z[i], d) * (z[j] - z[i])) +
         (1.0 - z[j] * z[j]) * pndleg(z[j], d) /
             ((double)d * (d + 1.0) * pnleg(z[i], d) * (z[j] - z[i]) * (z[j] - z[i]));
}

/* define_derivation_matrices (define_derivation_matrices.f90:28-100):
 * hprime_xx(i2,i1) = l'_{i1}(xi_{i2}); hprimewgll_xx(i2,i1) = hprime_xx(i2,i1) w(i2). */
void orc_derivation_matrices(realw *hprime_xx, realw *hprimewgll_xx, realw *wgllwgll_xy,
                             realw *wgllwgll_xz, realw *wgllwgll_yz, double *hprime_d) {
  double x[NGLL], w[NGLL];
  orc_gll(x, w);
  for (int i1 = 0; i1 < NGLL; ++i1)
    for (int i2 = 0; i2 < NGLL; ++i2) {
      double d = lagrange_deriv_gll(i1, i2, x);
      if (hprime_d) hprime_d[i2 + NGLL * i1] = d;
      hprime_xx[i2 + NGLL * i1] = (realw)d;
      hprimewgll_xx[i2 + NGLL * i1] = (realw)(d * w[i2]);
    }
  for (int i = 0; i < NGLL; ++i)
    for (int j = 0; j < NGLL; ++j) {
      wgllwgll_xy[i + NGLL * j] = (realw)(w[i] * w[j]);
      wgllwgll_xz[i + NGLL * j] = (realw)(w[i] * w[j]);
      wgllwgll_yz[i + NGLL * j] = (realw)(w[i] * w[j]);
    }
}

/* lagrange_any (lagrange_poly.f90:30-199): Lagrange interpolants and their
 * derivatives at xi, on the GLL points. */
void orc_lagrange_any(double xi, const double *xigll, double *h, double *hprime) {
  for (int dgr = 0; dgr < NGLL; ++dgr) {
    double prod1 = 1.0, prod2 = 1.0;
    for (int i = 0; i < NGLL; ++i) {
      if (i == dgr) continue;
      prod1 *= (xi - xigll[i]);
      prod2 *= (xigll[dgr] - xigll[i]);
    }
    h[dgr] = prod1 / prod2;
    double sum = 0.0;
    for (int i = 0; i < NGLL; ++i) {
      if (i == dgr) continue;
      double prod3 = 1.0;
      for (int j = 0; j < NGLL; ++j) {
        if (j == dgr || j == i) continue;
        prod3 *= (xi - xigll[j]);
      }
      sum += prod3;
    }
    hprime[dgr] = sum / prod2;
  }
}

/* ------------------------------------------------------------------------- */
/* 8-node hexahedron shape functions (get_shape3D.f90), node order            */
/* 1(-,-,-) 2(+,-,-) 3(+,+,-) 4(-,+,-) 5(-,-,+) 6(+,-,+) 7(+,+,+) 8(-,+,+)     */
/* ------------------------------------------------------------------------- */

static const int k_sx[8] = {-1, 1, 1, -1, -1, 1, 1, -1};
static const int k_sy[8] = {-1, -1, 1, 1, -1, -1, 1, 1};
static const int k_sz[8] = {-1, -1, -1, -1, 1, 1, 1, 1};

static void shape8(double xi, double eta, double ga, double *sh, double *dsh /* [3][8] */) {
  for (int a = 0; a < 8; ++a) {
    double fx = 1.0 + k_sx[a] * xi, fy = 1.0 + k_sy[a] * eta, fz = 1.0 + k_sz[a] * ga;
    sh[a] = 0.125 * fx * fy * fz;
    dsh[0 * 8 + a] = 0.125 * k_sx[a] * fy * fz;
    dsh[1 * 8 + a] = 0.125 * fx * k_sy[a] * fz;
    dsh[2 * 8 + a] = 0.125 * fx * fy * k_sz[a];
  }
}

/* ------------------------------------------------------------------------- */
/* regular layered block mesher (the internal-mesher geometry of the examples) */
/* ------------------------------------------------------------------------- */

/* Element order: x fastest, then y, then z from the bottom (the order of the
 * reference example's mesh_file, EXAMPLES/applications/homogeneous_halfspace_
 * HEX8_elastic_absorbing_Stacey_5sides/MESH-default).  zlev[0..nz] are the
 * vertical node levels.  anchors[(c + 3 a) + 24 ispec] for node a=0..7.
 * GLL coordinates follow calc_coords (calc_jacobian.f90:148-178). */
void orc_mesh_regular(int nx, int ny, int nz, double x0, double x1, double y0, double y1,
                      const double *zlev, double *anchors, double *xstore, double *ystore,
                      double *zstore) {
  double xg[NGLL], wg[NGLL];
  orc_gll(xg, wg);
  for (int ez = 0; ez < nz; ++ez)
    for (int ey = 0; ey < ny; ++ey)
      for (int ex = 0; ex < nx; ++ex) {
        long ispec = ex + (long)nx * (ey + (long)ny * ez);
        double xa = x0 + (x1 - x0) * ex / nx, xb = x0 + (x1 - x0) * (ex + 1) / nx;
        double ya = y0 + (y1 - y0) * ey / ny, yb = y0 + (y1 - y0) * (ey + 1) / ny;
        double za = zlev[ez], zb = zlev[ez + 1];
        double *an = anchors + 24 * ispec;
        for (int a = 0; a < 8; ++a) {
          an[3 * a + 0] = k_sx[a] < 0 ? xa : xb;
          an[3 * a + 1] = k_sy[a] < 0 ? ya : yb;
          an[3 * a + 2] = k_sz[a] < 0 ? za : zb;
        }
        for (int k = 0; k < NGLL; ++k)
          for (int j = 0; j < NGLL; ++j)
            for (int i = 0; i < NGLL; ++i) {
              double sh[8], dsh[24];
              shape8(xg[i], xg[j], xg[k], sh, dsh);
              double xm = 0, ym = 0, zm = 0;
              for (int a = 0; a < 8; ++a) { xm += sh[a] * an[3 * a]; ym += sh[a] * an[3 * a + 1]; zm += sh[a] * an[3 * a + 2]; }
              long p = IJK(i, j, k) + NGLL3 * ispec;
              xstore[p] = xm; ystore[p] = ym; zstore[p] = zm;
            }
      }
}

/* GLL point coordinates of any 8-node hexahedral mesh (calc_coords,
 * calc_jacobian.f90:148-178): anchors[(c + 3 a) + 24 ispec]. */
void orc_gll_coordinates(int nspec, const double *anchors, double *xstore, double *ystore, double *zstore) {
  double xg[NGLL], wg[NGLL];
  orc_gll(xg, wg);
  for (long ispec = 0; ispec < nspec; ++ispec) {
    const double *an = anchors + 24 * ispec;
    for (int k = 0; k < NGLL; ++k)
      for (int j = 0; j < NGLL; ++j)
        for (int i = 0; i < NGLL; ++i) {
          double sh[8], dsh[24];
          shape8(xg[i], xg[j], xg[k], sh, dsh);
          double xm = 0, ym = 0, zm = 0;
          for (int a = 0; a < 8; ++a) { xm += sh[a] * an[3 * a]; ym += sh[a] * an[3 * a + 1]; zm += sh[a] * an[3 * a + 2]; }
          long p = IJK(i, j, k) + NGLL3 * ispec;
          xstore[p] = xm; ystore[p] = ym; zstore[p] = zm;
        }
  }
}

/* ------------------------------------------------------------------------- */
/* global numbering: get_global + get_global_indirect_addressing               */
/* (get_global.f90:28-141, sort_array_coordinates.f90:30-128)                  */
/* ------------------------------------------------------------------------- */

typedef struct { double key[3]; long loc; } gpt;
static int g_axis;
static int cmp_gpt(const void *a, const void *b) {
  const gpt *p = (const gpt *)a, *q = (const gpt *)b;
  double u = p->key[g_axis], v = q->key[g_axis];
  if (u < v) return -1;
  if (u > v) return 1;
  return (p->loc < q->loc) ? -1 : (p->loc > q->loc);
}

/* Lexicographic segment sort with tolerance xtol (sort_array_coordinates), then
 * renumbering by first appearance in element order (get_global_indirect_addressing).
 * Returns nglob; ibool receives 1-based global indices. */
int orc_get_global(long npointot, const double *xp, const double *yp, const double *zp,
                   int *ibool, double xtol) {
  gpt *pts = (gpt *)malloc(sizeof(gpt) * npointot);
  char *ifseg = (char *)calloc(npointot, 1);
  long *ninseg = (long *)malloc(sizeof(long) * npointot);
  int *iglob = (int *)malloc(sizeof(int) * npointot);
  for (long i = 0; i < npointot; ++i) {
    pts[i].key[0] = xp[i]; pts[i].key[1] = yp[i]; pts[i].key[2] = zp[i]; pts[i].loc = i;
  }
  long nseg = 1;
  ifseg[0] = 1;
  ninseg[0] = npointot;
  for (int j = 0; j < 3; ++j) {
    long ioff = 0;
    g_axis = j;
    for (long iseg = 0; iseg < nseg; ++iseg) {
      qsort(pts + ioff, ninseg[iseg], sizeof(gpt), cmp_gpt);
      ioff += ninseg[iseg];
    }
    for (long i = 1; i < npointot; ++i)
      if (fabs(pts[i].key[j] - pts[i - 1].key[j]) > xtol) ifseg[i] = 1;
    nseg = 0;
    for (long i = 0; i < npointot; ++i) {
      if (ifseg[i]) { ninseg[nseg] = 1; nseg++; }
      else ninseg[nseg - 1]++;
    }
  }
  int ig = 0;
  for (long i = 0; i < npointot; ++i) {
    if (ifseg[i]) ig++;
    iglob[pts[i].loc] = ig;
  }
  int nglob = ig;
  /* indirect addressing: renumber by first appearance */
  int *mask = (int *)malloc(sizeof(int) * (nglob + 1));
  for (int i = 0; i <= nglob; ++i) mask[i] = -1;
  int inumber = 0;
  for (long p = 0; p < npointot; ++p) {
    int g = iglob[p];
    if (mask[g] == -1) { inumber++; mask[g] = inumber; }
    ibool[p] = mask[g];
  }
  free(mask); free(pts); free(ifseg); free(ninseg); free(iglob);
  return nglob;
}

/* ------------------------------------------------------------------------- */
/* Jacobian and regular/irregular element separation                          */
/* (calc_jacobian.f90:28-142, :184-360; create_regions_mesh.f90:693-716,1083) */
/* ------------------------------------------------------------------------- */

static void calc_jacobian_elem(const double *an, realw *out /* [10][125] */) {
  double xg[NGLL], wg[NGLL];
  orc_gll(xg, wg);
  for (int k = 0; k < NGLL; ++k)
    for (int j = 0; j < NGLL; ++j)
      for (int i = 0; i < NGLL; ++i) {
        double sh[8], dsh[24];
        shape8(xg[i], xg[j], xg[k], sh, dsh);
        double xxi = 0, xeta = 0, xgamma = 0, yxi = 0, yeta = 0, ygamma = 0, zxi = 0, zeta = 0, zgamma = 0;
        for (int a = 0; a < 8; ++a) {
          xxi += dsh[a] * an[3 * a]; xeta += dsh[8 + a] * an[3 * a]; xgamma += dsh[16 + a] * an[3 * a];
          yxi += dsh[a] * an[3 * a + 1]; yeta += dsh[8 + a] * an[3 * a + 1]; ygamma += dsh[16 + a] * an[3 * a + 1];
          zxi += dsh[a] * an[3 * a + 2]; zeta += dsh[8 + a] * an[3 * a + 2]; zgamma += dsh[16 + a] * an[3 * a + 2];
        }
        double jac = xxi * (yeta * zgamma - ygamma * zeta) - xeta * (yxi * zgamma - ygamma * zxi) +
                     xgamma * (yxi * zeta - yeta * zxi);
        double xix = (yeta * zgamma - ygamma * zeta) / jac;
        double xiy = (xgamma * zeta - xeta * zgamma) / jac;
        double xiz = (xeta * ygamma - xgamma * yeta) / jac;
        double etax = (ygamma * zxi - yxi * zgamma) / jac;
        double etay = (xxi * zgamma - xgamma * zxi) / jac;
        double etaz = (xgamma * yxi - xxi * ygamma) / jac;
        double gammax = (yxi * zeta - yeta * zxi) / jac;
        double gammay = (xeta * zxi - xxi * zeta) / jac;
        double gammaz = (xxi * yeta - xeta * yxi) / jac;
        jac = 1.0 / (xix * (etay * gammaz - etaz * gammay) - xiy * (etax * gammaz - etaz * gammax) +
                     xiz * (etax * gammay - etay * gammax));
        int p = IJK(i, j, k);
        out[0 * NGLL3 + p] = (realw)xix; out[1 * NGLL3 + p] = (realw)xiy; out[2 * NGLL3 + p] = (realw)xiz;
        out[3 * NGLL3 + p] = (realw)etax; out[4 * NGLL3 + p] = (realw)etay; out[5 * NGLL3 + p] = (realw)etaz;
        out[6 * NGLL3 + p] = (realw)gammax; out[7 * NGLL3 + p] = (realw)gammay; out[8 * NGLL3 + p] = (realw)gammaz;
        out[9 * NGLL3 + p] = (realw)jac;
      }
}

static int is_equal_number(float a, float b) { return fabsf(a - b) <= 1.1920929e-7f; }

/* Fills the 10 metric arrays (size 125*nspec, only the first nspec_irregular
 * element slots are meaningful afterwards), irregular_element_number (1-based
 * or 0) and the regular-element constants.  Returns nspec_irregular. */
int orc_calc_jacobian_all(int nspec, const double *anchors, realw **metric /* 10 ptrs */,
                          int *irregular_element_number, realw *xix_regular, realw *jacobian_regular) {
  int nspec_irregular = nspec;
  int any_regular = 0;
  double cube_edge_sq = 1.e9;
  realw buf[10 * NGLL3];
  int first_regular = -1;
  for (int ispec = 0; ispec < nspec; ++ispec) {
    const double *an = anchors + 24 * ispec;
    float xe[8], ye[8], ze[8];
    for (int a = 0; a < 8; ++a) { xe[a] = (float)an[3 * a]; ye[a] = (float)an[3 * a + 1]; ze[a] = (float)an[3 * a + 2]; }
    double d1 = (double)(xe[1] - xe[0]) * (xe[1] - xe[0]) + (double)(ye[1] - ye[0]) * (ye[1] - ye[0]) +
                (double)(ze[1] - ze[0]) * (ze[1] - ze[0]);
    double thr = 1.e-5 * cube_edge_sq;
    int regular = 0;
    if (!(any_regular && fabs(d1 - cube_edge_sq) > thr)) {
      int eq = is_equal_number(xe[0], xe[3]) && is_equal_number(xe[0], xe[4]) && is_equal_number(xe[0], xe[7]) &&
               is_equal_number(xe[1], xe[2]) && is_equal_number(xe[1], xe[5]) && is_equal_number(xe[1], xe[6]) &&
               is_equal_number(ye[0], ye[1]) && is_equal_number(ye[0], ye[4]) && is_equal_number(ye[0], ye[5]) &&
               is_equal_number(ye[2], ye[3]) && is_equal_number(ye[2], ye[6]) && is_equal_number(ye[2], ye[7]) &&
               is_equal_number(ze[0], ze[1]) && is_equal_number(ze[0], ze[2]) && is_equal_number(ze[0], ze[3]) &&
               is_equal_number(ze[4], ze[5]) && is_equal_number(ze[4], ze[6]) && is_equal_number(ze[4], ze[7]);
      if (eq) {
        double d2 = (double)(xe[4] - xe[0]) * (xe[4] - xe[0]) + (double)(ye[4] - ye[0]) * (ye[4] - ye[0]) +
                    (double)(ze[4] - ze[0]) * (ze[4] - ze[0]);
        double d3 = (double)(xe[3] - xe[0]) * (xe[3] - xe[0]) + (double)(ye[3] - ye[0]) * (ye[3] - ye[0]) +
                    (double)(ze[3] - ze[0]) * (ze[3] - ze[0]);
        double t2 = 1.e-5 * d1;
        if (fabs(d2 - d1) < t2 && fabs(d3 - d1) < t2) {
          double and_[24];
          for (int a = 0; a < 8; ++a) { and_[3 * a] = xe[a]; and_[3 * a + 1] = ye[a]; and_[3 * a + 2] = ze[a]; }
          calc_jacobian_elem(and_, buf);
          const double tz = 1.e-25;
          if (fabs((double)buf[0] - buf[4 * NGLL3]) < tz && fabs((double)buf[0] - buf[8 * NGLL3]) < tz &&
              fabs((double)buf[1 * NGLL3]) < tz && fabs((double)buf[2 * NGLL3]) < tz &&
              fabs((double)buf[3 * NGLL3]) < tz && fabs((double)buf[5 * NGLL3]) < tz &&
              fabs((double)buf[6 * NGLL3]) < tz && fabs((double)buf[7 * NGLL3]) < tz)
            regular = 1;
        }
      }
    }
    if (regular) {
      irregular_element_number[ispec] = 0;
      if (!any_regular) { cube_edge_sq = d1; any_regular = 1; first_regular = ispec; }
      nspec_irregular--;
    } else {
      irregular_element_number[ispec] = (ispec + 1) - (nspec - nspec_irregular);
    }
  }
  /* metric of irregular elements, compacted by their irregular number */
  for (int ispec = 0; ispec < nspec; ++ispec) {
    int ir = irregular_element_number[ispec];
    if (ir == 0) continue;
    calc_jacobian_elem(anchors + 24 * ispec, buf);
    for (int m = 0; m < 10; ++m) memcpy(metric[m] + (long)(ir - 1) * NGLL3, buf + m * NGLL3, sizeof(realw) * NGLL3);
  }
  *xix_regular = 0; *jacobian_regular = 0;
  if (first_regular >= 0) {
    calc_jacobian_elem(anchors + 24 * first_regular, buf);
    *xix_regular = buf[0];
    *jacobian_regular = buf[9 * NGLL3];
  }
  return nspec_irregular;
}

/* ------------------------------------------------------------------------- */
/* mass matrices (define_mass_matrices.f90:28-75, :353-442;                  */
/* prepare_timerun.F90:246-388)                                              */
/* ------------------------------------------------------------------------- */

void orc_mass_elastic(int nspec, int nglob, const int *ibool, const realw *rhostore,
                      const realw *jacobianstore, const int *irregular_element_number,
                      realw jacobian_regular, realw *rmass) {
  double xg[NGLL], w[NGLL];
  orc_gll(xg, w);
  for (int i = 0; i < nglob; ++i) rmass[i] = 0;
  for (int ispec = 0; ispec < nspec; ++ispec) {
    int ir = irregular_element_number[ispec];
    for (int k = 0; k < NGLL; ++k)
      for (int j = 0; j < NGLL; ++j)
        for (int i = 0; i < NGLL; ++i) {
          long p = IJK(i, j, k) + (long)NGLL3 * ispec;
          int iglob = ibool[p] - 1;
          double weight = w[i] * w[j] * w[k];
          realw jl = ir ? jacobianstore[IJK(i, j, k) + (long)NGLL3 * (ir - 1)] : jacobian_regular;
          rmass[iglob] = rmass[iglob] + (realw)((double)jl * weight * (double)rhostore[p]);
        }
  }
}

void orc_mass_stacey_elastic(int nglob, double DT, const int *ibool, const realw *rho_vp,
                             const realw *rho_vs, int nfaces, const int *abs_ispec,
                             const int *abs_ijk, const realw *abs_normal, const realw *abs_jw,
                             realw *rmassx, realw *rmassy, realw *rmassz) {
  realw deltatover2 = (realw)(0.5 * DT);
  for (int i = 0; i < nglob; ++i) rmassx[i] = rmassy[i] = rmassz[i] = 0;
  for (int f = 0; f < nfaces; ++f) {
    int ispec = abs_ispec[f] - 1;
    for (int g = 0; g < NGLL2; ++g) {
      int i = abs_ijk[0 + 3 * (g + NGLL2 * f)] - 1, j = abs_ijk[1 + 3 * (g + NGLL2 * f)] - 1,
          k = abs_ijk[2 + 3 * (g + NGLL2 * f)] - 1;
      long p = IJK(i, j, k) + (long)NGLL3 * ispec;
      realw nx = abs_normal[0 + 3 * (g + NGLL2 * f)], ny = abs_normal[1 + 3 * (g + NGLL2 * f)],
            nz = abs_normal[2 + 3 * (g + NGLL2 * f)];
      realw vn = deltatover2 * (nx + ny + nz);
      realw tx = rho_vp[p] * vn * nx + rho_vs[p] * (deltatover2 - vn * nx);
      realw ty = rho_vp[p] * vn * ny + rho_vs[p] * (deltatover2 - vn * ny);
      realw tz = rho_vp[p] * vn * nz + rho_vs[p] * (deltatover2 - vn * nz);
      realw jw = abs_jw[g + NGLL2 * f];
      int iglob = ibool[p] - 1;
      rmassx[iglob] += tx * jw; rmassy[iglob] += ty * jw; rmassz[iglob] += tz * jw;
    }
  }
}

/* rmass{x,y,z} = 1 / (M + C) with the Stacey term (prepare_timerun.F90:262-340). */
void orc_invert_mass(int nglob, const realw *rmass, realw *rmassx, realw *rmassy, realw *rmassz,
                     int with_stacey) {
  for (int i = 0; i < nglob; ++i) {
    realw mx = with_stacey ? rmass[i] + rmassx[i] : rmass[i];
    realw my = with_stacey ? rmass[i] + rmassy[i] : rmass[i];
    realw mz = with_stacey ? rmass[i] + rmassz[i] : rmass[i];
    if (mx <= 0) mx = 1;
    if (my <= 0) my = 1;
    if (mz <= 0) mz = 1;
    rmassx[i] = (realw)1 / mx; rmassy[i] = (realw)1 / my; rmassz[i] = (realw)1 / mz;
  }
}

/* ------------------------------------------------------------------------- */
/* boundary faces of a box (get_absorbing_boundary.F90:28-930,               */
/* get_element_face.f90:169-279, get_jacobian_boundaries.f90:28-297)          */
/* ------------------------------------------------------------------------- */

/* Face iface (1..6 = xmin,xmax,ymin,ymax,bottom,top) of element ispec:
 * ijk (3,25), jacobian2Dw(25), outward normal (3,25), computed from the element
 * anchors with 4-node bilinear face shape functions.  GLL order: first face
 * index fastest (get_element_face_gll_indices). */
void orc_face_geometry(const double *an, int iface, int *ijk, realw *jw, realw *normal) {
  double xg[NGLL], w[NGLL];
  orc_gll(xg, w);
  /* face corner nodes (a,b) = (-,-),(+,-),(+,+),(-,+) in the face's own axes */
  static const int faces[6][4] = {{0, 3, 7, 4}, {1, 2, 6, 5}, {0, 1, 5, 4}, {3, 2, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};
  const int *fc = faces[iface - 1];
  double cx[4][3];
  for (int c = 0; c < 4; ++c)
    for (int d = 0; d < 3; ++d) cx[c][d] = an[3 * fc[c] + d];
  /* element centre, to orient the normal outward (get_element_face_normal) */
  double ctr[3] = {0, 0, 0};
  for (int a = 0; a < 8; ++a)
    for (int d = 0; d < 3; ++d) ctr[d] += 0.125 * an[3 * a + d];
  int g = 0;
  for (int b = 0; b < NGLL; ++b)
    for (int a = 0; a < NGLL; ++a, ++g) {
      int i, j, k;
      switch (iface) {
        case 1: i = 0; j = a; k = b; break;
        case 2: i = NGLL - 1; j = a; k = b; break;
        case 3: i = a; j = 0; k = b; break;
        case 4: i = a; j = NGLL - 1; k = b; break;
        case 5: i = a; j = b; k = 0; break;
        default: i = a; j = b; k = NGLL - 1; break;
      }
      ijk[3 * g] = i + 1; ijk[3 * g + 1] = j + 1; ijk[3 * g + 2] = k + 1;
      double s = xg[a], t = xg[b];
      double dsa[4] = {-0.25 * (1 - t), 0.25 * (1 - t), 0.25 * (1 + t), -0.25 * (1 + t)};
      double dsb[4] = {-0.25 * (1 - s), -0.25 * (1 + s), 0.25 * (1 + s), 0.25 * (1 - s)};
      double sh[4] = {0.25 * (1 - s) * (1 - t), 0.25 * (1 + s) * (1 - t), 0.25 * (1 + s) * (1 + t), 0.25 * (1 - s) * (1 + t)};
      double e1[3] = {0, 0, 0}, e2[3] = {0, 0, 0}, px[3] = {0, 0, 0};
      for (int c = 0; c < 4; ++c)
        for (int d = 0; d < 3; ++d) { e1[d] += dsa[c] * cx[c][d]; e2[d] += dsb[c] * cx[c][d]; px[d] += sh[c] * cx[c][d]; }
      double n[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
      double jac2 = sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
      for (int d = 0; d < 3; ++d) n[d] /= jac2;
      double dot = n[0] * (px[0] - ctr[0]) + n[1] * (px[1] - ctr[1]) + n[2] * (px[2] - ctr[2]);
      if (dot < 0) for (int d = 0; d < 3; ++d) n[d] = -n[d];
      jw[g] = (realw)(jac2 * w[a] * w[b]);
      for (int d = 0; d < 3; ++d) normal[3 * g + d] = (realw)n[d];
    }
}

/* ------------------------------------------------------------------------- */
/* point location (locate_point.f90:32-416, :422-624)                         */
/* ------------------------------------------------------------------------- */

/* find_local_coordinates (locate_point.f90:422-624): up to 5 Newton steps on
 * (xi, eta, gamma) from GLL point (ix, iy, iz) of the element, stopping when the
 * distance stops decreasing; steps longer than 1 are cut to a third; the local
 * coordinates are clamped to [-1.01, 1.01].  d2 = final squared distance. */
static void find_local(const double *an, double xt, double yt, double zt, int ix, int iy, int iz,
                       double *xi_o, double *eta_o, double *ga_o, double *d2_o) {
  double xg[NGLL], wg[NGLL];
  orc_gll(xg, wg);
  double xi = xg[ix], eta = xg[iy], ga = xg[iz], dmin2 = 1e30;
  for (int it = 0; it < 5; ++it) {
    double sh[8], dsh[24], x = 0, y = 0, z = 0;
    double J[3][3] = {{0}};
    shape8(xi, eta, ga, sh, dsh);
    for (int a = 0; a < 8; ++a) {
      x += sh[a] * an[3 * a]; y += sh[a] * an[3 * a + 1]; z += sh[a] * an[3 * a + 2];
      for (int d = 0; d < 3; ++d)
        for (int e = 0; e < 3; ++e) J[e][d] += dsh[d * 8 + a] * an[3 * a + e];
    }
    double dx = xt - x, dy = yt - y, dz = zt - z, d2 = dx * dx + dy * dy + dz * dz;
    if (!(d2 < dmin2)) break;
    dmin2 = d2;
    double det = J[0][0] * (J[1][1] * J[2][2] - J[1][2] * J[2][1]) - J[0][1] * (J[1][0] * J[2][2] - J[1][2] * J[2][0]) +
                 J[0][2] * (J[1][0] * J[2][1] - J[1][1] * J[2][0]);
    double inv[3][3];
    inv[0][0] = (J[1][1] * J[2][2] - J[1][2] * J[2][1]) / det; inv[0][1] = (J[0][2] * J[2][1] - J[0][1] * J[2][2]) / det;
    inv[0][2] = (J[0][1] * J[1][2] - J[0][2] * J[1][1]) / det; inv[1][0] = (J[1][2] * J[2][0] - J[1][0] * J[2][2]) / det;
    inv[1][1] = (J[0][0] * J[2][2] - J[0][2] * J[2][0]) / det; inv[1][2] = (J[0][2] * J[1][0] - J[0][0] * J[1][2]) / det;
    inv[2][0] = (J[1][0] * J[2][1] - J[1][1] * J[2][0]) / det; inv[2][1] = (J[0][1] * J[2][0] - J[0][0] * J[2][1]) / det;
    inv[2][2] = (J[0][0] * J[1][1] - J[0][1] * J[1][0]) / det;
    double dxi = inv[0][0] * dx + inv[0][1] * dy + inv[0][2] * dz;
    double deta = inv[1][0] * dx + inv[1][1] * dy + inv[1][2] * dz;
    double dga = inv[2][0] * dx + inv[2][1] * dy + inv[2][2] * dz;
    if (dxi * dxi + deta * deta + dga * dga > 1.0) { dxi *= 0.33333333333; deta *= 0.33333333333; dga *= 0.33333333333; }
    xi += dxi; eta += deta; ga += dga;
    xi = xi > 1.01 ? 1.01 : (xi < -1.01 ? -1.01 : xi);
    eta = eta > 1.01 ? 1.01 : (eta < -1.01 ? -1.01 : eta);
    ga = ga > 1.01 ? 1.01 : (ga < -1.01 ? -1.01 : ga);
  }
  /* position and distance at the final local coordinates */
  double sh[8], dsh[24], x = 0, y = 0, z = 0;
  shape8(xi, eta, ga, sh, dsh);
  for (int a = 0; a < 8; ++a) { x += sh[a] * an[3 * a]; y += sh[a] * an[3 * a + 1]; z += sh[a] * an[3 * a + 2]; }
  *xi_o = xi; *eta_o = eta; *ga_o = ga;
  *d2_o = (xt - x) * (xt - x) + (yt - y) * (yt - y) + (zt - z) * (zt - z);
}

static int outside(double xi, double eta, double ga) { return fabs(xi) > 1.0 || fabs(eta) > 1.0 || fabs(ga) > 1.0; }

/* locate_point_in_mesh (locate_point.f90:32-416) with the brute-force first
 * guess: the closest GLL point over all elements (single-precision coordinates,
 * first strictly closer point in element, k, j, i order), Newton in that element;
 * unless the result lies strictly inside the element (or above the top of a
 * surface element), up to 3 rounds of find_best_neighbor (:630-804) over the
 * element's neighbours (CSR xadj/adjncy, 0-based; NULL = none).
 * surface_pt flags GLL points (per element, 125*nspec) on the mesh's outer
 * surface; is_acoustic flags fluid elements (NULL = all solid).
 * Returns ispec (1-based). */
int orc_locate_point(int nspec, const double *anchors, const double *xs, const double *ys,
                     const double *zs, const int *xadj, const int *adjncy, const unsigned char *surface_pt,
                     const int *is_acoustic, double xt, double yt, double zt, double *xi_out,
                     double *eta_out, double *gamma_out) {
  double dmin = 1e300;
  int isel = 0, ix = 0, iy = 0, iz = 0;
  for (int ispec = 0; ispec < nspec; ++ispec)
    for (int k = 0; k < NGLL; ++k)
      for (int j = 0; j < NGLL; ++j)
        for (int i = 0; i < NGLL; ++i) {
          long p = IJK(i, j, k) + (long)NGLL3 * ispec;
          double x = (float)xs[p], y = (float)ys[p], z = (float)zs[p];
          double d = (xt - x) * (xt - x) + (yt - y) * (yt - y) + (zt - z) * (zt - z);
          if (d < dmin) { dmin = d; isel = ispec; ix = i; iy = j; iz = k; }
        }
  double xi, eta, ga, d2;
  find_local(anchors + 24 * (long)isel, xt, yt, zt, ix, iy, iz, &xi, &eta, &ga, &d2);
  int search = !(fabs(xi) < 1.0 && fabs(eta) < 1.0 && fabs(ga) < 1.0);
  if (search && ga > 1.0 && surface_pt && surface_pt[IJK(ix, iy, iz) + (long)NGLL3 * isel]) search = 0;
  if (search && xadj) {
    for (int itry = 0; itry < 3; ++itry) {
      int e0 = isel;
      for (int q = xadj[e0]; q < xadj[e0 + 1]; ++q) {
        int e = adjncy[q];
        /* best GLL point of this neighbour as the starting guess */
        double dg = 1e300;
        int gx = NGLL / 2, gy = NGLL / 2, gz = NGLL / 2;
        for (int k = 0; k < NGLL; ++k)
          for (int j = 0; j < NGLL; ++j)
            for (int i = 0; i < NGLL; ++i) {
              long p = IJK(i, j, k) + (long)NGLL3 * e;
              double x = (float)xs[p], y = (float)ys[p], z = (float)zs[p];
              double d = (xt - x) * (xt - x) + (yt - y) * (yt - y) + (zt - z) * (zt - z);
              if (d < dg) { dg = d; gx = i; gy = j; gz = k; }
            }
        double nxi, neta, nga, nd2;
        find_local(anchors + 24 * (long)e, xt, yt, zt, gx, gy, gz, &nxi, &neta, &nga, &nd2);
        int better = 0;
        if (nd2 < 1e-10 && !outside(nxi, neta, nga)) {
          if (outside(xi, eta, ga)) better = 1;
          if (is_acoustic && is_acoustic[isel] && !is_acoustic[e]) better = 1;
        }
        /* a closer location: improvements below the reference's own 1e-15 tie
         * threshold count as ties (the earlier element stays), so that a point on
         * an element boundary does not move with rounding noise */
        if (nd2 < d2 - 1e-15) better = 1;
        if (better) { isel = e; xi = nxi; eta = neta; ga = nga; d2 = nd2; }
      }
      if (isel == e0) break;
      if (!outside(xi, eta, ga)) break;
    }
  }
  *xi_out = xi; *eta_out = eta; *gamma_out = ga;
  return isel + 1;
}

/* ------------------------------------------------------------------------- */
/* source arrays (compute_arrays_source.f90:29-149)                           */
/* ------------------------------------------------------------------------- */

/* Moment-tensor source array of one source in element ispec (1-based), given
 * Mxx..Myz in N.m (already scaled by 1e-7 from dyne.cm, get_cmt.f90:424). */
void orc_source_array_cmt(int ispec, const int *irregular_element_number, realw **metric,
                          realw xix_regular, double xi, double eta, double gamma, double Mxx,
                          double Myy, double Mzz, double Mxy, double Mxz, double Myz, realw *out) {
  double xg[NGLL], wg[NGLL], hx[NGLL], hpx[NGLL], he[NGLL], hpe[NGLL], hg[NGLL], hpg[NGLL];
  orc_gll(xg, wg);
  orc_lagrange_any(xi, xg, hx, hpx);
  orc_lagrange_any(eta, xg, he, hpe);
  orc_lagrange_any(gamma, xg, hg, hpg);
  double dxis_dx = 0, dxis_dy = 0, dxis_dz = 0, detas_dx = 0, detas_dy = 0, detas_dz = 0,
         dgammas_dx = 0, dgammas_dy = 0, dgammas_dz = 0;
  int ir = irregular_element_number[ispec - 1];
  for (int m = 0; m < NGLL; ++m)
    for (int l = 0; l < NGLL; ++l)
      for (int k = 0; k < NGLL; ++k) {
        double hl = hx[k] * he[l] * hg[m];
        if (ir) {
          long p = IJK(k, l, m) + (long)NGLL3 * (ir - 1);
          dxis_dx += hl * metric[0][p]; dxis_dy += hl * metric[1][p]; dxis_dz += hl * metric[2][p];
          detas_dx += hl * metric[3][p]; detas_dy += hl * metric[4][p]; detas_dz += hl * metric[5][p];
          dgammas_dx += hl * metric[6][p]; dgammas_dy += hl * metric[7][p]; dgammas_dz += hl * metric[8][p];
        } else {
          dxis_dx += hl * (double)xix_regular; detas_dy += hl * (double)xix_regular; dgammas_dz += hl * (double)xix_regular;
        }
      }
  for (int m = 0; m < NGLL; ++m)
    for (int l = 0; l < NGLL; ++l)
      for (int k = 0; k < NGLL; ++k) {
        double hxi = hpx[k] * he[l] * hg[m], heta = hx[k] * hpe[l] * hg[m], hga = hx[k] * he[l] * hpg[m];
        double dx = hxi * dxis_dx + heta * detas_dx + hga * dgammas_dx;
        double dy = hxi * dxis_dy + heta * detas_dy + hga * dgammas_dy;
        double dz = hxi * dxis_dz + heta * detas_dz + hga * dgammas_dz;
        int p = IJK(k, l, m);
        out[0 + 3 * p] = (realw)(Mxx * dx + Mxy * dy + Mxz * dz);
        out[1 + 3 * p] = (realw)(Mxy * dx + Myy * dy + Myz * dz);
        out[2 + 3 * p] = (realw)(Mxz * dx + Myz * dy + Mzz * dz);
      }
}

/* Point-force source array (compute_arrays_source.f90 force branch,
 * setup_sources_receivers.f90: sourcearray = factor * h_xi h_eta h_gamma). */
void orc_source_array_force(double xi, double eta, double gamma, double fx, double fy, double fz, realw *out) {
  double xg[NGLL], wg[NGLL], hx[NGLL], hpx[NGLL], he[NGLL], hpe[NGLL], hg[NGLL], hpg[NGLL];
  orc_gll(xg, wg);
  orc_lagrange_any(xi, xg, hx, hpx);
  orc_lagrange_any(eta, xg, he, hpe);
  orc_lagrange_any(gamma, xg, hg, hpg);
  for (int m = 0; m < NGLL; ++m)
    for (int l = 0; l < NGLL; ++l)
      for (int k = 0; k < NGLL; ++k) {
        double h = hx[k] * he[l] * hg[m];
        int p = IJK(k, l, m);
        out[0 + 3 * p] = (realw)(fx * h); out[1 + 3 * p] = (realw)(fy * h); out[2 + 3 * p] = (realw)(fz * h);
      }
}

/* Source time functions (comp_source_time_function.f90): kind 0 Heaviside
 * (error function, hdur_Gaussian = hdur/1.628), 1 Ricker (f0), 2 Gaussian. */
double orc_stf(int kind, double t, double p) {
  const double PI = 3.141592653589793;
  if (kind == 0) return 0.5 * (1.0 + erf(t / (p / 1.628)));
  if (kind == 1) { double a = PI * PI * p * p; return (1.0 - 2.0 * a * t * t) * exp(-a * t * t); }
  double hd = p / 1.628, a = 1.0 / (hd * hd);
  return exp(-a * t * t) / (sqrt(PI) * hd);
}

/* ------------------------------------------------------------------------- */
/* time loop                                                                  */
/* ------------------------------------------------------------------------- */

/* update_displ_elastic (update_displacement_scheme.f90:359-410) */
static void newmark_predictor(long n3, realw *d, realw *v, realw *a, realw dt, realw dt2, realw dtsq2) {
  for (long i = 0; i < n3; ++i) {
    d[i] = d[i] + dt * v[i] + dtsq2 * a[i];
    v[i] = v[i] + dt2 * a[i];
    a[i] = 0;
  }
}

/* Elastic stiffness of one element (compute_forces_viscoelastic.F90:250-860).
 * Writes into accel with the scatter-add of :788-806; with attenuation it uses
 * the strain of u + dt v (:396-417, :495-568), subtracts the memory variables
 * from the stress (:645-659) and then advances them with
 * compute_element_att_memory_second_order_rk (compute_element_att_memory.f90:28-157). */
static void element_forces(const orc_sim *s, int ispec, const realw *displ, const realw *veloc,
                           realw *accel, realw deltat, realw *R[6], realw *eps[6],
                           realw *eps_trace_over_3, int is_backward) {
  /* PML elements are computed by pml_element_forces (compute_forces_viscoelastic.F90:272-273) */
  if (!is_backward && s->nspec_cpml > 0 && s->is_cpml && s->is_cpml[ispec]) return;
  const realw *hp = s->hprime_xx, *hpw = s->hprimewgll_xx;
  realw ux[NGLL3], uy[NGLL3], uz[NGLL3];
  realw t1x[NGLL3], t2x[NGLL3], t3x[NGLL3], t1y[NGLL3], t2y[NGLL3], t3y[NGLL3], t1z[NGLL3], t2z[NGLL3], t3z[NGLL3];
  realw a1x[NGLL3], a2x[NGLL3], a3x[NGLL3], a1y[NGLL3], a2y[NGLL3], a3y[NGLL3], a1z[NGLL3], a2z[NGLL3], a3z[NGLL3];
  realw epsl[6][NGLL3];
  const int *ib = s->ibool + (long)NGLL3 * ispec;
  const int att = s->attenuation;
  (void)is_backward;
  const int store_strain = s->compute_and_store_strain;

  for (int p = 0; p < NGLL3; ++p) {
    long g = ib[p] - 1;
    ux[p] = displ[3 * g]; uy[p] = displ[3 * g + 1]; uz[p] = displ[3 * g + 2];
  }
  for (int k = 0; k < NGLL; ++k)
    for (int j = 0; j < NGLL; ++j)
      for (int i = 0; i < NGLL; ++i) {
        realw sx1 = 0, sx2 = 0, sx3 = 0, sy1 = 0, sy2 = 0, sy3 = 0, sz1 = 0, sz2 = 0, sz3 = 0;
        for (int l = 0; l < NGLL; ++l) {
          realw h1 = hp[i + NGLL * l], h2 = hp[j + NGLL * l], h3 = hp[k + NGLL * l];
          sx1 += ux[IJK(l, j, k)] * h1; sy1 += uy[IJK(l, j, k)] * h1; sz1 += uz[IJK(l, j, k)] * h1;
          sx2 += ux[IJK(i, l, k)] * h2; sy2 += uy[IJK(i, l, k)] * h2; sz2 += uz[IJK(i, l, k)] * h2;
          sx3 += ux[IJK(i, j, l)] * h3; sy3 += uy[IJK(i, j, l)] * h3; sz3 += uz[IJK(i, j, l)] * h3;
        }
        int p = IJK(i, j, k);
        t1x[p] = sx1; t2x[p] = sx2; t3x[p] = sx3; t1y[p] = sy1; t2y[p] = sy2; t3y[p] = sy3;
        t1z[p] = sz1; t2z[p] = sz2; t3z[p] = sz3;
      }
  if (store_strain && att) {
    /* compute_strain_in_element_att: derivative of (u + dt v) (:882-959) */
    realw vx[NGLL3], vy[NGLL3], vz[NGLL3];
    for (int p = 0; p < NGLL3; ++p) {
      long g = ib[p] - 1;
      vx[p] = deltat * veloc[3 * g]; vy[p] = deltat * veloc[3 * g + 1]; vz[p] = deltat * veloc[3 * g + 2];
    }
    for (int k = 0; k < NGLL; ++k)
      for (int j = 0; j < NGLL; ++j)
        for (int i = 0; i < NGLL; ++i) {
          int p = IJK(i, j, k);
          realw sx1 = t1x[p], sx2 = t2x[p], sx3 = t3x[p], sy1 = t1y[p], sy2 = t2y[p], sy3 = t3y[p], sz1 = t1z[p],
                sz2 = t2z[p], sz3 = t3z[p];
          for (int l = 0; l < NGLL; ++l) {
            realw h1 = hp[i + NGLL * l], h2 = hp[j + NGLL * l], h3 = hp[k + NGLL * l];
            sx1 += vx[IJK(l, j, k)] * h1; sy1 += vy[IJK(l, j, k)] * h1; sz1 += vz[IJK(l, j, k)] * h1;
            sx2 += vx[IJK(i, l, k)] * h2; sy2 += vy[IJK(i, l, k)] * h2; sz2 += vz[IJK(i, l, k)] * h2;
            sx3 += vx[IJK(i, j, l)] * h3; sy3 += vy[IJK(i, j, l)] * h3; sz3 += vz[IJK(i, j, l)] * h3;
          }
          a1x[p] = sx1; a2x[p] = sx2; a3x[p] = sx3; a1y[p] = sy1; a2y[p] = sy2; a3y[p] = sy3;
          a1z[p] = sz1; a2z[p] = sz2; a3z[p] = sz3;
        }
  }
  const int ir = s->irregular_element_number[ispec];
  const long mo = (long)NGLL3 * (ir - 1);
  const realw xr = s->xix_regular;
  for (int p = 0; p < NGLL3; ++p) {
    realw xixl, xiyl, xizl, etaxl, etayl, etazl, gammaxl, gammayl, gammazl, jacl;
    if (ir) {
      xixl = s->xix[mo + p]; xiyl = s->xiy[mo + p]; xizl = s->xiz[mo + p];
      etaxl = s->etax[mo + p]; etayl = s->etay[mo + p]; etazl = s->etaz[mo + p];
      gammaxl = s->gammax[mo + p]; gammayl = s->gammay[mo + p]; gammazl = s->gammaz[mo + p];
      jacl = s->jacobian[mo + p];
    } else {
      xixl = etayl = gammazl = xr; xiyl = xizl = etaxl = etazl = gammaxl = gammayl = 0; jacl = s->jacobian_regular;
    }
    realw duxdxl, duxdyl, duxdzl, duydxl, duydyl, duydzl, duzdxl, duzdyl, duzdzl;
    if (ir) {
      duxdxl = xixl * t1x[p] + etaxl * t2x[p] + gammaxl * t3x[p];
      duxdyl = xiyl * t1x[p] + etayl * t2x[p] + gammayl * t3x[p];
      duxdzl = xizl * t1x[p] + etazl * t2x[p] + gammazl * t3x[p];
      duydxl = xixl * t1y[p] + etaxl * t2y[p] + gammaxl * t3y[p];
      duydyl = xiyl * t1y[p] + etayl * t2y[p] + gammayl * t3y[p];
      duydzl = xizl * t1y[p] + etazl * t2y[p] + gammazl * t3y[p];
      duzdxl = xixl * t1z[p] + etaxl * t2z[p] + gammaxl * t3z[p];
      duzdyl = xiyl * t1z[p] + etayl * t2z[p] + gammayl * t3z[p];
      duzdzl = xizl * t1z[p] + etazl * t2z[p] + gammazl * t3z[p];
    } else {
      duxdxl = xr * t1x[p]; duxdyl = xr * t2x[p]; duxdzl = xr * t3x[p];
      duydxl = xr * t1y[p]; duydyl = xr * t2y[p]; duydzl = xr * t3y[p];
      duzdxl = xr * t1z[p]; duzdyl = xr * t2z[p]; duzdzl = xr * t3z[p];
    }
    if (store_strain) {
      realw dxx, dyy, dzz, dxy, dyx, dxz, dzx, dyz, dzy;
      if (att) {
        if (ir) {
          dxx = xixl * a1x[p] + etaxl * a2x[p] + gammaxl * a3x[p];
          dxy = xiyl * a1x[p] + etayl * a2x[p] + gammayl * a3x[p];
          dxz = xizl * a1x[p] + etazl * a2x[p] + gammazl * a3x[p];
          dyx = xixl * a1y[p] + etaxl * a2y[p] + gammaxl * a3y[p];
          dyy = xiyl * a1y[p] + etayl * a2y[p] + gammayl * a3y[p];
          dyz = xizl * a1y[p] + etazl * a2y[p] + gammazl * a3y[p];
          dzx = xixl * a1z[p] + etaxl * a2z[p] + gammaxl * a3z[p];
          dzy = xiyl * a1z[p] + etayl * a2z[p] + gammayl * a3z[p];
          dzz = xizl * a1z[p] + etazl * a2z[p] + gammazl * a3z[p];
        } else {
          dxx = xr * a1x[p]; dxy = xr * a2x[p]; dxz = xr * a3x[p];
          dyx = xr * a1y[p]; dyy = xr * a2y[p]; dyz = xr * a3y[p];
          dzx = xr * a1z[p]; dzy = xr * a2z[p]; dzz = xr * a3z[p];
        }
      } else {
        dxx = duxdxl; dxy = duxdyl; dxz = duxdzl; dyx = duydxl; dyy = duydyl; dyz = duydzl;
        dzx = duzdxl; dzy = duzdyl; dzz = duzdzl;
      }
      realw templ = (realw)(1.0 / 3.0) * (dxx + dyy + dzz);
      epsl[5][p] = dxx + dyy + dzz;
      if (eps_trace_over_3) eps_trace_over_3[(long)NGLL3 * ispec + p] = templ;
      epsl[0][p] = dxx - templ;
      epsl[1][p] = dyy - templ;
      epsl[2][p] = (realw)0.5 * (dxy + dyx);
      epsl[3][p] = (realw)0.5 * (dzx + dxz);
      epsl[4][p] = (realw)0.5 * (dzy + dyz);
    }
    realw dxy_yx = duxdyl + duydxl, dzx_xz = duzdxl + duxdzl, dzy_yz = duzdyl + duydzl;
    long q = (long)NGLL3 * ispec + p;
    realw kappal = s->kappastore[q], mul = s->mustore[q];
    realw l2m = kappal + (realw)(4.0 / 3.0) * mul;
    realw lambdal = l2m - (realw)2.0 * mul;
    realw sxx = l2m * duxdxl + lambdal * (duydyl + duzdzl);
    realw syy = l2m * duydyl + lambdal * (duxdxl + duzdzl);
    realw szz = l2m * duzdzl + lambdal * (duxdxl + duydyl);
    realw sxy = mul * dxy_yx, sxz = mul * dzx_xz, syz = mul * dzy_yz;
    if (s->cstore) {
      /* ANISOTROPY (compute_forces_viscoelastic.F90:578-611): c11..c66 at cstore[21 q + n] */
      const realw *c = s->cstore + 21 * q;
      realw c11 = c[0], c12 = c[1], c13 = c[2], c14 = c[3], c15 = c[4], c16 = c[5], c22 = c[6], c23 = c[7];
      realw c24 = c[8], c25 = c[9], c26 = c[10], c33 = c[11], c34 = c[12], c35 = c[13], c36 = c[14], c44 = c[15];
      realw c45 = c[16], c46 = c[17], c55 = c[18], c56 = c[19], c66 = c[20];
      sxx = c11 * duxdxl + c16 * dxy_yx + c12 * duydyl + c15 * dzx_xz + c14 * dzy_yz + c13 * duzdzl;
      syy = c12 * duxdxl + c26 * dxy_yx + c22 * duydyl + c25 * dzx_xz + c24 * dzy_yz + c23 * duzdzl;
      szz = c13 * duxdxl + c36 * dxy_yx + c23 * duydyl + c35 * dzx_xz + c34 * dzy_yz + c33 * duzdzl;
      sxy = c16 * duxdxl + c66 * dxy_yx + c26 * duydyl + c56 * dzx_xz + c46 * dzy_yz + c36 * duzdzl;
      sxz = c15 * duxdxl + c56 * dxy_yx + c25 * duydyl + c55 * dzx_xz + c45 * dzy_yz + c35 * duzdzl;
      syz = c14 * duxdxl + c46 * dxy_yx + c24 * duydyl + c45 * dzx_xz + c44 * dzy_yz + c34 * duzdzl;
    }
    if (att) {
      realw Rxx = 0, Ryy = 0, Rtr = 0, Rxy = 0, Rxz = 0, Ryz = 0;
      for (int sl = 0; sl < N_SLS; ++sl) {
        long r = sl + N_SLS * q;
        Rxx += R[0][r]; Ryy += R[1][r]; Rxy += R[2][r]; Rxz += R[3][r]; Ryz += R[4][r]; Rtr += R[5][r];
      }
      sxx = sxx - Rxx - Rtr;
      syy = syy - Ryy - Rtr;
      szz = szz + Rxx + Ryy - Rtr;
      sxy = sxy - Rxy; sxz = sxz - Rxz; syz = syz - Ryz;
    }
    if (ir) {
      t1x[p] = jacl * (sxx * xixl + sxy * xiyl + sxz * xizl);
      t1y[p] = jacl * (sxy * xixl + syy * xiyl + syz * xizl);
      t1z[p] = jacl * (sxz * xixl + syz * xiyl + szz * xizl);
      t2x[p] = jacl * (sxx * etaxl + sxy * etayl + sxz * etazl);
      t2y[p] = jacl * (sxy * etaxl + syy * etayl + syz * etazl);
      t2z[p] = jacl * (sxz * etaxl + syz * etayl + szz * etazl);
      t3x[p] = jacl * (sxx * gammaxl + sxy * gammayl + sxz * gammazl);
      t3y[p] = jacl * (sxy * gammaxl + syy * gammayl + syz * gammazl);
      t3z[p] = jacl * (sxz * gammaxl + syz * gammayl + szz * gammazl);
    } else {
      t1x[p] = jacl * sxx * xr; t1y[p] = jacl * sxy * xr; t1z[p] = jacl * sxz * xr;
      t2x[p] = jacl * sxy * xr; t2y[p] = jacl * syy * xr; t2z[p] = jacl * syz * xr;
      t3x[p] = jacl * sxz * xr; t3y[p] = jacl * syz * xr; t3z[p] = jacl * szz * xr;
    }
  }
  for (int k = 0; k < NGLL; ++k)
    for (int j = 0; j < NGLL; ++j)
      for (int i = 0; i < NGLL; ++i) {
        realw sx1 = 0, sx2 = 0, sx3 = 0, sy1 = 0, sy2 = 0, sy3 = 0, sz1 = 0, sz2 = 0, sz3 = 0;
        for (int l = 0; l < NGLL; ++l) {
          realw f1 = hpw[l + NGLL * i], f2 = hpw[l + NGLL * j], f3 = hpw[l + NGLL * k];
          sx1 += t1x[IJK(l, j, k)] * f1; sy1 += t1y[IJK(l, j, k)] * f1; sz1 += t1z[IJK(l, j, k)] * f1;
          sx2 += t2x[IJK(i, l, k)] * f2; sy2 += t2y[IJK(i, l, k)] * f2; sz2 += t2z[IJK(i, l, k)] * f2;
          sx3 += t3x[IJK(i, j, l)] * f3; sy3 += t3y[IJK(i, j, l)] * f3; sz3 += t3z[IJK(i, j, l)] * f3;
        }
        realw fac1 = s->wgllwgll_yz[j + NGLL * k], fac2 = s->wgllwgll_xz[i + NGLL * k], fac3 = s->wgllwgll_xy[i + NGLL * j];
        long g = ib[IJK(i, j, k)] - 1;
        realw ax = fac1 * sx1 + fac2 * sx2 + fac3 * sx3;
        realw ay = fac1 * sy1 + fac2 * sy2 + fac3 * sy3;
        realw az = fac1 * sz1 + fac2 * sz2 + fac3 * sz3;
#pragma omp atomic
        accel[3 * g] -= ax;
#pragma omp atomic
        accel[3 * g + 1] -= ay;
#pragma omp atomic
        accel[3 * g + 2] -= az;
      }
  if (att) {
    const realw *al = s->alphaval, *be = s->betaval, *ga = s->gammaval;
    for (int p = 0; p < NGLL3; ++p) {
      long q = (long)NGLL3 * ispec + p;
      for (int sl = 0; sl < N_SLS; ++sl) {
        long r = sl + N_SLS * q;
        realw fk = s->kappastore[q] * s->factor_common_kappa[r];
        R[5][r] = al[sl] * R[5][r] + fk * (be[sl] * eps[5][q] + ga[sl] * epsl[5][p]);
        realw fm = s->mustore[q] * s->factor_common[r];
        for (int c = 0; c < 5; ++c) R[c][r] = al[sl] * R[c][r] + fm * (be[sl] * eps[c][q] + ga[sl] * epsl[c][p]);
      }
    }
  }
  if (store_strain) {
    for (int p = 0; p < NGLL3; ++p) {
      long q = (long)NGLL3 * ispec + p;
      if (att) eps[5][q] = epsl[5][p];
      for (int c = 0; c < 5; ++c) if (eps[c]) eps[c][q] = epsl[c][p];
    }
  }
}

/* C-PML element (compute_forces_viscoelastic.F90:969-1400, compute_forces_viscoelastic_PML):
 * gradients of u, PML_displ_old and PML_displ_new; the convolution memory variables
 * and the non-symmetric stress (pml_compute_memory_variables.f90,
 * pml_compute_memory_variables_elastic); the layer's acceleration term
 * (pml_compute_accel_contribution.f90, pml_compute_accel_contribution_elastic); the
 * dot products with the metric, the transposed contractions and the scatter of
 * -(sum + acceleration term).  Memory variables rmem(48, 125, nspec_cpml): rows
 * 3n+q the three convolutions of dux_dxl_x, duy_dxl_y, duz_dxl_z, dux_dyl_x,
 * duy_dyl_y, duz_dyl_z, dux_dzl_x, duy_dzl_y, duz_dzl_z; rows 27-38 duz_dzl_y,
 * duz_dyl_y, duy_dzl_z, duy_dyl_z, duz_dzl_x, duz_dxl_x, dux_dzl_z, dux_dxl_z,
 * duy_dyl_x, duy_dxl_x, dux_dyl_y, dux_dxl_y; rows 39+3d+c the displacement. */
static void grad_ref(const realw *hp, const realw *f /* [3][125] */, realw T[NGLL3][3][3]) {
  for (int k = 0; k < NGLL; ++k)
    for (int j = 0; j < NGLL; ++j)
      for (int i = 0; i < NGLL; ++i) {
        const int p = IJK(i, j, k);
        for (int c = 0; c < 3; ++c) {
          realw s1 = 0, s2 = 0, s3 = 0;
          for (int l = 0; l < NGLL; ++l) {
            s1 += f[c * NGLL3 + IJK(l, j, k)] * hp[i + NGLL * l];
            s2 += f[c * NGLL3 + IJK(i, l, k)] * hp[j + NGLL * l];
            s3 += f[c * NGLL3 + IJK(i, j, l)] * hp[k + NGLL * l];
          }
          T[p][c][0] = s1; T[p][c][1] = s2; T[p][c][2] = s3;
        }
      }
}

static void pml_element_forces(const orc_sim *s, int ispec, realw *accel, realw *eps[6]) {
  const realw *hp = s->hprime_xx, *hpw = s->hprimewgll_xx;
  const int ec = s->spec_to_cpml[ispec] - 1;
  const int *ib = s->ibool + (long)NGLL3 * ispec;
  static realw Tu[NGLL3][3][3], To[NGLL3][3][3], Tn[NGLL3][3][3];
#pragma omp threadprivate(Tu, To, Tn)
  realw fu[3 * NGLL3], fo[3 * NGLL3], fn[3 * NGLL3];
  for (int p = 0; p < NGLL3; ++p) {
    long g = ib[p] - 1;
    for (int c = 0; c < 3; ++c) {
      fu[c * NGLL3 + p] = s->displ[3 * g + c];
      fo[c * NGLL3 + p] = s->pml_displ_old[c + 3 * (p + (long)NGLL3 * ec)];
      fn[c * NGLL3 + p] = s->pml_displ_new[c + 3 * (p + (long)NGLL3 * ec)];
    }
  }
  grad_ref(hp, fu, Tu);
  grad_ref(hp, fo, To);
  grad_ref(hp, fn, Tn);
  const int ir = s->irregular_element_number[ispec];
  const long mo = (long)NGLL3 * (ir - 1);
  const realw xr = s->xix_regular;
  realw t1x[NGLL3], t2x[NGLL3], t3x[NGLL3], t1y[NGLL3], t2y[NGLL3], t3y[NGLL3], t1z[NGLL3], t2z[NGLL3], t3z[NGLL3];
  realw acc[NGLL3][3];
  for (int p = 0; p < NGLL3; ++p) {
    realw m[9], jacl;
    if (ir) {
      m[0] = s->xix[mo + p]; m[1] = s->xiy[mo + p]; m[2] = s->xiz[mo + p];
      m[3] = s->etax[mo + p]; m[4] = s->etay[mo + p]; m[5] = s->etaz[mo + p];
      m[6] = s->gammax[mo + p]; m[7] = s->gammay[mo + p]; m[8] = s->gammaz[mo + p];
      jacl = s->jacobian[mo + p];
    } else {
      for (int q = 0; q < 9; ++q) m[q] = 0;
      m[0] = m[4] = m[8] = xr;
      jacl = s->jacobian_regular;
    }
    realw du[3][3], dold[3][3], dnew[3][3];
    for (int c = 0; c < 3; ++c)
      for (int x = 0; x < 3; ++x) {
        if (ir) {
          du[c][x] = m[x] * Tu[p][c][0] + m[3 + x] * Tu[p][c][1] + m[6 + x] * Tu[p][c][2];
          dold[c][x] = m[x] * To[p][c][0] + m[3 + x] * To[p][c][1] + m[6 + x] * To[p][c][2];
          dnew[c][x] = m[x] * Tn[p][c][0] + m[3 + x] * Tn[p][c][1] + m[6 + x] * Tn[p][c][2];
        } else {
          du[c][x] = xr * Tu[p][c][x];
          dold[c][x] = xr * To[p][c][x];
          dnew[c][x] = xr * Tn[p][c][x];
        }
      }
    const long q = (long)NGLL3 * ispec + p;
    if (s->compute_and_store_strain && eps[0]) {
      realw templ = (realw)(1.0 / 3.0) * (du[0][0] + du[1][1] + du[2][2]);
      eps[0][q] = du[0][0] - templ;
      eps[1][q] = du[1][1] - templ;
      eps[2][q] = (realw)0.5 * (du[0][1] + du[1][0]);
      eps[3][q] = (realw)0.5 * (du[2][0] + du[0][2]);
      eps[4][q] = (realw)0.5 * (du[2][1] + du[1][2]);
    }
    const long cp = p + (long)NGLL3 * ec;
#define CA(r) s->pml_coef_alpha[(r) + 9 * cp]
#define CB(r) s->pml_coef_beta[(r) + 9 * cp]
#define RM(r) s->pml_rmem[(r) + 48 * cp]
    /* sets of the three convolutions of the derivatives along x, y, z */
    for (int x = 0; x < 3; ++x)
      for (int c = 0; c < 3; ++c)
        for (int qq = 0; qq < 3; ++qq) {
          const int set = x == 0 ? (qq == 0 ? 6 : (qq == 1 ? 3 : -1)) : x == 1 ? (qq == 0 ? 0 : (qq == 1 ? 6 : -1))
                                                                                : (qq == 0 ? 0 : (qq == 1 ? 3 : -1));
          realw c0, c1, c2;
          if (set >= 0) { c0 = CA(set); c1 = CA(set + 1); c2 = CA(set + 2); }
          else { c0 = CB(3 * x); c1 = CB(3 * x + 1); c2 = CB(3 * x + 2); }
          realw *r = &RM(3 * (3 * x + c) + qq);
          *r = c0 * *r + dnew[c][x] * c1 + dold[c][x] * c2;
        }
    const int srow[12] = {0, 0, 0, 0, 3, 3, 3, 3, 6, 6, 6, 6};
    const int sc[12] = {2, 2, 1, 1, 2, 2, 0, 0, 1, 1, 0, 0};
    const int sx[12] = {2, 1, 2, 1, 2, 0, 2, 0, 1, 0, 1, 0};
    for (int n = 0; n < 12; ++n) {
      realw *r = &RM(27 + n);
      *r = CA(srow[n]) * *r + dnew[sc[n]][sx[n]] * CA(srow[n] + 1) + dold[sc[n]][sx[n]] * CA(srow[n] + 2);
    }
    const realw *A = s->pml_coef_strain + 18 * cp;   /* A6 .. A23 */
    realw duxdxl_x = A[0] * du[0][0] + A[1] * RM(0) + A[2] * RM(1) + A[3] * RM(2);
    realw duxdyl_x = A[4] * du[0][1] + A[5] * RM(9) + A[6] * RM(10) + A[7] * RM(11);
    realw duxdzl_x = A[8] * du[0][2] + A[9] * RM(18) + A[10] * RM(19) + A[11] * RM(20);
    realw duzdzl_x = A[14] * du[2][2] + A[15] * RM(31);
    realw duzdxl_x = A[14] * du[2][0] + A[15] * RM(32);
    realw duydyl_x = A[16] * du[1][1] + A[17] * RM(35);
    realw duydxl_x = A[16] * du[1][0] + A[17] * RM(36);
    realw duydxl_y = A[0] * du[1][0] + A[1] * RM(3) + A[2] * RM(4) + A[3] * RM(5);
    realw duydyl_y = A[4] * du[1][1] + A[5] * RM(12) + A[6] * RM(13) + A[7] * RM(14);
    realw duydzl_y = A[8] * du[1][2] + A[9] * RM(21) + A[10] * RM(22) + A[11] * RM(23);
    realw duzdzl_y = A[12] * du[2][2] + A[13] * RM(27);
    realw duzdyl_y = A[12] * du[2][1] + A[13] * RM(28);
    realw duxdyl_y = A[16] * du[0][1] + A[17] * RM(37);
    realw duxdxl_y = A[16] * du[0][0] + A[17] * RM(38);
    realw duzdxl_z = A[0] * du[2][0] + A[1] * RM(6) + A[2] * RM(7) + A[3] * RM(8);
    realw duzdyl_z = A[4] * du[2][1] + A[5] * RM(15) + A[6] * RM(16) + A[7] * RM(17);
    realw duzdzl_z = A[8] * du[2][2] + A[9] * RM(24) + A[10] * RM(25) + A[11] * RM(26);
    realw duydzl_z = A[12] * du[1][2] + A[13] * RM(29);
    realw duydyl_z = A[12] * du[1][1] + A[13] * RM(30);
    realw duxdzl_z = A[14] * du[0][2] + A[15] * RM(33);
    realw duxdxl_z = A[14] * du[0][0] + A[15] * RM(34);
    realw kappal = s->kappastore[q], mul = s->mustore[q];
    realw l2m = kappal + (realw)(4.0 / 3.0) * mul, lam = l2m - (realw)2 * mul;
    realw sxx = l2m * duxdxl_x + lam * duydyl_x + lam * duzdzl_x;
    realw syx = mul * duxdyl_x + mul * duydxl_x;
    realw szx = mul * duzdxl_x + mul * duxdzl_x;
    realw sxy = mul * duxdyl_y + mul * duydxl_y;
    realw syy = lam * duxdxl_y + l2m * duydyl_y + lam * duzdzl_y;
    realw szy = mul * duzdyl_y + mul * duydzl_y;
    realw sxz = mul * duzdxl_z + mul * duxdzl_z;
    realw syz = mul * duzdyl_z + mul * duydzl_z;
    realw szz = lam * duxdxl_z + lam * duydyl_z + l2m * duzdzl_z;
    /* displacement memory variables and the layer's acceleration term */
    realw rd[3][3];
    for (int d = 0; d < 3; ++d)
      for (int c = 0; c < 3; ++c) {
        realw *r = &RM(39 + 3 * d + c);
        *r = CA(3 * d) * *r + fn[c * NGLL3 + p] * CA(3 * d + 1) + fo[c * NGLL3 + p] * CA(3 * d + 2);
        rd[c][d] = *r;
      }
    const realw *Ab = s->pml_coef_abar + 5 * cp;
    const realw wrj = s->wgll_cube[p] * s->rhostore[q] * jacl;
    for (int c = 0; c < 3; ++c)
      acc[p][c] = wrj * (Ab[0] * s->veloc[3 * (ib[p] - 1) + c] + Ab[1] * fu[c * NGLL3 + p] + Ab[2] * rd[c][0] +
                         Ab[3] * rd[c][1] + Ab[4] * rd[c][2]);
#undef CA
#undef CB
#undef RM
    /* dot products with the metric rows, non-symmetric form */
    t1x[p] = jacl * (sxx * m[0] + syx * m[1] + szx * m[2]);
    t1y[p] = jacl * (sxy * m[0] + syy * m[1] + szy * m[2]);
    t1z[p] = jacl * (sxz * m[0] + syz * m[1] + szz * m[2]);
    t2x[p] = jacl * (sxx * m[3] + syx * m[4] + szx * m[5]);
    t2y[p] = jacl * (sxy * m[3] + syy * m[4] + szy * m[5]);
    t2z[p] = jacl * (sxz * m[3] + syz * m[4] + szz * m[5]);
    t3x[p] = jacl * (sxx * m[6] + syx * m[7] + szx * m[8]);
    t3y[p] = jacl * (sxy * m[6] + syy * m[7] + szy * m[8]);
    t3z[p] = jacl * (sxz * m[6] + syz * m[7] + szz * m[8]);
  }
  for (int k = 0; k < NGLL; ++k)
    for (int j = 0; j < NGLL; ++j)
      for (int i = 0; i < NGLL; ++i) {
        realw sx1 = 0, sx2 = 0, sx3 = 0, sy1 = 0, sy2 = 0, sy3 = 0, sz1 = 0, sz2 = 0, sz3 = 0;
        for (int l = 0; l < NGLL; ++l) {
          realw f1 = hpw[l + NGLL * i], f2 = hpw[l + NGLL * j], f3 = hpw[l + NGLL * k];
          sx1 += t1x[IJK(l, j, k)] * f1; sy1 += t1y[IJK(l, j, k)] * f1; sz1 += t1z[IJK(l, j, k)] * f1;
          sx2 += t2x[IJK(i, l, k)] * f2; sy2 += t2y[IJK(i, l, k)] * f2; sz2 += t2z[IJK(i, l, k)] * f2;
          sx3 += t3x[IJK(i, j, l)] * f3; sy3 += t3y[IJK(i, j, l)] * f3; sz3 += t3z[IJK(i, j, l)] * f3;
        }
        realw fac1 = s->wgllwgll_yz[j + NGLL * k], fac2 = s->wgllwgll_xz[i + NGLL * k], fac3 = s->wgllwgll_xy[i + NGLL * j];
        const int p = IJK(i, j, k);
        long g = ib[p] - 1;
        realw ax = fac1 * sx1 + fac2 * sx2 + fac3 * sx3 + acc[p][0];
        realw ay = fac1 * sy1 + fac2 * sy2 + fac3 * sy3 + acc[p][1];
        realw az = fac1 * sz1 + fac2 * sz2 + fac3 * sz3 + acc[p][2];
#pragma omp atomic
        accel[3 * g] -= ax;
#pragma omp atomic
        accel[3 * g + 1] -= ay;
#pragma omp atomic
        accel[3 * g + 2] -= az;
      }
}

/* update_displ_elastic_PML (update_displacement_scheme.f90:417-455) */
static void pml_store_displ(orc_sim *s, realw *out) {
  const realw theta = (realw)0.125;
  for (int ec = 0; ec < s->nspec_cpml; ++ec) {
    const int ispec = s->cpml_to_spec[ec] - 1;
    for (int p = 0; p < NGLL3; ++p) {
      long g = s->ibool[(long)NGLL3 * ispec + p] - 1;
      for (int c = 0; c < 3; ++c)
        out[c + 3 * (p + (long)NGLL3 * ec)] = s->displ[3 * g + c] +
                                              s->deltatover2 * ((realw)1 - (realw)2 * theta) * s->veloc[3 * g + c] +
                                              s->deltatsqover2 * ((realw)1 - theta) * s->accel[3 * g + c];
    }
  }
}

/* pml_impose_boundary_condition_elastic (pml_compute_accel_contribution.f90 /
 * pml_impose_boundary_condition_cuda_kernel.cu): u, v, a and the stored
 * predictions zero on the outer faces of the layers */
static void pml_boundary(orc_sim *s) {
  for (int f = 0; f < s->num_abs_boundary_faces; ++f) {
    const int ispec = s->abs_boundary_ispec[f] - 1;
    if ((s->ispec_is_acoustic && s->ispec_is_acoustic[ispec]) || !s->is_cpml[ispec]) continue;
    const int ec = s->spec_to_cpml[ispec] - 1;
    for (int g = 0; g < NGLL2; ++g) {
      const int *ijk = s->abs_boundary_ijk + 3 * (g + NGLL2 * f);
      const int p = IJK(ijk[0] - 1, ijk[1] - 1, ijk[2] - 1);
      long ig = s->ibool[p + (long)NGLL3 * ispec] - 1;
      for (int c = 0; c < 3; ++c) {
        s->displ[3 * ig + c] = 0;
        s->veloc[3 * ig + c] = 0;
        s->accel[3 * ig + c] = 0;
        s->pml_displ_old[c + 3 * (p + (long)NGLL3 * ec)] = 0;
        s->pml_displ_new[c + 3 * (p + (long)NGLL3 * ec)] = 0;
      }
    }
  }
}

/* All elements' stiffness contribution (one phase covers the whole slice). */
void orc_compute_forces_elastic(orc_sim *s, int backward) {
  realw *R[6] = {s->R_xx, s->R_yy, s->R_xy, s->R_xz, s->R_yz, s->R_trace};
  realw *eps[6] = {s->epsilondev_xx, s->epsilondev_yy, s->epsilondev_xy, s->epsilondev_xz, s->epsilondev_yz, s->epsilondev_trace};
  realw *bep[6] = {s->b_epsilondev_xx, s->b_epsilondev_yy, s->b_epsilondev_xy, s->b_epsilondev_xz, s->b_epsilondev_yz, NULL};
  const realw *d = backward ? s->b_displ : s->displ;
  const realw *v = backward ? s->b_veloc : s->veloc;
  realw *a = backward ? s->b_accel : s->accel;
  realw dt = backward ? s->b_deltat : s->deltat;
  realw **E = backward ? bep : eps;
  realw *tr3 = backward ? s->b_epsilon_trace_over_3 : s->epsilon_trace_over_3;
  const int n = s->n_elastic < 0 ? s->nspec : s->n_elastic;
#ifdef _OPENMP
  omp_set_num_threads(s->nthreads > 0 ? s->nthreads : 1);
#pragma omp parallel for schedule(static)
#endif
  for (int q = 0; q < n; ++q) {
    const int ispec = s->n_elastic < 0 ? q : s->elastic_list[q] - 1;
    element_forces(s, ispec, d, v, a, dt, R, E, tr3, backward);
  }
  if (!backward && s->nspec_cpml > 0) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int ec = 0; ec < s->nspec_cpml; ++ec) pml_element_forces(s, s->cpml_to_spec[ec] - 1, a, E);
  }
}

/* compute_stacey_viscoelastic_forward (compute_stacey_viscoelastic.F90:32-206) */
void orc_stacey_elastic(orc_sim *s, const realw *veloc, realw *accel) {
  for (int f = 0; f < s->num_abs_boundary_faces; ++f) {
    int ispec = s->abs_boundary_ispec[f] - 1;
    if (s->ispec_is_acoustic && s->ispec_is_acoustic[ispec]) continue;
    for (int g = 0; g < NGLL2; ++g) {
      const int *ijk = s->abs_boundary_ijk + 3 * (g + NGLL2 * f);
      long p = IJK(ijk[0] - 1, ijk[1] - 1, ijk[2] - 1) + (long)NGLL3 * ispec;
      long ig = s->ibool[p] - 1;
      realw vx = veloc[3 * ig], vy = veloc[3 * ig + 1], vz = veloc[3 * ig + 2];
      const realw *n = s->abs_boundary_normal + 3 * (g + NGLL2 * f);
      realw vn = vx * n[0] + vy * n[1] + vz * n[2];
      realw tx = s->rho_vp[p] * vn * n[0] + s->rho_vs[p] * (vx - vn * n[0]);
      realw ty = s->rho_vp[p] * vn * n[1] + s->rho_vs[p] * (vy - vn * n[1]);
      realw tz = s->rho_vp[p] * vn * n[2] + s->rho_vs[p] * (vz - vn * n[2]);
      realw jw = s->abs_boundary_jacobian2Dw[g + NGLL2 * f];
      accel[3 * ig] -= tx * jw; accel[3 * ig + 1] -= ty * jw; accel[3 * ig + 2] -= tz * jw;
    }
  }
}

/* compute_add_sources_viscoelastic (compute_add_sources_viscoelastic.F90:30-140):
 * stf is precomputed in FP64 per step and rounded to CUSTOM_REAL. */
void orc_add_sources(orc_sim *s, realw *accel, int it) {
  for (int isrc = 0; isrc < s->nsources; ++isrc) {
    realw stf = (realw)s->stf[isrc + (long)s->nsources * (it - 1)];
    int ispec = s->ispec_selected_source[isrc] - 1;
    if (s->ispec_is_acoustic && s->ispec_is_acoustic[ispec]) continue;
    for (int p = 0; p < NGLL3; ++p) {
      long ig = s->ibool[(long)NGLL3 * ispec + p] - 1;
      for (int c = 0; c < 3; ++c)
        accel[3 * ig + c] += s->sourcearrays[isrc + (long)s->nsources * (c + 3 * p)] * stf;
    }
  }
}

/* compute_seismograms + compute_interpolated_dva_viscoelast
 * (compute_seismograms.f90:29-265, compute_interpolated_dva.f90:28-110). */
/* (1/rho) grad chi at the GLL points of one fluid element
 * (compute_gradient_in_acoustic.f90:28-200), then interpolated at the receiver
 * with its Lagrange weights (compute_interpolated_dva_acoust). */
static void fluid_vector_seismogram(const orc_sim *s, const realw *chi, int r, int ispec, double u[3]) {
  const int ir = s->irregular_element_number[ispec];
  u[0] = u[1] = u[2] = 0.0;
  for (int k = 0; k < NGLL; ++k)
    for (int j = 0; j < NGLL; ++j)
      for (int i = 0; i < NGLL; ++i) {
        realw t1 = 0, t2 = 0, t3 = 0;
        for (int l = 0; l < NGLL; ++l) {
          t1 += chi[s->ibool[IJK(l, j, k) + (long)NGLL3 * ispec] - 1] * s->hprime_xx[i + NGLL * l];
          t2 += chi[s->ibool[IJK(i, l, k) + (long)NGLL3 * ispec] - 1] * s->hprime_xx[j + NGLL * l];
          t3 += chi[s->ibool[IJK(i, j, l) + (long)NGLL3 * ispec] - 1] * s->hprime_xx[k + NGLL * l];
        }
        const int p = IJK(i, j, k);
        const realw rho_inv = (realw)1 / s->rhostore[p + (long)NGLL3 * ispec];
        realw g[3];
        if (ir) {
          const long q = p + (long)NGLL3 * (ir - 1);
          g[0] = rho_inv * (s->xix[q] * t1 + s->etax[q] * t2 + s->gammax[q] * t3);
          g[1] = rho_inv * (s->xiy[q] * t1 + s->etay[q] * t2 + s->gammay[q] * t3);
          g[2] = rho_inv * (s->xiz[q] * t1 + s->etaz[q] * t2 + s->gammaz[q] * t3);
        } else {
          g[0] = rho_inv * s->xix_regular * t1;
          g[1] = rho_inv * s->xix_regular * t2;
          g[2] = rho_inv * s->xix_regular * t3;
        }
        const double h = s->hxir[i + NGLL * r] * s->hetar[j + NGLL * r] * s->hgammar[k + NGLL * r];
        for (int c = 0; c < 3; ++c) u[c] += h * (double)g[c];
      }
}

void orc_seismograms(orc_sim *s, const realw *field, int it) {
  for (int r = 0; r < s->nrec; ++r) {
    int ispec = s->ispec_selected_rec[r] - 1;
    if (s->rec_is_acoustic && s->rec_is_acoustic[r] && s->fluid_vector) {
      const realw *chi = s->record_what == 2 ? s->potential_dot
                         : (s->record_what == 3 ? s->potential_dot_dot : s->potential);
      double u[3];
      fluid_vector_seismogram(s, chi, r, ispec, u);
      const double *nu = s->nu_rec ? s->nu_rec + 9 * r : NULL;
      for (int c = 0; c < 3; ++c) {
        double v = nu ? nu[c + 0] * u[0] + nu[c + 3] * u[1] + nu[c + 6] * u[2] : u[c];
        s->seismograms[c + 3 * (r + (long)s->nrec * (it - 1))] = (double)(realw)v;
      }
      continue;
    }
    if (s->rec_is_acoustic && s->rec_is_acoustic[r]) {
      /* pressure = - sum h chi_dot_dot (compute_interpolated_dva.f90:280-300) */
      double pd = 0.0;
      for (int k = 0; k < NGLL; ++k)
        for (int j = 0; j < NGLL; ++j)
          for (int i = 0; i < NGLL; ++i) {
            double h = s->hxir[i + NGLL * r] * s->hetar[j + NGLL * r] * s->hgammar[k + NGLL * r];
            long ig = s->ibool[IJK(i, j, k) + (long)NGLL3 * ispec] - 1;
            pd -= h * (double)s->potential_dot_dot[ig];
          }
      for (int c = 0; c < 3; ++c)
        s->seismograms[c + 3 * (r + (long)s->nrec * (it - 1))] = c == 0 ? (double)(realw)pd : 0.0;
      continue;
    }
    double u[3] = {0, 0, 0};
    for (int k = 0; k < NGLL; ++k)
      for (int j = 0; j < NGLL; ++j)
        for (int i = 0; i < NGLL; ++i) {
          double h = s->hxir[i + NGLL * r] * s->hetar[j + NGLL * r] * s->hgammar[k + NGLL * r];
          long ig = s->ibool[IJK(i, j, k) + (long)NGLL3 * ispec] - 1;
          for (int c = 0; c < 3; ++c) u[c] += (double)field[3 * ig + c] * h;
        }
    const double *nu = s->nu_rec ? s->nu_rec + 9 * r : NULL;
    for (int c = 0; c < 3; ++c) {
      double v = nu ? nu[c + 0] * u[0] + nu[c + 3] * u[1] + nu[c + 6] * u[2] : u[c];
      s->seismograms[c + 3 * (r + (long)s->nrec * (it - 1))] = (double)(realw)v;
    }
  }
}

/* One forward time step (iterate_time.F90:219-330 with
 * compute_forces_viscoelastic_calling_routine.F90:107-417): predictor,
 * iphase 1 (Stacey, sources; no outer elements on one slice), iphase 2
 * (stiffness of all elements), mass matrix, corrector, seismograms. */
void orc_step(orc_sim *s) {
  long n3 = 3L * s->nglob;
  const int pml = s->nspec_cpml > 0;
  if (pml) pml_store_displ(s, s->pml_displ_old);
  newmark_predictor(n3, s->displ, s->veloc, s->accel, s->deltat, s->deltatover2, s->deltatsqover2);
  if (pml) pml_store_displ(s, s->pml_displ_new);
  if (s->stacey && s->num_abs_boundary_faces > 0) orc_stacey_elastic(s, s->veloc, s->accel);
  if (s->nsources > 0 && s->stf) orc_add_sources(s, s->accel, s->it);
  orc_compute_forces_elastic(s, 0);
  if (pml) pml_boundary(s);
  for (long g = 0; g < s->nglob; ++g) {
    s->accel[3 * g] *= s->rmassx[g];
    s->accel[3 * g + 1] *= s->rmassy[g];
    s->accel[3 * g + 2] *= s->rmassz[g];
  }
  for (long i = 0; i < n3; ++i) s->veloc[i] += s->deltatover2 * s->accel[i];
  if (s->nrec > 0 && s->seismograms) {
    const realw *f = s->record_what == 2 ? s->veloc : (s->record_what == 3 ? s->accel : s->displ);
    orc_seismograms(s, f, s->it);
  }
  s->it++;
}

void orc_run(orc_sim *s, int nsteps) {
  for (int n = 0; n < nsteps; ++n) orc_step(s);
}

/* ------------------------------------------------------------------------- */
/* attenuation model (shared/get_attenuation_model.f90)                       */
/* ------------------------------------------------------------------------- */

#define ATT_NF 100
static double g_att_f[ATT_NF], g_att_tau_s[N_SLS], g_att_iQ;

/* attenuation_maxwell + attenuation_eval (get_attenuation_model.f90:1100-1215) */
static double att_eval(const double *tau_eps) {
  const double PI = 3.14159265358979;
  double sum = 0.0, iQ2 = g_att_iQ * g_att_iQ;
  for (int i = 0; i < ATT_NF; ++i) {
    double w = 2.0 * PI * pow(10.0, g_att_f[i]), A = 0.0, B = 0.0;
    for (int j = 0; j < N_SLS; ++j) {
      double denom = 1.0 + w * w * g_att_tau_s[j] * g_att_tau_s[j];
      A += (1.0 + (w * w * tau_eps[j] * g_att_tau_s[j])) / denom;
      B += w * (tau_eps[j] - g_att_tau_s[j]) / denom;
    }
    double td = B / A;
    sum += sqrt(((td - g_att_iQ) * (td - g_att_iQ)) / iQ2);
  }
  return sum;
}

/* bubble sort of fv with permutation (qsort_local, :1558-1607) */
static void att_sort(double *fv, int *place, int n) {
  for (int j = 0; j < n; ++j) place[j] = j;
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < n - 1 - j; ++k)
      if (fv[k + 1] < fv[k]) {
        double r = fv[k]; fv[k] = fv[k + 1]; fv[k + 1] = r;
        int t = place[k]; place[k] = place[k + 1]; place[k + 1] = t;
      }
}

/* Nelder-Mead search of fminsearch (:1222-1473) with tolx = tolf = 1e-4. */
static void att_fminsearch(double *x) {
  const int n = N_SLS;
  const double rho = 1.0, chi = 2.0, psi = 0.5, sigma = 0.5, tolx = 1.0e-4, tolf = 1.0e-4;
  const int maxiter = 200 * n, maxfun = 200 * n;
  double v[N_SLS][N_SLS + 1], fv[N_SLS + 1], vt[N_SLS][N_SLS + 1];
  int place[N_SLS + 1];
  for (int i = 0; i < n; ++i) v[i][0] = x[i];
  fv[0] = att_eval(x);
  for (int j = 0; j < n; ++j) {
    double y[N_SLS];
    for (int i = 0; i < n; ++i) y[i] = x[i];
    y[j] = y[j] != 0.0 ? (1.0 + 0.05) * y[j] : 0.00025;
    for (int i = 0; i < n; ++i) v[i][j + 1] = y[i];
    fv[j + 1] = att_eval(y);
  }
  att_sort(fv, place, n + 1);
  for (int j = 0; j <= n; ++j) for (int i = 0; i < n; ++i) vt[i][j] = v[i][place[j]];
  memcpy(v, vt, sizeof(v));
  int itercount = 1, func_evals = n + 1;
  while (func_evals < maxfun && itercount < maxiter) {
    double ms = 0.0, mv = 0.0;
    for (int i = 0; i < n; ++i) for (int j = 1; j <= n; ++j) { double z = fabs(v[i][j] - v[i][0]); if (z > ms) ms = z; }
    for (int j = 1; j <= n; ++j) { double z = fabs(fv[0] - fv[j]); if (z > mv) mv = z; }
    if (ms <= tolx && mv <= tolf) break;
    double xbar[N_SLS], xr[N_SLS], xe[N_SLS], xc[N_SLS], xcc[N_SLS];
    for (int i = 0; i < n; ++i) { xbar[i] = 0; for (int j = 0; j < n; ++j) xbar[i] += v[i][j]; xbar[i] /= (double)n; }
    for (int i = 0; i < n; ++i) xr[i] = (1 + rho) * xbar[i] - rho * v[i][n];
    double fxr = att_eval(xr); func_evals++;
    int shrink = 0;
    if (fxr < fv[0]) {
      for (int i = 0; i < n; ++i) xe[i] = (1 + rho * chi) * xbar[i] - rho * chi * v[i][n];
      double fxe = att_eval(xe); func_evals++;
      if (fxe < fxr) { for (int i = 0; i < n; ++i) v[i][n] = xe[i]; fv[n] = fxe; }
      else { for (int i = 0; i < n; ++i) v[i][n] = xr[i]; fv[n] = fxr; }
    } else if (fxr < fv[n - 1]) {
      for (int i = 0; i < n; ++i) v[i][n] = xr[i];
      fv[n] = fxr;
    } else {
      if (fxr < fv[n]) {
        for (int i = 0; i < n; ++i) xc[i] = (1 + psi * rho) * xbar[i] - psi * rho * v[i][n];
        double fxc = att_eval(xc); func_evals++;
        if (fxc <= fxr) { for (int i = 0; i < n; ++i) v[i][n] = xc[i]; fv[n] = fxc; } else shrink = 1;
      } else {
        for (int i = 0; i < n; ++i) xcc[i] = (1 - psi) * xbar[i] + psi * v[i][n];
        double fxcc = att_eval(xcc); func_evals++;
        if (fxcc < fv[n]) { for (int i = 0; i < n; ++i) v[i][n] = xcc[i]; fv[n] = fxcc; } else shrink = 1;
      }
      if (shrink) {
        for (int j = 1; j <= n; ++j) {
          double xx[N_SLS];
          for (int i = 0; i < n; ++i) { v[i][j] = v[i][0] + sigma * (v[i][j] - v[i][0]); xx[i] = v[i][j]; }
          fv[j] = att_eval(xx);
        }
        func_evals += n;
      }
    }
    att_sort(fv, place, n + 1);
    for (int j = 0; j <= n; ++j) for (int i = 0; i < n; ++i) vt[i][j] = v[i][place[j]];
    memcpy(v, vt, sizeof(v));
    itercount++;
  }
  for (int i = 0; i < n; ++i) x[i] = v[i][0];
}

/* get_attenuation_periods / _tau_sigma / _source_freq (:702-810) from the
 * minimum resolved period; outputs tau_sigma (double), f_c_source, band. */
void orc_attenuation_constants(double min_resolved_period_f32, double *tau_sigma, double *f_c_source,
                               double *min_period, double *max_period) {
  const double PI = 3.14159265358979;
  float minp = (float)(0.99f * (float)min_resolved_period_f32);
  *min_period = minp;
  *max_period = *min_period * pow(10.0, 1.75);
  double f1 = 1.0 / *max_period, f2 = 1.0 / *min_period;
  double e1 = log10(f1), e2 = log10(f2), d = (e2 - e1) / ((double)N_SLS - 1);
  for (int i = 0; i < N_SLS; ++i) tau_sigma[i] = 1.0 / (PI * 2.0 * pow(10.0, e1 + i * 1.0 * d));
  *f_c_source = pow(10.0, 0.5 * (log10(f1) + log10(f2)));
}

/* get_attenuation_tau_eps via attenuation_invert_by_simplex (:838-1058) and the
 * derived factors (get_attenuation_property_values, _scale_factor, :599-694).
 * Outputs beta(N_SLS), one_minus_sum_beta, scale_factor for one Q value. */
void orc_attenuation_factors(double Q, const double *tau_sigma, double min_period, double max_period,
                             double f_c_source, double f0_reference, double *beta, double *one_minus_sum_beta,
                             double *scale_factor, double *tau_eps_out) {
  const double PI = 3.141592653589793, TWO_PI = 2.0 * PI;
  double tau_eps[N_SLS];
  double f1 = 1.0 / max_period, f2 = 1.0 / min_period, e1 = log10(f1), e2 = log10(f2);
  for (int i = 0; i < ATT_NF; ++i) g_att_f[i] = e1 + (i * 1.0 * (e2 - e1) / ((ATT_NF - 1) * 1.0));
  for (int i = 0; i < N_SLS; ++i) g_att_tau_s[i] = tau_sigma[i];
  g_att_iQ = 1.0 / Q;
  for (int i = 0; i < N_SLS; ++i) tau_eps[i] = tau_sigma[i] + (tau_sigma[i] * 2.0 / Q);
  att_fminsearch(tau_eps);
  double s = 0.0;
  for (int i = 0; i < N_SLS; ++i) { beta[i] = tau_eps[i] / tau_sigma[i]; s += beta[i]; beta[i] -= 1.0; }
  *one_minus_sum_beta = s;
  double mu0 = 1.0 + 2.0 * log(f_c_source / f0_reference) / (PI * Q);
  double x1 = 1.0, x2 = 1.0;
  for (int i = 0; i < N_SLS; ++i) {
    double ak = tau_eps[i] / tau_sigma[i] - 1.0;
    x1 += ak / N_SLS;
    x2 += ak / (1.0 + 1.0 / pow(TWO_PI * f_c_source * tau_sigma[i], 2)) / N_SLS;
  }
  *scale_factor = (x1 / x2) * mu0;
  if (tau_eps_out) for (int i = 0; i < N_SLS; ++i) tau_eps_out[i] = tau_eps[i];
}

/* get_attenuation_memory_values (:464-493) in CUSTOM_REAL. */
void orc_attenuation_memory_values(const realw *tau_s, realw deltat, realw *alphaval, realw *betaval,
                                   realw *gammaval) {
  for (int i = 0; i < N_SLS; ++i) {
    realw ti = (realw)-1 / tau_s[i];
    realw d2 = deltat * deltat, d3 = d2 * deltat, d4 = d3 * deltat;
    alphaval[i] = (realw)1.0 + deltat * ti + d2 * (ti * ti) / (realw)2 + d3 * (ti * ti * ti) / (realw)6 +
                  d4 * (ti * ti * ti * ti) / (realw)24;
    betaval[i] = deltat / (realw)2 + d2 * ti / (realw)3 + d3 * (ti * ti) / (realw)8 + d4 * (ti * ti * ti) / (realw)24;
    gammaval[i] = deltat / (realw)2 + d2 * ti / (realw)6 + d3 * (ti * ti) / (realw)24;
  }
}

/* ------------------------------------------------------------------------- */
/* acoustic domain and fluid-solid coupling                                   */
/* ------------------------------------------------------------------------- */

/* Acoustic stiffness of one element (compute_forces_acoustic.F90:130-340):
 * chi_dot_dot -= w . hprimewgll^T (J/rho grad(xi) . grad chi). */
static void element_forces_acoustic(const orc_sim *s, int ispec, const realw *pot, realw *pot_dd) {
  const realw *hp = s->hprime_xx, *hpw = s->hprimewgll_xx;
  realw chi[NGLL3], t1[NGLL3], t2[NGLL3], t3[NGLL3];
  const int *ib = s->ibool + (long)NGLL3 * ispec;
  for (int p = 0; p < NGLL3; ++p) chi[p] = pot[ib[p] - 1];
  for (int k = 0; k < NGLL; ++k)
    for (int j = 0; j < NGLL; ++j)
      for (int i = 0; i < NGLL; ++i) {
        realw a = 0, b = 0, c = 0;
        for (int l = 0; l < NGLL; ++l) {
          a += chi[IJK(l, j, k)] * hp[i + NGLL * l];
          b += chi[IJK(i, l, k)] * hp[j + NGLL * l];
          c += chi[IJK(i, j, l)] * hp[k + NGLL * l];
        }
        int p = IJK(i, j, k);
        t1[p] = a; t2[p] = b; t3[p] = c;
      }
  const int ir = s->irregular_element_number[ispec];
  const long mo = (long)NGLL3 * (ir - 1);
  for (int p = 0; p < NGLL3; ++p) {
    realw rho_inv = (realw)1.0 / s->rhostore[(long)NGLL3 * ispec + p];
    if (ir) {
      realw xixl = s->xix[mo + p], xiyl = s->xiy[mo + p], xizl = s->xiz[mo + p];
      realw etaxl = s->etax[mo + p], etayl = s->etay[mo + p], etazl = s->etaz[mo + p];
      realw gxl = s->gammax[mo + p], gyl = s->gammay[mo + p], gzl = s->gammaz[mo + p];
      realw jl = s->jacobian[mo + p];
      realw dx = xixl * t1[p] + etaxl * t2[p] + gxl * t3[p];
      realw dy = xiyl * t1[p] + etayl * t2[p] + gyl * t3[p];
      realw dz = xizl * t1[p] + etazl * t2[p] + gzl * t3[p];
      t1[p] = rho_inv * jl * (xixl * dx + xiyl * dy + xizl * dz);
      t2[p] = rho_inv * jl * (etaxl * dx + etayl * dy + etazl * dz);
      t3[p] = rho_inv * jl * (gxl * dx + gyl * dy + gzl * dz);
    } else {
      realw f = rho_inv * s->jacobian_regular * s->xix_regular * s->xix_regular;
      t1[p] = f * t1[p]; t2[p] = f * t2[p]; t3[p] = f * t3[p];
    }
  }
  for (int k = 0; k < NGLL; ++k)
    for (int j = 0; j < NGLL; ++j)
      for (int i = 0; i < NGLL; ++i) {
        realw a = 0, b = 0, c = 0;
        for (int l = 0; l < NGLL; ++l) {
          a += t1[IJK(l, j, k)] * hpw[l + NGLL * i];
          b += t2[IJK(i, l, k)] * hpw[l + NGLL * j];
          c += t3[IJK(i, j, l)] * hpw[l + NGLL * k];
        }
        long g = ib[IJK(i, j, k)] - 1;
        realw add = s->wgllwgll_yz[j + NGLL * k] * a + s->wgllwgll_xz[i + NGLL * k] * b + s->wgllwgll_xy[i + NGLL * j] * c;
#pragma omp atomic
        pot_dd[g] -= add;
      }
}

void orc_compute_forces_acoustic(orc_sim *s) {
#ifdef _OPENMP
  omp_set_num_threads(s->nthreads > 0 ? s->nthreads : 1);
#pragma omp parallel for schedule(static)
#endif
  for (int q = 0; q < s->n_acoustic; ++q) element_forces_acoustic(s, s->acoustic_list[q] - 1, s->potential, s->potential_dot_dot);
}

/* compute_stacey_acoustic_forward (compute_stacey_acoustic.f90:79-125) */
static void stacey_acoustic(orc_sim *s) {
  for (int f = 0; f < s->num_abs_boundary_faces; ++f) {
    int ispec = s->abs_boundary_ispec[f] - 1;
    if (!s->ispec_is_acoustic || !s->ispec_is_acoustic[ispec]) continue;
    for (int g = 0; g < NGLL2; ++g) {
      const int *ijk = s->abs_boundary_ijk + 3 * (g + NGLL2 * f);
      long p = IJK(ijk[0] - 1, ijk[1] - 1, ijk[2] - 1) + (long)NGLL3 * ispec;
      long ig = s->ibool[p] - 1;
      realw rhol = s->rhostore[p];
      realw cpl = (realw)sqrt((double)(s->kappastore[p] / rhol));
      realw jw = s->abs_boundary_jacobian2Dw[g + NGLL2 * f];
      realw absorbl = s->potential_dot[ig] * jw / cpl / rhol;
      s->potential_dot_dot[ig] -= absorbl;
    }
  }
}

/* compute_coupling_acoustic_el (compute_coupling_acoustic_el.f90:70-150):
 * chi_dot_dot += jw (u . n), n pointing out of the fluid. */
static void coupling_acoustic_el(orc_sim *s) {
  for (int f = 0; f < s->num_coupling_faces; ++f) {
    int ispec = s->coupling_ispec[f] - 1;
    for (int g = 0; g < NGLL2; ++g) {
      const int *ijk = s->coupling_ijk + 3 * (g + NGLL2 * f);
      long ig = s->ibool[IJK(ijk[0] - 1, ijk[1] - 1, ijk[2] - 1) + (long)NGLL3 * ispec] - 1;
      const realw *n = s->coupling_normal + 3 * (g + NGLL2 * f);
      realw dn = s->displ[3 * ig] * n[0] + s->displ[3 * ig + 1] * n[1] + s->displ[3 * ig + 2] * n[2];
      s->potential_dot_dot[ig] += s->coupling_jacobian2Dw[g + NGLL2 * f] * dn;
    }
  }
}

/* compute_coupling_viscoelastic_ac (compute_coupling_viscoelastic_ac.f90:70-160):
 * accel += jw n (-chi_dot_dot). */
static void coupling_elastic_ac(orc_sim *s) {
  for (int f = 0; f < s->num_coupling_faces; ++f) {
    int ispec = s->coupling_ispec[f] - 1;
    for (int g = 0; g < NGLL2; ++g) {
      const int *ijk = s->coupling_ijk + 3 * (g + NGLL2 * f);
      long ig = s->ibool[IJK(ijk[0] - 1, ijk[1] - 1, ijk[2] - 1) + (long)NGLL3 * ispec] - 1;
      const realw *n = s->coupling_normal + 3 * (g + NGLL2 * f);
      realw pr = -s->potential_dot_dot[ig];
      realw jw = s->coupling_jacobian2Dw[g + NGLL2 * f];
      s->accel[3 * ig] += jw * n[0] * pr;
      s->accel[3 * ig + 1] += jw * n[1] * pr;
      s->accel[3 * ig + 2] += jw * n[2] * pr;
    }
  }
}

/* compute_add_sources_acoustic (compute_add_sources_acoustic.f90:100-126):
 * chi_dot_dot -= sourcearray(1) stf / kappa for sources in fluid elements. */
static void add_sources_acoustic(orc_sim *s, int it) {
  for (int isrc = 0; isrc < s->nsources; ++isrc) {
    int ispec = s->ispec_selected_source[isrc] - 1;
    if (!s->ispec_is_acoustic || !s->ispec_is_acoustic[ispec]) continue;
    realw stf = (realw)s->stf[isrc + (long)s->nsources * (it - 1)];
    for (int p = 0; p < NGLL3; ++p) {
      long q = (long)NGLL3 * ispec + p;
      long ig = s->ibool[q] - 1;
      s->potential_dot_dot[ig] -= s->sourcearrays[isrc + (long)s->nsources * (0 + 3 * p)] * stf / s->kappastore[q];
    }
  }
}

/* acoustic_enforce_free_surface (compute_forces_acoustic_calling_routine.f90:754-810) */
static void enforce_free_surface(orc_sim *s) {
  for (int f = 0; f < s->num_free_surface_faces; ++f) {
    int ispec = s->free_surface_ispec[f] - 1;
    if (!s->ispec_is_acoustic[ispec]) continue;
    for (int g = 0; g < NGLL2; ++g) {
      const int *ijk = s->free_surface_ijk + 3 * (g + NGLL2 * f);
      long ig = s->ibool[IJK(ijk[0] - 1, ijk[1] - 1, ijk[2] - 1) + (long)NGLL3 * ispec] - 1;
      s->potential[ig] = 0; s->potential_dot[ig] = 0; s->potential_dot_dot[ig] = 0;
    }
  }
}

/* One coupled fluid-solid step (iterate_time.F90:219-300 with
 * compute_forces_acoustic_calling_routine.f90:54-343 then
 * compute_forces_viscoelastic_calling_routine.F90:107-417). */
void orc_step_coupled(orc_sim *s) {
  long n3 = 3L * s->nglob;
  newmark_predictor(n3, s->displ, s->veloc, s->accel, s->deltat, s->deltatover2, s->deltatsqover2);
  newmark_predictor(s->nglob, s->potential, s->potential_dot, s->potential_dot_dot, s->deltat, s->deltatover2,
                    s->deltatsqover2);
  /* fluid */
  enforce_free_surface(s);
  if (s->stacey) stacey_acoustic(s);
  if (s->num_coupling_faces) coupling_acoustic_el(s);
  if (s->nsources > 0 && s->stf) add_sources_acoustic(s, s->it);
  orc_compute_forces_acoustic(s);
  for (long g = 0; g < s->nglob; ++g) {
    s->potential_dot_dot[g] *= s->rmass_acoustic[g];
    s->potential_dot[g] += s->deltatover2 * s->potential_dot_dot[g];
  }
  enforce_free_surface(s);
  /* solid */
  if (s->stacey && s->num_abs_boundary_faces > 0) orc_stacey_elastic(s, s->veloc, s->accel);
  if (s->num_coupling_faces) coupling_elastic_ac(s);
  if (s->nsources > 0 && s->stf) orc_add_sources(s, s->accel, s->it);
  orc_compute_forces_elastic(s, 0);
  for (long g = 0; g < s->nglob; ++g) {
    s->accel[3 * g] *= s->rmassx[g];
    s->accel[3 * g + 1] *= s->rmassy[g];
    s->accel[3 * g + 2] *= s->rmassz[g];
  }
  for (long i = 0; i < n3; ++i) s->veloc[i] += s->deltatover2 * s->accel[i];
  if (s->nrec > 0 && s->seismograms) {
    const realw *f = s->record_what == 2 ? s->veloc : (s->record_what == 3 ? s->accel : s->displ);
    orc_seismograms(s, f, s->it);
  }
  s->it++;
}

void orc_run_coupled(orc_sim *s, int nsteps) {
  for (int n = 0; n < nsteps; ++n) orc_step_coupled(s);
}
