/*
 * CPU oracle for the SPECFEM3D Cartesian spectral-element time step.
 *
 * TEST INFRASTRUCTURE ONLY.  The GB300 CUDA path is tested against this
 * library: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * may load it.  The product library never links or calls it.
 *
 * It restates, in plain C, the reference solver's CPU algorithms (file:line
 * citations are given on each function in sem_oracle.c).  It is compiled twice:
 * REALW=float  -> liboracle_f32.so  (the reference built with CUSTOM_REAL=4)
 * REALW=double -> liboracle_f64.so  (the reference built with
 *                                   --enable-double-precision, CUSTOM_REAL=8)
 *
 * Array layouts are the reference's Fortran column-major layouts, 0-based in C
 * but holding the reference's 1-based index values (ibool, ijk, ispec):
 *   ibool(i,j,k,ispec)          -> ibool[i + 5j + 25k + 125 ispec]
 *   displ(3,NGLOB)              -> displ[c + 3 iglob]
 *   R_xx(N_SLS,i,j,k,ispec)     -> R_xx[s + 3 (ijk + 125 ispec)]
 *   abs_boundary_ijk(3,25,nf)   -> ijk[c + 3 (igll + 25 iface)]
 *   sourcearrays(NSOURCES,3,i,j,k) -> sa[isrc + NSRC (c + 3 ijk)]
 */
#ifndef SEM_ORACLE_H
#define SEM_ORACLE_H

#ifdef ORACLE_DOUBLE
typedef double realw;
#else
typedef float realw;
#endif

#define NGLL 5
#define NGLL2 25
#define NGLL3 125
#define N_SLS 3

typedef struct orc_sim {
  /* sizes and switches */
  int nspec, nglob, nspec_irregular;
  int nsources, nrec, nstep, it;
  int attenuation, stacey, compute_and_store_strain;
  int simulation_type;      /* 1 forward, 3 adjoint + reconstructed forward */
  int nthreads;
  int record_what;          /* 1 displacement, 2 velocity, 3 acceleration */

  /* mesh */
  int *ibool, *irregular_element_number;
  realw *xix, *xiy, *xiz, *etax, *etay, *etaz, *gammax, *gammay, *gammaz, *jacobian;
  realw xix_regular, jacobian_regular;
  realw *kappastore, *mustore, *rho_vp, *rho_vs, *rhostore;
  realw *rmassx, *rmassy, *rmassz;
  realw *hprime_xx, *hprimewgll_xx, *wgllwgll_xy, *wgllwgll_xz, *wgllwgll_yz;

  /* Stacey */
  int num_abs_boundary_faces;
  int *abs_boundary_ispec, *abs_boundary_ijk;
  realw *abs_boundary_normal, *abs_boundary_jacobian2Dw;

  /* attenuation */
  realw *alphaval, *betaval, *gammaval;  /* N_SLS */
  realw *factor_common, *factor_common_kappa;
  realw *R_xx, *R_yy, *R_xy, *R_xz, *R_yz, *R_trace;
  realw *epsilondev_xx, *epsilondev_yy, *epsilondev_xy, *epsilondev_xz, *epsilondev_yz;
  realw *epsilondev_trace, *epsilon_trace_over_3;

  /* sources / receivers */
  realw *sourcearrays;
  int *ispec_selected_source;
  double *stf;              /* (nsources, nstep): stf[isrc + nsources*(it-1)] */
  int *ispec_selected_rec;
  double *hxir, *hetar, *hgammar;   /* (5, nrec) */
  double *nu_rec;                   /* (3,3,nrec) */
  double *seismograms;              /* (3, nrec, nstep) */

  /* wavefields */
  realw *displ, *veloc, *accel;
  realw deltat, deltatover2, deltatsqover2;

  /* adjoint (SIMULATION_TYPE=3): reconstructed/backward field and kernels */
  realw *b_displ, *b_veloc, *b_accel;
  realw *b_epsilondev_xx, *b_epsilondev_yy, *b_epsilondev_xy, *b_epsilondev_xz, *b_epsilondev_yz;
  realw *b_epsilon_trace_over_3;
  realw b_deltat, b_deltatover2, b_deltatsqover2;
  double *rho_kl, *mu_kl, *kappa_kl;   /* (125, nspec) accumulated in FP64 */
  realw *source_adjoint;               /* (3, nrec, nstep) adjoint source traces */
  double *hxir_adj, *hetar_adj, *hgammar_adj;

  /* acoustic domain and fluid-solid coupling */
  int n_elastic, n_acoustic;           /* element lists (1-based ispec); n_elastic<0: all elastic */
  int *elastic_list, *acoustic_list;
  int *ispec_is_acoustic;              /* (nspec) 0/1 */
  realw *potential, *potential_dot, *potential_dot_dot, *rmass_acoustic;
  int num_coupling_faces, *coupling_ispec, *coupling_ijk;
  realw *coupling_normal, *coupling_jacobian2Dw;
  int num_free_surface_faces, *free_surface_ispec, *free_surface_ijk;
  int *rec_is_acoustic;                /* (nrec) records pressure when 1 */
  int fluid_vector;                    /* 1: fluid receivers record (1/rho) grad of the potential */
  realw *cstore;                       /* ANISOTROPY: (21, 125*nspec) c11..c66 per point, or NULL */

  /* C-PML layers, forward field (prepare_timerun_pml, compute_forces_viscoelastic_PML) */
  int nspec_cpml;
  int *is_cpml;                        /* (nspec) 0/1 */
  int *cpml_to_spec;                   /* (nspec_cpml) 1-based */
  int *spec_to_cpml;                   /* (nspec) 1-based, 0 outside the layers */
  realw *pml_coef_alpha, *pml_coef_beta;   /* (9, 125, nspec_cpml) */
  realw *pml_coef_abar;                /* (5, 125, nspec_cpml) */
  realw *pml_coef_strain;              /* (18, 125, nspec_cpml) */
  realw *wgll_cube;                    /* (125) */
  realw *pml_displ_old, *pml_displ_new;    /* (3, 125, nspec_cpml) */
  realw *pml_rmem;                     /* (48, 125, nspec_cpml) convolution memory variables */
} orc_sim;

#endif
