/*
 * specfem3d_gb300 — C ABI of the GB300 (sm_103a) spectral-element time step.
 *
 * Two layers:
 *
 * 1. Drop-in entry points with the exact names and argument lists of the
 *    reference's Fortran-callable GPU layer (the .cu files of src/gpu, declared through
 *    FC_FUNC_(name,NAME), which gfortran resolves to `name_`).  Every argument
 *    is passed by reference, Fortran LOGICALs arrive as int*, index arrays hold
 *    the Fortran 1-based values, host arrays keep the Fortran layouts listed in
 *    the comments.  Each declaration cites the reference function it replaces.
 *    Like the reference these return void; on an error they record a status
 *    (read it with sf3d_last_error) instead of aborting, unless the environment
 *    variable SF3D_ABORT_ON_ERROR=1 asks for the reference's exit(1).
 *
 * 2. sf3d_* entry points of this library (status-returning): error queries,
 *    whole-run time loops captured in CUDA graphs, and the batched-shot API.
 *
 * realw is float (the reference GPU build is single precision only,
 * src/gpu/mesh_constants_gpu.h:80-87).
 */
#ifndef SPECFEM3D_GB300_H
#define SPECFEM3D_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef float realw;

/* ---------------------------------------------------------------------------
 * status API (no reference counterpart: the reference aborts on any error)
 * ------------------------------------------------------------------------- */
#define SF3D_OK 0
#define SF3D_ERR_ARG 1      /* invalid argument or size */
#define SF3D_ERR_CUDA 2     /* CUDA runtime error */
#define SF3D_ERR_STATE 3    /* call out of order / handle not prepared */
#define SF3D_ERR_UNSTABLE 4 /* wavefield blew up (NaN/Inf or above threshold) */
#define SF3D_ERR_UNSUPPORTED 5 /* entry point of a feature this library does not provide */

int sf3d_last_error(char *msg, int msg_len);  /* returns last status, copies message */
void sf3d_clear_error(void);
int sf3d_version(void);

/* ---------------------------------------------------------------------------
 * setup — src/gpu/initialize_gpu.cu, src/gpu/prepare_mesh_constants_cuda.cu
 * ------------------------------------------------------------------------- */

/* initialize_gpu_device (initialize_gpu.cu:535): selects device myrank % count,
 * returns the visible device count. */
void initialize_gpu_device_(int *myrank_f, int *ncuda_devices);

/* prepare_constants_device (prepare_mesh_constants_cuda.cu:70-119, argument list
 * as called from specfem3D/prepare_gpu.f90:67-101).  Allocates the Mesh handle
 * and stores it in *Mesh_pointer.  Layouts: xix..gammaz (5,5,5,NSPEC_IRREGULAR),
 * ibool (5,5,5,NSPEC_AB), abs_boundary_ijk (3,25,nfaces), abs_boundary_normal
 * (3,25,nfaces), abs_boundary_jacobian2Dw (25,nfaces), sourcearrays
 * (NSOURCES,3,5,5,5), xir/etar/gammar (5,nrec_local), nu_rec/nu_source
 * (3,3,nrec)/(3,3,NSOURCES) in double. */
void prepare_constants_device_(long *Mesh_pointer, int *h_NGLLX, int *NSPEC_AB, int *NGLOB_AB,
                               int *NSPEC_IRREGULAR, int *h_irregular_element_number,
                               realw *h_xix, realw *h_xiy, realw *h_xiz, realw *h_etax,
                               realw *h_etay, realw *h_etaz, realw *h_gammax, realw *h_gammay,
                               realw *h_gammaz, realw *xix_regular, realw *jacobian_regular,
                               int *h_ibool, int *num_interfaces_ext_mesh,
                               int *max_nibool_interfaces_ext_mesh,
                               int *h_nibool_interfaces_ext_mesh, int *h_ibool_interfaces_ext_mesh,
                               realw *h_hprime_xx, realw *h_hprimewgll_xx, realw *h_wgllwgll_xy,
                               realw *h_wgllwgll_xz, realw *h_wgllwgll_yz,
                               int *STACEY_ABSORBING_CONDITIONS, int *h_abs_boundary_ispec,
                               int *h_abs_boundary_ijk, realw *h_abs_boundary_normal,
                               realw *h_abs_boundary_jacobian2Dw, int *h_num_abs_boundary_faces,
                               int *h_ispec_is_inner, int *NSOURCES, int *nsources_local_f,
                               realw *h_sourcearrays, int *h_islice_selected_source,
                               int *h_ispec_selected_source, int *h_ispec_selected_rec, int *nrec,
                               int *nrec_local, int *SIMULATION_TYPE, int *USE_MESH_COLORING_GPU_f,
                               int *nspec_acoustic, int *nspec_elastic, int *ispec_is_acoustic,
                               int *ispec_is_elastic, int *h_myrank, int *SAVE_FORWARD,
                               realw *h_xir, realw *h_etar, realw *h_gammar, double *nu_rec,
                               double *nu_source, int *h_islice_selected_rec,
                               int *nlength_seismogram, int *SAVE_SEISMOGRAMS_DISPLACEMENT,
                               int *SAVE_SEISMOGRAMS_VELOCITY, int *SAVE_SEISMOGRAMS_ACCELERATION,
                               int *SAVE_SEISMOGRAMS_PRESSURE, int *h_NB_RUNS_ACOUSTIC_GPU,
                               int *FAULT_SIMULATION, int *UNDO_ATTENUATION_AND_OR_PML,
                               int *PML_CONDITIONS);

/* prepare_fields_elastic_device (prepare_mesh_constants_cuda.cu:657-998;
 * specfem3D/prepare_gpu.f90:138-165).  rmass{x,y,z} (NGLOB), rho_vp/rho_vs/
 * kappav/muv (5,5,5,NSPEC), phase_ispec_inner_elastic (num_phase_ispec,2),
 * R_* / factor_common* (N_SLS,5,5,5,NSPEC), epsilondev_* (5,5,5,NSPEC),
 * alphaval/betaval/gammaval (N_SLS). */
void prepare_fields_elastic_device_(long *Mesh_pointer, realw *rmassx, realw *rmassy, realw *rmassz,
                                    realw *rho_vp, realw *rho_vs, realw *h_kappav, realw *h_muv,
                                    int *num_phase_ispec_elastic, int *phase_ispec_inner_elastic,
                                    realw *b_absorb_field, int *b_reclen_field,
                                    int *COMPUTE_AND_STORE_STRAIN, realw *epsilondev_xx,
                                    realw *epsilondev_yy, realw *epsilondev_xy,
                                    realw *epsilondev_xz, realw *epsilondev_yz, int *ATTENUATION,
                                    int *R_size, realw *R_xx, realw *R_yy, realw *R_xy,
                                    realw *R_xz, realw *R_yz, realw *factor_common,
                                    realw *R_trace, realw *epsilondev_trace,
                                    realw *factor_common_kappa, realw *alphaval, realw *betaval,
                                    realw *gammaval, int *APPROXIMATE_OCEAN_LOAD,
                                    realw *rmass_ocean_load, int *NOISE_TOMOGRAPHY,
                                    realw *free_surface_normal, int *free_surface_ispec,
                                    int *free_surface_ijk, int *num_free_surface_faces,
                                    int *ACOUSTIC_SIMULATION, int *num_colors_outer_elastic,
                                    int *num_colors_inner_elastic, int *num_elem_colors_elastic,
                                    int *ANISOTROPY, realw *c11store, realw *c12store,
                                    realw *c13store, realw *c14store, realw *c15store,
                                    realw *c16store, realw *c22store, realw *c23store,
                                    realw *c24store, realw *c25store, realw *c26store,
                                    realw *c33store, realw *c34store, realw *c35store,
                                    realw *c36store, realw *c44store, realw *c45store,
                                    realw *c46store, realw *c55store, realw *c56store,
                                    realw *c66store);

/* prepare_cleanup_device (prepare_mesh_constants_cuda.cu:1552): frees the handle. */
void prepare_cleanup_device_(long *Mesh_pointer, int *ACOUSTIC_SIMULATION, int *ELASTIC_SIMULATION,
                             int *NOISE_TOMOGRAPHY);

/* ---------------------------------------------------------------------------
 * hot path — one call each per time step, in iterate_time.F90 order
 * ------------------------------------------------------------------------- */

/* update_displacement_cuda (update_displacement_cuda.cu:39-188): Newmark predictor
 * u += dt v + dt^2/2 a; v += dt/2 a; a = 0 on the forward (1), backward (3) or both (0) fields. */
void update_displacement_cuda_(long *Mesh_pointer, realw *deltat_F, realw *deltatover2_F,
                               realw *deltatsqover2_F, int *FORWARD_OR_ADJOINT);

/* compute_forces_viscoelastic_cuda (compute_forces_viscoelastic_cuda.cu:1115-1278):
 * elastic stiffness of the elements of phase iphase (1 outer, 2 inner), gathered
 * through ibool and scatter-added into accel; attenuation memory variables and
 * strain updated when requested. */
void compute_forces_viscoelastic_cuda_(long *Mesh_pointer, int *iphase, realw *deltat,
                                       int *nspec_outer_elastic, int *nspec_inner_elastic,
                                       int *COMPUTE_AND_STORE_STRAIN, int *ATTENUATION,
                                       int *FORWARD_OR_ADJOINT_f);

/* compute_stacey_viscoelastic_cuda (compute_stacey_viscoelastic_cuda.cu:39-222):
 * absorbing traction on the Stacey faces (iphase 1 only). */
void compute_stacey_viscoelastic_cuda_(long *Mesh_pointer, int *iphasef, realw *b_absorb_field,
                                       int *FORWARD_OR_ADJOINT_f);

/* compute_add_sources_el_cuda (compute_add_sources_viscoelastic_cuda.cu:39-100):
 * accel += sourcearrays * stf, stf given per source for this step (FP64 host). */
void compute_add_sources_el_cuda_(long *Mesh_pointer, double *h_stf_pre_compute, int *h_NSOURCES);

/* compute_add_sources_el_s3_cuda (compute_add_sources_viscoelastic_cuda.cu:~105):
 * same on the backward/reconstructed field. */
void compute_add_sources_el_s3_cuda_(long *Mesh_pointer, double *h_stf_pre_compute, int *h_NSOURCES);

/* kernel_3_a_cuda (update_displacement_cuda.cu:287-380): a *= rmass{x,y,z};
 * v += dt/2 a (fused mass + corrector without ocean load).  The pass is
 * deferred and fused with the next update_displacement_cuda of the same field
 * (one streaming pass instead of two); every other entry point applies it
 * first, so callers observe the reference's fields. */
void kernel_3_a_cuda_(long *Mesh_pointer, realw *deltatover2_F, realw *b_deltatover2_F,
                      int *APPROXIMATE_OCEAN_LOAD, int *FORWARD_OR_ADJOINT);

/* kernel_3_b_cuda (update_displacement_cuda.cu:382): corrector only (ocean-load path). */
void kernel_3_b_cuda_(long *Mesh_pointer, realw *deltatover2_F, realw *b_deltatover2_F,
                      int *FORWARD_OR_ADJOINT);

/* compute_seismograms_cuda (write_seismograms_cuda.cu:34-373): receiver
 * interpolation into the device trace buffer (NDIM,nrec_local,nlength); the
 * buffer is copied to the host arrays when full or at it == it_end. */
void compute_seismograms_cuda_(long *Mesh_pointer_f, realw *seismograms_d, realw *seismograms_v,
                               realw *seismograms_a, realw *seismograms_p, int *seismo_currentf,
                               int *nlength_seismogramf, int *itf, int *it_endf,
                               int *ACOUSTIC_SIMULATION, int *ELASTIC_SIMULATION,
                               int *USE_TRICK_FOR_BETTER_PRESSURE);

/* ---------------------------------------------------------------------------
 * fluid domain and fluid-solid coupling — src/gpu/compute_forces_acoustic_cuda.cu,
 * compute_stacey_acoustic_cuda.cu, compute_coupling_cuda.cu, update_displacement_cuda.cu
 * ------------------------------------------------------------------------- */

/* prepare_fields_acoustic_device (prepare_mesh_constants_cuda.cu:434): rmass_acoustic
 * (NGLOB), rhostore/kappastore (5,5,5,NSPEC), phase lists (num,2), free-surface and
 * coupling faces (ispec, ijk (3,25,nf), normal (3,25,nf) pointing out of the fluid). */
void prepare_fields_acoustic_device_(long *Mesh_pointer, realw *rmass_acoustic, realw *rhostore,
                                     realw *kappastore, int *num_phase_ispec_acoustic,
                                     int *phase_ispec_inner_acoustic, int *NOISE_TOMOGRAPHY,
                                     int *num_free_surface_faces, int *free_surface_ispec,
                                     int *free_surface_ijk, int *b_reclen_potential,
                                     realw *b_absorb_potential, int *ELASTIC_SIMULATION,
                                     int *num_coupling_ac_el_faces, int *coupling_ac_el_ispec,
                                     int *coupling_ac_el_ijk, realw *coupling_ac_el_normal,
                                     realw *coupling_ac_el_jacobian2Dw, int *num_colors_outer_acoustic,
                                     int *num_colors_inner_acoustic, int *num_elem_colors_acoustic);
/* compute_forces_acoustic_cuda (compute_forces_acoustic_cuda.cu:238): fluid stiffness. */
void compute_forces_acoustic_cuda_(long *Mesh_pointer, int *iphase, int *nspec_outer_acoustic,
                                   int *nspec_inner_acoustic, int *FORWARD_OR_ADJOINT_f);
/* acoustic_enforce_free_surf_cuda (compute_forces_acoustic_cuda.cu:334). */
void acoustic_enforce_free_surf_cuda_(long *Mesh_pointer, int *ABSORB_INSTEAD_OF_FREE_SURFACE,
                                      int *FORWARD_OR_ADJOINT);
/* update_displacement_ac_cuda (update_displacement_cuda.cu:192): potential predictor. */
void update_displacement_ac_cuda_(long *Mesh_pointer, realw *deltat_F, realw *deltatover2_F,
                                  realw *deltatsqover2_F, int *FORWARD_OR_ADJOINT);
/* kernel_3_acoustic_cuda (update_displacement_cuda.cu:448): mass + corrector. */
void kernel_3_acoustic_cuda_(long *Mesh_pointer, realw *deltatover2_F, realw *b_deltatover2_F,
                             int *FORWARD_OR_ADJOINT_f);
/* compute_stacey_acoustic_cuda (compute_stacey_acoustic_cuda.cu:39). */
void compute_stacey_acoustic_cuda_(long *Mesh_pointer, int *iphasef, realw *h_b_absorb_potential,
                                   int *FORWARD_OR_ADJOINT_f);
/* compute_coupling_ac_el_cuda / compute_coupling_el_ac_cuda (compute_coupling_cuda.cu:39, :135). */
void compute_coupling_ac_el_cuda_(long *Mesh_pointer, int *iphasef, int *num_coupling_ac_el_facesf,
                                  int *FORWARD_OR_ADJOINT);
void compute_coupling_el_ac_cuda_(long *Mesh_pointer, int *iphasef, int *num_coupling_ac_el_facesf,
                                  int *FORWARD_OR_ADJOINT);
/* compute_add_sources_ac_cuda (compute_add_sources_acoustic_cuda.cu:65): pressure sources. */
void compute_add_sources_ac_cuda_(long *Mesh_pointer, int *NSOURCESf, double *h_stf_pre_compute,
                                  int *run_number_of_the_source);
/* transfer_fields_ac_to_device / _from_device (transfer_fields_cuda.cu): potentials (NGLOB). */
void transfer_fields_ac_to_device_(int *size, realw *potential_acoustic, realw *potential_dot_acoustic,
                                   realw *potential_dot_dot_acoustic, long *Mesh_pointer);
void transfer_fields_ac_from_device_(int *size, realw *potential_acoustic, realw *potential_dot_acoustic,
                                     realw *potential_dot_dot_acoustic, long *Mesh_pointer);

/* ---------------------------------------------------------------------------
 * transfers — src/gpu/transfer_fields_cuda.cu
 * ------------------------------------------------------------------------- */
void transfer_fields_el_to_device_(int *size, realw *displ, realw *veloc, realw *accel, long *Mesh_pointer);   /* :45 */
void transfer_fields_el_from_device_(int *size, realw *displ, realw *veloc, realw *accel, long *Mesh_pointer); /* :95 */
void transfer_b_fields_to_device_(int *size, realw *b_displ, realw *b_veloc, realw *b_accel, long *Mesh_pointer);
void transfer_b_fields_from_device_(int *size, realw *b_displ, realw *b_veloc, realw *b_accel, long *Mesh_pointer);
void transfer_displ_from_device_(int *size, realw *displ, long *Mesh_pointer);
void transfer_displ_to_device_(int *size, realw *displ, long *Mesh_pointer);
void transfer_veloc_from_device_(int *size, realw *veloc, long *Mesh_pointer);
void transfer_veloc_to_device_(int *size, realw *veloc, long *Mesh_pointer);
void transfer_accel_from_device_(int *size, realw *accel, long *Mesh_pointer);
void transfer_accel_to_device_(int *size, realw *accel, long *Mesh_pointer);
void transfer_b_displ_from_device_(int *size, realw *b_displ, long *Mesh_pointer);
void transfer_b_displ_to_device_(int *size, realw *b_displ, long *Mesh_pointer);
/* transfer_rmemory_from_device / transfer_strain_from_device
 * (transfer_fields_cuda.cu:~560-640): R_* (N_SLS,5,5,5,NSPEC), epsilondev_* (5,5,5,NSPEC). */
void transfer_rmemory_from_device_(long *Mesh_pointer, realw *R_xx, realw *R_yy, realw *R_xy,
                                   realw *R_xz, realw *R_yz, realw *R_trace, int *size_R);
void transfer_strain_from_device_(long *Mesh_pointer, realw *epsilondev_xx, realw *epsilondev_yy,
                                  realw *epsilondev_xy, realw *epsilondev_xz, realw *epsilondev_yz,
                                  realw *epsilondev_trace, int *size_epsilondev);

/* ---------------------------------------------------------------------------
 * adjoint (SIMULATION_TYPE = 3) — src/gpu/compute_kernels_cuda.cu,
 * prepare_mesh_constants_cuda.cu:999 and :1306
 * ------------------------------------------------------------------------- */
void prepare_fields_elastic_adj_dev_(long *Mesh_pointer, int *size_f, realw *epsilon_trace_over_3,
                                     realw *b_epsilondev_xx, realw *b_epsilondev_yy,
                                     realw *b_epsilondev_xy, realw *b_epsilondev_xz,
                                     realw *b_epsilondev_yz, realw *b_epsilon_trace_over_3,
                                     int *R_size, realw *b_R_xx, realw *b_R_yy, realw *b_R_xy,
                                     realw *b_R_xz, realw *b_R_yz, realw *b_R_trace,
                                     realw *b_epsilondev_trace, realw *b_alphaval,
                                     realw *b_betaval, realw *b_gammaval, int *ANISOTROPIC_KL,
                                     int *APPROXIMATE_HESS_KL);
void prepare_sim2_or_3_const_device_(long *Mesh_pointer, int *nadj_rec_local,
                                     int *NTSTEP_BETWEEN_READ_ADJSRC, realw *hxir_adjstore,
                                     realw *hetar_adjstore, realw *hgammar_adjstore, int *nrec,
                                     int *h_islice_selected_rec, int *h_ispec_selected_rec);
/* add_sources_el_sim_type_2_or_3 (compute_add_sources_viscoelastic_cuda.cu:224):
 * h_source_adjoint (3, nadj_rec_local, NTSTEP_BETWEEN_READ_ADJSRC). */
void add_sources_el_sim_type_2_or_3_(long *Mesh_pointer, realw *h_source_adjoint, int *nrec,
                                     int *nadj_rec_local, int *NTSTEP_BETWEEN_READ_ADJSRC, int *it);
/* compute_strain_cuda (compute_strain_cuda.cu): deviatoric strain and trace/3 of the
 * forward (1) or backward (3) displacement, used by the checkpointed adjoint. */
void compute_strain_cuda_(long *Mesh_pointer, int *FORWARD_OR_ADJOINT);
/* compute_kernels_elastic_cuda (compute_kernels_cuda.cu:39): rho/mu/kappa kernels
 * accumulated on the device in FP64. */
void compute_kernels_elastic_cuda_(long *Mesh_pointer, realw *deltat_f);
/* transfer_kernels_el_to_host (transfer_fields_cuda.cu:~700): (5,5,5,NSPEC). */
void transfer_kernels_el_to_host_(long *Mesh_pointer, realw *h_rho_kl, realw *h_mu_kl,
                                  realw *h_kappa_kl, realw *h_cijkl_kl, int *NSPEC_AB);

/* APPROXIMATE_HESS_KL (compute_kernels_cuda.cu:350-470): accumulate the
 * elastic Hessian kernels hess_kl += dt a_adj . b_a, hess_rho_kl += dt
 * b_v . b_v, hess_kappa_kl and hess_mu_kl from the backward strain
 * (compute_kernels.f90:513-545); acoustic Hessian kernels are not supported. */
void compute_kernels_hess_cuda_(long *Mesh_pointer, realw *deltat_f, int *ELASTIC_SIMULATION,
                                int *ACOUSTIC_SIMULATION);
void transfer_kernels_hess_el_tohost_(long *Mesh_pointer, realw *h_hess_kl, realw *h_hess_rho_kl,
                                      realw *h_hess_kappa_kl, realw *h_hess_mu_kl, int *NSPEC_AB);

/* FP64 accumulators of ANISOTROPIC_KL ((21,5,5,5,NSPEC), the strain products of
 * compute_strain_product) and APPROXIMATE_HESS_KL ((5,5,5,NSPEC) x 4: hess,
 * hess_rho, hess_kappa, hess_mu); either pointer may be NULL.  Library-only. */
int sf3d_get_extra_kernels_f64(long *Mesh_pointer, double *h_cijkl_kl, double *h_hess);

/* ---- Gaussian smoothing of kernels (xsmooth_sem GPU mode) ----------------
 * Replace prepare_smooth_gpu / compute_smooth_gpu / get_smooth_gpu
 * (src/gpu/smooth_cuda.cu:40-248).  *Container receives a handle; the
 * coordinates are per element GLL point (5,5,5,nspec); sigma_h2 = 2 sigma_h^2,
 * sigma_h3 = the horizontal search radius (smooth_sem.F90:524-559), nker <= 8.
 * compute_smooth_gpu adds the contributions of one slice (call it for this
 * slice and each neighbour); data_other is (5,5,5,nspec_other,nker).
 * get_smooth_gpu normalises, copies (5,5,5,nspec_me,nker) back and releases
 * the handle. */
void prepare_smooth_gpu_(long *Container, realw *xstore_me, realw *ystore_me, realw *zstore_me,
                         realw *sigma_h2, realw *sigma_v2, realw *sigma_h3, realw *sigma_v3, int *nspec_me,
                         int *nker);
void compute_smooth_gpu_(long *smooth_pointer, realw *data_other, realw *integ_factor, realw *xstore_other,
                         realw *ystore_other, realw *zstore_other, const int *nspec_other_f);
void get_smooth_gpu_(long *smooth_pointer, realw *data_smooth);

/* FP64 sensitivity kernels (5,5,5,NSPEC) straight from the device accumulators
 * (no reference counterpart: the reference accumulates in single precision). */
int sf3d_get_kernels_f64(long *Mesh_pointer, double *h_rho_kl, double *h_mu_kl, double *h_kappa_kl);

/* ---------------------------------------------------------------------------
 * library entry points (no reference counterpart)
 * ------------------------------------------------------------------------- */

/* Upload a whole-run source time function table (NSOURCES, nstep) in FP64;
 * the device copy is rounded to FP32 like the per-step stf of the reference. */
int sf3d_set_stf_table(long *Mesh_pointer, const double *h_stf, int nsources, int nstep);

/* Replace the sources of a prepared mesh (another shot on the same mesh and
 * model): ispec_selected_source (1-based), sourcearrays in the layout of
 * prepare_constants_device (NSOURCES,3,5,5,5), and the whole-run stf table as
 * sf3d_set_stf_table takes it.  Waits for the compute stream first. */
int sf3d_set_sources(long *Mesh_pointer, int nsources, const int *ispec_selected_source,
                     const realw *sourcearrays, const double *h_stf, int nstep);

/* Run time steps it_begin..it_end (1-based, inclusive) of the forward scheme
 * entirely on the device: fused corrector+predictor, Stacey, sources,
 * stiffness, displacement seismograms (trace slot (it-1) mod nlength_seismogram);
 * with a fluid domain (prepare_fields_acoustic_device) also the fluid step,
 * both coupling terms and the pressure traces, in the order of
 * iterate_time.F90.  Steps are captured in CUDA graphs of
 * steps_per_graph steps (0 = no graphs).  Leaves the fields as the per-call
 * ABI leaves them after the same steps.  On a fluid-solid mesh the solid
 * predictor/corrector passes cover the span of global points of the solid
 * elements and the fluid passes that of the fluid elements (the first call
 * finds the spans): the solid fields at points of fluid elements alone, and the
 * potentials at points of solid elements alone, are not touched (they stay zero
 * from rest; the per-call entry points advance every point, as the reference
 * does).  flags bit 0: record the device time of every stiffness launch (read
 * back with sf3d_last_timing). */
int sf3d_iterate_time(long *Mesh_pointer, int it_begin, int it_end, realw deltat, int steps_per_graph,
                      int flags);

/* Copy the device trace buffer (3, nrec_local, nlength) to the host (pressure
 * runs: pressure in component 0, as compute_seismograms_cuda returns it). */
int sf3d_get_seismograms(long *Mesh_pointer, realw *h_seismograms);

/* One kind of the device seismogram buffers, (NDIM, nrec_local, nlength):
 * kind 0 displacement, 1 velocity, 2 acceleration (the kinds enabled by
 * SAVE_SEISMOGRAMS_* at prepare time), 3 pressure (component 1, the others 0).
 * Receivers in fluid elements hold (1/rho) grad of chi, chi_dot, chi_dot_dot
 * (compute_seismograms.f90:127-144).  Library-only: the Fortran solver gets
 * these arrays from compute_seismograms_cuda. */
int sf3d_get_seismograms_kind(long *Mesh_pointer, int kind, realw *h_seismograms);

/* Device time of the stiffness kernel launches of the last sf3d_iterate_time
 * call with flags bit 0 set, in ms (a pair of CUDA events recorded on the
 * compute stream around each step's stiffness launches), their count, and the
 * event-timed total of the call. */
int sf3d_last_timing(long *Mesh_pointer, float *stiffness_ms, int *stiffness_launches,
                     float *total_ms, int *total_launches);

/* Select the elastic stiffness kernel.  All variants compute the same
 * arithmetic in the same order:
 *   0, 2, 3, 4: one 128-thread CTA per element, compiled for 4, 5, 6, 7
 *               resident CTAs per SM (register budget 128, 96, 80, 72);
 *   1:          persistent CTAs fed by a three-stage bulk-copy (TMA) pipeline;
 *   5, 6, 7:    one CTA per element with the memory variables, strains and
 *               attenuation factors staged in shared memory by cp.async, for
 *               6, 7, 8 CTAs per SM (register budget 80, 72, 64);
 *   8, 9:       one CTA per element, evict-first cache hints on the element
 *               streams (read and written once per launch), 6 and 7 CTAs/SM;
 *   10, 11:     three threads per GLL point (one per displacement component),
 *               384-thread CTAs, 3 and 4 CTAs/SM;
 *   12, 13, 14: one CTA per element with the memory variables, strains and
 *               attenuation factors brought into shared memory by 14 bulk
 *               copies (one thread, one mbarrier with a bounded wait), for 8,
 *               9, 10 CTAs per SM (register budget 64, 56, 48); without
 *               attenuation the plain build at 8, 10, 12 CTAs per SM;
 *   15, 16:     without attenuation or strain storage, FP32 arrays: a thread per
 *               (element, z-line) holding its five points in registers, five
 *               elements per 125-thread CTA, for 8 and 7 CTAs per SM (register
 *               budget 64, 72); every other case runs the default build
 *               (variant 3) under these numbers.
 * Under a packed geometry format (sf3d_set_geometry_format) the variant picks
 * the packed build: 4 at 7 CTAs/SM; 5, 6, 7 with the memory variables and
 * strains staged by cp.async and the factors read from the element record, at
 * 8, 9, 10 CTAs/SM (register budget 64, 56, 48); 12, 13, 14 the same with the
 * memory variables and strains bulk-copied, at 8, 9, 10 CTAs/SM; any other at 6.
 * Default 3; the autotuner picks among all of them (the bulk-copy builds are
 * the fastest on GB300 for the layered viscoelastic workload).
 * No reference counterpart (the reference compiles one Kernel_2 per
 * configuration). */
int sf3d_set_stiffness_variant(long *Mesh_pointer, int variant);

/* Storage of the stiffness kernel's static per-element streams (nine metric
 * rows of irregular elements, kappa, mu and, with attenuation, factor_common
 * and factor_common_kappa of the three solids), in packed form:
 *   0: the FP32 arrays (default);
 *   1: FP16, 2: BF16: a stream constant over an element is stored once, exactly,
 *      in a 160-byte per-element record; a varying stream gets a 125-value row
 *      value = offset + scale * h, offset/scale = (max +- min)/2 over the element,
 *      h in [-1, 1] in FP16 (error <= scale * 2^-11) or BF16 (scale * 2^-8);
 *   3: FP32 rows for the varying streams (lossless).
 * Fields, memory variables and arithmetic stay FP32.  Isotropic meshes only.
 * No reference counterpart (the reference stores CUSTOM_REAL arrays only). */
int sf3d_set_geometry_format(long *Mesh_pointer, int format);

/* 32: format 0; 16: format 1 of sf3d_set_geometry_format. */
int sf3d_set_geometry_precision(long *Mesh_pointer, int bits);

/* Payload rows and device bytes (records + rows) of the packed format in use
 * (0, 0 for the FP32 arrays).  No reference counterpart. */
int sf3d_geometry_pack_info(long *Mesh_pointer, long *payload_rows, long *device_bytes);

/* Time every stiffness variant over `reps` full passes and keep the fastest.
 * Must run on a wavefield at rest (after prepare_fields_elastic_device, before
 * the first step): zero fields make the passes leave every array unchanged;
 * returns SF3D_ERR_STATE otherwise.  ms_per_variant (17 floats) and
 * best_variant may be NULL.  No reference counterpart. */
int sf3d_autotune_stiffness(long *Mesh_pointer, int reps, float *ms_per_variant, int *best_variant);

/* ------------------------------------------------------------------------
 * Inter-slice assembly of accel through the MPI interface buffers
 * (assemble_MPI_vector_cuda.cu; called from
 * compute_forces_viscoelastic_calling_routine.F90:140-160,286-310 and
 * assemble_MPI_vector.f90:790-880).  Buffers are (NDIM, max_nibool_interfaces_ext_mesh,
 * num_interfaces_ext_mesh); the interface lists come from prepare_constants_device. */
/* assemble_MPI_vector_cuda.cu:42 — pack accel (or b_accel) and copy to the host */
void transfer_boun_accel_from_device_(long *Mesh_pointer, realw *send_accel_buffer,
                                      const int *FORWARD_OR_ADJOINT);
/* assemble_MPI_vector_cuda.cu:120 — pack accel and start the copy to pinned memory */
void transfer_boundary_from_device_a_(long *Mesh_pointer, const int *nspec_outer_elastic);
/* assemble_MPI_vector_cuda.cu:449 — wait for that copy, hand the buffer to MPI (iphase 2) */
void sync_copy_from_device_(long *Mesh_pointer, int *iphase, realw *send_buffer);
/* assemble_MPI_vector_cuda.cu:174 — start the upload of the received buffer */
void transfer_boundary_to_device_a_(long *Mesh_pointer, realw *buffer_recv_vector_ext_mesh,
                                    const int *num_interfaces_ext_mesh,
                                    const int *max_nibool_interfaces_ext_mesh);
/* assemble_MPI_vector_cuda.cu:205 — upload the received buffer and add it into accel */
void transfer_asmbl_accel_to_device_(long *Mesh_pointer, realw *buffer_recv_vector_ext_mesh,
                                     const int *num_interfaces_ext_mesh,
                                     const int *max_nibool_interfaces_ext_mesh,
                                     const int *nibool_interfaces_ext_mesh,
                                     const int *ibool_interfaces_ext_mesh, const int *FORWARD_OR_ADJOINT);
/* assemble_MPI_vector_cuda.cu:305 — add the buffer uploaded by transfer_boundary_to_device_a */
void transfer_sync_accel_to_device_(long *Mesh_pointer, realw *buffer_recv_vector_ext_mesh,
                                    const int *num_interfaces_ext_mesh,
                                    const int *max_nibool_interfaces_ext_mesh,
                                    const int *nibool_interfaces_ext_mesh,
                                    const int *ibool_interfaces_ext_mesh, const int *FORWARD_OR_ADJOINT);

/* ------------------------------------------------------------------------
 * Checkpointed discrete-adjoint gradient of a waveform misfit (elastic, no
 * attenuation).  Replaces the reference's SIMULATION_TYPE=3 pairing of an
 * adjoint run with a backward reconstruction (iterate_time.F90:219-330,
 * compute_kernels.f90:67-226) by forward recomputation from HBM checkpoints
 * (the scheme of iterate_time_undoatt.F90:29-632).  The gradient is the exact
 * derivative of the discrete misfit J(seismograms) with respect to rho, kappa
 * and mu at every GLL point, accumulated in FP64.  No reference counterpart
 * as a single call; the kernel formulas are compute_kernels.f90:151-186.
 *
 * Order: sf3d_gradient_setup -> sf3d_gradient_forward (from rest, records the
 * displacement seismograms, which needs nlength_seismogram >= nstep) -> the
 * caller forms dJ/d(seismogram) -> sf3d_gradient_set_residual ->
 * sf3d_gradient_backward -> sf3d_gradient_get.  The backward pass recomputes
 * the forward field, so the forward wavefield arrays hold an intermediate
 * state afterwards. */
/* Allocate checkpoints every checkpoint_every steps plus one segment of
 * recomputed fields; *device_bytes receives the HBM footprint. */
int sf3d_gradient_setup(long *Mesh_pointer, int nstep, int checkpoint_every, double *device_bytes);
/* Forward run of nstep steps from rest with checkpoints (stf from sf3d_set_stf_table). */
int sf3d_gradient_forward(long *Mesh_pointer, realw deltat);
/* dJ/d(seismogram sample), layout (3, nrec_local, nstep) like seismograms_d. */
int sf3d_gradient_set_residual(long *Mesh_pointer, const realw *residual);
/* Reverse sweep: recompute each segment, apply the transposed steps, accumulate. */
int sf3d_gradient_backward(long *Mesh_pointer, realw deltat);
/* 1 (default): the transposed stiffness K p and the gradient terms of an element
 * in one kernel; 0: the stiffness kernel on p, then a separate gradient kernel. */
int sf3d_gradient_set_fused(long *Mesh_pointer, int fused);
/* dJ/drho, dJ/dkappa, dJ/dmu per GLL point, layout (5,5,5,NSPEC); any may be NULL. */
int sf3d_gradient_get(long *Mesh_pointer, double *g_rho, double *g_kappa, double *g_mu);
/* Free the gradient buffers (also freed by prepare_cleanup_device). */
int sf3d_gradient_release(long *Mesh_pointer);

/* Max |x| over the first n values of a device array of floats (NaN if any is
 * NaN), computed on `stream` (NULL: the default stream) without allocating:
 * the reduction's scratch is a fixed 256 KB device array inside the library.
 * No reference counterpart (it is the reduction of sf3d_check_stability /
 * check_stability.f90:408 for callers that must not allocate device memory).
 * Limits and rules:
 *   - 1 <= n <= 536854528 (one partial per 16384 values in the fixed scratch);
 *     larger n returns SF3D_ERR_ARG with a message;
 *   - nothing has to be zeroed beforehand: every scratch slot the call reads
 *     is written earlier in the same call;
 *   - the first call on a device looks up the scratch address
 *     (cudaGetSymbolAddress) with that device current; make that first call
 *     before any stream capture begins;
 *   - calls that overlap in time on one device (other streams or host
 *     threads) share the scratch and race: serialise them;
 *   - a non-null `stream` must belong to the current device (SF3D_ERR_ARG
 *     otherwise); a process that resets the device (cudaDeviceReset) must
 *     not call this entry point afterwards (the cached address is gone);
 *   - returns after the result is on the host (synchronises `stream`). */
int sf3d_field_maxabs_noalloc(const realw *d_field, long n, void *stream, realw *max_abs);

/* Self-check of the bounded mbarrier wait behind every bulk copy of the
 * stiffness, C-PML and adjoint kernels: one CTA waits, with a limit of limit_s
 * seconds (0 < limit_s <= 2), on an mbarrier that expects 16 bytes no copy
 * delivers; *timed_out = 1 when the wait gave up and set the error word the way
 * the kernels do, *waited_s (may be NULL) the time the wait took.  Nothing is
 * in flight and nothing faults; the context stays usable.  No reference
 * counterpart. */
int sf3d_check_bounded_wait(double limit_s, int *timed_out, double *waited_s);

/* ------------------------------------------------------------------------
 * Misfit post-processing on the device (FP64).  No Mesh handle needed. */
/* Adjoint sources of the reference's tools utils/adjoint_sources/
 * {waveform,traveltime,amplitude}/create_adjsrc_*.f90 for all traces at once:
 * kind 0 waveform (cosine-tapered window, adj = (syn - dat) tw), 1 cross-
 * correlation traveltime (adj = -v tw / norm, v the centred time derivative of
 * syn), 2 amplitude (adj = syn tw / norm).  Traces (nrec, 3, nstep) C order
 * (component innermost of the first two, samples contiguous); window from
 * ts, te with samples t0 + (j - 1) dt; component 0 keeps all components, 1-3
 * only that one (ifile of the tools).  h_dat is used by kind 0 only.  norms
 * (nrec, 3) = dt sum(tw signal^2).  Errors: window outside the trace; a
 * waveform window shorter than 20 samples (the tool's taper divides by zero
 * there). */
int sf3d_adjoint_sources(int kind, int nrec, int nstep, double dt, double t0, double ts, double te,
                         int component, const double *h_syn, const double *h_dat, double *h_adj,
                         double *h_norms);
/* Sum of nker event kernels of n values each (src/tomography/sum_kernels.f90:
 * 215-315), each optionally multiplied by its source mask (USE_SOURCE_MASK;
 * h_masks NULL: none), accumulated in FP64 on the device; h_total (n) FP64 and,
 * if not NULL, h_total_f32 (n) rounded to CUSTOM_REAL; h_norms (nker) = sum(k^2)
 * of each event kernel before masking (the tool prints its square root). */
int sf3d_sum_kernels(int nker, long n, const realw *const *h_kernels, const realw *const *h_masks,
                     double *h_total, realw *h_total_f32, double *h_norms);

/* ------------------------------------------------------------------------
 * Many shots on one prepared mesh (elastic, no attenuation).  The reference
 * runs shots as independent simulations (NUMBER_OF_SIMULTANEOUS_RUNS,
 * parallel.f90:2171-2260); here the shots' wavefields are stacked
 * shot-innermost and advance together, one stiffness pass per step reading
 * the mesh once for a tile of shots.  No reference counterpart as calls.
 * Receivers are the mesh's (prepare_constants_device), shared by all shots. */
/* Per-shot sources: ispec_selected_source (nshots, 1-based), sourcearrays in the
 * layout of prepare_constants_device (nshots,3,5,5,5), stf (nshots, nstep) FP64;
 * seismogram buffer of nlength samples; *device_bytes receives the footprint. */
int sf3d_batch_prepare(long *Mesh_pointer, int nshots, const int *ispec_selected_source,
                       const realw *sourcearrays, const double *stf, int nstep, int nlength,
                       double *device_bytes);
/* Tiling of the batched stiffness kernel: shots per CTA (1, 2, 4, 8; divides
 * nshots) x elements per CTA (1, 2, 4) x shots per thread (1, or 4 with 4 or 8
 * shots per CTA: float4 rows and vector atomics); shots_per_thread 0 selects the
 * register-blocked pencil kernel with shots_per_block 8, 16 or 32 shots per CTA
 * (dividing nshots) and elements_per_block 1. */
int sf3d_batch_set_tiling(long *Mesh_pointer, int shots_per_block, int elements_per_block,
                          int shots_per_thread);
/* Time every valid tiling over `reps` stiffness passes on wavefields at rest and
 * keep the fastest; ms_table (27 floats: 0-23 [shots per thread 1,4] x [shots per
 * CTA 1,2,4,8] x [elements 1,2,4], 24-26 the pencil kernel with 8, 16, 32 shots
 * per CTA; -1 where invalid) and the outputs may be NULL.  The pencil kernel is
 * reported as shots_per_thread 0. */
int sf3d_batch_autotune(long *Mesh_pointer, int reps, float *ms_table, int *best_shots_per_block,
                        int *best_elements_per_block, int *best_shots_per_thread);
/* 1: every kernel of a step covers all shots (default); 2: the two halves of the
 * shots advance on two streams, the second half's corrector/predictor running
 * while the first half's stiffness runs and the first half's next one while the
 * second half's stiffness runs (needs the pencil kernel and nshots / 2 divisible
 * by its shots per CTA).  Results do not depend on the choice. */
int sf3d_batch_set_halves(long *Mesh_pointer, int halves);
/* Steps it_begin..it_end of all shots, graph-captured in blocks of steps_per_graph. */
int sf3d_batch_iterate(long *Mesh_pointer, int it_begin, int it_end, realw deltat, int steps_per_graph);
/* Device time (CUDA events on the compute stream) and launches of the last sf3d_batch_iterate. */
int sf3d_batch_timing(long *Mesh_pointer, float *total_ms, int *launches);
/* Displacement seismograms, layout (3, nrec_local, nshots, nlength). */
int sf3d_batch_get_seismograms(long *Mesh_pointer, realw *h_seismograms);
/* Stacked displacement, layout (nshots, 3, NGLOB) Fortran order (shot fastest). */
int sf3d_batch_get_displ(long *Mesh_pointer, realw *h_displ);
/* Free the batch (also freed by prepare_cleanup_device). */
int sf3d_batch_release(long *Mesh_pointer);

/* Host-side checks, norms and memory reports (check_fields_cuda.cu). The *_gpu checks and
 * get_max_accel reduce the device field; the others reduce the host array passed in. */
void check_error_vectors_(int *sizef, realw *vector1, realw *vector2);
void check_max_norm_vector_(int *size, realw *vector1, int *announceID);
void check_max_norm_displ_(int *size, realw *displ, int *announceID);
void check_max_norm_b_displ_(int *size, realw *b_displ, int *announceID);
void check_max_norm_b_accel_(int *size, realw *b_accel, int *announceID);
void check_max_norm_displ_gpu_(int *size, realw *displ, long *Mesh_pointer, int *announceID);
void check_max_norm_b_displ_gpu_(int *size, realw *b_displ, long *Mesh_pointer, int *announceID);
void check_max_norm_b_accel_gpu_(int *size, realw *b_accel, long *Mesh_pointer, int *announceID);
void check_max_norm_b_veloc_gpu_(int *size, realw *b_veloc, long *Mesh_pointer, int *announceID);
void get_max_accel_(int *itf, int *sizef, long *Mesh_pointer);
void get_norm_elastic_from_device_(realw *norm, long *Mesh_pointer, int *type);
void get_norm_acoustic_from_device_(realw *norm, long *Mesh_pointer, int *sim_type);
void get_free_device_memory_(realw *free_mb, realw *used, realw *total);
void output_free_device_memory_(int *myrank);
void make_displ_rand_(long *Mesh_pointer, realw *h_displ);
void pause_for_debug_(void);
void register_host_array_(int *size, realw *h_array);
void unregister_host_array_(realw *h_array);

/* Field transfers (transfer_fields_cuda.cu), host arrays in the reference's layout. */
void transfer_b_accel_from_device_(int *size, realw *b_accel, long *Mesh_pointer);
void transfer_b_accel_to_device_(int *size, realw *b_accel, long *Mesh_pointer);
void transfer_b_veloc_from_device_(int *size, realw *b_veloc, long *Mesh_pointer);
void transfer_b_veloc_to_device_(int *size, realw *b_veloc, long *Mesh_pointer);
void transfer_potential_ac_from_device_(int *size, realw *potential_acoustic, long *Mesh_pointer);
void transfer_dot_dot_from_device_(int *size, realw *potential_dot_dot_acoustic, long *Mesh_pointer);
void transfer_dot_dot_to_device_(int *size, realw *potential_dot_dot_acoustic, long *Mesh_pointer);
void transfer_b_strain_to_device_(long *Mesh_pointer, realw *b_epsilondev_xx, realw *b_epsilondev_yy,
                                  realw *b_epsilondev_xy, realw *b_epsilondev_xz, realw *b_epsilondev_yz,
                                  realw *b_epsilondev_trace, int *size_epsilondev);
void transfer_b_rmemory_to_device_(long *Mesh_pointer, realw *b_R_xx, realw *b_R_yy, realw *b_R_xy,
                                   realw *b_R_xz, realw *b_R_yz, realw *b_R_trace, int *size_R);
void transfer_compute_kernel_answers_from_device_(long *Mesh_pointer, realw *rho_kl, int *size_rho,
                                                  realw *mu_kl, int *size_mu, realw *kappa_kl,
                                                  int *size_kappa);
void transfer_compute_kernel_fields_from_device_(long *Mesh_pointer, realw *accel, int *size_accel,
                                                 realw *b_displ, int *size_b_displ, realw *epsilondev_xx,
                                                 realw *epsilondev_yy, realw *epsilondev_xy,
                                                 realw *epsilondev_xz, realw *epsilondev_yz,
                                                 int *size_epsilondev, realw *b_epsilondev_xx,
                                                 realw *b_epsilondev_yy, realw *b_epsilondev_xy,
                                                 realw *b_epsilondev_xz, realw *b_epsilondev_yz,
                                                 int *size_b_epsilondev, realw *rho_kl, int *size_rho,
                                                 realw *mu_kl, int *size_mu, realw *kappa_kl,
                                                 int *size_kappa, realw *epsilon_trace_over_3,
                                                 realw *b_epsilon_trace_over_3,
                                                 int *size_epsilon_trace_over_3);
void transfer_boun_pot_from_device_(long *Mesh_pointer, realw *send_potential_dot_dot_buffer,
                                    const int *FORWARD_OR_ADJOINT);
void transfer_asmbl_pot_to_device_(long *Mesh_pointer, realw *buffer_recv_scalar_ext_mesh,
                                   const int *FORWARD_OR_ADJOINT);

/* Stacey passes of the undo-attenuation scheme (compute_stacey_viscoelastic_cuda.cu,
 * compute_stacey_acoustic_cuda.cu): the same boundary term without a boundary record. */
void compute_stacey_viscoelastic_undoatt_cuda_(long *Mesh_pointer, int *iphasef, int *FORWARD_OR_ADJOINT_f);
void compute_stacey_acoustic_undoatt_cuda_(long *Mesh_pointer, int *iphasef, int *FORWARD_OR_ADJOINT_f);

/* SIMULATION_TYPE = 3 in fluid elements (prepare_mesh_constants_cuda.cu,
 * compute_add_sources_acoustic_cuda.cu, compute_kernels_cuda.cu, transfer_fields_cuda.cu):
 * backward potentials (FORWARD_OR_ADJOINT = 3 on every acoustic entry point, Stacey
 * record b_absorb_potential(NGLL2, nfaces) stored by SAVE_FORWARD runs and replayed),
 * adjoint sources of receivers in fluid elements, and the rho / kappa kernels
 * rho_ac_kl += dt grad(chi_adj).grad(b_chi), kappa_ac_kl += dt chi_adj b_chi_dd
 * (FP64 accumulators); with APPROXIMATE_HESS_KL, compute_kernels_hess_cuda with
 * ACOUSTIC_SIMULATION also accumulates hess_ac_kl, hess_rho_ac_kl, hess_kappa_ac_kl. */
void transfer_kernels_hess_ac_tohost_(long *Mesh_pointer, realw *h_hess_ac_kl, realw *h_hess_rho_ac_kl,
                                      realw *h_hess_kappa_ac_kl, int *NSPEC_AB);
void add_sources_ac_sim_2_or_3_cuda_(long *Mesh_pointer, realw *h_source_adjoint, int *nrec,
                                     int *nadj_rec_local, int *NTSTEP_BETWEEN_READ_ADJSRC, int *it);
void compute_add_sources_ac_s3_cuda_(long *Mesh_pointer, int *NSOURCESf, double *h_stf_pre_compute,
                                     int *run_number_of_the_source);
void compute_kernels_acoustic_cuda_(long *Mesh_pointer, realw *deltat_f);
void prepare_fields_acoustic_adj_dev_(long *Mesh_pointer, int *APPROXIMATE_HESS_KL);
void transfer_b_dot_dot_from_device_(int *size, realw *b_potential_dot_dot_acoustic, long *Mesh_pointer);
void transfer_b_fields_ac_from_device_(int *size, realw *b_potential_acoustic,
                                       realw *b_potential_dot_acoustic, realw *b_potential_dot_dot_acoustic,
                                       long *Mesh_pointer);
void transfer_b_fields_ac_to_device_(int *size, realw *b_potential_acoustic,
                                     realw *b_potential_dot_acoustic, realw *b_potential_dot_dot_acoustic,
                                     long *Mesh_pointer);
void transfer_b_potential_ac_from_device_(int *size, realw *b_potential_acoustic, long *Mesh_pointer);
void transfer_b_potential_ac_to_device_(int *size, realw *b_potential_acoustic, long *Mesh_pointer);
void transfer_b_potential_dot_dot_ac_from_device_(int *size, realw *b_potential_dot_dot_acoustic,
                                                  long *Mesh_pointer);
void transfer_b_potential_dot_dot_ac_to_device_(int *size, realw *b_potential_dot_dot_acoustic,
                                                long *Mesh_pointer);
void transfer_kernels_ac_to_host_(long *Mesh_pointer, realw *h_rho_ac_kl, realw *h_kappa_ac_kl,
                                  int *NSPEC_AB);
/* Fluid kernel pairing: 0 (default) the reference's chi_adj; 1 chi_adj_dd, whose
 * kernels are the discrete derivative of the misfit (same host scaling). */
int sf3d_set_acoustic_kernel_pairing(long *Mesh_pointer, int discrete);
/* FP64 acoustic accumulators, (5,5,5,NSPEC) each (library extension). */
int sf3d_get_kernels_ac_f64(long *Mesh_pointer, double *h_rho_ac_kl, double *h_kappa_ac_kl);

/* ------------------------------------------------------------------------
 * C-PML absorbing layers of elastic elements (forward runs).
 * prepare_fields_elastic_pml (prepare_mesh_constants_cuda.cu:1176; called from
 * prepare_gpu.f90:191): the CPML element lists (1-based CPML_to_spec /
 * spec_to_CPML, is_CPML per element) and the recursive-convolution coefficients
 * of pml_compute_memory_variables.f90 per CPML element and point
 * (coef_alpha / _beta (9, NGLL3, NSPEC_CPML), coef_abar (5, ...),
 * coef_strain (18, ...)); rhostore and wgll_cube for the PML mass terms.  The
 * CPML elements' stiffness, memory variables and acceleration contribution
 * (pml_compute_accel_contribution.f90, compute_forces_viscoelastic_PML) then
 * run inside compute_forces_viscoelastic_cuda and sf3d_iterate_time, the
 * PML_displ_old/_new stores around the predictor inside
 * update_displacement_cuda.  Rejected with SF3D_ERR_UNSUPPORTED: attenuation,
 * anisotropy, mesh colouring, SIMULATION_TYPE = 3.
 * pml_impose_boundary_condition_elastic_cuda (pml_compute_accel_cuda.cu:245,
 * called from pml_compute_accel_contribution.f90:695): displ, veloc and accel
 * set to zero on the outer faces of the layers (the absorbing face lists of
 * prepare_constants_device).
 * transfer_pml_displ_from_device / _to_device (transfer_fields_cuda.cu:292,307):
 * PML_displ_old / _new (3, NGLL3, NSPEC_CPML). */
void pml_impose_boundary_condition_elastic_cuda_(long *Mesh_pointer);
void prepare_fields_elastic_pml_(long *Mesh_pointer, int *NSPEC_CPML, int *is_CPML, int *CPML_to_spec,
                                 int *spec_to_CPML, realw *pml_convolution_coef_alpha,
                                 realw *pml_convolution_coef_beta, realw *pml_convolution_coef_abar,
                                 realw *pml_convolution_coef_strain, realw *h_wgll_cube, realw *rhostore);
void transfer_pml_displ_from_device_(int *size, realw *PML_displ_old, realw *PML_displ_new,
                                     long *Mesh_pointer);
void transfer_pml_displ_to_device_(int *size, realw *PML_displ_old, realw *PML_displ_new,
                                   long *Mesh_pointer);

/* Not provided: each records SF3D_ERR_UNSUPPORTED through sf3d_last_error (noise
 * tomography, gravity, ocean load, faults);
 * prepare_fields_gravity_device with GRAVITY = 0 and prepare_fault_device without
 * Kelvin-Voigt damping are accepted no-ops. */
void add_source_main_rec_noise_cu_(long *Mesh_pointer, int *it_f, int *irec_main_noise_f,
                                   int *islice_selected_rec);
void compute_coupling_ocean_cuda_(long *Mesh_pointer, int *FORWARD_OR_ADJOINT);
void compute_kernels_strgth_noise_cu_(long *Mesh_pointer, realw *h_noise_surface_movie, realw *deltat);
void fault_solver_gpu_(long *Mesh_pointer, long *Fault_pointer, realw *dt, int *it);
void initialize_fault_data_gpu_(long *Fault_solver, int *fault_index, int *iglob, int *num_of_records,
                                int *ndat, int *NT_RECORD_LENGTH);
void initialize_fault_solver_gpu_(long *Fault_solver, int *num_of_faults, realw *v_healing, realw *v_rupt,
                                  int *RATE_AND_STATE);
void noise_read_add_surface_movie_cu_(long *Mesh_pointer, realw *h_noise_surface_movie,
                                      int *NOISE_TOMOGRAPHYf);
void prepare_fault_device_(long *Mesh_pointer, int *KELVIN_VOIGT_DAMPING, realw *Kelvin_Voigt_eta);
void prepare_fields_gravity_device_(long *Mesh_pointer, int *GRAVITY, realw *minus_deriv_gravity,
                                    realw *minus_g, realw *h_wgll_cube, realw *rhostore);
void prepare_fields_noise_device_(long *Mesh_pointer, int *NSPEC_AB, int *NGLOB_AB, int *free_surface_ispec,
                                  int *free_surface_ijk, int *num_free_surface_faces, int *NOISE_TOMOGRAPHY,
                                  int *NSTEP, realw *noise_sourcearray, realw *normal_x_noise,
                                  realw *normal_y_noise, realw *normal_z_noise, realw *mask_noise,
                                  realw *free_surface_jacobian2Dw);
void transfer_datat_to_host_(long *Fault_pointer, int *fault_index, realw *h_dataT, int *it_in);
void transfer_fault_data_to_device_(long *Fault_pointer, int *fault_index, int *NSPEC_FLT, int *NGLOB_FLT,
                                    realw *D, realw *T0, realw *T, realw *B, realw *R, realw *V0, realw *Z,
                                    realw *invM1, realw *invM2, int *ibulk1, int *ibulk2,
                                    int *allow_opening);
void transfer_fault_data_to_host_(long *Fault_pointer, int *fault_index, int *NSPEC_FLT, int *NGLOB_FLT,
                                  realw *D, realw *V, realw *T);
void transfer_kernels_noise_to_host_(long *Mesh_pointer, realw *h_sigma_kl, int *NSPEC_AB);
void transfer_rsf_data_todevice_(long *Fault_pointer, int *fault_index, int *NGLOB_FLT, realw *Fload,
                                 realw *V0, realw *f0, realw *V_init, realw *a, realw *b, realw *L,
                                 realw *theta, realw *T, realw *C, realw *fw, realw *Vw, int *StateLaw);
void transfer_rsf_data_tohost_(long *Fault_pointer, int *fault_index, int *NGLOB_FLT, realw *V0, realw *f0,
                               realw *V_init, realw *a, realw *b, realw *L, realw *theta, realw *T,
                               realw *C, realw *fw, realw *Vw);
void transfer_sigma_from_device_(int *size, realw *sigma_kl, long *Mesh_pointer);
void transfer_surface_to_host_(long *Mesh_pointer, realw *h_noise_surface_movie);
void transfer_swf_data_todevice_(long *Fault_pointer, int *fault_index, int *NGLOB_FLT, realw *Dc,
                                 realw *mus, realw *mud, realw *T, realw *C, realw *theta);
void transfer_swf_data_tohost_(long *Fault_pointer, int *fault_index, int *NGLOB_FLT, realw *Dc, realw *mus,
                               realw *mud, realw *T, realw *C, realw *theta);

/* Synchronise the compute stream and report the first stored status. */
int sf3d_synchronize(long *Mesh_pointer);

/* Raw device pointer of a named field ("displ", "veloc", "accel", ...) for
 * in-HBM benchmarking and zero-copy interop; NULL if unknown. */
void *sf3d_device_ptr(long *Mesh_pointer, const char *name);

/* Stability check (check_stability.f90:408): max |displ| over the device field;
 * returns SF3D_ERR_UNSTABLE if NaN/Inf or above threshold. */
int sf3d_check_stability(long *Mesh_pointer, realw threshold, realw *max_norm);

#ifdef __cplusplus
}
#endif
#endif
