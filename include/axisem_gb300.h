/*
 * axisem_gb300.h -- C-ABI of the GB300 (sm_103a) AxiSEM solver time loop.
 *
 * The library replaces the body of the reference's `time_loop`
 * (SOLVER/time_evol_wave.F90:231-245, Newmark path `sf_time_loop_newmark`
 * SOLVER/time_evol_wave.F90:264-502) and, for the stiffness/assembly
 * micro-benchmark, the pair `glob_stiffness_{mono,di,quad}_4` +
 * `pdistsum_solid` (SOLVER/stiffness_*.f90, SOLVER/commun.F90:69-171).
 *
 * Everything the Fortran host computes before the loop (mesh database,
 * precomputed metric terms, source, receivers, attenuation constants) is
 * handed over through `axg_mesh_desc` as plain pointers to the module
 * arrays, in the reference's own Fortran column-major layouts and
 * `realkind = 4` (float) precision.  The library copies what it needs to
 * HBM in `axg_create`; the caller keeps ownership of every host array.
 *
 * All entry points return an `int` status (AXG_OK == 0); none of them
 * calls exit()/abort().  A handle is single-caller: calls on one handle
 * must not overlap.  Every function is `extern "C"`, takes plain pointers
 * and sizes, and can be bound from Fortran with `bind(c)` interfaces: the
 * descriptor is a `bind(c)` derived type holding `c_loc` of the module
 * arrays, and the calls are `bind(c, name='axg_...')` interfaces, as the
 * reference binds its NetCDF helpers (SOLVER/nc_routines.F90:291-300).
 */
#ifndef AXISEM_GB300_H
#define AXISEM_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define AXG_ABI_VERSION 3
#define AXG_NPOL 4   /* only npol = 4 (5x5 GLL points) is supported, as the *_4 kernels */

/* ---- status codes ---------------------------------------------------- */
enum axg_status {
  AXG_OK = 0,
  AXG_ERR_BAD_DESC = 1,      /* inconsistent sizes, null required array, bad index */
  AXG_ERR_OOM = 2,           /* device allocation failed */
  AXG_ERR_CUDA = 3,          /* any other CUDA runtime error */
  AXG_ERR_BLOWUP = 4,        /* |disp(1,1,:,:)| > 10 |magnitude| (runtime_info) */
  AXG_ERR_TIMEOUT = 5,       /* a bounded device wait ran out */
  AXG_ERR_NO_DEVICE = 6,     /* no CUDA device / extension cannot run here */
  AXG_ERR_BAD_ARG = 7,       /* bad argument to a call other than axg_create */
  AXG_ERR_UNSUPPORTED = 8    /* valid input the library does not implement */
};

/* src_type(1) of the reference (SOLVER/data_source.f90; mapping in
 * SOLVER/source.f90:63-80). */
enum axg_pole { AXG_MONOPOLE = 0, AXG_DIPOLE = 1, AXG_QUADPOLE = 2 };

/* Solid metric arrays of module data_matr (SOLVER/data_matr.f90:45-76),
 * each real(0:4,0:4,nel_solid).  Which ones a pole type reads:
 *   monopole  : M_1..M_4, M_w1, M11s M21s M41s M12s M22s M32s M42s M11z M21z M41z (15)
 *   dipole    : + M_5..M_8, M_w2, M_w3, M13s, M33s, M43s                         (24)
 *   quadrupole: + M_5..M_8, M_w2..M_w5, M1phi, M2phi, M4phi                      (26)
 * Arrays a pole does not read may be NULL. */
enum axg_solid_term {
  AXG_M_1 = 0, AXG_M_2, AXG_M_3, AXG_M_4, AXG_M_5, AXG_M_6, AXG_M_7, AXG_M_8,
  AXG_M_W1, AXG_M_W2, AXG_M_W3, AXG_M_W4, AXG_M_W5,
  AXG_M11S, AXG_M21S, AXG_M41S, AXG_M12S, AXG_M22S, AXG_M32S, AXG_M42S,
  AXG_M11Z, AXG_M21Z, AXG_M41Z,
  AXG_M13S, AXG_M33S, AXG_M43S,
  AXG_M1PHI, AXG_M2PHI, AXG_M4PHI,
  AXG_N_SOLID_TERMS
};

/* Axial vectors M0_w1..M0_w10, each real(0:4,nel_solid) (SOLVER/data_matr.f90:78-83).
 * monopole reads w1..w3, dipole w1..w4,w6..w10, quadrupole w1..w6. */
enum axg_axial_term {
  AXG_M0_W1 = 0, AXG_M0_W2, AXG_M0_W3, AXG_M0_W4, AXG_M0_W5,
  AXG_M0_W6, AXG_M0_W7, AXG_M0_W8, AXG_M0_W9, AXG_M0_W10,
  AXG_N_AXIAL_TERMS
};

/* Fluid metric arrays (SOLVER/data_matr.f90:86-89), real(0:4,0:4,nel_fluid);
 * M_w_fl only for dipole/quadrupole. */
enum axg_fluid_term { AXG_M1CHI = 0, AXG_M2CHI, AXG_M4CHI, AXG_M_W_FL, AXG_N_FLUID_TERMS };

/* Everything the time loop reads.  Field names are the reference's; all
 * element/point indices are the reference's 1-based values. */
typedef struct axg_mesh_desc {
  int32_t abi_version;       /* = AXG_ABI_VERSION */
  int32_t npol;              /* = 4 */
  int32_t src_type;          /* enum axg_pole: src_type(1) */
  int32_t fluid_src;         /* source sits in the fluid (add_source_fl) */

  int32_t nel_solid, nel_fluid;
  int32_t nglob_solid, nglob_fluid;
  int32_t naxel_solid, naxel_fluid;
  int32_t nel_bdry;
  int32_t nelsrc;            /* <= 8 */

  int32_t niter;             /* length of stf */
  int32_t seis_it;           /* receiver sampling every seis_it steps */
  int32_t num_rec;
  int32_t have_absorbing_bc;

  double deltat;             /* data_time: deltat (FP64) */
  double magnitude;          /* blow-up threshold = 10*|magnitude| */

  /* numbering (SOLVER/data_mesh.f90:57-58): igloc(25*nel), walk ipol fastest */
  const int32_t *igloc_solid, *igloc_fluid;
  const int32_t *ax_el_solid, *ax_el_fluid;      /* (naxel_*) element numbers */

  /* spectral matrices (SOLVER/data_spec.f90) */
  const float *G0;                               /* (0:4) */
  const float *G1, *G1T, *G2, *G2T;              /* (0:4,0:4) */

  const float *m_solid[AXG_N_SOLID_TERMS];
  const float *m0_solid[AXG_N_AXIAL_TERMS];
  const float *m_fluid[AXG_N_FLUID_TERMS];
  const float *m0_w_fl;                          /* (0:4,nel_fluid), non-monopole */

  const float *inv_mass_rho;                     /* (0:4,0:4,nel_solid) */
  const float *inv_mass_fluid;                   /* (0:4,0:4,nel_fluid) */
  const float *fluid_free_surface_mask;          /* (0:4,0:4,nel_fluid) or NULL (= 1) */
  const float *solid_absorbing_gamma;            /* (0:4,0:4,nel_solid), if have_absorbing_bc */
  const float *fluid_absorbing_gamma;            /* (0:4,0:4,nel_fluid), if have_absorbing_bc */

  /* solid-fluid boundary (SOLVER/data_mesh.f90:106-110, data_matr bdry_matr) */
  const float *bdry_matr;                        /* (0:4,nel_bdry,2) */
  const int32_t *bdry_solid_el, *bdry_fluid_el;  /* (nel_bdry) */
  const int32_t *bdry_jpol_solid, *bdry_jpol_fluid;

  /* source (SOLVER/data_source.f90): ielsrc(8), source_term_el(0:4,0:4,8,3)
   * or source_term_fl(0:4,0:4,8), stf(niter) */
  const int32_t *ielsrc;
  const float *source_term_el;
  const float *source_term_fl;
  const float *stf;

  /* receivers: recfile_el(num_rec,3) = (element, ipol, jpol), column-major */
  const int32_t *recfile_el;

  /* coarse-grained (cg4) attenuation (SOLVER/attenuation.f90:81-202) */
  int32_t anel_true;
  int32_t n_sls;                                 /* n_sls_attenuation, 1..8 */
  int32_t do_corr_lowq;
  int32_t att_coarse_grained;                    /* 1: cg4 (below); 0: every GLL point (end of the struct) */
  const double *y_j_attenuation;                 /* (n_sls) */
  const double *exp_w_j_deltat;                  /* (n_sls) */
  const double *ts_fac_t, *ts_fac_tm1;           /* (n_sls) */
  const float *Q_mu, *Q_kappa;                   /* (nel_solid) */
  const float *delta_mu_cg4, *delta_kappa_cg4;   /* (1:4,nel_solid) */
  const float *Y_cg4, *V_s_eta_cg4, *V_s_xi_cg4, *V_z_eta_cg4, *V_z_xi_cg4;  /* (1:4,nel_solid) */
  const float *DsDeta_over_J_sol_cg4, *DzDeta_over_J_sol_cg4;
  const float *DsDxi_over_J_sol_cg4, *DzDxi_over_J_sol_cg4;                  /* (1:4,nel_solid) */
  const float *inv_s_solid;                      /* (0:4,0:4,nel_solid) */

  /* FP64 copies (optional; NULL: none) of the terms the compensated mode
   * (axg_set_compensated) applies in FP64: the assembled inverse masses and
   * the solid source term as the precompute forms them before the cast to
   * realkind (SOLVER/def_precomp_terms.f90:735-800 without the FP32
   * assembly, SOLVER/source.f90:985-1226).  No counterpart in the reference,
   * which stores them in realkind. */
  const double *inv_mass_rho_dp;                 /* (0:4,0:4,nel_solid) */
  const double *inv_mass_fluid_dp;               /* (0:4,0:4,nel_fluid) */
  const double *source_term_el_dp;               /* (0:4,0:4,8,3) */

  /* attenuation at every GLL point, when att_coarse_grained = 0
   * (time_step_memvars_4, glob_anel_stiffness_{mono,di,quad}_4,
   * SOLVER/attenuation.f90:210-334, 542-606); NULL otherwise.  Q_mu,
   * Q_kappa and inv_s_solid are the fields above; the strain takes the
   * data_pointwise mapping terms. */
  const float *delta_mu, *delta_kappa;           /* (0:4,0:4,nel_solid) */
  const float *Y, *V_s_eta, *V_s_xi, *V_z_eta, *V_z_xi;        /* (0:4,0:4,nel_solid) */
  const float *Y0, *V0_s_eta, *V0_s_xi, *V0_z_eta, *V0_z_xi;   /* (0:4,nel_solid) */
  const float *DsDeta_over_J_sol, *DzDeta_over_J_sol;
  const float *DsDxi_over_J_sol, *DzDxi_over_J_sol;            /* (0:4,0:4,nel_solid) */
} axg_mesh_desc;

typedef struct axg_handle axg_handle;

/* State arrays for axg_get_state / axg_set_state, returned in the reference's
 * element-local layouts disp(0:4,0:4,nel_solid,3), chi(0:4,0:4,nel_fluid),
 * memory_var_cg4(1:4,6,n_sls,nel_solid), and the attenuation source terms of
 * the previous step src_tr_tm1_glob_cg4(1:4,nel_solid),
 * src_dev_tm1_glob_cg4(1:4,6,nel_solid) (SOLVER/attenuation.f90:153-154,
 * 196-197).  The three attenuation fields need a handle created with
 * anel_true. */
enum axg_field {
  AXG_FIELD_DISP = 0, AXG_FIELD_VELO, AXG_FIELD_ACC0,
  AXG_FIELD_CHI, AXG_FIELD_DCHI, AXG_FIELD_DDCHI0,
  AXG_FIELD_MEMVAR, AXG_FIELD_ATT_SRC_TR, AXG_FIELD_ATT_SRC_DEV,
  /* compensated mode (axg_set_compensated): the running compensation terms
   * of disp, velo (solid layout) and chi, dchi (fluid layout) */
  AXG_FIELD_DISP_COMP, AXG_FIELD_VELO_COMP, AXG_FIELD_CHI_COMP, AXG_FIELD_DCHI_COMP
};

/* Library build/version string; never NULL. */
const char *axg_version(void);

/* Number of CUDA devices visible (0 when none); never fails. */
int axg_device_count(void);

/* Copies the mesh, metric terms, source and receiver tables to HBM and builds
 * the element patches, the patch colouring and the point renumbering.
 * Replaces the data hand-over before SOLVER/time_evol_wave.F90:264 (the
 * Fortran module arrays of data_matr / data_mesh / data_source).
 * `*out` is set to a handle (or NULL on failure, with the reason in
 * axg_last_error(NULL)). */
int axg_create(const axg_mesh_desc *desc, axg_handle **out);

/* Zeroes the wavefields, memory variables and seismogram buffer and records
 * the iter-0 seismogram sample (SOLVER/time_evol_wave.F90:310-344). */
int axg_reset(axg_handle *h);

/* Advances n_iter Newmark steps, iterations first_iter .. first_iter+n_iter-1
 * (1-based, as `iter` in SOLVER/time_evol_wave.F90:353), using stf(iter).
 * Steps are launched in CUDA graphs of `steps_per_graph` (axg_set_tuning).
 * Returns AXG_ERR_BLOWUP when the blow-up guard of runtime_info
 * (SOLVER/time_evol_wave.F90:1042) fired; the flag is polled once per graph. */
int axg_run(axg_handle *h, int32_t first_iter, int32_t n_iter);

/* Seismograms so far, in the NetCDF layout recdumpvar(nseismo,3,num_rec)
 * (SOLVER/nc_routines.F90:531-538), column-major; `nseismo_cap` is the first
 * extent of `out`; components as nc_compute_recfile_seis_bare
 * (SOLVER/seismograms.f90:783-820).  *nseismo_out = samples written. */
int axg_get_receivers(axg_handle *h, float *out, int32_t nseismo_cap, int32_t *nseismo_out);

/* Copies a state field to the host in the reference's element-local layout. */
int axg_get_state(axg_handle *h, int32_t field, float *out);

/* Sets a state field from the reference's element-local layout (the value of
 * each global point is taken from its first element-local copy). */
int axg_set_state(axg_handle *h, int32_t field, const float *in);

/* Stiffness + assembly, the config-2 micro-benchmark operation:
 * u is gvec-layout displacement (nglob_solid,3) column-major in the
 * reference's global numbering (igloc), f receives the assembled
 *   f = pdistsum_solid( axis_mask( glob_stiffness_<pole>(u) ) )
 * in the same layout (SOLVER/stiffness_*_4, SOLVER/apply_masks.f90,
 * SOLVER/commun.F90:69-171).  Host pointers; copies are included. */
int axg_stiffness_assembled(axg_handle *h, const float *u_gvec, float *f_gvec);

/* The same operation on device-resident buffers of the handle: reads the
 * handle's displacement field and writes the handle's force buffer; used to
 * time the kernels alone.  `stream` may be NULL (the handle's stream). */
int axg_stiffness_assembled_device(axg_handle *h, void *stream);

/* Stiffness + assembly (the same operation and result as
 * axg_stiffness_assembled, from the same descriptor and host buffers) for
 * callers that cannot allocate device memory, e.g. code running where
 * cudaMalloc is unavailable or forbidden.  This entry point has no
 * counterpart in the reference.  It makes no cudaMalloc/cudaFree call and
 * uses no allocating library routine: all device data (plan, element blocks,
 * u, f) lives in one 32 MiB static device array that every GPU loading the
 * library holds until exit, which limits the mesh to roughly 11 000
 * quadrupole elements (larger meshes return AXG_ERR_BAD_ARG naming the size
 * needed).  Of the descriptor it reads only what a stiffness + assembly
 * needs: abi_version, npol, src_type, nel_solid, nglob_solid, igloc_solid,
 * G0, G1, G2, the pole's solid metric arrays, naxel_solid, ax_el_solid and
 * the pole's axial vectors.  The first call on a device (and the first after
 * the device's context was replaced, e.g. by cudaDeviceReset) looks up the
 * array's device address and sets kernel attributes; make that first call
 * before any stream capture.  All calls share the array, which keeps the
 * last call's contents (the force region is cleared on every call): calls
 * that overlap on the GPU race (host threads are serialised).  Uses the
 * legacy default stream; host memory is used for planning. */
int axg_stiffness_assembled_noalloc(const axg_mesh_desc *desc, const float *u_gvec, float *f_gvec);

/* Uploads a gvec-layout displacement (nglob_solid,3) into the handle's
 * displacement field / downloads the handle's force buffer as gvec layout. */
int axg_upload_gvec_disp(axg_handle *h, const float *u_gvec);
int axg_download_gvec_force(axg_handle *h, float *f_gvec);

/* Tuning knobs after creation: steps per CUDA graph (0 = keep).  The patch
 * shape is fixed at creation (axg_create_tuned); patch_elems must be 0 or the
 * handle's value. */
int axg_set_tuning(axg_handle *h, int32_t patch_elems, int32_t steps_per_graph);

/* Measured choice of the steps per CUDA graph: the handle's step (its scheme
 * and modes as set) is timed with CUDA events in graphs of 2, 4, ..., 64
 * steps (those that fit in niter), from a saved copy of the solve's state
 * that is restored afterwards, so the solve continues as if untouched.  The
 * fastest becomes the handle's steps_per_graph (*chosen).  Together with the
 * planner's tuner of the patch shape (axg_create), this is the autotuner of
 * the launch shapes. */
int axg_autotune(axg_handle *h, int32_t *chosen);

/* A further solve on the mesh of an existing handle (serving: meshes stay
 * resident, solves come and go).  `desc` must describe the same mesh -- sizes,
 * pole type, global numbering, axial elements, attenuation layout are
 * checked; metric terms, masses and boundary terms are taken from `mesh_of`
 * -- while its source, stf, receivers, niter, seis_it, deltat and magnitude
 * are this solve's.  Element blocks, plans, masses, coupling tables and
 * attenuation constants stay shared (freed with the last handle of the
 * mesh); the new handle has its own wavefields, stream and CUDA graph.
 * No counterpart in the reference. */
int axg_create_sharing(axg_handle *mesh_of, const axg_mesh_desc *desc, axg_handle **out);

/* axg_run without waiting: the steps are queued on the handle's stream (so
 * the solves of several handles run concurrently); axg_poll sets *done
 * once they finished, axg_wait blocks until then.  Both then report a
 * blow-up or a bounded-wait timeout as axg_run does. */
int axg_run_async(axg_handle *h, int32_t first_iter, int32_t n_iter);
int axg_poll(axg_handle *h, int32_t *done);
int axg_wait(axg_handle *h);

/* Batches: several solves advanced together, on the same or on different
 * meshes (uneven element counts).  A batch step makes one launch per colour
 * and kernel class for all its solves -- the kernels take a work list of
 * (solve, patch) items -- and is captured once in a CUDA graph that every
 * step replays.  Solves of a batch may differ in pole, precision mode
 * (plain or compensated), attenuation (cg4) and time scheme: a symplectic
 * solve's stages run as phases of the batch step (stage i of every solve
 * with more than i stages in one launch per colour and kernel class).  They
 * share the GLL derivative matrices; solves that dump wavefields or
 * checkpoint seismograms run alone.  Each solve's results are bit-for-bit
 * those it gets alone.  The handles must stay open while the batch exists
 * and are neither run nor reconfigured (time scheme, precision mode) by
 * other calls meanwhile; their later calls are ordered after the batch's
 * work.  No counterpart in the reference. */
typedef struct axg_batch axg_batch;
int axg_batch_create(axg_handle *const *hs, int32_t n, axg_batch **out);
/* Queue n_iter steps of every solve, solve k from iteration first_iters[k]
 * (each within 1..niter of its solve); returns at once. */
int axg_batch_run_async(axg_batch *b, const int32_t *first_iters, int32_t n_iter);
/* *done = 1 once the queued steps finished; then (and in axg_batch_wait)
 * a blow-up or timeout of any solve is reported as axg_run reports it. */
int axg_batch_poll(axg_batch *b, int32_t *done);
int axg_batch_wait(axg_batch *b);
/* kernel launches of one batch step */
int axg_batch_launches_per_step(axg_batch *b, int64_t *n);
void axg_batch_destroy(axg_batch *b);
const char *axg_batch_last_error(axg_batch *b);

/* Time schemes of the reference (time_scheme in inparam_advanced,
 * SOLVER/time_evol_wave.F90:231-245, 516-967). */
enum axg_scheme {
  AXG_SCHEME_NEWMARK2 = 0,  /* the default */
  AXG_SCHEME_SYMPLEC4,      /* 4th order PEFRL, 4 stages */
  AXG_SCHEME_ML_SO4M5,      /* 4th order McLachlan, 5 stages */
  AXG_SCHEME_ML_SO6M7,      /* 6th order McLachlan, 7 stages */
  AXG_SCHEME_KL_O8M17,      /* 8th order Kahan-Li, 17 stages */
  AXG_SCHEME_SS_35O10       /* 10th order Sofroniou-Spaletta, 35 stages */
};

/* The drift / kick coefficients of a symplectic scheme times deltat, as
 * symplectic_coefficients computes them: coefd[0..nstages], coefv[0..nstages-1]
 * and the stage times coeff[i] = sum(coefd[0..i]) (host only; arrays of at
 * least 36 entries).  A caller evaluates its source time function at
 * t_(iter-1) + coeff[i] for axg_set_time_scheme. */
int axg_symplectic_coefficients(int32_t scheme, double deltat, double *coefd, double *coefv, double *coeff,
                                int32_t *nstages);

/* Selects the time scheme of the handle's time loop.  For a symplectic
 * scheme, stf_stages(niter, nstages) (column-major) holds the source time
 * function at the stage times of every step (compute_stf_t at
 * t - deltat + coeff(i)); the Newmark scheme ignores it.  The symplectic
 * schemes follow symplectic_time_loop, with attenuation (anelastic stiffness
 * in every stage, memory variables once per step after the final drift) and
 * the compensated mode; a fluid source and a fluid free surface, which the
 * reference's symplectic loop does not apply, are refused
 * (AXG_ERR_UNSUPPORTED).  Resets the state. */
int axg_set_time_scheme(axg_handle *h, int32_t scheme, const float *stf_stages);

/* Compensated time integration on (1) or off (0): the predictor
 * disp += dt velo + dt^2/2 acc0 and the corrector velo += dt/2 (acc0 + acc1)
 * (and chi, dchi in the fluid) -- or a symplectic scheme's drifts
 * disp += coefd velo and kicks velo += coefv acc -- use Kahan's compensated summation in FP32, with
 * a running compensation per point kept in HBM, so that rounding does not
 * accumulate over 1e4-1e5 steps.  When the descriptor carried the FP64
 * inverse masses and source term, the compensated mode also multiplies by
 * the inverse mass and subtracts the source in FP64 (one rounding to FP32
 * each).  Stiffness, coupling and attenuation are unchanged.  The first call
 * allocates the compensation (zero; axg_reset zeroes it too).  No
 * counterpart in the reference. */
int axg_set_compensated(axg_handle *h, int32_t on);

/* axg_create with the patch shape chosen by the caller: patch_elems 1..64
 * elements per patch and growth 0 (compact: most shared points first) or 1
 * (layered: breadth-first layers, square patches on structured blocks).
 * 0 / -1 leave the choice to the planner's tuner, which axg_create always
 * uses: it compares patch sizes {32,40,48,56,64} x both growths on the first
 * 65 536 elements of each domain by a model of the kernels' warp iterations
 * (patch overhead, conflict-free sub-rounds of 8 warps, patch points).
 * This entry point has no counterpart in the reference. */
int axg_create_tuned(const axg_mesh_desc *desc, int32_t patch_elems, int32_t growth, axg_handle **out);

/* Introspection for tests and the benchmark. */
typedef struct axg_info {
  int64_t n_patches_solid, n_patches_fluid;
  int32_t n_colours_solid, n_colours_fluid;
  int32_t max_subrounds_solid, max_subrounds_fluid;
  int64_t device_bytes;               /* bytes the handle holds in HBM */
  int64_t kernels_per_step;           /* kernel launches in one Newmark step */
  int64_t kernels_per_force;          /* kernel launches in one stiffness+assembly */
  int64_t patch_points_solid;         /* sum over patches of their point counts */
  int32_t patch_elems_solid, growth_solid;  /* patch shape the planner used */
  int32_t patch_elems_fluid, growth_fluid;
  int32_t ctas_per_sm_force, ctas_per_sm_step;  /* resident solid-kernel CTAs per SM */
  int64_t mesh_bytes;                 /* part of device_bytes shared by the handles of one mesh */
  int32_t steps_per_graph;            /* steps per CUDA graph (axg_set_tuning / axg_autotune) */
} axg_info;
int axg_get_info(axg_handle *h, axg_info *info);

/* Per-element patch colour of the solid elements (1-based reference order);
 * for validation of the atomic-free colouring. */
int axg_get_solid_colouring(axg_handle *h, int32_t *patch_of_elem, int32_t *colour_of_patch,
                            int64_t n_patch_cap);

/* Plans (patch_elems 0 / growth -1 = tuned, as axg_create) the patch
 * colouring of the solid (and fluid) domain on the host only
 * -- no GPU is touched -- and checks every invariant the kernels rely on:
 * each element in one patch, no two patches of one colour sharing a global
 * point, no two elements of one sub-round sharing a point, exactly one first
 * and one last writer per point.  `info` receives the plan sizes
 * (device_bytes = 0).  Returns AXG_ERR_BAD_DESC with the violated invariant. */
int axg_plan_check(const axg_mesh_desc *desc, int32_t patch_elems, int32_t growth, axg_info *info);
/* The same, tuned as axg_create tunes on a device with `ctas` resident CTAs
 * of the solid kernel (two per SM): a mesh of fewer than two rounds of
 * 64-element patches per colour gets the patch size (8 to 64 elements) of
 * least modelled colour latency.  ctas = 0 (axg_plan_check) assumes launches
 * the mesh fills. */
int axg_plan_check_ctas(const axg_mesh_desc *desc, int32_t patch_elems, int32_t growth, int32_t ctas,
                        axg_info *info);

/* Kernel wavefield dumps (dump_wavefields / dump_type of inparam_advanced;
 * dump_stuff, SOLVER/time_evol_wave.F90:1201-1249).  After every step with
 * mod(iter, strain_it) == 0 the fields of `dump_type` are computed on the GPU
 * from the state at the end of the step and copied into snapshot
 * iter / strain_it - 1 of `out`, while the following steps run.  A snapshot
 * holds the solid fields, then the fluid fields (none without a fluid); each
 * field covers the points (ibeg:iend, jbeg:jend) of every element in the
 * reference's element order, i.e. pack(f(ibeg:iend, jbeg:jend, :)) as
 * nc_dump_field_solid/fluid receive it (SOLVER/wavefields_io.f90:787-836).
 * axg_wavefield_dump_layout names the fields with the reference's variable
 * names.  Fields per type (p components and the last two strain terms only for
 * the dipole and quadrupole):
 *   DISPL_ONLY   dump_disp_global:  disp_sol_s, _p, _z (dipole in s, phi);
 *                                   disp_flu_s, _p (zero), _z = grad(chi) / rho
 *   STRAIN_ONLY  compute_strain:    strain_dsus, strain_dsuz, strain_dpup,
 *                                   straintrace, strain_dsup, strain_dzup (_sol, _flu)
 *   DISPL_VELO   dump_disp + dump_velo_dchi: disp_sol_s, _p, _z and velo_sol_s,
 *                                   _p, _z as stored; chi_flu, dchi_flu
 *   FULLFIELDS   compute_strain + dump_velo_global: the strain terms, then
 *                                   velo_sol_s, _p, _z; velo_flu_s, _p (zero), _z
 * The values of compute_strain's fields are the reference's; with kwf_mask
 * and mapping_ijel_ikwf the fields come in the kernel wavefield point layout
 * of its NetCDF 'displ_only' / 'strain_only' output (kwf_mapping_*) instead
 * of the packed one.  `out` should be page-locked host
 * memory (cudaHostAlloc / cudaHostRegister) for the copies to overlap the
 * steps.  A dumping solve runs alone (not in a batch). */
enum axg_dump_type {
  AXG_DUMP_NONE = 0,
  AXG_DUMP_DISPL_ONLY,
  AXG_DUMP_STRAIN_ONLY,
  AXG_DUMP_DISPL_VELO,
  AXG_DUMP_FULLFIELDS
};

typedef struct axg_dump_desc {
  int32_t dump_type;                 /* AXG_DUMP_*; AXG_DUMP_NONE switches the dumps off */
  int32_t strain_it;                 /* dump interval in steps (>= 1) */
  int32_t ibeg, iend, jbeg, jend;    /* points of each element, 0 <= beg <= end <= 4 */
  /* data_pointwise, (0:4,0:4,nel) column-major; the fluid ones only with a fluid */
  const float *DsDeta_over_J_sol, *DzDeta_over_J_sol, *DsDxi_over_J_sol, *DzDxi_over_J_sol;
  const float *inv_s_solid;
  const float *DsDeta_over_J_flu, *DzDeta_over_J_flu, *DsDxi_over_J_flu, *DzDxi_over_J_flu;
  const float *inv_s_fluid, *inv_rho_fluid;
  float *out;                        /* capacity snapshots of floats_per_snapshot floats */
  int64_t capacity;
  /* Optional (NULL: the packed layout above): the kernel wavefield point
   * layout of the NetCDF 'displ_only' / 'strain_only' output
   * (kwf_mapping_sol / kwf_mapping_flu, SOLVER/wavefields_io.f90:743-780,
   * built in SOLVER/meshes_io.F90:543-630).  Both are (0:4,0:4,nel_solid +
   * nel_fluid), the fluid's elements after the solid's; kwf_mask nonzero marks
   * the one element point that writes each output point, mapping_ijel_ikwf
   * its 1-based position (fluid positions after npoint_solid_kwf).  Each field
   * then holds npoint_solid_kwf (solid) or npoint_fluid_kwf (fluid) values. */
  const int32_t *kwf_mask;
  const int32_t *mapping_ijel_ikwf;
  int32_t npoint_solid_kwf, npoint_fluid_kwf;
  /* src_dump_type = 'mask' (the reference's default, SOLVER/parameters.F90:
   * 399): 1 zeroes every solid field on the points of the source elements
   * ielsrc (eradicate_src_elem_values / _vec_values,
   * SOLVER/wavefields_io.f90:1123-1153); 0 dumps them as computed. */
  int32_t src_dump_mask;
} axg_dump_desc;

int axg_set_wavefield_dump(axg_handle *h, const axg_dump_desc *dd);
/* Fields per snapshot and their names, comma-separated into `names` (NUL
 * terminated, truncated to names_cap bytes; names may be NULL). */
int axg_wavefield_dump_layout(axg_handle *h, int32_t *n_solid_fields, int32_t *n_fluid_fields,
                              int64_t *floats_per_snapshot, char *names, int32_t names_cap);

/* Seismogram checkpoints (the reference's check_it = niter / 20,
 * SOLVER/parameters.F90:932, flushing the receivers at
 * SOLVER/time_evol_wave.F90:1142-1146 through nc_rec_checkpoint,
 * SOLVER/nc_routines.F90:588): during every later run, after the steps up to
 * each multiple of check_it the seismogram samples recorded so far (sample 0
 * is iteration 0, then one every seis_it steps) are copied into `out`, in the
 * layout of axg_get_receivers with first extent nseismo_cap, on a copy stream
 * while the following steps run.  check_it 0 switches the checkpoints off.
 * `out` should be page-locked host memory (cudaHostAlloc / cudaHostRegister)
 * for the copies to overlap the steps.  axg_reset restarts them. */
int axg_set_seismogram_checkpoint(axg_handle *h, int32_t check_it, float *out, int32_t nseismo_cap);
/* Samples (from sample 0) whose checkpoint copies have completed. */
int axg_seismogram_checkpoint_samples(axg_handle *h, int32_t *n_samples);

/* Event-timed repeat of axg_stiffness_assembled_device: n launches, returns the
 * average device time in ms of one stiffness+assembly (all colour launches). */
int axg_time_stiffness(axg_handle *h, int32_t n, float *ms_avg);

/* Debug builds compiled with -DAXG_DEVICE_CHECKS check every device index
 * against its bound and record the first violation instead of accessing
 * memory.  Fills out8 = {flag, kernel id, source line, 0, index lo, index hi,
 * bound lo, bound hi}; returns AXG_ERR_UNSUPPORTED in normal builds. */
int axg_device_check_report(int32_t *out8);

/* Self-test of the kernels' bounded device wait: one GPU thread waits on an
 * mbarrier that nothing arrives at (no copy is involved), through the same
 * wait the patch kernels use.  *status receives what the wait recorded
 * (AXG_ERR_TIMEOUT when it gave up as designed) and *elapsed_s how long it
 * waited (about one second).  No counterpart in the reference. */
int axg_selftest_wait_timeout(int32_t *status, double *elapsed_s);

void axg_destroy(axg_handle *h);

/* Message of the last error on `h` (or of the last failed axg_create when h is
 * NULL); never NULL. */
const char *axg_last_error(axg_handle *h);

#ifdef __cplusplus
}
#endif
#endif /* AXISEM_GB300_H */
