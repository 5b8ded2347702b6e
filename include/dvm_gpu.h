/*
 * dvm_gpu.h -- C ABI of the GB300 (sm_103a) DVM time step.
 *
 * The time step of the discrete-velocity Boltzmann solver is
 *   collisions (Monte Carlo, variance reduced or full)  -> convection (first-order
 *   upwind, with wall / inflow boundary conditions)     -> per-cell moments.
 * Every entry point takes plain pointers, sizes and POD structs so that a Fortran
 * host can bind it with iso_c_binding (value scalars, assumed-size arrays), the same
 * way the reference binds GSL (utils/random_number_generation.f90:46-80).
 *
 * Reference: aarthisekaran11/2D_DVM_microflows, software/trunk/src (2-D code) and
 * software/code_versions/grid_ref_code/src (1-D code). File:line citations below are
 * relative to software/trunk/src unless they say grid_ref.
 *
 * Layout: f[cell][v], v = i + Nx*(j + Ny*k), cell = nx + nx_space*ny (0-based), the
 * column-major order of DistFuncType%value(i,j,k) (grid/velocity_grid.f90:714-726) and of
 * phi(nx,ny) (solver/dvm_solver.f90:55-64).
 *
 * Every call returns an int status (DVM_OK = 0). Calls are ordered on the context's CUDA
 * stream; the ones that return host data synchronise.
 */
#ifndef DVM_GPU_H
#define DVM_GPU_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DVM_ABI_VERSION 2

/* ---- status codes ------------------------------------------------------------------ */
enum {
  DVM_OK = 0,
  DVM_ERR_PARAM = 1,      /* invalid parameter (the reference prints and stops)     */
  DVM_ERR_OOM = 2,        /* device allocation failed                                */
  DVM_ERR_CUDA = 3,       /* CUDA runtime / launch error                             */
  DVM_ERR_NUMERIC = 4,    /* device error word set (see dvm_get_error_word)          */
  DVM_ERR_TIMEOUT = 5,    /* a bounded device wait ran out                           */
  DVM_ERR_NODEVICE = 6,   /* no CUDA device                                          */
  DVM_ERR_TOO_LARGE = 7,  /* problem exceeds a fixed scratch or a server's budget     */
  DVM_ERR_IO = 8          /* an output file could not be opened or written            */
};

/* Bits of the device error word. */
enum {
  DVM_EW_SEARCH = 1,      /* CDF inversion left its bucket (reference would loop)    */
  DVM_EW_REMAP = 2,       /* remap found no exterior node (remapping.f90:348 stops)  */
  DVM_EW_NONFINITE = 4,   /* non-finite moment                                       */
  DVM_EW_NEGDENS = 8,     /* non-positive cell density                               */
  DVM_EW_WAIT = 16        /* a bounded device wait (bulk copy barrier) ran out       */
};

/* iColl (collisions/collision_integral.f90:35-38) */
enum { DVM_COLL_NONE = 0, DVM_COLL_FMC = 2, DVM_COLL_VR = 3 };
/* iConv (convection/convection.f90:34-35) */
enum { DVM_CONV_NONE = 0, DVM_CONV_UPWIND1 = 1 };
/* physical-space dimensionality */
enum { DVM_GEOM_0D = 0, DVM_GEOM_1D = 1, DVM_GEOM_2D = 2 };
/* 2-D wall condition numbering (conditions/boundary_conditions.f90:56-59) */
enum { DVM_BC2D_WALL = 1, DVM_BC2D_INOUT = 2, DVM_BC2D_ZEROGRAD = 3, DVM_BC2D_COUETTE = 4 };
/* 1-D end condition numbering (grid_ref conditions/boundary_conditions.f90:43-46) */
enum { DVM_BC1D_SPECULAR = 1, DVM_BC1D_DIFFUSE = 2, DVM_BC1D_INOUT = 3, DVM_BC1D_ZEROGRAD = 4 };
/* pi used by Maxwellian normalisation and scattering azimuth (utils/constants.f90:30) */
enum { DVM_PI_REFERENCE = 0, DVM_PI_EXACT = 1 };
/* how many samples a cell-step draws */
enum { DVM_SAMPLES_FORMULA = 0,   /* compute_num_coll_pairs, collision_utilities.f90:106-140 */
       DVM_SAMPLES_FIXED = 1 };   /* samples_per_step total per cell-step, split over the
                                     sub-integrals in proportion to densA*densB             */
/* arithmetic of the collision sampling and scatter (not in the reference) */
enum { DVM_PREC_FP64 = 0,         /* plain method: everything in FP64                       */
       DVM_PREC_FP32 = 1 };       /* sampling and scatter in FP32 into an FP32 increment,
                                     then a per-cell FP64 projection that restores mass,
                                     momentum and energy conservation; f, CDFs, moments FP64 */
/* wall index in dvm_params.bc / .wall */
enum { DVM_WALL_LEFT = 0, DVM_WALL_RIGHT = 1, DVM_WALL_BOTTOM = 2, DVM_WALL_TOP = 3 };
/* wall property index in dvm_params.wall[w][...] */
enum { DVM_WP_DENS = 0, DVM_WP_U = 1, DVM_WP_V = 2, DVM_WP_W = 3, DVM_WP_TEMP = 4 };

/* Per-cell property record (dist_funcs/physical_props.f90:41-69, monatomic subset). */
enum {
  DVM_P_DENS = 0, DVM_P_U = 1, DVM_P_V = 2, DVM_P_W = 3,
  DVM_P_TEMP = 4,          /* translational temperature, compute_temperature :1033-1087 */
  DVM_P_SPECIES_TEMP = 5,  /* compute_overall_temperature :1428-1457 (monatomic)        */
  DVM_P_AVG_SPEED = 6,     /* compute_avg_speed :1459-1507                               */
  DVM_P_PRESSURE = 7,      /* 0.5*n*T :357                                               */
  DVM_P_QX = 8, DVM_P_QY = 9, DVM_P_QZ = 10,            /* compute_heat_flux :1914-1986   */
  DVM_P_TXX = 11, DVM_P_TYY = 12, DVM_P_TZZ = 13,       /* compute_viscous_stress          */
  DVM_P_TXY = 14, DVM_P_TXZ = 15, DVM_P_TYZ = 16,       /*   :1988-2071                    */
  DVM_NPROP = 20
};

/* Velocity grid: node coordinates per axis (grid/velocity_grid.f90:35-73). The node
 * volumes (compute_beta :486-540), zero/neg/pos indices (find_zero_point :653-689) and
 * beta3_min (:542-597) are derived from these by dvm_create. */
typedef struct dvm_vgrid {
  int32_t nx, ny, nz;
  const double* x;   /* [nx], increasing */
  const double* y;   /* [ny] */
  const double* z;   /* [nz] */
} dvm_vgrid;

/* Solver parameters; one field per input-deck key the step reads
 * (input_output/read_input_2D.f90:75-777). Single species (every supported
 * configuration is monatomic). */
typedef struct dvm_params {
  int32_t geometry;        /* DVM_GEOM_*                                           */
  int32_t nx_space;        /* cells in x (1 for 0-D)                               */
  int32_t ny_space;        /* cells in y (2-D); 1-D: independent rows of nx_space  */
                           /* cells, each with both ends (1 = one 1-D domain)      */
  int32_t coll_method;     /* iColl                                                */
  int32_t conv_method;     /* iConv                                                */
  int32_t num_repl;        /* NRepl (replenishing_collisions.f90:134-354)          */
  int32_t samples_mode;    /* DVM_SAMPLES_*                                        */
  int32_t pi_mode;         /* DVM_PI_*                                             */
  int32_t bc[4];           /* per wall, DVM_BC2D_* (2-D) or DVM_BC1D_* (1-D)       */
  int64_t samples_per_step;/* per cell-step, DVM_SAMPLES_FIXED                     */
  uint64_t seed;           /* Philox key                                           */
  double dx, dy;           /* cell sizes (mean free paths)                         */
  double dt;               /* deltat (solver/time_stepping.f90)                    */
  double Kn;               /* Knudsen number (solver/scaling.f90)                  */
  double mass;             /* scaled molecular mass                                */
  double omega;            /* VHS viscosity exponent                               */
  double alpha;            /* VSS scattering exponent (1 = isotropic)              */
  double sigma;            /* cross-section from calculate_cross_section           */
                           /* (solver/scaling.f90:163-201)                          */
  double coln_rms;         /* ColnRMS (collision_integral.f90:79-96)               */
  double cdf_tolerance;    /* variance_reduction.f90:316-322                       */
  double acc_coeff;        /* accommodation coefficient                            */
  double wall[4][5];       /* per wall: density, u, v, w, temperature              */
  int32_t precision;       /* DVM_PREC_*                                           */
  int32_t reserved;        /* zero                                                 */
} dvm_params;

/* Recorded collision list for one cell-step (same list applied to every cell).
 * Sub-integral s: VR uses s = 0 (eq x dev), 1 (dev x eq), 2 (dev x dev)
 * (variance_reduction.f90:669-816, 822-961, 967-1116); FMC uses s = 0 only.
 * Partners are given either as 0-based node indices (glA/glB) or as the uniforms fed
 * to pick_collision_partner (rA/rB, collision_utilities.f90:142-186); r_phi/r_cos hold
 * num_repl values per sample, in the order pick_random_velocity_on_sphere draws them
 * (azimuth first, collision_utilities.f90:308 then :332). */
typedef struct dvm_pairlist {
  int64_t count[3];
  const int32_t* glA[3];
  const int32_t* glB[3];
  const double* rA[3];
  const double* rB[3];
  const double* r_phi[3];  /* [count * num_repl] */
  const double* r_cos[3];  /* [count * num_repl] */
} dvm_pairlist;

typedef struct dvm_ctx dvm_ctx;

/* ---- lifetime ----------------------------------------------------------------------- */
/* Replaces initialize_solver's allocations (solver/dvm_solver.f90:55-64), create_velocity_grid
 * (grid/velocity_grid.f90:271-350) and create_collision_integral (collision_integral.f90:98). */
int dvm_create(const dvm_params* params, const dvm_vgrid* grid, dvm_ctx** out);
/* Replaces destroy_solver (solver/dvm_solver.f90:371). */
int dvm_destroy(dvm_ctx* ctx);
const char* dvm_strerror(int status);
int dvm_abi_version(void);

/* ---- state -------------------------------------------------------------------------- */
/* f[cells][Nv] host array, copied to the device (phi and delta_phi both take it). */
int dvm_upload_f(dvm_ctx* ctx, const double* f);
int dvm_download_f(dvm_ctx* ctx, double* f);
int dvm_num_velocity_points(const dvm_ctx* ctx);
int dvm_num_cells(const dvm_ctx* ctx);

/* ---- the hot path ------------------------------------------------------------------- */
/* compute_collision_integral for every cell (collisions/collision_integral.f90:163-274,
 * called per cell from solver/dvm_solver.f90:305-315). Uses the properties held by the
 * context (the last dvm_calculate_physical_properties or dvm_set_properties). step is the
 * Philox counter; pairs != NULL replays a recorded list instead of drawing. */
int dvm_compute_collision_integral(dvm_ctx* ctx, uint64_t step, const dvm_pairlist* pairs);
/* compute_convection with its boundary conditions (convection/convection.f90:69-117,
 * conditions/boundary_conditions.f90:537-1656; 1-D: grid_ref convection.f90:111-256 and
 * grid_ref conditions/boundary_conditions.f90:319-913). */
int dvm_compute_convection(dvm_ctx* ctx);
/* calculate_physical_properties per cell (dist_funcs/physical_props.f90:285-485) plus heat
 * flux and stress (:1914-2071), on the device; results stay on the device. */
int dvm_calculate_physical_properties(dvm_ctx* ctx);
/* props[cells][DVM_NPROP] */
int dvm_get_properties(dvm_ctx* ctx, double* props);
int dvm_set_properties(dvm_ctx* ctx, const double* props);
/* One solve() iteration per step: collisions, convection, moments
 * (solver/dvm_solver.f90:299-357). first_step is the Philox step counter of the first. */
int dvm_step(dvm_ctx* ctx, uint64_t first_step, int nsteps);
/* No reference counterpart: dvm_upload_f(f_in), dvm_step(first_step, nsteps) and
 * dvm_download_f(f_out) in one call, for a host that keeps f in its own memory between
 * steps (the reference's phi). When f_in / f_out are page-locked (cudaHostAlloc,
 * cudaHostRegister), the device reads f_in in the moments pass that starts the call (which
 * writes the device's copy as it goes) and writes f_out in the moments pass that ends it,
 * instead of separate copies; other host memory goes through copies. f_in and f_out may be
 * the same buffer. Returns after f_out is written. */
int dvm_step_host(dvm_ctx* ctx, uint64_t first_step, int nsteps, const double* f_in,
                  double* f_out);
/* Collision samples drawn by the last collision call, summed over cells (tot_colls). */
int dvm_last_collision_count(dvm_ctx* ctx, int64_t* count);
/* Scatter adds into f made by the last collision call, counted by the collide kernel: two
 * depletions per sample plus the written stencil nodes of each replenishment (4 to 7;
 * replenishing_collisions.f90:356-434). FP32 adds into the increment in the precision
 * form. Divided by the collision count, it is the atomics per sample behind the kernel's
 * atomic roofline. */
int dvm_last_scatter_count(dvm_ctx* ctx, int64_t* count);

/* Convergence residual of the last dvm_calculate_physical_properties: the largest, over
 * cells, relative change of n, u (on the thermal speed), T and the stress tensor (on the
 * pressure) since the moments before it.
 * No reference counterpart (the reference runs a fixed number of steps). */
int dvm_get_residual(dvm_ctx* ctx, double* residual);

/* ---- checkpoint / restart ------------------------------------------------------------ */
/* Replaces the reference's restart files (input_output/restart.f90:93-250, ntime and phi):
 * the checkpoint holds ntime, f, the properties and the cached equilibrium with its CDF
 * and bucket table, so that a context restored from it continues the run exactly as the
 * saved one would (the Philox stream is indexed by ntime). The buffer is host memory of
 * dvm_checkpoint_size bytes; dvm_checkpoint_load checks that it belongs to a context of
 * the same cells, grid size, geometry and collision method. */
int dvm_checkpoint_size(dvm_ctx* ctx, uint64_t* bytes);
int dvm_checkpoint_save(dvm_ctx* ctx, uint64_t ntime, void* buf, uint64_t bytes);
int dvm_checkpoint_load(dvm_ctx* ctx, const void* buf, uint64_t bytes, uint64_t* ntime);

/* ---- batched instances ----------------------------------------------------------------- */
/* Many independent 0-D relaxations (the reference's homogeneous case, nx_space = ny_space =
 * 1, run for many initial states and grids at once), or, with params->geometry =
 * DVM_GEOM_1D, many 1-D solves of params->nx_space cells each, all with the end conditions
 * of params (each instance is one row of a multi-row 1-D context). No reference
 * counterpart. Instances on
 * the same velocity grid form one group (one context whose cells are the instances). One
 * step of every instance is one launch each of the CDF build, the sample plan, the
 * persistent collision kernel (the precision form adds the projection) and the moments, over
 * all groups at once (up to 8 grids per launch; each CTA runs its own group's grid), and that
 * step is captured into a single CUDA graph on the first dvm_batch_step and replayed after.
 * A timing autotuner picks the CDF CTA width and the collision kernel's CTAs per SM at that
 * point; the collision CTAs are dealt to the groups in proportion to their samples.
 * params gives the common settings (collision method, dt, Kn, species, precision, seed);
 * samples_per_grid[g] is the fixed sample count per instance-step on grid g. */
typedef struct dvm_batch dvm_batch;
int dvm_batch_create(const dvm_params* params, const dvm_vgrid* grids, int ngrids,
                     const int32_t* instance_grid, int ninstances,
                     const int64_t* samples_per_grid, dvm_batch** out);
int dvm_batch_destroy(dvm_batch* b);
/* f of one instance ([Nv] of its grid; 1-D: [nx_space][Nv]); properties are computed at
 * the next step. */
int dvm_batch_upload_f(dvm_batch* b, int instance, const double* f);
int dvm_batch_download_f(dvm_batch* b, int instance, double* f);
int dvm_batch_step(dvm_batch* b, int nsteps);
/* props[ninstances][DVM_NPROP] (1-D: [ninstances][nx_space][DVM_NPROP]) */
int dvm_batch_get_properties(dvm_batch* b, double* props);
/* Device time of nsteps graph replays (ms) and the samples they drew. */
int dvm_batch_time_steps(dvm_batch* b, int nsteps, double* ms, int64_t* collisions);
/* The launch shape the autotuner chose (after the first step; 0 before it): threads per CDF
 * CTA and collision CTAs per SM; launches per step of the graph. */
int dvm_batch_launch_shape(dvm_batch* b, int* cdf_threads, int* collide_ctas_per_sm,
                           int* launches_per_step);

/* ---- request server ------------------------------------------------------------------ */
/* Device bytes a context for (params, vgrid) allocates; the server admits by this figure.
 * No reference counterpart. */
int dvm_footprint_bytes(const dvm_params* params, const dvm_vgrid* vgrid, uint64_t* bytes);

/* Independent solves (any geometry, grid, Knudsen or Mach number) served with continuous
 * batching. No reference counterpart: the reference runs one solve per process. Native
 * host threads admit submitted requests in arrival order while the admitted footprints fit in
 * hbm_budget_bytes and fewer than max_active run; each admitted request keeps its state on
 * the device in its own context and stream and advances up to steps_per_turn steps per turn
 * (one launch of a CUDA graph whose conditional while loop tests the residual on the device
 * after every step, or every two steps with convection, and stops there), so the turns of
 * different requests overlap on the device. A request ends when the convergence residual
 * (dvm_get_residual) is <= residual_tol or after max_steps steps. Its result depends only
 * on its own parameters, seed and step count. */
typedef struct dvm_server dvm_server;
typedef struct dvm_request_info {
  int32_t status;         /* DVM_OK or the status that ended the request               */
  int32_t converged;      /* 1: the residual reached the tolerance                     */
  int32_t steps;          /* steps taken                                               */
  int32_t preempted;      /* times checkpointed and requeued (dvm_server_set_preemption) */
  double residual;        /* residual after the last step                              */
  double queue_ms;        /* submission to admission                                   */
  double latency_ms;      /* submission to result ready on the host                    */
  int64_t collisions;     /* Monte Carlo samples drawn                                 */
  uint64_t device_bytes;  /* bytes the request's context allocated                     */
} dvm_request_info;

int dvm_server_create(uint64_t hbm_budget_bytes, int max_active, int steps_per_turn,
                      dvm_server** out);
/* Waits for every submitted request to finish, then frees the server. */
int dvm_server_destroy(dvm_server* server);
/* f0[cells][Nv] is copied; returns DVM_ERR_TOO_LARGE if the request alone exceeds the
 * budget. */
int dvm_server_submit(dvm_server* server, const dvm_params* params, const dvm_vgrid* vgrid,
                      const double* f0, int32_t max_steps, double residual_tol, int64_t* id);
/* Blocks until request id has finished. */
int dvm_server_wait(dvm_server* server, int64_t id, dvm_request_info* info);
/* Copies the finished request's properties [cells][DVM_NPROP] and f [cells][Nv] (either may
 * be NULL) and forgets the request. */
int dvm_server_result(dvm_server* server, int64_t id, double* props, double* f);
int dvm_server_stats(dvm_server* server, int64_t* completed, int32_t* peak_active,
                     uint64_t* peak_bytes);
/* Preemption through the checkpoint (input_output/restart.f90:93-250): a request that has
 * run `turns` turns since its admission while another request waits is checkpointed to
 * host memory, its device memory and slot are released, and it is queued again behind the
 * waiting requests; readmitted, it resumes from the checkpoint with its step counter, so
 * its result is that of an uninterrupted run. 0 (the default) turns preemption off. */
int dvm_server_set_preemption(dvm_server* server, int32_t turns);

/* ---- errors, synchronisation, instrumentation -------------------------------------- */
int dvm_synchronize(dvm_ctx* ctx);
/* Reads and clears the device error word (DVM_EW_* bits). */
int dvm_get_error_word(dvm_ctx* ctx, uint32_t* word);
/* When enabled, every kernel launch is bracketed by CUDA events on the context's stream. */
int dvm_profile_enable(dvm_ctx* ctx, int enable);
/* kernel ids */
enum { DVM_K_CDF = 0, DVM_K_PLAN = 1, DVM_K_COLLIDE = 2, DVM_K_WALL = 3, DVM_K_GHOST = 4,
       DVM_K_CONVECT = 5, DVM_K_BC1D = 6, DVM_K_MOMENTS = 7, DVM_K_PROJECT = 8,
       DVM_K_COUNT = 9 };
const char* dvm_kernel_name(int kernel_id);
/* Sums the event-timed durations (ms) and launch counts since the last reset; synchronises. */
int dvm_profile_read(dvm_ctx* ctx, int kernel_id, double* total_ms, int64_t* launches);
int dvm_profile_reset(dvm_ctx* ctx);
/* Total kernels this context launched (profiled or not). */
int dvm_launch_count(dvm_ctx* ctx, int64_t* launches);
/* Events around nsteps of dvm_step on the context's stream: elapsed device time in ms. */
int dvm_time_steps(dvm_ctx* ctx, uint64_t first_step, int nsteps, double* ms);
/* Writes a buffer of bytes > L2 on the context's stream (cold-cache timing). */
int dvm_flush_l2(dvm_ctx* ctx);
/* FP64 atomic-add throughput (adds per second) of pseudo-random addresses in a window of
 * window_bytes of device memory: the roofline of a scatter whose target stays in L2.
 * Instrumentation; no reference counterpart. */
int dvm_atomic_rate(dvm_ctx* ctx, uint64_t window_bytes, double* per_s);
/* Failure-path check of the bounded device waits: runs a wait on a barrier that nothing
 * completes, on the context's stream. The wait gives up after its bounded number of polls
 * and sets DVM_EW_WAIT in the error word (read it with dvm_get_error_word); the context
 * stays usable. */
int dvm_wait_selftest(dvm_ctx* ctx);

/* ---- Tecplot output (input_output/visualization.f90) --------------------------------- */
/* The reference's output files for one monatomic species, written on the host from data the
 * caller downloaded; no device work. Replaces write_headers (visualization.f90:514-762),
 * write_properties (:1591-1716, with get_data_to_output :2296-2633) and write_df
 * (:920-1230). Given f, every property is formed from it on the host with the reference's
 * formulas and summation order (physical_props.f90:285-485, 1779-2071), so an f equal to
 * the reference's gives the same bytes; without f (props only) the device moments are
 * written and the columns formed from phi (Temp. X/Y/Z, Entropy) are refused. */
enum { DVM_VIS_NPROP = 27 };  /* property_names(1:27), visualization.f90:314-340        */
enum { DVM_VIS_DF_1D = 1, DVM_VIS_DF_2D = 2, DVM_VIS_DF_3D = 3 };  /* df_output_dimension */
typedef struct dvm_vis {
  char properties_filename[128]; /* properties_vis_filename: <name>.dat (mixture) and
                                    <name>_1.dat (the species)                            */
  char df_filename[128];         /* df_vis_filename: <name>_1_<x>_<y>.dat per location    */
  int32_t enable_properties;     /* enable_properties_vis                                 */
  int32_t properties_to_output[DVM_VIS_NPROP]; /* write_dens ... write_pressure, in the
                                    order of property_names                               */
  int32_t write_stress;          /* stress columns written (0..6)                         */
  int32_t stress_directions[6];  /* 11, 22, 33, 12, 13 or 23 each                         */
  int32_t write_moment;          /* moment columns of the species file (0..6)             */
  int32_t moment_numbers[6];     /* moment_numbers: orders of compute_moment              */
  int32_t nx_space, ny_space;
  double dx, dy;                 /* delta_x, delta_y                                      */
  int32_t end_time;              /* ntstep (zone count of a one-cell run)                 */
  int32_t properties_dump_freq;  /* properties_vis_dump_freq                              */
  int32_t enable_vel_df, enable_rot_df, enable_vib_df;
  int32_t df_dimension;          /* DVM_VIS_DF_*                                          */
  int32_t num_locations;         /* df output cells (1..16), 1-based like the reference  */
  int32_t x_locations[16], y_locations[16];
  int32_t rot_levels, vib_levels;/* num_rot_levels, num_vib_levels (columns of zeros)     */
  int32_t pi_mode;               /* DVM_PI_* of the Maxwellian in the deviation column    */
  double mass, omega;            /* molecule mass and viscosity exponent                  */
  double cZr, cZv;               /* collision numbers of the analytic relaxation columns  */
  double right_wall_dens;        /* gamma and molecular mass of the Mach column           */
  double right_wall_temp_rot, right_wall_temp_vib;
} dvm_vis;
/* Creates (truncates) the files and writes their title, variables and, for a one-cell run,
 * zone lines. */
int dvm_vis_write_headers(const dvm_vis* vis);
/* Appends one output time: props[cells][DVM_NPROP] and/or f[cells][Nv] (either may be NULL,
 * not both; grid is needed with f). */
int dvm_vis_write_properties(const dvm_vis* vis, double time, const double* props,
                             const double* f, const dvm_vgrid* grid);
/* Appends one output time of the distribution function at the chosen cells. */
int dvm_vis_write_df(const dvm_vis* vis, double time, const double* f, const dvm_vgrid* grid);
/* One Ew.d field as the reference's format statements write it (for checking the format). */
int dvm_vis_format_e(double x, int w, int d, char* out, int out_len);

/* ---- collisions without device allocation ------------------------------------------ */
/* No counterpart in the reference. The collision integral of dvm_compute_collision_integral
 * for callers that cannot allocate device memory -- a host that owns all device memory and
 * forbids allocation behind its back, a memory pool held at a fixed budget, a real-time loop
 * that must not enter the allocator. It allocates nothing: the caller passes, in device
 * memory, f[ncells][Nv] (updated in place) and props[ncells][DVM_NPROP] (the cell
 * properties, e.g. from dvm_get_properties); every intermediate lives in one fixed 32 MiB
 * device array that the library holds on each GPU that loads it, until exit.
 *   Limit: the grid tables (under 0.2 MB) plus 16*(Nv+1) + 16112 bytes per cell must fit
 *   in 32 MiB: at most 410 cells of 16^3, 141 of 24^3, 61 of 32^3 or 32 of 40^3; larger
 *   problems get DVM_ERR_TOO_LARGE before anything is launched.
 *   The first call on a device looks up that array's address (cudaGetSymbolAddress) with
 *   the device current and keeps it; make that first call before any stream capture, and
 *   do not use this entry point across a cudaDeviceReset of that device.
 *   Every call shares the array and rebuilds what it needs (the equilibrium is recomputed,
 *   as on a new context's first call); calls that overlap on the GPU race on it.
 *   Work is queued on `stream` (a cudaStream_t; NULL = default stream). If `collisions` is
 *   not NULL the call synchronises that stream, stores the samples drawn, and returns
 *   DVM_ERR_NUMERIC if the device error word is set; the word collects the bits of every
 *   call since the last call that read it, so a fault in a call made with `collisions`
 *   NULL is reported by the next call that passes it. */
int dvm_collide_noalloc(const dvm_params* params, const dvm_vgrid* grid, double* f,
                        const double* props, int ncells, uint64_t step, void* stream,
                        int64_t* collisions);

#ifdef __cplusplus
}
#endif
#endif /* DVM_GPU_H */
