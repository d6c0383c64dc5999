/*
 * gfmd_gb300 — C ABI of the GB300-native GFMD elastic force evaluation.
 *
 * This is the boundary a LAMMPS `fix gfmd` solver style (static/gb300,
 * dynamic/gb300) or any other host code binds to.  Plain C types only; all
 * pointers are either host memory or CUDA device memory as stated per call.
 * Every call returns an int status (GFMD_OK = 0) and never aborts, traps or
 * exits; gfmd_last_error() gives a message for the last failure on the
 * calling thread.  A handle is not thread-safe: one host thread per handle.
 *
 * Grid layout (that of the reference, src/main/fix_gfmd.cpp:763 and
 * src/solvers/gfmd_solver_fft.cpp:72-80): displacement and force arrays are
 * [ndof][nx*ny] with the grid index ix*ny + iy (y fastest).
 *
 * Transform conventions (reference with LAMMPS >= patch_10Feb2021):
 * forward exp(-i q.r) unscaled, backward exp(+i q.r) unscaled, Phi(q)
 * pre-scaled by 1/(nx*ny) (src/main/gfmd_misc.cpp:88-97).
 */
#ifndef GFMD_GB300_H
#define GFMD_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes -------------------------------------------------------- */
#define GFMD_OK 0
#define GFMD_EINVAL 1        /* bad argument or state */
#define GFMD_ENOMEM 2        /* device or host allocation failed */
#define GFMD_ECUDA 3         /* a CUDA runtime call failed */
#define GFMD_ENONFINITE 4    /* NaN or Inf in the energy or a norm */
#define GFMD_ETIMEDOUT 5     /* a bounded device wait gave up */
#define GFMD_ENOTCONVERGED 6 /* iteration cap reached before tolerance */
#define GFMD_ENOPHI 7        /* no stiffness table uploaded yet */

/* ---- arithmetic of a solver handle -------------------------------------- */
#define GFMD_PREC_F64 0      /* plain FP64 everywhere (drop-in parity path) */
#define GFMD_PREC_F32 1      /* FP32 transforms and Phi products with
                                compensated twiddles; FP64 energy */

/* ---- Phi table layouts accepted by gfmd_set_phi ------------------------- */
#define GFMD_PHI_FULL 0      /* [nx*ny][ndof][ndof] complex (re,im), index
                                ix*ny+iy: what fill_phi_buffer produces */
#define GFMD_PHI_HALF 1      /* [nx][ny/2+1][ndof][ndof] complex (re,im) */

typedef struct gfmd_solver *gfmd_handle_t;
typedef struct gfmd_kernel *gfmd_kernel_t;

const char *gfmd_last_error(void);

/* Library version string. */
const char *gfmd_version(void);

/* ---- solver handle ------------------------------------------------------- */

/* Create a solver for an nx x ny grid with ndof = 3*nu degrees of freedom per
 * grid point (ndof <= 24, nx, ny in [1, 8192]).  Allocates all device scratch
 * on the current CUDA device.
 * Replaces: GFMDSolverStatic::GFMDSolverStatic + GFMDSolver::set_grid_size
 * (src/solvers/gfmd_solver_static.cpp:49-84, src/main/gfmd_solver.cpp:79-136)
 * for a single process that owns the whole grid. */
int gfmd_create(int nx, int ny, int ndof, int precision, gfmd_handle_t *out);

/* Release the handle and its device memory. */
int gfmd_destroy(gfmd_handle_t h);

/* Run all later work of this handle on the given cudaStream_t (NULL = the
 * legacy default stream). */
int gfmd_set_stream(gfmd_handle_t h, void *cuda_stream);

/* Upload the stiffness table once (host memory, FP64).  phi is pre-scaled by
 * 1/(nx*ny) as fill_phi_buffer leaves it; layout is GFMD_PHI_FULL or
 * GFMD_PHI_HALF; linf holds ndof/3 linear forces per layer (NULL = zeros).
 * The table is packed on the host into the Hermitian half-spectrum form the
 * kernels read and copied to the device; the caller keeps ownership of phi.
 * Replaces: GFMDSolverStatic::set_kernel (src/solvers/gfmd_solver_static.cpp:90-136),
 * which fills phi via fill_phi_buffer (src/main/gfmd_misc.cpp:32-101). */
int gfmd_set_phi(gfmd_handle_t h, const double *phi, int layout, const double *linf);

/* One force evaluation on device buffers (FP64, [ndof][nx*ny]); u and f must
 * not alias.  Writes the elastic energy to *epot (host) and synchronizes the
 * handle's stream.
 * Replaces: GFMDSolverStatic::post_force (src/solvers/gfmd_solver_static.cpp:145-249),
 * the GPU form of which took device double pointers with pitch nxy_loc
 * (src/cuda/gfmd_solver_cuda.cpp:394-504). */
int gfmd_post_force(gfmd_handle_t h, const double *d_u, double *d_f, double *epot);

/* The same on host buffers: copies u in and f out inside the call.
 * Replaces: GFMDSolverStatic::post_force with the CPU double** buffers
 * allocated by FixGFMD (src/main/fix_gfmd.cpp:613-617). */
int gfmd_post_force_host(gfmd_handle_t h, const double *u, double *f, double *epot);

/* Asynchronous force evaluation on device-resident state, no host sync.
 * d_epot (device, one double) receives the energy.  gfmd_force_f64 needs a
 * GFMD_PREC_F64 handle, gfmd_force_f32 a GFMD_PREC_F32 handle. */
int gfmd_force_f64(gfmd_handle_t h, const double *d_u, double *d_f, double *d_epot);
int gfmd_force_f32(gfmd_handle_t h, const float *d_u, float *d_f, double *d_epot);

/* u(q=0) of the last force evaluation, ndof doubles, host.
 * Replaces: GFMDSolver::get_u0 (src/main/gfmd_solver.h:89-91). */
int gfmd_get_u0(gfmd_handle_t h, double *u0);

/* Launch plan of the fused path: rows per block of the shared-memory row
 * transforms and the Phi prefetch depth of the column kernel (both chosen by
 * the autotuner at gfmd_set_phi); 0, 0 on the general path.  No counterpart
 * in the reference. */
int gfmd_plan_info(gfmd_handle_t h, int *rows_per_block, int *phi_prefetch);

/* Device bytes held by the handle (with the preconditioner gfmd_prec_gradient
 * keeps for it, once built).
 * Replaces: GFMDSolver::memory_usage (src/main/gfmd_solver.h:97). */
int gfmd_memory_usage(gfmd_handle_t h, double *bytes);

/* Kernel launches one force evaluation of this handle makes, and whether it
 * runs the fused power-of-two path (1) or the general-size path (0).  No
 * counterpart in the reference (introspection for benchmarks and tests). */
int gfmd_solver_info(gfmd_handle_t h, int *launches_per_eval, int *fused);

/* Device time of each kernel launch of one force evaluation: records CUDA
 * events around the launches on the handle's stream, synchronizes, and
 * writes gfmd_solver_info's launches_per_eval times (milliseconds) to ms
 * (nmax entries available) and their count to *nk.  u and f are device
 * buffers of the handle's arithmetic type (double for GFMD_PREC_F64, float
 * for GFMD_PREC_F32); d_epot receives the energy.  No counterpart in the
 * reference (measurement). */
int gfmd_force_kernel_times(gfmd_handle_t h, const void *d_u, void *d_f, double *d_epot, float *ms,
                            int nmax, int *nk);

/* Kernels of the fused FP32 path: row_warp_tma = 1 when the row transforms
 * run one warp per row with TMA-staged spectrum tiles (rows of ny = 2048),
 * col_cluster = blocks per ky of the thread-block-cluster column kernel
 * (0: the single-block column kernel), phi_vector = the packed stiffness
 * table's vector width (4: 16-byte vectors).  No counterpart in the
 * reference (introspection). */
int gfmd_kernel_plan(gfmd_handle_t h, int *row_warp_tma, int *col_cluster, int *phi_vector);

/* Storage pattern of the uploaded table, chosen by gfmd_set_phi from the
 * pairs that are exactly zero at every wavevector: 0 every pair; 1
 * layer-tridiagonal (3x3 blocks of layers two or more apart are zero); 2 as 1
 * with the blocks of all layers but the last diagonal (a slab with
 * nearest-neighbour interactions).  Used at ndof 12 by the FP32
 * register-transform column kernel and by the general path's Phi application
 * (both precisions); reals_per_wavevector = reals streamed per wavevector.
 * Forces are the same with every pattern (the skipped products are zero and
 * the kept ones are summed in the same order).  No counterpart in the
 * reference (introspection). */
int gfmd_phi_pattern(gfmd_handle_t h, int *pattern, int *reals_per_wavevector);

/* ---- solver loops ----------------------------------------------------- */

/* Obstacles acting on every atom of the grid.  The position of the atom of
 * layer l at grid site (ix, iy) is (ix*lattice[0], iy*lattice[1], 0) +
 * layer_offset[l] + u.  No counterpart as one struct in the reference: it
 * carries the parameters of the obstacle fixes listed per kind. */
#define GFMD_OBST_NONE 0
#define GFMD_OBST_SPHERE_EXP 1 /* e = eps exp(-g/sigma) on the gap g = |r-c| - R
                                  (exponential wall of FixWallMap::eval_exp,
                                  src/extras/fix_wall_map.cpp:575-582, on a sphere) */
#define GFMD_OBST_SPHERE_LJ 2  /* LJ 12-6 on the gap, shifted at cutoff
                                  (FixContactSphere, src/extras/fix_contact_sphere.cpp:207-264) */
#define GFMD_OBST_MAP_EXP 3    /* exponential wall on dz = norm (z - (map + map_z0)),
                                  map height at the grid site, normal force only
                                  (FixWallMap::pre_force, src/extras/fix_wall_map.cpp:686-817,
                                  for small lateral displacements and slopes) */
#define GFMD_OBST_MAP_BICUBIC 4 /* the same wall with FixWallMap's bicubic map table
                                  (corner values, central-difference slopes, zero cross
                                  derivatives; src/mathutils/table2d.cpp:176-260)
                                  evaluated at the atom's displaced (x, y) (map pixel
                                  (i, j) at (i lattice[0], j lattice[1])), and the
                                  lateral force -f_z dz/dx, -f_z dz/dy
                                  (fix_wall_map.cpp:686-817, 1381); with GFMD_MIN_CG
                                  and gfmd_obstacle_force */

typedef struct {
  int kind;
  double center[3];     /* sphere centre */
  double radius;        /* sphere radius */
  double epsilon;       /* energy scale */
  double sigma;         /* length scale (decay length of the exponential) */
  double cutoff;        /* on the gap; <= 0: none */
  const double *d_map;  /* MAP_EXP: rigid surface heights [nx*ny], device */
  double map_z0;        /* MAP_EXP: offset added to the map */
  int norm;             /* MAP_EXP: +1 wall below the atoms, -1 above (0 = +1) */
  double lattice[2];    /* grid spacing along x and y (<= 0: 1) */
  int nlayer;           /* layers (from l = 0) that feel the obstacle (<= 0: all) */
  double layer_offset[8][3];
  double fz_ext;        /* constant external force along +z on every atom the
                           obstacle acts on (load control: pressure x area per
                           atom); energy -fz_ext * sum u_z */
} gfmd_obstacle_t;

#define GFMD_MIN_CG 0   /* Polak-Ribiere CG, Newton line search (LAMMPS min_style cg
                           as used on fix gfmd by tests/TEST_Hertz_x/lammps.in) */
#define GFMD_MIN_FIRE 1 /* FIRE (FixFIRE, src/cuda/fix_fire.cpp:117-297) */
#define GFMD_MIN_TR 2   /* trust region on the preconditioned gradient (min_style
                           tr/gfmd, src/extras/min_tr_gfmd.cpp:95-241) */

typedef struct {
  int method;           /* GFMD_MIN_CG, GFMD_MIN_FIRE or GFMD_MIN_TR */
  double ftol;          /* converged when max |f_i| <= ftol (per component) */
  int maxiter;          /* <= 0: 100000 */
  int recompute;        /* CG: recompute F_el(u) from scratch every n iterations (<= 0: 50) */
  gfmd_handle_t refine; /* optional FP64 handle (same grid and table): when the
                           loop converges, forces are recomputed with it and the
                           loop continues until it also converges */
  /* FIRE parameters (<= 0: the defaults of FixFIRE, src/cuda/fix_fire.cpp:63-69) */
  int fire_minsteps;
  double fire_incfac, fire_decfac, fire_mix, fire_mixdec, fire_dtmax, fire_dt, fire_xlimit;
  gfmd_handle_t precond; /* CG: optional preconditioner from gfmd_make_preconditioner
                            (same grid and precision as the handle): Polak-Ribiere
                            on z = (Phi + shift)^{-1} g, the reference's min_style
                            cg/gfmd (src/extras/min_cg_gfmd.cpp:96-207);
                            TR: the preconditioner of the step (none: identity) */
  /* TR parameters (<= 0: defaults): largest trust radius (LAMMPS min_modify
     dmax, default 0.1) and the acceptance ratio (0.01, min_tr_gfmd.cpp:76) */
  double tr_dmax, tr_rho_tol;
  /* CG: largest move of any displacement component in one line-search step
     (LAMMPS min_modify dmax, which the reference's Hertz inputs leave at its
     default 0.1); <= 0: no cap */
  double dmax;
} gfmd_min_params_t;

typedef struct {
  int status;           /* GFMD_OK or the failure code */
  int iterations;
  int force_evals;      /* FFT force evaluations */
  double energy;        /* elastic + obstacle energy at the end */
  double fmax;          /* max |f_i| at the end (from freshly computed forces) */
  double fnorm;         /* |f|_2 at the end (LAMMPS' fnorm) */
  double seconds;       /* wall time of the call */
} gfmd_min_report_t;

/* Preconditioner for CG: a new handle (same grid and precision) whose force
 * evaluation returns -(Phi(q) + shift I)^{-1} u(q), no gamma-point term.
 * Restates precondition_gradient (src/main/gfmd_misc.h:40-133) with
 * Cavg = shift I; the block inverses are computed once, on the host, from
 * h's uploaded table.  shift > 0 (it regularizes q = 0 and stands in for the
 * obstacle stiffness).  Destroy with gfmd_destroy. */
int gfmd_make_preconditioner(gfmd_handle_t h, double shift, gfmd_handle_t *out);

/* Preconditioned gradient, device buffers [ndof][nx*ny] FP64, on h's stream:
 *   gP = IFFT( (Phi(q) + Cavg)^{-1} FFT(g) )
 * with Phi(q) the uploaded table (divided by nx*ny) and both transforms
 * unscaled, as the reference computes it.  Cavg: ndof*ndof doubles (host),
 * symmetric, added to every block.  The block inverses are built on the host
 * on the first call and again whenever Cavg or the table changes.
 * As in the reference, when ndof > 3 only the first three components are
 * preconditioned and the others are returned as nx*ny*g (the reference's
 * loop writes back three components, src/main/gfmd_misc.h:121-124).
 * Replaces: GFMDSolverStatic::prec_gradient (src/solvers/gfmd_solver_static.cpp:253-269)
 * with precondition_gradient<DEF_G> (src/main/gfmd_misc.h:40-133). */
int gfmd_prec_gradient(gfmd_handle_t h, const double *cavg, const double *d_g, double *d_gP);

/* The same on host buffers [ndof][nx*ny] (copies in and out inside the call).
 * Replaces: GFMDSolverStatic::prec_gradient with FixGFMD's CPU double** buffers. */
int gfmd_prec_gradient_host(gfmd_handle_t h, const double *cavg, const double *g, double *gP);

/* Static minimization of elastic + obstacle energy from the displacements in
 * d_u (device, [ndof][nx*ny], FP64; updated in place).  Replaces LAMMPS'
 * minimize driving fix gfmd through min_pre_force/min_post_force
 * (src/main/fix_gfmd.cpp:1078-1088) and FixFIRE. */
int gfmd_minimize(gfmd_handle_t h, const gfmd_obstacle_t *obst, const gfmd_min_params_t *params,
                  double *d_u, gfmd_min_report_t *report);

/* Batched static minimization: n independent surfaces (any grid sizes and
 * kernels), solved concurrently by CG in one CUDA graph per phase: every
 * surface is a branch of the graph running its restart and a device-driven
 * WHILE loop of CG iterations.  Mixed precision when the items' handles are
 * FP32 and carry an FP64 `refine` handle (all items alike).  params->method
 * must be GFMD_MIN_CG; params->refine is ignored (per item); every handle
 * may appear in one item only (each owns its scratch).  Returns
 * GFMD_OK when every item converged, else the first failing item's status;
 * each item's report is filled either way.  No counterpart in the reference
 * (one surface per LAMMPS run). */
typedef struct {
  gfmd_handle_t handle;           /* force evaluation (FP64, or FP32 for mixed) */
  gfmd_handle_t refine;           /* FP64 handle of the same grid, or NULL */
  const gfmd_obstacle_t *obstacle;/* may be NULL */
  double *d_u;                    /* displacements [ndof][nx*ny], device FP64, in/out */
  gfmd_min_report_t report;       /* out */
  gfmd_handle_t precond;          /* optional preconditioner (all items alike) */
} gfmd_batch_item_t;

int gfmd_minimize_batch(int n, gfmd_batch_item_t *items, const gfmd_min_params_t *params);

/* Damped velocity Verlet (unit masses): v_h = v + dt/2 (f - gamma v),
 * u += dt v_h, v = (v_h + dt/2 f) / (1 + dt gamma/2); gamma = 0 is fix nve.
 * d_u, d_v device FP64 [ndof][nx*ny] updated in place; energies (host,
 * nsteps+1 doubles, may be NULL) receives the total energy before the first
 * and after every step.  Replaces the fix nve + fix gfmd loop of the
 * reference's dynamics runs (tests/TEST_energy_conservation_x/lammps.in). */
int gfmd_run_dynamics(gfmd_handle_t h, const gfmd_obstacle_t *obst, double dt, double gamma,
                      int nsteps, double *d_u, double *d_v, double *energies,
                      gfmd_min_report_t *report);

/* Force of an obstacle on every atom of the grid at displacements d_u
 * (device, FP64 [ndof][nx*ny]) into d_f (same layout; zero on layers the
 * obstacle does not act on) and its energy into *d_energy (device, one
 * double), summed in a fixed order.  Synchronizes cuda_stream.
 * Replaces: the per-atom evaluations of FixWallMap::pre_force
 * (src/extras/fix_wall_map.cpp:686-817) and FixContactSphere::post_force
 * (src/extras/fix_contact_sphere.cpp:207-264) for a fix that keeps its
 * atoms on the device as a grid. */
int gfmd_obstacle_force(int nx, int ny, int ndof, const gfmd_obstacle_t *ob, const double *d_u,
                        double *d_f, double *d_energy, void *cuda_stream);

/* ---- allocation-free force evaluation ------------------------------------- */

/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a host whose pooling allocator owns the device memory, or a time-critical
 * loop where an allocation's implicit synchronization is not acceptable):
 * the FP64 force evaluation of gfmd_post_force without a handle and without
 * allocating.  Inputs and outputs are the caller's device memory:
 *   d_phi_half  [nx][ny/2+1][ndof][ndof] complex (re,im), GFMD_PHI_HALF layout,
 *               scaled by 1/(nx*ny), Phi(-q) = conj Phi(q) assumed off the
 *               ky = 0 and ky = ny/2 columns;
 *   d_linf      ndof/3 linear forces, or NULL;
 *   d_u, d_f    [ndof][nx*ny], must not alias;  d_epot: one double.
 * Scratch (twiddles, spectrum, energy partials) lives in one fixed 16 MiB
 * device array inside the library, held on every GPU that loads it until the
 * process exits; grids that need more (e.g. beyond 512 x 512 at ndof 6) are
 * rejected with GFMD_EINVAL.  Calls share that array: calls that overlap on
 * the GPU race.  The first call on each device looks up the array's address;
 * make it before any stream capture (later calls on a stream that is not
 * capturing look it up again, so a device reset does not leave it stale).
 * Buffers that the device cannot reach (plain host memory) are refused with
 * GFMD_EINVAL.  Asynchronous on cuda_stream. */
int gfmd_post_force_noalloc(int nx, int ny, int ndof, const double *d_phi_half,
                            const double *d_linf, const double *d_u, double *d_f,
                            double *d_epot, void *cuda_stream);

/* ---- stiffness-kernel tables (host) ------------------------------------- */

/* Parse the stiffness-kernel part of a `fix gfmd` line, e.g.
 * "ft fcc100 1.0 2 pair-potential 1 1.0 height 64".  Supported here: the
 * `ft` style on the sc100, fcc100 and fcc111 surfaces with `pair-potential`
 * force constants, the analytic `sc100` and `fcc100` styles, and the
 * continuum `isotropic` and `nonperiodic` styles.  Other styles are produced
 * by the reference's own fill_phi_buffer and uploaded with gfmd_set_phi.
 * Replaces: stiffness_kernel_factory (src/main/surface_stiffness.cpp:440-481). */
int gfmd_kernel_create(const char *args, gfmd_kernel_t *out);
int gfmd_kernel_destroy(gfmd_kernel_t k);

/* Kernel dimension ndof (get_dimension) and substrate height (get_height). */
int gfmd_kernel_info(gfmd_kernel_t k, int *ndof, int *height);

/* Lateral box lengths of the surface (LAMMPS domain->xprd, domain->yprd),
 * which the isotropic (q = 0 term, square boxes only) and nonperiodic (grid
 * spacing xprd/nx, yprd/ny) styles read.  0 (the default) means one length
 * unit per grid point, xprd = nx and yprd = ny of each table filled.
 * Replaces: the Domain pointer handed to stiffness_kernel_factory
 * (src/main/surface_stiffness.cpp:440-444). */
int gfmd_kernel_set_box(gfmd_kernel_t k, double xprd, double yprd);

/* Fill a Phi table for an nx x ny grid, scaled by 1/(nx*ny), in
 * GFMD_PHI_FULL or GFMD_PHI_HALF layout (host memory the caller allocates:
 * 2*ndof*ndof doubles per stored q), and linf (ndof/3 doubles, may be NULL).
 * nthreads <= 0 uses every host core.
 * Replaces: fill_phi_buffer + StiffnessKernel::get_force_at_gamma_point
 * (src/main/gfmd_misc.cpp:32-101, src/main/surface_stiffness.cpp:430-435). */
int gfmd_kernel_phi(gfmd_kernel_t k, int nx, int ny, int layout, double *phi,
                    double *linf, int nthreads);

/* ---- Atom list <-> grid -------------------------------------------------
 * For a fix that keeps its atoms on the device (one rank owning the grid).
 * gid: [natoms][3] ints (ix, iy, iu) as atom->gid; x, xeq, v: [natoms][3].
 * Replaces: FixGFMD::pre_force, orthogonal box (src/main/fix_gfmd.cpp:659-858):
 * u[3 iu + c][ix' ny + iy'] = x - xeq (minimum image in x, y), with
 * ix' = (ix - dxshift) mod nx, iy' = (iy - dyshift) mod ny; v (may be NULL)
 * copied into vgrid the same way.  d_slot_count (may be NULL): [ndof/3][nx*ny]
 * int scratch that, when given, checks that atoms and slots match one to one.
 * status (host, may be NULL): [0] atoms with iu outside [0, ndof/3), [1] empty
 * slots, [2] slots filled twice or more (-1 without d_slot_count).
 * GFMD_EINVAL when any of them is nonzero.  Synchronizes the stream. */
int gfmd_atoms_to_grid(int natoms, const double *d_x, const double *d_xeq, const double *d_v,
                       const int *d_gid, int nx, int ny, int ndof, double xprd, double yprd,
                       int dxshift, int dyshift, double *d_u, double *d_vgrid, int *d_slot_count,
                       int *status, void *cuda_stream);
/* Replaces: FixGFMD::grid_to_list (src/main/fix_gfmd.cpp:952-1074): the grid
 * force f[3 iu + c][ix ny + iy] of every atom into (accumulate: added to)
 * d_fatoms [natoms][3]; fsum (host, may be NULL) gets the force summed over
 * the atoms (FP64, fixed order).  GFMD_EINVAL for ids outside the grid.
 * Synchronizes the stream.  The fix's `fix_center` option (fix_gfmd.cpp:913-927)
 * is then the caller's f[i][c] -= fsum[c] / natoms on its total forces. */
int gfmd_grid_to_atoms(int natoms, const int *d_gid, const double *d_f, int nx, int ny, int ndof,
                       double *d_fatoms, int accumulate, double *fsum, void *cuda_stream);

/* ---- Self-affine rough surfaces ------------------------------------------
 * No counterpart in the reference, which only reads height maps
 * (FixWallMap, src/extras/fix_wall_map.cpp:1123-1190) and low-pass filters
 * them (:1220-1310).  Random-phase synthesis: on the half spectrum
 * (kx, ky >= 0) of the nx x ny grid with spacing a,
 *   C(q) = (q / q_L)^(-2-2H)  for q_L <= q <= q_s, else 0,
 *   q_L = 2 pi / lambda_long, q_s = 2 pi / lambda_short,
 *   Z(q) = sqrt(C(q)) exp(2 pi i u(q)), u uniform in [0,1) from a counter-
 *   based hash of (seed, q) (SplitMix64 finaliser), Hermitian on the ky = 0
 *   and ky = ny/2 columns,
 *   h(r) = s * sum_q Z(q) exp(i q.r),  s such that the spectral rms slope
 *   sqrt(sum_q |q|^2 |Z(q)|^2) equals rms_slope.
 * Writes h[nx*ny] (x slow, y fast) on the device; synchronous. */
typedef struct {
  double lattice;          /* grid spacing a (> 0) */
  double hurst;            /* Hurst exponent H */
  double rms_slope;        /* spectral rms slope of the result (> 0) */
  double lambda_short;     /* short-wavelength cut-off (> 0) */
  double lambda_long;      /* long-wavelength cut-off (>= lambda_short) */
  unsigned long long seed;
} gfmd_surface_params_t;

int gfmd_rough_surface(int nx, int ny, const gfmd_surface_params_t *params, double *d_h,
                       void *cuda_stream);

/* ---- Learned warm start ----------------------------------------------------
 * No counterpart in the reference.  A BF16 convolutional encoder-decoder
 * (4 levels, base_ch channels at full resolution, 2 base_ch below; periodic
 * 3x3 convolutions, 2x2 average pooling, nearest upsampling with additive
 * skips) mapping in_ch input channels to out_ch output channels, run and
 * trained by the library's own tensor-core kernels (BF16 operands, FP32
 * accumulation, FP32 master weights, Adam).  Tensors are device FP32 NHWC
 * [batch][H][W][C], H and W multiples of 8.  Not thread-safe per handle. */
typedef struct gfmd_ws_net *gfmd_ws_handle_t;

int gfmd_ws_create(int in_ch, int out_ch, int base_ch, unsigned long long seed, gfmd_ws_handle_t *out);
int gfmd_ws_destroy(gfmd_ws_handle_t net);
int gfmd_ws_set_stream(gfmd_ws_handle_t net, void *cuda_stream);
int gfmd_ws_num_params(gfmd_ws_handle_t net, long long *count);
/* Copy parameters and/or the last gradient to host FP32 arrays (may be NULL);
 * layout per layer: W[cout][9][cin] (tap = 3 (dy+1) + (dx+1)), then b[cout]. */
int gfmd_ws_get_params(gfmd_ws_handle_t net, float *host_w, float *host_grad);
int gfmd_ws_set_params(gfmd_ws_handle_t net, const float *host_w);
int gfmd_ws_forward(gfmd_ws_handle_t net, int batch, int H, int W, const float *d_in, float *d_out);
/* Forward, mean-squared-error loss against d_target, backward; the gradient
 * stays in the handle for gfmd_ws_adam_step; *loss (may be NULL) is FP64. */
int gfmd_ws_loss_grad(gfmd_ws_handle_t net, int batch, int H, int W, const float *d_in,
                      const float *d_target, double *loss);
int gfmd_ws_adam_step(gfmd_ws_handle_t net, float lr, float beta1, float beta2, float eps);
/* Layout conversions between a solver grid [channels][nsite] (FP64) and one
 * NHWC image (FP32), with a scale factor. */
int gfmd_ws_to_nhwc(const double *d_u, int channels, int nsite, float scale, float *d_out,
                    void *cuda_stream);
int gfmd_ws_from_nhwc(const float *d_in, int channels, int nsite, double scale, double *d_u,
                      void *cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* GFMD_GB300_H */
