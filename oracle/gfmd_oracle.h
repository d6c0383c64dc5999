/*
 * ORACLE — test infrastructure, not product code.
 *
 * Plain-C FP64 restatement of the USER-GFMD force evaluation
 * (GFMDSolverStatic::post_force, src/solvers/gfmd_solver_static.cpp:145-249)
 * and of the solver loops built around it.  Only tests/, the smoke check and
 * the CPU-baseline leg of bench.py may load this library; the product path
 * never links or calls it.
 *
 * Parity status: pinned.  The restatement is checked against outputs of the
 * reference's own, unmodified GFMDSolverStatic::post_force and
 * fill_phi_buffer (compiled from the reference sources by oracle/ref/Makefile
 * into oracle/_ref/), stored as fixtures under tests/golden/.
 *
 * Conventions (those of the reference with LAMMPS >= patch_10Feb2021,
 * README.md:36-38 of the reference):
 *   forward  transform  u(q) = sum_r u(r) exp(-i q.r), unscaled;
 *   backward transform  f(r) = sum_q f(q) exp(+i q.r), unscaled;
 *   Phi(q) pre-scaled by 1/(nx*ny) (src/main/gfmd_misc.cpp:88-97).
 * Grid layout: index = ix*ny + iy (y fastest), as FFT3d(1, ny, nx) in
 * src/solvers/gfmd_solver_fft.cpp:72-80.
 */
#ifndef GFMD_ORACLE_H
#define GFMD_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* 1-D complex FFT plan (mixed radix 2/3/4/5/generic, Stockham). */
typedef struct orc_fft_plan orc_fft_plan;

orc_fft_plan *orc_fft_plan_create(int n);
void orc_fft_plan_destroy(orc_fft_plan *p);
/* In-place transform of n interleaved complex values.  sign = -1 gives
 * exp(-i...), +1 gives exp(+i...); unscaled.  work holds 2n doubles. */
void orc_fft_exec(const orc_fft_plan *p, double *data, double *work, int sign);

/* 2-D complex FFT over an nx*ny grid (index ix*ny+iy), interleaved complex.
 * flag = +1 forward (exp(-i)), -1 backward (exp(+i)): the semantics of
 * LAMMPS FFT3d::compute(in, out, flag) with scaled = 0.  Returns 0 on
 * success.  nthreads <= 0 uses all available threads. */
int orc_fft2d(double *data, int nx, int ny, int flag, int nthreads);

/* Restatement of GFMDSolverStatic::post_force for a single process
 * (xlo_loc = ylo_loc = 0, gammai_ = 0).
 *   phi : [nx*ny][ndof*ndof] complex interleaved, row-major per q (MEL),
 *         pre-scaled by 1/(nx*ny) as fill_phi_buffer leaves it;
 *   linf: [ndof/3] linear force per layer (may be NULL = zeros);
 *   u   : [ndof][nx*ny] displacements;  f: [ndof][nx*ny] forces (out);
 *   u0  : [ndof] q=0 displacement (out, may be NULL).
 * Returns the elastic energy. */
double orc_post_force(int nx, int ny, int ndof, const double *phi,
                      const double *linf, const double *u, double *f,
                      double *u0, int nthreads);

/* The same with the table given on the stored half spectrum
 * [nx][ny/2+1][ndof][ndof] (the layout the GPU path uploads): entries with
 * ky > ny/2 are read as conj Phi(-q), the relation fill_phi_buffer's tables
 * satisfy for the ft kernels.  Identical arithmetic to orc_post_force on the
 * expanded table, without its nx*ny*ndof^2 complex memory (9.7 GB at 2048^2,
 * ndof 12). */
double orc_post_force_half(int nx, int ny, int ndof, const double *phi_half,
                           const double *linf, const double *u, double *f,
                           double *u0, int nthreads);

/* Fills a full-grid table [nx*ny][ndof][ndof] with seeded pseudo-random
 * Hermitian matrices (diagonal 2*scale + U(-scale/2, scale/2), off-diagonal
 * parts U(-scale/2, scale/2)) that satisfy Phi(-q) = conj Phi(q) exactly.
 * Timing input only: the operation count of orc_post_force does not depend
 * on the table's values. */
void orc_synthetic_phi_full(int nx, int ny, int ndof, unsigned long long seed, double scale,
                            double *full, int nthreads);

/* Expand a half-spectrum table [nx][ny/2+1][ndof][ndof] to the full grid
 * [nx*ny][ndof][ndof] using Phi(-q) = conj Phi(q) (test and baseline input
 * preparation; the reference itself computes every grid point). */
void orc_phi_half_to_full(int nx, int ny, int ndof, const double *half, double *full,
                          int nthreads);

/* Number of threads the oracle uses when nthreads <= 0. */
int orc_max_threads(void);

#ifdef __cplusplus
}
#endif

#endif
