// GFMDSolverGB300: see gfmd_solver_gb300.h.
#include "gfmd_solver_gb300.h"

#include <cstring>
#include <vector>

#include "error.h"
#include "gfmd_misc.h"
#include "memory.h"
#include "surface_stiffness.h"

using namespace LAMMPS_NS;

GFMDSolverGB300::GFMDSolverGB300(LAMMPS *lmp, int narg, int *carg, char **arg) : GFMDSolver(lmp) {
  strcpy(name, "static/gb300");
  if (carg && arg && *carg < narg && !strcmp(arg[*carg], "f32")) {
    precision_ = GFMD_PREC_F32;
    (*carg)++;
  }
}

GFMDSolverGB300::~GFMDSolverGB300() {
  if (pre_) gfmd_destroy(pre_);
  if (h_) gfmd_destroy(h_);
  delete[] scratch_;
}

void GFMDSolverGB300::check(int rc) {
  if (rc != GFMD_OK) error->one(FLERR, gfmd_last_error());
}

void GFMDSolverGB300::set_grid_size(int in_nx, int in_ny, int in_ndof) {
  GFMDSolver::set_grid_size(in_nx, in_ny, in_ndof);  // xlo_loc ... for the fix
  if (nprocs != 1) error->all(FLERR, "static/gb300 owns the whole grid: run it on one rank");
  if (h_) gfmd_destroy(h_);
  h_ = nullptr;
  check(gfmd_create(nx, ny, ndof, precision_, &h_));
}

void GFMDSolverGB300::set_kernel(StiffnessKernel *kernel, bool normalize) {
  double_complex **phi = create_complex_operator_buffer("static/gb300:phi");
  fill_phi_buffer(ndof, nx, xlo_loc, xhi_loc, ny, ylo_loc, yhi_loc, kernel, phi, normalize, error);
  std::vector<double> linf(ndof / 3, 0.0);
  kernel->get_force_at_gamma_point(linf.data());
  check(gfmd_set_phi(h_, reinterpret_cast<double *>(&phi[0][0]), GFMD_PHI_FULL, linf.data()));
  destroy_complex_operator_buffer(phi);  // the library keeps its own packed copy
  if (pre_) gfmd_destroy(pre_);
  pre_ = nullptr;
  pre_shift_ = -1.0;
}

double GFMDSolverGB300::post_force(void *u, void *f, char *dump_prefix) {
  if (dump_prefix) error->all(FLERR, "static/gb300 does not write q-space dumps");
  double e = 0.0;
  check(gfmd_post_force_host(h_, &static_cast<double **>(u)[0][0], &static_cast<double **>(f)[0][0], &e));
  check(gfmd_get_u0(h_, u0));
  return e;
}

void GFMDSolverGB300::prec_gradient(double *cavg, double **g, double **gP) {
  const int nsq = ndof * ndof;
  for (int i = 0; i < nsq; i++)
    if (cavg[i] != ((i % (ndof + 1)) == 0 ? cavg[0] : 0.0))
      error->all(FLERR, "static/gb300 preconditions with Cavg = c I only");
  const double N = (double)nx * (double)ny;
  const double shift = N * cavg[0];
  if (!pre_ || shift != pre_shift_) {
    if (pre_) gfmd_destroy(pre_);
    pre_ = nullptr;
    check(gfmd_make_preconditioner(h_, shift, &pre_));
    pre_shift_ = shift;
  }
  const size_t n = (size_t)ndof * nxy_loc;
  if (!scratch_) scratch_ = new double[n];
  double e = 0.0;
  // the handle's evaluation returns -(Phi + shift)^{-1} g
  check(gfmd_post_force_host(pre_, &g[0][0], scratch_, &e));
  const double s = -N * N;
  for (size_t i = 0; i < n; i++) gP[0][i] = s * scratch_[i];
}

double GFMDSolverGB300::memory_usage() {
  double b = 0.0, p = 0.0;
  if (h_) gfmd_memory_usage(h_, &b);
  if (pre_) gfmd_memory_usage(pre_, &p);
  return b + p;
}
