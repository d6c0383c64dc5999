// GFMDSolverGB300: see gfmd_solver_gb300.h.
#include "gfmd_solver_gb300.h"

#include <cstdlib>
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
  if (h_) gfmd_destroy(h_);
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
}

double GFMDSolverGB300::post_force(void *u, void *f, char *dump_prefix) {
  // q-space dumps (dumpq_every) need the spectra on the host; this style
  // keeps them on the device, so it refuses rather than writing nothing
  if (dump_prefix) error->all(FLERR, "static/gb300 does not write q-space dumps (unset dumpq_every)");
  double e = 0.0;
  check(gfmd_post_force_host(h_, &static_cast<double **>(u)[0][0], &static_cast<double **>(f)[0][0], &e));
  check(gfmd_get_u0(h_, u0));
  return e;
}

void GFMDSolverGB300::prec_gradient(double *cavg, double **g, double **gP) {
  check(gfmd_prec_gradient_host(h_, cavg, &g[0][0], &gP[0][0]));
}

double GFMDSolverGB300::memory_usage() {
  double b = 0.0;
  if (h_) gfmd_memory_usage(h_, &b);
  return b;
}

GFMDSolverGB300Dynamic::GFMDSolverGB300Dynamic(LAMMPS *lmp, int narg, int *carg, char **arg)
    : GFMDSolverGB300(lmp, narg, carg, arg) {
  strcpy(name, "dynamic/gb300");
  if (carg && arg && *carg + 1 < narg && !strcmp(arg[*carg], "gamma")) {
    char *end = nullptr;
    gamma_ = strtod(arg[*carg + 1], &end);
    if (!end || *end != '\0' || !(gamma_ >= 0.0)) error->all(FLERR, "dynamic/gb300: gamma must be a number >= 0");
    *carg += 2;
  }
}

double GFMDSolverGB300Dynamic::post_force(void *u, void *f, char *dump_prefix) {
  double *fp = &static_cast<double **>(f)[0][0];
  const size_t n = (size_t)ndof * nx * ny;
  if (gamma_ > 0.0) v_.assign(fp, fp + n);  // the fix's velocities
  const double e = GFMDSolverGB300::post_force(u, f, dump_prefix);
  if (gamma_ > 0.0)
    for (size_t i = 0; i < n; i++) fp[i] -= gamma_ * v_[i];
  return e;
}
