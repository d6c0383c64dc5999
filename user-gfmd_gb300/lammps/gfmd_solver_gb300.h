// USER-GFMD solver style "static/gb300": the reference's GFMDSolver interface
// (src/main/gfmd_solver.h:34-123) implemented over the C ABI of
// libgfmd_gb300 (include/gfmd_gb300.h).  Drop into USER-GFMD's src/solvers/
// and register in gfmd_solver_factory (src/main/gfmd_solver.cpp:209-256):
//   else if (!strcmp(solver_name, "static/gb300"))
//     solver = new GFMDSolverGB300(lmp, narg, carg, arg);
// Input syntax is unchanged (`fix ... gfmd ... solver static/gb300`, or the
// `static` style with `-sf gb300`).  One rank owns the whole grid.
#ifndef GFMD_SOLVER_GB300_H
#define GFMD_SOLVER_GB300_H

#include <vector>

#include "gfmd_gb300.h"
#include "gfmd_solver.h"

namespace LAMMPS_NS {

class GFMDSolverGB300 : public GFMDSolver {
 public:
  // Optional argument (carg points at it in arg): "f32" for the FP32
  // compensated-twiddle evaluation; FP64 otherwise.
  GFMDSolverGB300(LAMMPS *lmp, int narg, int *carg, char **arg);
  ~GFMDSolverGB300() override;

  void set_grid_size(int nx, int ny, int ndof) override;
  // GFMDSolverStatic::set_kernel (src/solvers/gfmd_solver_static.cpp:90-136):
  // the table from fill_phi_buffer, uploaded once
  void set_kernel(StiffnessKernel *kernel, bool normalize = true) override;
  // GFMDSolverStatic::post_force (gfmd_solver_static.cpp:145-249); u and f
  // are FixGFMD's contiguous double** [ndof][nxy] (memory->create)
  double post_force(void *u, void *f, char *dump_prefix) override;
  // GFMDSolverStatic::prec_gradient (gfmd_solver_static.cpp:253-269):
  // gP = IFFT((Phi/N + Cavg)^{-1} FFT(g)), unnormalised transforms, Cavg a
  // symmetric ndof x ndof matrix (gfmd_prec_gradient_host)
  void prec_gradient(double *cavg, double **g, double **gP) override;
  double memory_usage() override;

  gfmd_handle_t handle() const { return h_; }

 private:
  gfmd_handle_t h_ = nullptr;
  int precision_ = GFMD_PREC_F64;
  void check(int rc);
};

// USER-GFMD solver style "dynamic/gb300": damped GFMD dynamics for a fix
// gfmd integrated by LAMMPS (fix nve).  FixGFMD hands a dynamic solver the
// atoms' velocities in the force buffer (src/main/fix_gfmd.cpp:782-793,
// "Velocities are needed for the dynamic GFMD only"); this style returns the
// elastic force of u minus the linear damping force, f = F_el(u) - gamma v
// (unit masses), the same damping gfmd_run_dynamics integrates.  Register
// beside static/gb300:
//   else if (!strcmp(solver_name, "dynamic/gb300"))
//     solver = new GFMDSolverGB300Dynamic(lmp, narg, carg, arg);
// Arguments after the style name: optional "f32", then optional
// "gamma <value>" (default 0: undamped).
class GFMDSolverGB300Dynamic : public GFMDSolverGB300 {
 public:
  GFMDSolverGB300Dynamic(LAMMPS *lmp, int narg, int *carg, char **arg);
  double post_force(void *u, void *f, char *dump_prefix) override;
  double gamma() const { return gamma_; }

 private:
  double gamma_ = 0.0;
  std::vector<double> v_;  // velocities taken from the force buffer
};

}  // namespace LAMMPS_NS

#endif
