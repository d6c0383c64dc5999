// Builds GFMDSolverGB300 the way USER-GFMD's fix does (constructor, grid,
// kernel) in the oracle's LAMMPS stand-in environment and reports how far it
// got: "ok" when the library accepted the grid and the table, or the
// library's error message (e.g. no GPU).  Used by tests/test_lammps_shim.py.
#include <cstdio>
#include <exception>
#include <stdexcept>
#include <sstream>
#include <string>
#include <vector>

#include "comm.h"
#include "domain.h"
#include "error.h"
#include "force.h"
#include "gfmd_solver_gb300.h"
#include "memory.h"
#include "surface_stiffness.h"
#include "update.h"

using namespace LAMMPS_NS;

int main(int argc, char **argv) {
  Error error;
  Memory memory{&error};
  Comm comm;
  Domain domain;
  Update update;
  LAMMPS lmp;
  lmp.memory = &memory;
  lmp.error = &error;
  lmp.comm = &comm;
  lmp.domain = &domain;
  lmp.update = &update;
  lmp.screen = nullptr;
  const char *kargs = argc > 1 ? argv[1] : "ft sc100 1.0 1 pair-potential 2 1.0 1.0 height 16";
  std::vector<std::string> tok;
  std::istringstream is(kargs);
  for (std::string t; is >> t;) tok.push_back(t);
  std::vector<char *> av;
  for (auto &t : tok) av.push_back(&t[0]);
  try {
    int carg = 0;
    GFMDSolverGB300 solver(&lmp, 0, &carg, av.data());
    int karg = 1;
    StiffnessKernel *k = stiffness_kernel_factory(av[karg], (int)av.size(), &karg, av.data(), &domain,
                                                  nullptr, &memory, &error);
    std::string styles = "static/gb300";
    if (argc > 2 && std::string(argv[2]) == "dynamic") {
      // the dynamic style: gamma parsed, velocities in f damped
      char g0[] = "gamma", g1[] = "0.25";
      char *dargs[] = {g0, g1};
      int dc = 0;
      GFMDSolverGB300Dynamic dyn(&lmp, 2, &dc, dargs);
      if (dc != 2 || dyn.gamma() != 0.25) throw std::runtime_error("dynamic/gb300: arguments not parsed");
      styles = dyn.get_name();
      dyn.set_grid_size(16, 16, k->get_dimension());
      dyn.set_kernel(k, true);
    } else {
      solver.set_grid_size(16, 16, k->get_dimension());
      solver.set_kernel(k, true);
    }
    std::printf("ok %s\n", styles.c_str());
  } catch (const std::exception &e) {
    std::printf("error %s\n", e.what());
  }
  return 0;
}
