/* ORACLE harness shim (project code): the members of LAMMPS' Comm that the
 * GFMD solver reads (src/main/gfmd_solver.cpp:67-68, 111-122). */
#ifndef GFMD_REF_SHIM_COMM_H
#define GFMD_REF_SHIM_COMM_H
namespace LAMMPS_NS {
class Comm {
 public:
  int me = 0, nprocs = 1;
  int procgrid[3] = {1, 1, 1};
};
}  // namespace LAMMPS_NS
#endif
