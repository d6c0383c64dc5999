/*
 * ORACLE harness shim (project code): a minimal LAMMPS instance and the
 * Pointers base class, carrying only the members the GFMD solver classes
 * touch (memory, error, comm, domain, screen, world, suffix).
 */
#ifndef GFMD_REF_SHIM_POINTERS_H
#define GFMD_REF_SHIM_POINTERS_H
#include <stdio.h>
#include "mpi.h"
#include "lmptype.h"
#include "error.h"
#include "memory.h"
#include "domain.h"
#include "comm.h"
#include "update.h"

namespace LAMMPS_NS {

class LAMMPS {
 public:
  Memory *memory = nullptr;
  Error *error = nullptr;
  Comm *comm = nullptr;
  Domain *domain = nullptr;
  Update *update = nullptr;
  FILE *screen = nullptr;
  FILE *logfile = nullptr;
  MPI_Comm world = MPI_COMM_WORLD;
  int suffix_enable = 0;
  char *suffix = nullptr;
};

class Pointers {
 public:
  explicit Pointers(LAMMPS *ptr)
      : lmp(ptr), memory(ptr->memory), error(ptr->error), comm(ptr->comm),
        domain(ptr->domain), update(ptr->update), screen(ptr->screen),
        logfile(ptr->logfile), world(ptr->world) {}
  virtual ~Pointers() {}

 protected:
  LAMMPS *lmp;
  Memory *memory;
  Error *error;
  Comm *comm;
  Domain *domain;
  Update *update;
  FILE *screen;
  FILE *logfile;
  MPI_Comm world;
};

}  // namespace LAMMPS_NS
#endif
