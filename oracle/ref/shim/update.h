/* ORACLE harness shim (project code): LAMMPS' Update, step counter only. */
#ifndef GFMD_REF_SHIM_UPDATE_H
#define GFMD_REF_SHIM_UPDATE_H
#include "lmptype.h"
namespace LAMMPS_NS {
class Update {
 public:
  bigint ntimestep = 0;
};
}  // namespace LAMMPS_NS
#endif
