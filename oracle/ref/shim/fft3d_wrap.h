/*
 * ORACLE harness shim (project code): LAMMPS' FFT3d with the semantics the
 * GFMD solver relies on (src/solvers/gfmd_solver_fft.cpp:72-80, 116, 181):
 * a serial 3-D complex transform with nfast = 1, i.e. a 2-D transform over
 * (nslow = nx) x (nmid = ny), y fastest; flag = +1 forward exp(-i),
 * flag = -1 backward exp(+i); unscaled (scaled = 0).  The arithmetic is the
 * oracle's own FFT (oracle/gfmd_oracle.c).
 */
#ifndef GFMD_REF_SHIM_FFT3D_WRAP_H
#define GFMD_REF_SHIM_FFT3D_WRAP_H
#include <string.h>
#include <stdexcept>
#include "pointers.h"
#include "gfmd_oracle.h"

namespace LAMMPS_NS {

class FFT3d : protected Pointers {
 public:
  FFT3d(LAMMPS *lmp, MPI_Comm, int nfast, int nmid, int nslow,
        int, int, int, int, int, int,
        int, int, int, int, int, int,
        int scaled, int, int *nbuf, int)
      : Pointers(lmp), nfast_(nfast), nmid_(nmid), nslow_(nslow) {
    if (nfast != 1 || scaled != 0)
      throw std::runtime_error("FFT3d shim: only nfast = 1, unscaled");
    if (nbuf) *nbuf = nmid * nslow;
  }
  void compute(double *in, double *out, int flag) {
    if (in != out) memcpy(out, in, sizeof(double) * 2 * (size_t)nmid_ * nslow_);
    if (orc_fft2d(out, nslow_, nmid_, flag, 1) != 0)
      throw std::runtime_error("FFT3d shim: transform failed");
  }
 private:
  int nfast_, nmid_, nslow_;
};

}  // namespace LAMMPS_NS
#endif
