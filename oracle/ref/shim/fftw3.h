/*
 * ORACLE harness shim (project code): the three FFTW3 calls the reference's
 * NonperiodicStiffnessKernel makes (src/stiffness_kernels/
 * nonperiodic_stiffness.cpp:114-189): an in-place 2-D complex transform over
 * n0 x n1 (n1 fastest), unscaled, sign -1 = exp(-i), +1 = exp(+i) as FFTW
 * defines them.  The arithmetic is the oracle's own FFT (oracle/gfmd_oracle.c),
 * whose flag has the opposite sense (+1 = exp(-i)).  FFTW itself is not
 * installed on these machines.
 */
#ifndef GFMD_REF_SHIM_FFTW3_H
#define GFMD_REF_SHIM_FFTW3_H
#include <stdexcept>
#include "gfmd_oracle.h"

typedef double fftw_complex[2];

struct gfmd_shim_fftw_plan {
  int n0, n1, sign;
};
typedef gfmd_shim_fftw_plan *fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_ESTIMATE (1U << 6)

inline fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex *, fftw_complex *, int sign,
                                  unsigned) {
  return new gfmd_shim_fftw_plan{n0, n1, sign};
}

inline void fftw_execute_dft(const fftw_plan p, fftw_complex *in, fftw_complex *out) {
  if (in != out) throw std::runtime_error("fftw3 shim: in-place transforms only");
  if (orc_fft2d(&in[0][0], p->n0, p->n1, -p->sign, 1) != 0)
    throw std::runtime_error("fftw3 shim: transform failed");
}

inline void fftw_destroy_plan(fftw_plan p) { delete p; }

#endif
