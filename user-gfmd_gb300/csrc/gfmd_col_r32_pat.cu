// Launches of the register-transform column kernel (gfmd_col_cluster.cuh)
// for ndof 12 tables stored in a layer-tridiagonal pattern (pat_keeps): the
// same kernel streaming only the pairs of the pattern.
#include <cuda_runtime.h>

#include "gfmd_internal.h"
#include "gfmd_col_cluster.cuh"

namespace gfmd {

cudaError_t enqueue_col_r32_pat(gfmd_solver *h, float2 *W, double *d_epot) {
  const int CL = h->col_cl;
  const bool n2k = h->g.nx == 2048;
  if (h->g.ndof != 12) return cudaErrorInvalidValue;
  if (CL == 6 && n2k) {
    if (h->phi_pat == 2) return launch_col_r32<12, 6, 11, 4, 2>(h, W, d_epot);
    if (h->phi_pat == 1) return launch_col_r32<12, 6, 11, 4, 1>(h, W, d_epot);
  }
  if (CL == 2 && !n2k) {
    if (h->phi_pat == 2) return launch_col_r32<12, 2, 10, 3, 2>(h, W, d_epot);
    if (h->phi_pat == 1) return launch_col_r32<12, 2, 10, 3, 1>(h, W, d_epot);
  }
  return cudaErrorInvalidValue;
}

}  // namespace gfmd
