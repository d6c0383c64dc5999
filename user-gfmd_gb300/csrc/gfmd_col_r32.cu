// Launches of the register-transform column kernel (gfmd_col_cluster.cuh)
// with every-pair tables, in a translation unit of their own so the build
// compiles them beside the other kernels.
#include <cuda_runtime.h>

#include "gfmd_internal.h"
#include "gfmd_col_cluster.cuh"

namespace gfmd {

cudaError_t enqueue_col_r32(gfmd_solver *h, float2 *W, double *d_epot) {
  const int D = h->g.ndof, CL = h->col_cl;
  const bool n2k = h->g.nx == 2048;
  if (D == 12 && h->phi_pat != 0) return enqueue_col_r32_pat(h, W, d_epot);
  if (D == 12 && CL == 6 && n2k) return launch_col_r32<12, 6, 11, 4>(h, W, d_epot);
  if (D == 12 && CL == 2 && !n2k) return launch_col_r32<12, 2, 10, 3>(h, W, d_epot);
  if (D == 6 && CL == 2 && n2k) return launch_col_r32<6, 2, 11, 3>(h, W, d_epot);
  if (D == 6 && CL == 1 && !n2k) return launch_col_r32<6, 1, 10, 3>(h, W, d_epot);
  if (D == 3 && CL == 1 && n2k) {  // 2048 / 1025 one-ky blocks: the residency sets the last wave
    if (h->col_minb == 4) return launch_col_r32<3, 1, 11, 4>(h, W, d_epot);
    if (h->col_minb == 2) return launch_col_r32<3, 1, 11, 2>(h, W, d_epot);
    return launch_col_r32<3, 1, 11, 3>(h, W, d_epot);
  }
  if (D == 3 && CL == 1 && !n2k) return launch_col_r32<3, 1, 10, 3>(h, W, d_epot);
  return cudaErrorInvalidValue;
}

}  // namespace gfmd
