// Launches of the fused shared-memory column kernel (gfmd_fast_kernels.cuh)
// for FP64 handles, one instance per ndof, in a translation unit of
// their own so the build compiles them beside the other kernels.
#include <cuda_runtime.h>

#include "gfmd_internal.h"
#include "gfmd_fast_kernels.cuh"

namespace gfmd {

namespace {

template <typename T, int D>
cudaError_t launch_col_fast(gfmd_solver *h, C<T> *W, size_t sm, double *d_epot) {
  using E = typename TwE<T>::type;
  auto kf = k_col_phi_fast<T, D>;
  cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  kf<<<h->g.nyc, ColThreads<T, D>::value, sm, h->stream>>>(
      W, reinterpret_cast<const T *>(h->d_phi), h->g, h->p2_col,
      reinterpret_cast<const E *>(h->d_ftw) + h->ftw_col_off, h->d_linf, h->d_epart, h->d_scal,
      h->d_counter, d_epot);
  return cudaSuccess;
}

}  // namespace

cudaError_t enqueue_col_fast_f64(gfmd_solver *h, void *W, size_t smem, double *d_epot) {
  C<double> *w = reinterpret_cast<C<double> *>(W);
  switch (h->g.ndof) {
    case 3: return launch_col_fast<double, 3>(h, w, smem, d_epot);
    case 6: return launch_col_fast<double, 6>(h, w, smem, d_epot);
    case 9: return launch_col_fast<double, 9>(h, w, smem, d_epot);
    case 12: return launch_col_fast<double, 12>(h, w, smem, d_epot);
    case 15: return launch_col_fast<double, 15>(h, w, smem, d_epot);
    case 18: return launch_col_fast<double, 18>(h, w, smem, d_epot);
    case 21: return launch_col_fast<double, 21>(h, w, smem, d_epot);
    case 24: return launch_col_fast<double, 24>(h, w, smem, d_epot);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace gfmd
