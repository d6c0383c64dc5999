// Launches of the per-wavevector Phi application of the general-size path
// (k_phi_apply, gfmd_plain_kernels.cuh) for FP32 handles, one instance per
// ndof, in a translation unit of their own so the build compiles them beside
// the other kernels.
#include <cuda_runtime.h>

#include "gfmd_internal.h"
#include "gfmd_fft.cuh"
#include "gfmd_plain_kernels.cuh"

namespace gfmd {

namespace {

template <typename T, int D, int PAT = 0> cudaError_t launch_phi(gfmd_solver *h, dim3 grid) {
  k_phi_apply<T, D, PAT><<<grid, kPhiThreads, 0, h->stream>>>(reinterpret_cast<C<T> *>(h->d_W),
                                                         reinterpret_cast<const T *>(h->d_phi), h->g, h->d_linf,
                                                         h->d_epart, h->d_scal);
  return cudaGetLastError();
}

template <typename T> cudaError_t phi_t(gfmd_solver *h, dim3 grid) {
  switch (h->g.ndof) {
    case 3: return launch_phi<T, 3>(h, grid);
    case 6: return launch_phi<T, 6>(h, grid);
    case 9: return launch_phi<T, 9>(h, grid);
    case 12:  // layer-tridiagonal tables stream and multiply only their kept pairs
      if (h->phi_pat == 2) return launch_phi<T, 12, 2>(h, grid);
      if (h->phi_pat == 1) return launch_phi<T, 12, 1>(h, grid);
      return launch_phi<T, 12>(h, grid);
    case 15: return launch_phi<T, 15>(h, grid);
    case 18: return launch_phi<T, 18>(h, grid);
    case 21: return launch_phi<T, 21>(h, grid);
    case 24: return launch_phi<T, 24>(h, grid);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t enqueue_phi_plain_f32(gfmd_solver *h, dim3 grid) { return phi_t<float>(h, grid); }

}  // namespace gfmd
