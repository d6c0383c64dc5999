// Launches of the thread-block-cluster column kernel (gfmd_col_cluster.cuh):
// CL blocks per ky exchanging their columns through distributed shared
// memory; the register-transform variant is launched from gfmd_col_r32.cu.
#include <cuda_runtime.h>

#include "gfmd_internal.h"
#include "gfmd_col_cluster.cuh"

namespace gfmd {

namespace {

template <int D, int CL, int V>
cudaError_t launch_col_cl(gfmd_solver *h, float2 *W, double *d_epot) {
  auto kf = k_col_phi_cl<D, CL, V>;
  const size_t sm = (size_t)(D / CL) * h->g.nx * sizeof(float2);
  cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(h->g.nyc * CL);
  cfg.blockDim = dim3(colcl::kThreads);
  cfg.dynamicSmemBytes = sm;
  cfg.stream = h->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kf, W, reinterpret_cast<const float *>(h->d_phi), h->g, h->p2_col,
                            reinterpret_cast<const float4 *>(h->d_ftw) + h->ftw_col_off,
                            (const double *)h->d_linf, h->d_epart, h->d_scal, h->d_counter, d_epot);
}

}  // namespace

cudaError_t enqueue_col_cl(gfmd_solver *h, float2 *W, double *d_epot) {
  const int D = h->g.ndof, CL = h->col_cl;
  if (h->col_r32) return enqueue_col_r32(h, W, d_epot);
  if (D == 3 && CL == 1) return launch_col_cl<3, 1, 1>(h, W, d_epot);
  if (D == 6 && CL == 1) return launch_col_cl<6, 1, 4>(h, W, d_epot);
  if (D == 6 && CL == 2) return launch_col_cl<6, 2, 4>(h, W, d_epot);
  if (D == 12 && CL == 1) return launch_col_cl<12, 1, 4>(h, W, d_epot);
  if (D == 12 && CL == 2) return launch_col_cl<12, 2, 4>(h, W, d_epot);
  if (D == 12 && CL == 4) return launch_col_cl<12, 4, 4>(h, W, d_epot);
  return cudaErrorInvalidValue;
}

}  // namespace gfmd
