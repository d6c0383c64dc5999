// Launches of the warp-per-row row transforms with TMA-staged spectrum tiles
// (gfmd_rows_warp.cuh; FP32 handles, rows of ny = 2048).
#include <cuda_runtime.h>

#include <algorithm>

#include "gfmd_internal.h"
#include "gfmd_rows_warp.cuh"

namespace gfmd {

namespace {

// Persistent blocks: as many as fit on the GPU (2 per SM with 8-row blocks,
// 1 with 16-row blocks), at most one per row set.
inline int row_blocks(const gfmd_solver *h, int rb) {
  const int nsets = h->g.nx / rb * h->g.ndof;
  return std::max(1, std::min(nsets, (rb == 8 ? 2 : 1) * std::max(1, h->sm_count)));
}

template <typename Tin, int RB> cudaError_t launch_row_fwd32(gfmd_solver *h, const void *d_u) {
  using K = rows32::Cfg<RB>;
  auto kf = k_row_fwd_w32<Tin, RB>;
  cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K::kSmemBytes);
  if (e != cudaSuccess) return e;
  const float4 *tw = reinterpret_cast<const float4 *>(h->d_tw32);
  kf<<<row_blocks(h, RB), K::kThreads, K::kSmemBytes, h->stream>>>(
      reinterpret_cast<const Tin *>(d_u), reinterpret_cast<float2 *>(h->d_W), h->tm_w[RB == 8 ? 0 : 1], h->g, tw,
      tw + 1024);
  return cudaSuccess;
}
template <typename Tout, int RB> cudaError_t launch_row_inv32(gfmd_solver *h, void *d_f) {
  using K = rows32::Cfg<RB>;
  auto kf = k_row_inv_w32<Tout, RB>;
  cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)K::kSmemBytes);
  if (e != cudaSuccess) return e;
  const float4 *tw = reinterpret_cast<const float4 *>(h->d_tw32);
  kf<<<row_blocks(h, RB), K::kThreads, K::kSmemBytes, h->stream>>>(
      reinterpret_cast<const float2 *>(h->d_W), h->tm_w[RB == 8 ? 0 : 1], reinterpret_cast<Tout *>(d_f), h->g, tw,
      tw + 1024, h->d_err);
  return cudaSuccess;
}

}  // namespace

cudaError_t enqueue_row_fwd32(gfmd_solver *h, const void *d_u, int in_t) {
  if (h->row_rb == 16)
    return in_t == 0 ? launch_row_fwd32<double, 16>(h, d_u) : launch_row_fwd32<float, 16>(h, d_u);
  return in_t == 0 ? launch_row_fwd32<double, 8>(h, d_u) : launch_row_fwd32<float, 8>(h, d_u);
}
cudaError_t enqueue_row_inv32(gfmd_solver *h, void *d_f, int out_t) {
  if (h->row_rb == 16)
    return out_t == 0 ? launch_row_inv32<double, 16>(h, d_f) : launch_row_inv32<float, 16>(h, d_f);
  return out_t == 0 ? launch_row_inv32<double, 8>(h, d_f) : launch_row_inv32<float, 8>(h, d_f);
}

}  // namespace gfmd
