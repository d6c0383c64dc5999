// Force evaluation kernels: u(r) -> u(q) -> F(q) = -Phi(q) u(q) -> f(r).
//
// Pipeline (one evaluation), all on the handle's stream:
//   row_fwd   real rows along y -> half spectrum, written transposed into
//             W[ky][dof][x] (so every column along x is contiguous);
//   col_fft   forward complex transforms of the columns along x;
//   phi_apply per wavevector: energy partial, F = Phi_eff u, W = -F, linear
//             gamma-point force;
//   reduce    fixed-order sum of the energy partials (deterministic);
//   col_fft   backward transforms of the columns;
//   row_inv   half spectrum -> real rows, written to f[dof][x][y].
//
// Restates GFMDSolverStatic::post_force (src/solvers/gfmd_solver_static.cpp:145-249)
// with the per-DOF full complex FFTs of GFMDSolverFFT (src/solvers/gfmd_solver_fft.cpp:96-195)
// replaced by real-to-half-complex transforms.  The half spectrum is exact for
// the reference's result because gfmd_set_phi stores
// Phi_eff(k) = (Phi(k) + conj Phi(-k)) / 2, see gfmd_capi.cu.
#include <cuda_runtime.h>

#include <algorithm>

#include "gfmd_fft.cuh"
#include "gfmd_internal.h"
#include "gfmd_fast_kernels.cuh"
#include "gfmd_col_cluster.cuh"
#include "gfmd_plain_kernels.cuh"
#include "gfmd_rows_warp.cuh"

namespace gfmd {

namespace {

template <typename T> size_t csize() { return sizeof(C<T>); }

int rows_per_block(const Geom &g, size_t elem, size_t smem_max) {
  size_t per_row = 2 * (size_t)(g.nrow + 1) * elem;
  int rb = 8;
  while (rb > 1 && rb * per_row > smem_max) rb /= 2;
  return rb;
}

int cols_per_block(const Geom &g, size_t elem, size_t smem_max) {
  size_t per_col = 2 * (size_t)g.nx * elem;
  int cb = 4;
  while (cb > 1 && cb * per_col > smem_max) cb /= 2;
  return cb;
}

template <typename T, int D>
void launch_phi(gfmd_solver *h, dim3 grid, double *d_epot_unused) {
  (void)d_epot_unused;
  k_phi_apply<T, D><<<grid, kPhiThreads, 0, h->stream>>>(
      reinterpret_cast<C<T> *>(h->d_W), reinterpret_cast<const T *>(h->d_phi), h->g, h->d_linf,
      h->d_epart, h->d_scal);
}

template <typename T, int D>
void launch_col_fast(gfmd_solver *h, C<T> *W, size_t sm, double *d_epot) {
  using E = typename TwE<T>::type;
  auto kf = k_col_phi_fast<T, D>;
  cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  kf<<<h->g.nyc, ColThreads<T, D>::value, sm, h->stream>>>(
      W, reinterpret_cast<const T *>(h->d_phi), h->g, h->p2_col,
      reinterpret_cast<const E *>(h->d_ftw) + h->ftw_col_off, h->d_linf, h->d_epart, h->d_scal,
      h->d_counter, d_epot);
}

// Event i of a timed evaluation (gfmd_force_kernel_times), before launch i.
inline void mark(gfmd_solver *h, int i) {
  if (h->mark && i < h->nmark) cudaEventRecord(h->mark[i], h->stream);
}

// Cluster column kernel: CL blocks per ky (a thread-block cluster).
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

// Register-transform column kernel (nx = 2^LGN in {1024, 2048}).
template <int D, int CL, int LGN, int MINB>
cudaError_t launch_col_r32(gfmd_solver *h, float2 *W, double *d_epot) {
  constexpr int NT = (D / CL) * (1 << LGN) / 32;
  auto kf = k_col_phi_r32<D, CL, LGN, MINB>;
  const size_t sm = (size_t)(D / CL) * (1 << LGN) * sizeof(float2);
  cudaError_t e = cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(h->g.nyc * CL);
  cfg.blockDim = dim3(NT);
  cfg.dynamicSmemBytes = sm;
  cfg.stream = h->stream;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = CL;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kf, W, reinterpret_cast<const float *>(h->d_phi), h->g,
                            reinterpret_cast<const float4 *>(h->d_twc), (const double *)h->d_linf, h->d_epart,
                            h->d_scal, h->d_counter, d_epot, h->col_pf);
}

cudaError_t enqueue_col_cl(gfmd_solver *h, float2 *W, double *d_epot) {
  const int D = h->g.ndof, CL = h->col_cl;
  if (h->col_r32) {
    const bool n2k = h->g.nx == 2048;
    const bool m3 = h->col_minb == 3;
    if (D == 12 && CL == 3 && n2k)
      return m3 ? launch_col_r32<12, 3, 11, 3>(h, W, d_epot) : launch_col_r32<12, 3, 11, 2>(h, W, d_epot);
    if (D == 12 && CL == 2 && !n2k) return launch_col_r32<12, 2, 10, 3>(h, W, d_epot);
    if (D == 6 && CL == 2 && n2k) return launch_col_r32<6, 2, 11, 3>(h, W, d_epot);
    if (D == 6 && CL == 1 && !n2k) return launch_col_r32<6, 1, 10, 3>(h, W, d_epot);
    if (D == 3 && CL == 1 && n2k) return launch_col_r32<3, 1, 11, 3>(h, W, d_epot);
    if (D == 3 && CL == 1 && !n2k) return launch_col_r32<3, 1, 10, 3>(h, W, d_epot);
    return cudaErrorInvalidValue;
  }
  if (D == 3 && CL == 1) return launch_col_cl<3, 1, 1>(h, W, d_epot);
  if (D == 6 && CL == 1) return launch_col_cl<6, 1, 4>(h, W, d_epot);
  if (D == 6 && CL == 2) return launch_col_cl<6, 2, 4>(h, W, d_epot);
  if (D == 12 && CL == 1) return launch_col_cl<12, 1, 4>(h, W, d_epot);
  if (D == 12 && CL == 2) return launch_col_cl<12, 2, 4>(h, W, d_epot);
  if (D == 12 && CL == 4) return launch_col_cl<12, 4, 4>(h, W, d_epot);
  return cudaErrorInvalidValue;
}

// Persistent blocks of the warp-per-row kernels: as many as fit on the GPU
// (2 per SM with 8-row blocks, 1 with 16-row blocks), at most one per row set.
inline int row_blocks(const gfmd_solver *h, int rb) {
  const int nsets = h->g.nx / rb * h->g.ndof;
  return std::max(1, std::min(nsets, (rb == 8 ? 2 : 1) * std::max(1, h->sm_count)));
}

// Warp-per-row row kernels with TMA tiles (FP32 handles, ny = 2048).
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
template <int RB> cudaError_t row_fwd32(gfmd_solver *h, const void *d_u, int in_t) {
  return in_t == 0 ? launch_row_fwd32<double, RB>(h, d_u) : launch_row_fwd32<float, RB>(h, d_u);
}
template <int RB> cudaError_t row_inv32(gfmd_solver *h, void *d_f, int out_t) {
  return out_t == 0 ? launch_row_inv32<double, RB>(h, d_f) : launch_row_inv32<float, RB>(h, d_f);
}

// Fused power-of-two path: three launches.  FP32 handles use the
// warp-per-row TMA row kernels where the row length allows (rows32) and the
// cluster column kernel where it has an instance (col_cl > 0).
template <typename T>
cudaError_t enqueue_fast(gfmd_solver *h, const void *d_u, int in_t, void *d_f, int out_t,
                         double *d_epot) {
  using E = typename TwE<T>::type;
  const Geom &g = h->g;
  const E *tab_row = reinterpret_cast<const E *>(h->d_ftw);
  C<T> *W = reinterpret_cast<C<T> *>(h->d_W);
  const int rb = h->fast_rb;
  const size_t smr = (size_t)h->p2_row.tsize * sizeof(E) + srev_bytes(g.nrow) +
                     (size_t)rb * (g.nrow + 1) * sizeof(C<T>);
  dim3 gridr((g.nx + rb - 1) / rb, g.ndof);
  constexpr bool f32 = sizeof(T) == 4;
  cudaError_t e = cudaSuccess;

  mark(h, 0);
  if (f32 && h->rows32) {
    e = h->row_rb == 16 ? row_fwd32<16>(h, d_u, in_t) : row_fwd32<8>(h, d_u, in_t);
  } else if (in_t == 0) {
    auto kf = k_row_fwd_fast<T, double>;
    cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr);
    kf<<<gridr, kRowThreads, smr, h->stream>>>(reinterpret_cast<const double *>(d_u), W, g, h->p2_row, tab_row, rb);
  } else {
    auto kf = k_row_fwd_fast<T, float>;
    cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr);
    kf<<<gridr, kRowThreads, smr, h->stream>>>(reinterpret_cast<const float *>(d_u), W, g, h->p2_row, tab_row, rb);
  }
  if (e != cudaSuccess) return e;

  mark(h, 1);
  if (f32 && h->col_cl > 0) {
    e = enqueue_col_cl(h, reinterpret_cast<float2 *>(W), d_epot);
  } else {
    const size_t smc = (size_t)h->p2_col.tsize * sizeof(E) + (size_t)g.ndof * g.nx * sizeof(C<T>);
    switch (g.ndof) {
      case 3: launch_col_fast<T, 3>(h, W, smc, d_epot); break;
      case 6: launch_col_fast<T, 6>(h, W, smc, d_epot); break;
      case 9: launch_col_fast<T, 9>(h, W, smc, d_epot); break;
      case 12: launch_col_fast<T, 12>(h, W, smc, d_epot); break;
      case 15: launch_col_fast<T, 15>(h, W, smc, d_epot); break;
      case 18: launch_col_fast<T, 18>(h, W, smc, d_epot); break;
      case 21: launch_col_fast<T, 21>(h, W, smc, d_epot); break;
      case 24: launch_col_fast<T, 24>(h, W, smc, d_epot); break;
      default: return cudaErrorInvalidValue;
    }
  }
  if (e != cudaSuccess) return e;

  mark(h, 2);
  if (f32 && h->rows32) {
    e = h->row_rb == 16 ? row_inv32<16>(h, d_f, out_t) : row_inv32<8>(h, d_f, out_t);
  } else if (out_t == 0) {
    auto kf = k_row_inv_fast<T, double>;
    cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr);
    kf<<<gridr, kRowThreads, smr, h->stream>>>(W, reinterpret_cast<double *>(d_f), g, h->p2_row, tab_row, rb);
  } else {
    auto kf = k_row_inv_fast<T, float>;
    cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr);
    kf<<<gridr, kRowThreads, smr, h->stream>>>(W, reinterpret_cast<float *>(d_f), g, h->p2_row, tab_row, rb);
  }
  if (e != cudaSuccess) return e;
  mark(h, 3);
  return cudaGetLastError();
}

template <typename T>
cudaError_t enqueue_t(gfmd_solver *h, const void *d_u, int in_t, void *d_f, int out_t,
                      double *d_epot) {
  if (h->fast) return enqueue_fast<T>(h, d_u, in_t, d_f, out_t, d_epot);
  const Geom &g = h->g;
  Tw<T> tw;
  tw.hi = reinterpret_cast<decltype(tw.hi)>(h->d_tw_hi);
  if constexpr (sizeof(T) == 4) tw.lo = reinterpret_cast<const float2 *>(h->d_tw_lo);
  else tw.lo_unused = nullptr;
  C<T> *W = reinterpret_cast<C<T> *>(h->d_W);
  const size_t smax = h->smem_optin;

  // row_fwd
  mark(h, 0);
  {
    int rb = rows_per_block(g, sizeof(C<T>), smax);
    size_t sm = 2 * (size_t)rb * (g.nrow + 1) * sizeof(C<T>);
    dim3 grid((g.nx + rb - 1) / rb, g.ndof);
    if (in_t == 0) {
      auto kf = k_row_fwd<T, double>;
      cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      kf<<<grid, kThreads, sm, h->stream>>>(reinterpret_cast<const double *>(d_u), W, g, h->plan_row, tw, rb);
    } else {
      auto kf = k_row_fwd<T, float>;
      cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      kf<<<grid, kThreads, sm, h->stream>>>(reinterpret_cast<const float *>(d_u), W, g, h->plan_row, tw, rb);
    }
  }
  // col_fft forward
  mark(h, 1);
  int cb = cols_per_block(g, sizeof(C<T>), smax);
  size_t smc = 2 * (size_t)cb * g.nx * sizeof(C<T>);
  dim3 gridc((g.nyc * g.ndof + cb - 1) / cb);
  cudaFuncSetAttribute(k_col_fft<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc);
  k_col_fft<T><<<gridc, kThreads, smc, h->stream>>>(W, g, h->plan_col, tw, cb, -1);
  // phi
  mark(h, 2);
  dim3 gridp((g.nx + kPhiThreads - 1) / kPhiThreads, g.nyc);
  switch (g.ndof) {
    case 3: launch_phi<T, 3>(h, gridp, d_epot); break;
    case 6: launch_phi<T, 6>(h, gridp, d_epot); break;
    case 9: launch_phi<T, 9>(h, gridp, d_epot); break;
    case 12: launch_phi<T, 12>(h, gridp, d_epot); break;
    case 15: launch_phi<T, 15>(h, gridp, d_epot); break;
    case 18: launch_phi<T, 18>(h, gridp, d_epot); break;
    case 21: launch_phi<T, 21>(h, gridp, d_epot); break;
    case 24: launch_phi<T, 24>(h, gridp, d_epot); break;
    default: return cudaErrorInvalidValue;
  }
  mark(h, 3);
  k_reduce<<<1, 256, 0, h->stream>>>(h->d_epart, (int)(gridp.x * gridp.y), d_epot);
  // col_fft backward
  mark(h, 4);
  k_col_fft<T><<<gridc, kThreads, smc, h->stream>>>(W, g, h->plan_col, tw, cb, +1);
  // row_inv
  mark(h, 5);
  {
    int rb = rows_per_block(g, sizeof(C<T>), smax);
    size_t sm = 2 * (size_t)rb * (g.nrow + 1) * sizeof(C<T>);
    dim3 grid((g.nx + rb - 1) / rb, g.ndof);
    if (out_t == 0) {
      auto kf = k_row_inv<T, double>;
      cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      kf<<<grid, kThreads, sm, h->stream>>>(W, reinterpret_cast<double *>(d_f), g, h->plan_row, tw, rb);
    } else {
      auto kf = k_row_inv<T, float>;
      cudaFuncSetAttribute(kf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      kf<<<grid, kThreads, sm, h->stream>>>(W, reinterpret_cast<float *>(d_f), g, h->plan_row, tw, rb);
    }
  }
  mark(h, 6);
  return cudaGetLastError();
}

}  // namespace

void force_layout(const Geom &g, int precision, size_t *w_bytes, size_t *phi_bytes, int *n_epart) {
  size_t s = precision == GFMD_PREC_F64 ? 8 : 4;
  *w_bytes = (size_t)g.nyc * g.ndof * g.nxp * 2 * s;
  *phi_bytes = (size_t)g.nyc * g.npk * g.nxp * s;
  // plain path: one partial per phi_apply block; fused paths: one per
  // column block (up to 4 per ky for the cluster column kernel)
  *n_epart = std::max((g.nx + kPhiThreads - 1) / kPhiThreads, 4) * g.nyc;
}

int force_launches(const gfmd_solver *h) { return h->fast ? 3 : 6; }

cudaError_t enqueue_force(gfmd_solver *h, const void *d_u, int in_t, void *d_f, int out_t,
                          double *d_epot) {
  if (h->precision == GFMD_PREC_F64) return enqueue_t<double>(h, d_u, in_t, d_f, out_t, d_epot);
  return enqueue_t<float>(h, d_u, in_t, d_f, out_t, d_epot);
}

cudaError_t enqueue_force_opts(gfmd_solver *h, const void *d_u, int in_t, void *d_f, int out_t,
                               double *d_epot, bool with_linf) {
  double *keep = h->d_linf;
  if (!with_linf) h->d_linf = h->d_zero;
  cudaError_t e = enqueue_force(h, d_u, in_t, d_f, out_t, d_epot);
  h->d_linf = keep;
  return e;
}

}  // namespace gfmd
