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

// Event i of a timed evaluation (gfmd_force_kernel_times), before launch i.
inline void mark(gfmd_solver *h, int i) {
  if (h->mark && i < h->nmark) cudaEventRecord(h->mark[i], h->stream);
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
    e = enqueue_row_fwd32(h, d_u, in_t);
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
    e = f32 ? enqueue_col_fast_f32(h, W, smc, d_epot) : enqueue_col_fast_f64(h, W, smc, d_epot);
  }
  if (e != cudaSuccess) return e;

  mark(h, 2);
  if (f32 && h->rows32) {
    e = enqueue_row_inv32(h, d_f, out_t);
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
  {
    const cudaError_t ep = sizeof(T) == 8 ? enqueue_phi_plain_f64(h, gridp) : enqueue_phi_plain_f32(h, gridp);
    if (ep != cudaSuccess) return ep;
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
