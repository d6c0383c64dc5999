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

namespace gfmd {

namespace {

constexpr int kThreads = 256;
constexpr int kPhiThreads = 128;

template <typename X> __device__ __forceinline__ double to_d(X v) { return (double)v; }

// ---------------------------------------------------------------------------
// row_fwd: `rb` rows (consecutive x of one dof) per block.
// Even ny: z[k] = x[2k] + i x[2k+1] (length ny/2), Z = FFT(z),
//   X[k] = (Z[k] + conj Z[n-k]) / 2 - i e^{-2 pi i k/ny} (Z[k] - conj Z[n-k]) / 2.
// Odd ny: complex transform of the real row, keep k = 0..(ny-1)/2.
template <typename T, typename Tin>
__global__ void __launch_bounds__(kThreads) k_row_fwd(const Tin *__restrict__ u, C<T> *__restrict__ W,
                                                       Geom g, FftPlan p, Tw<T> tw, int rb) {
  extern __shared__ unsigned char smem_raw[];
  C<T> *bufA = reinterpret_cast<C<T> *>(smem_raw);
  const int rs = g.nrow + 1;  // row stride in shared memory
  C<T> *bufB = bufA + (size_t)rb * rs;
  const int dof = blockIdx.y;
  const int ix0 = blockIdx.x * rb;
  const int nr = min(rb, g.nx - ix0);
  const Tin *src = u + ((size_t)dof * g.nx + ix0) * g.ny;
  const int tid = threadIdx.x, nth = blockDim.x;

  if (g.ny_even) {
    const int half = g.ny / 2;
    for (int idx = tid; idx < nr * half; idx += nth) {
      int r = idx / half, k = idx - r * half;
      bufA[r * rs + k] = mk<T>((T)src[(size_t)r * g.ny + 2 * k], (T)src[(size_t)r * g.ny + 2 * k + 1]);
    }
  } else {
    for (int idx = tid; idx < nr * g.ny; idx += nth) {
      int r = idx / g.ny, k = idx - r * g.ny;
      bufA[r * rs + k] = mk<T>((T)src[idx], (T)0);
    }
  }
  __syncthreads();
  C<T> *Z = fft_block<T>(bufA, bufB, p, nr, rs, tw, -1);

  const int n = g.nrow;
  for (int idx = tid; idx < nr * g.nyc; idx += nth) {
    int ky = idx / nr, r = idx - ky * nr;
    C<T> X;
    if (g.ny_even) {
      C<T> zk = Z[r * rs + (ky == n ? 0 : ky)];
      C<T> zc = cconj<T>(Z[r * rs + (ky == 0 ? 0 : n - ky)]);
      C<T> A = cadd<T>(zk, zc), B = csub<T>(zk, zc);
      C<T> wB = tw.mul(B, g.rpost + ky, -1);  // e^{-2 pi i ky/ny} B
      X = mk<T>((T)0.5 * (A.x + wB.y), (T)0.5 * (A.y - wB.x));
    } else {
      X = Z[r * rs + ky];
    }
    W[((size_t)ky * g.ndof + dof) * g.nxp + ix0 + r] = X;
  }
}

// ---------------------------------------------------------------------------
// row_inv: inverse of row_fwd, keeping the real part the reference keeps
// (imaginary parts of the ky = 0 and ky = ny/2 bins are dropped).
template <typename T, typename Tout>
__global__ void __launch_bounds__(kThreads) k_row_inv(const C<T> *__restrict__ W, Tout *__restrict__ f,
                                                       Geom g, FftPlan p, Tw<T> tw, int rb) {
  extern __shared__ unsigned char smem_raw[];
  C<T> *bufA = reinterpret_cast<C<T> *>(smem_raw);
  const int rs = g.nrow + 1;
  C<T> *bufB = bufA + (size_t)rb * rs;
  const int dof = blockIdx.y;
  const int ix0 = blockIdx.x * rb;
  const int nr = min(rb, g.nx - ix0);
  const int tid = threadIdx.x, nth = blockDim.x;
  const int n = g.nrow;

  for (int idx = tid; idx < nr * g.nyc; idx += nth) {
    int ky = idx / nr, r = idx - ky * nr;
    bufB[r * rs + ky] = W[((size_t)ky * g.ndof + dof) * g.nxp + ix0 + r];
  }
  __syncthreads();
  if (g.ny_even) {
    for (int idx = tid; idx < nr * n; idx += nth) {
      int r = idx / n, k = idx - r * n;
      C<T> xk = bufB[r * rs + k];
      C<T> xm = bufB[r * rs + n - k];
      if (k == 0) {
        xk.y = 0;
        xm.y = 0;
      }
      C<T> xc = cconj<T>(xm);
      C<T> A = cadd<T>(xk, xc), B = csub<T>(xk, xc);
      C<T> wB = tw.mul(B, g.rpost + k, +1);  // e^{+2 pi i k/ny} B
      bufA[r * rs + k] = mk<T>(A.x - wB.y, A.y + wB.x);
    }
  } else {
    const int h = (g.ny - 1) / 2;
    for (int idx = tid; idx < nr * g.ny; idx += nth) {
      int r = idx / g.ny, k = idx - r * g.ny;
      C<T> v;
      if (k == 0) {
        v = bufB[r * rs];
        v.y = 0;
      } else if (k <= h) {
        v = bufB[r * rs + k];
      } else {
        v = cconj<T>(bufB[r * rs + g.ny - k]);
      }
      bufA[r * rs + k] = v;
    }
  }
  __syncthreads();
  C<T> *z = fft_block<T>(bufA, bufB, p, nr, rs, tw, +1);
  Tout *dst = f + ((size_t)dof * g.nx + ix0) * g.ny;
  if (g.ny_even) {
    const int half = g.ny / 2;
    for (int idx = tid; idx < nr * half; idx += nth) {
      int r = idx / half, k = idx - r * half;
      C<T> v = z[r * rs + k];
      dst[(size_t)r * g.ny + 2 * k] = (Tout)v.x;
      dst[(size_t)r * g.ny + 2 * k + 1] = (Tout)v.y;
    }
  } else {
    for (int idx = tid; idx < nr * g.ny; idx += nth) {
      int r = idx / g.ny, k = idx - r * g.ny;
      dst[idx] = (Tout)z[r * rs + k].x;
    }
  }
}

// ---------------------------------------------------------------------------
// col_fft: `cb` contiguous columns (length nx, pitch nxp) per block, in place.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_col_fft(C<T> *__restrict__ W, Geom g, FftPlan p,
                                                       Tw<T> tw, int cb, int sign) {
  extern __shared__ unsigned char smem_raw[];
  C<T> *bufA = reinterpret_cast<C<T> *>(smem_raw);
  const int rs = g.nx;
  C<T> *bufB = bufA + (size_t)cb * rs;
  const int ncol = g.nyc * g.ndof;
  const int c0 = blockIdx.x * cb;
  const int nc = min(cb, ncol - c0);
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int idx = tid; idx < nc * g.nx; idx += nth) {
    int c = idx / g.nx, x = idx - c * g.nx;
    bufA[c * rs + x] = W[(size_t)(c0 + c) * g.nxp + x];
  }
  __syncthreads();
  C<T> *res = fft_block<T>(bufA, bufB, p, nc, rs, tw, sign);
  for (int idx = tid; idx < nc * g.nx; idx += nth) {
    int c = idx / g.nx, x = idx - c * g.nx;
    W[(size_t)(c0 + c) * g.nxp + x] = res[c * rs + x];
  }
}

// ---------------------------------------------------------------------------
// phi_apply: one thread per wavevector (x = kx, blockIdx.y = ky).
// Packed Hermitian Phi: p < D -> Re H_pp; then for i < j in row-major order
// the pair (Re H_ij, Im H_ij).  F_i = sum_j H_ij u_j with H_ji = conj H_ij.
// e = w(ky) Re(conj(F).u) (weight 2 for ky with a mirror partner in the
// stored half, else 1), accumulated in FP64.
template <typename T, int D>
__global__ void __launch_bounds__(kPhiThreads) k_phi_apply(C<T> *__restrict__ W, const T *__restrict__ phi,
                                                           Geom g, const double *__restrict__ linf,
                                                           double *__restrict__ epart,
                                                           double *__restrict__ scal) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int ky = blockIdx.y;
  double e = 0.0;
  if (x < g.nx) {
    const size_t cs = (size_t)g.nxp;
    C<T> *col = W + (size_t)ky * D * cs + x;
    const T *ph = phi + (size_t)ky * g.npk * cs + x;
    C<T> uq[D], F[D];
#pragma unroll
    for (int j = 0; j < D; j++) {
      uq[j] = col[j * cs];
      F[j] = mk<T>(0, 0);
    }
#pragma unroll
    for (int i = 0; i < D; i++) {
      T h = ph[i * cs];
      F[i].x += h * uq[i].x;
      F[i].y += h * uq[i].y;
    }
    int pidx = D;
#pragma unroll
    for (int i = 0; i < D; i++) {
#pragma unroll
      for (int j = i + 1; j < D; j++) {
        T hr = ph[pidx * cs], hi = ph[(pidx + 1) * cs];
        pidx += 2;
        // F_i += H_ij u_j ; F_j += conj(H_ij) u_i
        F[i].x += hr * uq[j].x - hi * uq[j].y;
        F[i].y += hr * uq[j].y + hi * uq[j].x;
        F[j].x += hr * uq[i].x + hi * uq[i].y;
        F[j].y += hr * uq[i].y - hi * uq[i].x;
      }
    }
    const bool mirror_self = (ky == 0) || (g.ny_even && ky == g.ny / 2);
    const double w = mirror_self ? 1.0 : 2.0;
    double es = 0.0;
#pragma unroll
    for (int i = 0; i < D; i++) es += to_d(F[i].x) * to_d(uq[i].x) + to_d(F[i].y) * to_d(uq[i].y);
    e = w * es;
    if (ky == 0 && x == 0) {
      // u(q=0) (gfmd_solver_static.cpp:169-177); gamma-point energy (:193-197)
      // and linear force (:228-231)
#pragma unroll
      for (int j = 0; j < D; j++) scal[1 + j] = to_d(uq[j].x);
      for (int l = 0; l < D / 3; l++) {
        e -= 2.0 * linf[l] * to_d(uq[3 * l + 2].x);
        F[3 * l + 2].x -= (T)linf[l];
      }
    }
#pragma unroll
    for (int i = 0; i < D; i++) col[i * cs] = mk<T>(-F[i].x, -F[i].y);
  }
  // block reduction of e (fixed order)
  __shared__ double red[kPhiThreads / 32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    epart[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = s;
  }
}

// Fixed-order sum of the energy partials; E = 0.5 * sum (:236).
__global__ void __launch_bounds__(256) k_reduce(const double *__restrict__ epart, int n,
                                                double *__restrict__ out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += epart[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = 0.5 * red[0];
}

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

template <typename T>
cudaError_t enqueue_t(gfmd_solver *h, const void *d_u, int in_t, void *d_f, int out_t,
                      double *d_epot) {
  const Geom &g = h->g;
  Tw<T> tw;
  tw.hi = reinterpret_cast<decltype(tw.hi)>(h->d_tw_hi);
  if constexpr (sizeof(T) == 4) tw.lo = reinterpret_cast<const float2 *>(h->d_tw_lo);
  else tw.lo_unused = nullptr;
  C<T> *W = reinterpret_cast<C<T> *>(h->d_W);
  const size_t smax = h->smem_optin;

  // row_fwd
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
  int cb = cols_per_block(g, sizeof(C<T>), smax);
  size_t smc = 2 * (size_t)cb * g.nx * sizeof(C<T>);
  dim3 gridc((g.nyc * g.ndof + cb - 1) / cb);
  cudaFuncSetAttribute(k_col_fft<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc);
  k_col_fft<T><<<gridc, kThreads, smc, h->stream>>>(W, g, h->plan_col, tw, cb, -1);
  // phi
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
  k_reduce<<<1, 256, 0, h->stream>>>(h->d_epart, (int)(gridp.x * gridp.y), d_epot);
  // col_fft backward
  k_col_fft<T><<<gridc, kThreads, smc, h->stream>>>(W, g, h->plan_col, tw, cb, +1);
  // row_inv
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
  return cudaGetLastError();
}

}  // namespace

void force_layout(const Geom &g, int precision, size_t *w_bytes, size_t *phi_bytes, int *n_epart) {
  size_t s = precision == GFMD_PREC_F64 ? 8 : 4;
  *w_bytes = (size_t)g.nyc * g.ndof * g.nxp * 2 * s;
  *phi_bytes = (size_t)g.nyc * g.npk * g.nxp * s;
  *n_epart = ((g.nx + kPhiThreads - 1) / kPhiThreads) * g.nyc;
}

cudaError_t enqueue_force(gfmd_solver *h, const void *d_u, int in_t, void *d_f, int out_t,
                          double *d_epot) {
  if (h->precision == GFMD_PREC_F64) return enqueue_t<double>(h, d_u, in_t, d_f, out_t, d_epot);
  return enqueue_t<float>(h, d_u, in_t, d_f, out_t, d_epot);
}

}  // namespace gfmd
