// Kernels of the plain force-evaluation pipeline (row_fwd, col_fft,
// phi_apply, reduce, row_inv), shared by the translation units that launch
// them.  Each includer gets its own internal-linkage instantiations.
#ifndef GFMD_GB300_PLAIN_KERNELS_CUH
#define GFMD_GB300_PLAIN_KERNELS_CUH

#include <cuda_runtime.h>

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
template <typename T, int D, int PAT = 0>
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
    // reals per wavevector: every pair, or the kept pairs of the pattern
    const size_t npk = PAT == 0 ? (size_t)g.npk : (size_t)(D + 2 * pat_pairs(D, PAT));
    const T *ph = phi + (size_t)ky * npk * cs + x;
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
    // F_i += H_ij u_j ; F_j += conj(H_ij) u_i
    if constexpr (PAT == 0) HermPairs<T, D>::run(ph, cs, uq, F);
    else HermPairsPat<T, D, PAT>::run(ph, cs, uq, F);
    const bool mirror_self = (ky == 0) || (g.ny_even && ky == g.ny / 2);
    const double w = mirror_self ? 1.0 : 2.0;
    T es = 0;
#pragma unroll
    for (int i = 0; i < D; i++) es = fma(F[i].x, uq[i].x, fma(F[i].y, uq[i].y, es));
    e = w * (double)es;
    if (ky == 0 && x == 0) {
      // u(q=0) (gfmd_solver_static.cpp:169-177); gamma-point energy (:193-197)
      // and linear force (:228-231)
#pragma unroll
      for (int j = 0; j < D; j++) scal[1 + j] = to_d(uq[j].x);
#pragma unroll
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
static __global__ void __launch_bounds__(256) k_reduce(const double *__restrict__ epart, int n,
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

}  // namespace

}  // namespace gfmd

#endif
