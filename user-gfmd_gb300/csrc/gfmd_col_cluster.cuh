// Column phase of the FP32 force path, split over a thread-block cluster.
//
// For one ky the D spectral columns along x (D x nx complex) and the
// per-wavevector product F = -Phi u couple every degree of freedom, so the
// earlier column kernel kept all D columns of a ky in one block (196 KB at
// nx = 2048, D = 12): one block per SM, whose transforms and Phi stream
// alternated instead of overlapping.  Here the columns of a ky are spread
// over a cluster of CL blocks, DL = D / CL columns each (96 KB at D = 12,
// CL = 2), so two blocks share an SM and one streams Phi while the other
// transforms:
//
//   1. forward DIF FFT of the block's own DL columns (natural order in,
//      digit-reversed out), in XOR-swizzled shared memory;
//   2. cluster barrier;
//   3. the block's 1/CL share of the wavevectors: u of all D columns
//      (own columns from shared memory, the others from the peer blocks'
//      shared memory through distributed shared memory), F = Phi u with the
//      energy, -F written back to the owning blocks;
//   4. cluster barrier;
//   5. backward DIT FFT of the own columns, written to W.
//
// Twiddles are read from global memory (L1-resident) so that shared memory
// holds only the columns.  Phi is streamed as 16-byte vectors from the
// layout [ky][x/32][D*D/4][32][4] over digit-reversed positions x (each
// lane one wavevector, a warp reads 512 contiguous bytes per vector); the
// first round of the block's Phi is prefetched into L2 before its forward
// transform.  The energy partials of all blocks are summed in a fixed order
// by the last block to finish (deterministic).
#ifndef GFMD_GB300_COL_CLUSTER_CUH
#define GFMD_GB300_COL_CLUSTER_CUH

#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <utility>

#include "gfmd_fast_kernels.cuh"
#include "gfmd_fft.cuh"
#include "gfmd_internal.h"
#include "gfmd_rows_warp.cuh"

namespace gfmd {

namespace colcl {

constexpr int kThreads = 256;

template <int R>
__device__ __forceinline__ void dif_task_g(float2 *col, int base, int S, int j, const float4 *__restrict__ tws) {
  float2 v[R];
#pragma unroll
  for (int r = 0; r < R; r++) v[r] = col[swz(base + r * S)];
  Dft<float, R>::run(v, -1);
#pragma unroll
  for (int m = 0; m < R; m++) {
    float2 y = v[m];
    if (m > 0 && j > 0) y = twmul(y, __ldg(&tws[m * S]), -1);
    col[swz(base + m * S)] = y;
  }
}

template <int R>
__device__ __forceinline__ void dit_task_g(float2 *col, int base, int S, int j, const float4 *__restrict__ tws) {
  float2 v[R];
#pragma unroll
  for (int m = 0; m < R; m++) {
    float2 y = col[swz(base + m * S)];
    if (m > 0 && j > 0) y = twmul(y, __ldg(&tws[m * S]), +1);
    v[m] = y;
  }
  Dft<float, R>::run(v, +1);
#pragma unroll
  for (int r = 0; r < R; r++) col[swz(base + r * S)] = v[r];
}

// Forward transform of nb columns of length p.n (stride cs) in place,
// natural -> digit-reversed; tab: stage tables (global).  Ends with a
// block barrier.
inline __device__ void fft_dif_g(float2 *buf, int nb, int cs, const P2Plan &p, const float4 *__restrict__ tab) {
  int lgL = p.lgn;
#pragma unroll
  for (int s = 0; s < kP2MaxStages; s++) {
    if (s >= p.nst) break;
    const int lgR = p.lg[s], lgS = lgL - lgR, S = 1 << lgS;
    const int lgper = p.lgn - lgR;
    const int total = nb << lgper;
    const float4 *ts = tab + p.toff[s];
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int c = t >> lgper, q = t & ((1 << lgper) - 1);
      const int b = q >> lgS, j = q & (S - 1);
      float2 *col = buf + (size_t)c * cs;
      const int base = (b << lgL) + j;
      switch (lgR) {
        case 4: dif_task_g<16>(col, base, S, j, ts + j); break;
        case 3: dif_task_g<8>(col, base, S, j, ts + j); break;
        case 2: dif_task_g<4>(col, base, S, j, ts + j); break;
        default: dif_task_g<2>(col, base, S, j, ts + j); break;
      }
    }
    __syncthreads();
    lgL = lgS;
  }
}

// Backward transform in place, digit-reversed -> natural (unscaled).
inline __device__ void fft_dit_g(float2 *buf, int nb, int cs, const P2Plan &p, const float4 *__restrict__ tab) {
#pragma unroll
  for (int s = kP2MaxStages - 1; s >= 0; s--) {
    if (s >= p.nst) continue;
    int lgL = p.lgn;
#pragma unroll
    for (int q = 0; q < kP2MaxStages; q++)
      if (q < s) lgL -= p.lg[q];
    const int lgR = p.lg[s], lgS = lgL - lgR, S = 1 << lgS;
    const int lgper = p.lgn - lgR;
    const int total = nb << lgper;
    const float4 *ts = tab + p.toff[s];
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int c = t >> lgper, q = t & ((1 << lgper) - 1);
      const int b = q >> lgS, j = q & (S - 1);
      float2 *col = buf + (size_t)c * cs;
      const int base = (b << lgL) + j;
      switch (lgR) {
        case 4: dit_task_g<16>(col, base, S, j, ts + j); break;
        case 3: dit_task_g<8>(col, base, S, j, ts + j); break;
        case 2: dit_task_g<4>(col, base, S, j, ts + j); break;
        default: dit_task_g<2>(col, base, S, j, ts + j); break;
      }
    }
    __syncthreads();
  }
}

// Packed-element meaning: element e < D is Re H_ee; element D + 2p (+1) is
// Re (Im) H_IJ of the p-th pair I < J in row-major order.
constexpr int pair_row(int D, int p) {
  int i = 0;
  while (p >= D - 1 - i) {
    p -= D - 1 - i;
    i++;
  }
  return i;
}
constexpr int pair_col(int D, int p) {
  int i = 0;
  while (p >= D - 1 - i) {
    p -= D - 1 - i;
    i++;
  }
  return i + 1 + p;
}

// F += H u from the packed table of one wavevector.  V = 4: the D*D
// elements come as float4 vectors at ph[g * 32] (g = element / 4); V = 1:
// scalars at ph[e * 32].  D even with V = 4 keeps every (Re, Im) pair
// inside one vector.
template <int D, int V, int PAT = 0> struct PhiApply {
  static_assert(PAT == 0 || V == 4, "table patterns use the vector layout");
  template <int E>
  static __device__ __forceinline__ void item(float h0, float h1, const float2 *uq, float2 *F) {
    if constexpr (E < D) {  // two diagonal entries (E, E + 1) or one
      F[E].x = fmaf(h0, uq[E].x, F[E].x);
      F[E].y = fmaf(h0, uq[E].y, F[E].y);
      if constexpr (E + 1 < D) {
        F[E + 1].x = fmaf(h1, uq[E + 1].x, F[E + 1].x);
        F[E + 1].y = fmaf(h1, uq[E + 1].y, F[E + 1].y);
      }
    } else if constexpr ((E - D) / 2 < pat_pairs(D, PAT)) {  // else: padding
      constexpr int P = (E - D) / 2, I = pat_pair(D, PAT, P, 0), J = pat_pair(D, PAT, P, 1);
      const float hr = h0, hi = h1;
      F[I].x = fmaf(hr, uq[J].x, fmaf(-hi, uq[J].y, F[I].x));
      F[I].y = fmaf(hr, uq[J].y, fmaf(hi, uq[J].x, F[I].y));
      F[J].x = fmaf(hr, uq[I].x, fmaf(hi, uq[I].y, F[J].x));
      F[J].y = fmaf(hr, uq[I].y, fmaf(-hi, uq[I].x, F[J].y));
    }
  }
  template <int G>
  static __device__ __forceinline__ void group(const float *__restrict__ ph, const float2 *uq, float2 *F) {
    if constexpr (V == 4) {
      const float4 v = __ldcs(reinterpret_cast<const float4 *>(ph) + G * 32);
      item<4 * G>(v.x, v.y, uq, F);
      item<4 * G + 2>(v.z, v.w, uq, F);
    } else {
      // scalar layout: items start at 0 (diagonals, one at a time) and at
      // D + 2p (pairs); G enumerates items
      if constexpr (G < D) {
        const float h = __ldcs(ph + G * 32);
        F[G].x = fmaf(h, uq[G].x, F[G].x);
        F[G].y = fmaf(h, uq[G].y, F[G].y);
      } else {
        constexpr int E = D + 2 * (G - D);
        const float hr = __ldcs(ph + E * 32), hi = __ldcs(ph + (E + 1) * 32);
        item<E>(hr, hi, uq, F);
      }
    }
  }
  template <int... Gs>
  static __device__ __forceinline__ void all(const float *__restrict__ ph, const float2 *uq, float2 *F,
                                             std::integer_sequence<int, Gs...>) {
    (group<Gs>(ph, uq, F), ...);
  }
  // number of groups: float4 vectors of the pattern, or D diagonals + D(D-1)/2 pairs
  static constexpr int kGroups = V == 4 ? pat_floats(D, PAT) / 4 : D + D * (D - 1) / 2;
  static __device__ __forceinline__ void run(const float *__restrict__ ph, const float2 *uq, float2 *F) {
    all(ph, uq, F, std::make_integer_sequence<int, kGroups>{});
  }
};

}  // namespace colcl

// One cluster of CL blocks per ky; block rank r owns columns [r DL, (r+1) DL).
// phi: packed FP32 table (layout per V, see PhiApply); tab: column stage
// twiddles (global); epart: one partial per block.
template <int D, int CL, int V>
__global__ void __launch_bounds__(colcl::kThreads, 2)
    k_col_phi_cl(float2 *__restrict__ W, const float *__restrict__ phi, Geom g, P2Plan p,
                 const float4 *__restrict__ tab, const double *__restrict__ linf, double *__restrict__ epart,
                 double *__restrict__ scal, unsigned *__restrict__ counter, double *__restrict__ d_epot) {
  namespace cg = cooperative_groups;
  constexpr int DL = D / CL;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[colcl::kThreads / 32];
  __shared__ int is_last;
  float2 *sm = reinterpret_cast<float2 *>(smem_raw);
  const int n = g.nx;
  const int rank = (int)(blockIdx.x % CL), ky = (int)(blockIdx.x / CL);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  constexpr int kPerPos = D * D;                          // floats per wavevector
  constexpr unsigned kBlk = (unsigned)(kPerPos * 32 * 4);  // bytes per 32 wavevectors
  const int nkb = g.nxp >> 5;
  const float *phik = phi + (size_t)ky * nkb * (kPerPos * 32);
  // this block's share of the 32-wavevector blocks
  const int nkb_used = (n + 31) >> 5;
  const int kb0 = (nkb_used * rank) / CL, kb1 = (nkb_used * (rank + 1)) / CL;

  float2 *colg = W + ((size_t)ky * D + rank * DL) * g.nxp;
  for (int i = threadIdx.x; i < DL * n; i += blockDim.x) {
    const int c = i >> p.lgn, x = i & (n - 1);
    cp_async<8>(&sm[c * n + swz(x)], &colg[(size_t)c * g.nxp + x]);
  }
  if (lane == 0 && kb0 + warp < kb1) prefetch_l2(phik + (size_t)(kb0 + warp) * (kPerPos * 32), kBlk);
  cp_async_wait_all();
  __syncthreads();
  colcl::fft_dif_g(sm, DL, n, p, tab);

  cg::cluster_group cluster = cg::this_cluster();
  if constexpr (CL > 1) cluster.sync();
  float2 *part[CL];
#pragma unroll
  for (int q = 0; q < CL; q++) part[q] = (q == rank) ? sm : cluster.map_shared_rank(sm, q);

  const bool mirror_self = (ky == 0) || (g.ny_even && ky == g.ny / 2);
  const double wgt = mirror_self ? 1.0 : 2.0;
  double e = 0.0;
  for (int kb = kb0 + warp; kb < kb1; kb += nwarp) {
    if (lane == 0 && kb + nwarp < kb1) prefetch_l2(phik + (size_t)(kb + nwarp) * (kPerPos * 32), kBlk);
    const int q = (kb << 5) + lane;  // position in the digit-reversed order
    if (q >= n) continue;
    const int pos = swz(q);
    const float *ph = phik + (size_t)kb * (kPerPos * 32) + lane * V;
    float2 uq[D], F[D];
#pragma unroll
    for (int j = 0; j < D; j++) {
      uq[j] = part[j / DL][(j % DL) * n + pos];
      F[j] = make_float2(0.0f, 0.0f);
    }
    colcl::PhiApply<D, V>::run(ph, uq, F);
    float es = 0.0f;
#pragma unroll
    for (int i = 0; i < D; i++) es = fmaf(F[i].x, uq[i].x, fmaf(F[i].y, uq[i].y, es));
    e += wgt * (double)es;
    if (ky == 0 && q == 0) {  // kx = 0 sits at position 0
#pragma unroll
      for (int j = 0; j < D; j++) scal[1 + j] = (double)uq[j].x;
#pragma unroll
      for (int l = 0; l < D / 3; l++) {
        e -= 2.0 * linf[l] * (double)uq[3 * l + 2].x;
        F[3 * l + 2].x -= (float)linf[l];
      }
    }
#pragma unroll
    for (int i = 0; i < D; i++) part[i / DL][(i % DL) * n + pos] = make_float2(-F[i].x, -F[i].y);
  }
  if constexpr (CL > 1) cluster.sync();
  else __syncthreads();
  colcl::fft_dit_g(sm, DL, n, p, tab);
  for (int i = threadIdx.x; i < DL * n; i += blockDim.x) {
    const int c = i >> p.lgn, x = i & (n - 1);
    colg[(size_t)c * g.nxp + x] = sm[c * n + swz(x)];
  }

  // energy: block partial, then the last block sums all partials in order
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  if (lane == 0) red[warp] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < nwarp; w++) s += red[w];
    epart[blockIdx.x] = s;
    __threadfence();
    unsigned prev = atomicAdd(counter, 1u);
    is_last = (prev == gridDim.x - 1) ? 1 : 0;
  }
  __syncthreads();
  if (is_last) {
    __threadfence();
    double s = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x) s += ((volatile double *)epart)[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    __syncthreads();
    if (lane == 0) red[warp] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < nwarp; w++) t += red[w];
      *d_epot = 0.5 * t;
      *counter = 0u;
    }
  }
}

// ---------------------------------------------------------------------------
// Register-transform column kernel for nx = 32 P, P in {32, 64} (nx = 1024,
// 2048).  A column x[t + P m] (t < P, m < 32) is transformed in two passes
// held in registers:
//   pass A (thread t of the column): 32-point DFT over m, straight from the
//     coalesced global loads of W, times the compensated twiddle w_nx^(t k1),
//     written transposed to shared memory S[k1][t] (XOR-swizzled);
//   pass B (thread (k1, s), s = t mod 2 for P = 64): 32-point DFT over the
//     column's t of that parity and, for P = 64, one radix-2 step across the
//     thread pair by warp shuffles; the spectrum X[k1 + 32 k2] is stored at
//     position q = P k1 + k2 (swizzled q ^ ((q >> 5) & 15)), the order in
//     which the stiffness table is packed for this kernel.
// The backward transform runs the passes in reverse; its pass A stores the
// column to W with coalesced stores, so the kernel reads and writes W once
// and stages nothing but the transposes in shared memory.
namespace colr {

template <int P> __device__ __forceinline__ int swa(int k1) { return P == 64 ? 2 * (k1 & 7) : (k1 & 15); }
__device__ __forceinline__ int physq(int q) { return q ^ ((q >> 5) & 15); }

// (cos, sin) of 2 pi k / 64, k = 0..31
__device__ __forceinline__ float2 w64(int k) {
  const float c[32] = {1.00000000000000000000f, 0.99518472667219692873f, 0.98078528040323043058f, 0.95694033573220882438f, 0.92387953251128673848f, 0.88192126434835504956f, 0.83146961230254523567f, 0.77301045336273699338f, 0.70710678118654757274f, 0.63439328416364548779f, 0.55557023301960228867f, 0.47139673682599780857f, 0.38268343236508983729f, 0.29028467725446233105f, 0.19509032201612833135f, 0.09801714032956077016f, 0.0f, -0.09801714032956064526f, -0.19509032201612819257f, -0.29028467725446216452f, -0.38268343236508972627f, -0.47139673682599769755f, -0.55557023301960195560f, -0.63439328416364537677f, -0.70710678118654746172f, -0.77301045336273699338f, -0.83146961230254534669f, -0.88192126434835493853f, -0.92387953251128673848f, -0.95694033573220882438f, -0.98078528040323043058f, -0.99518472667219681771f};
  const float sn[32] = {0.00000000000000000000f, 0.09801714032956060363f, 0.19509032201612824808f, 0.29028467725446233105f, 0.38268343236508978178f, 0.47139673682599764204f, 0.55557023301960217765f, 0.63439328416364548779f, 0.70710678118654746172f, 0.77301045336273699338f, 0.83146961230254523567f, 0.88192126434835493853f, 0.92387953251128673848f, 0.95694033573220893540f, 0.98078528040323043058f, 0.99518472667219681771f, 1.00000000000000000000f, 0.99518472667219692873f, 0.98078528040323043058f, 0.95694033573220893540f, 0.92387953251128673848f, 0.88192126434835504956f, 0.83146961230254545772f, 0.77301045336273710440f, 0.70710678118654757274f, 0.63439328416364548779f, 0.55557023301960217765f, 0.47139673682599786408f, 0.38268343236508989280f, 0.29028467725446238656f, 0.19509032201612860891f, 0.09801714032956082567f};
  return make_float2(c[k], sn[k]);
}

}  // namespace colr

// One cluster of CL blocks per ky, block rank r owning columns
// [r DL, (r+1) DL), DL * P threads (thread c P + t: column c, index t).
// twa: [k1][t] compensated w_nx^(t k1); phi packed [ky][q/32][D*D/4][32][4]
// (V = 4) or [ky][q/32][D*D][32] (V = 1) over the storage positions q.
template <int D, int CL, int LGN, int MINB, int PAT = 0>
__global__ void __launch_bounds__((D / CL) * (1 << LGN) / 32, MINB)
    k_col_phi_r32(float2 *__restrict__ W, const float *__restrict__ phi, Geom g, const float4 *__restrict__ twa,
                  const double *__restrict__ linf, double *__restrict__ epart, double *__restrict__ scal,
                  unsigned *__restrict__ counter, double *__restrict__ d_epot, int pf) {
  namespace cg = cooperative_groups;
  constexpr int n = 1 << LGN, P = n / 32, DL = D / CL, NT = DL * P;
  constexpr int V = (D * D) % 4 == 0 ? 4 : 1;
  constexpr int kPerPos = V == 4 ? pat_floats(D, PAT) : D * D;  // floats per wavevector
  constexpr unsigned kBlk = (unsigned)(kPerPos * 32 * 4);
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[NT / 32];
  __shared__ int is_last;
  float2 *sm = reinterpret_cast<float2 *>(smem_raw);
  const int rank = (int)(blockIdx.x % CL), ky = (int)(blockIdx.x / CL);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = NT / 32;
  const int c = threadIdx.x / P, t = threadIdx.x % P;
  float2 *S = sm + c * n;
  float2 *colg = W + ((size_t)ky * D + rank * DL + c) * g.nxp;
  const int nkb = g.nxp >> 5;
  const float *phik = phi + (size_t)ky * nkb * (kPerPos * 32);
  constexpr int kbn = n / 32;
  const int kb0 = (kbn * rank) / CL, kb1 = (kbn * (rank + 1)) / CL;
  // pass-B roles: k1 and the parity s of t (P = 64)
  const int k1b = P == 64 ? (t >> 1) : t, sb = P == 64 ? (t & 1) : 0;

  // the first pf rounds of this block's Phi stream go to L2 during the
  // forward transform (pf is tuned per grid: deeper rounds of all resident
  // blocks compete for L2)
  if (lane == 0)
    for (int r = 0; r < pf; r++)
      if (kb0 + warp + r * nwarp < kb1) prefetch_l2(phik + (size_t)(kb0 + warp + r * nwarp) * (kPerPos * 32), kBlk);
  float2 x[32];
  // ---- forward pass A ----
#pragma unroll
  for (int m = 0; m < 32; m++) x[m] = __ldcs(colg + t + P * m);
  rows32::dft32<-1>(x);
#pragma unroll
  for (int k1 = 1; k1 < 32; k1++) x[k1] = rows32::twc<-1>(x[k1], __ldg(&twa[k1 * P + t]));
#pragma unroll
  for (int k1 = 0; k1 < 32; k1++) S[k1 * P + (t ^ colr::swa<P>(k1))] = x[k1];
  __syncthreads();
  // ---- forward pass B ----
#pragma unroll
  for (int tp = 0; tp < 32; tp++) {
    const int tt = P == 64 ? 2 * tp + sb : tp;
    x[tp] = S[k1b * P + (tt ^ colr::swa<P>(k1b))];
  }
  rows32::dft32<-1>(x);
  if constexpr (P == 64) {
#pragma unroll
    for (int k = 0; k < 32; k++) {
      const float2 own = x[k];
      const float2 oth = make_float2(__shfl_xor_sync(0xffffffffu, own.x, 1), __shfl_xor_sync(0xffffffffu, own.y, 1));
      const float2 a = sb ? oth : own, b = sb ? own : oth;  // D_0, D_1
      const float2 w = colr::w64(k);
      const float2 wb = make_float2(fmaf(b.x, w.x, b.y * w.y), fmaf(b.y, w.x, -b.x * w.y));  // b e^{-2 pi i k/64}
      x[k] = sb ? make_float2(a.x - wb.x, a.y - wb.y) : make_float2(a.x + wb.x, a.y + wb.y);
    }
  }
  __syncthreads();  // pass-B reads of S done
#pragma unroll
  for (int k = 0; k < 32; k++) S[colr::physq(P * k1b + 32 * sb + k)] = x[k];

  cg::cluster_group cluster = cg::this_cluster();
  if constexpr (CL > 1) cluster.sync();
  else __syncthreads();
  float2 *part[CL];
#pragma unroll
  for (int q = 0; q < CL; q++) part[q] = (q == rank) ? sm : cluster.map_shared_rank(sm, q);

  // ---- F = -Phi u over this block's share of the positions ----
  const bool mirror_self = (ky == 0) || (g.ny_even && ky == g.ny / 2);
  const double wgt = mirror_self ? 1.0 : 2.0;
  double e = 0.0;
  for (int kb = kb0 + warp; kb < kb1; kb += nwarp) {
    if (lane == 0 && kb + pf * nwarp < kb1) prefetch_l2(phik + (size_t)(kb + pf * nwarp) * (kPerPos * 32), kBlk);
    const int q = (kb << 5) + lane;
    const int pos = colr::physq(q);
    const float *ph = phik + (size_t)kb * (kPerPos * 32) + lane * V;
    float2 uq[D], F[D];
#pragma unroll
    for (int j = 0; j < D; j++) {
      uq[j] = part[j / DL][(j % DL) * n + pos];
      F[j] = make_float2(0.0f, 0.0f);
    }
    colcl::PhiApply<D, V, PAT>::run(ph, uq, F);
    float es = 0.0f;
#pragma unroll
    for (int i = 0; i < D; i++) es = fmaf(F[i].x, uq[i].x, fmaf(F[i].y, uq[i].y, es));
    e += wgt * (double)es;
    if (ky == 0 && q == 0) {  // kx = 0 sits at position 0
#pragma unroll
      for (int j = 0; j < D; j++) scal[1 + j] = (double)uq[j].x;
#pragma unroll
      for (int l = 0; l < D / 3; l++) {
        e -= 2.0 * linf[l] * (double)uq[3 * l + 2].x;
        F[3 * l + 2].x -= (float)linf[l];
      }
    }
#pragma unroll
    for (int i = 0; i < D; i++) part[i / DL][(i % DL) * n + pos] = make_float2(-F[i].x, -F[i].y);
  }
  if constexpr (CL > 1) cluster.sync();
  else __syncthreads();

  // ---- backward pass B ----
#pragma unroll
  for (int k = 0; k < 32; k++) x[k] = S[colr::physq(P * k1b + 32 * sb + k)];
  if constexpr (P == 64) {
#pragma unroll
    for (int k = 0; k < 32; k++) {
      const float2 own = x[k];
      const float2 oth = make_float2(__shfl_xor_sync(0xffffffffu, own.x, 1), __shfl_xor_sync(0xffffffffu, own.y, 1));
      if (sb == 0) {
        x[k] = make_float2(own.x + oth.x, own.y + oth.y);  // X_0 + X_1
      } else {
        const float2 d = make_float2(oth.x - own.x, oth.y - own.y);  // X_0 - X_1
        const float2 w = colr::w64(k);
        x[k] = make_float2(fmaf(d.x, w.x, -d.y * w.y), fmaf(d.y, w.x, d.x * w.y));  // d e^{+2 pi i k/64}
      }
    }
  }
  rows32::dft32<+1>(x);
  __syncthreads();  // reads of the spectrum done
#pragma unroll
  for (int tp = 0; tp < 32; tp++) {
    const int tt = P == 64 ? 2 * tp + sb : tp;
    S[k1b * P + (tt ^ colr::swa<P>(k1b))] = x[tp];
  }
  __syncthreads();
  // ---- backward pass A ----
#pragma unroll
  for (int k1 = 0; k1 < 32; k1++) x[k1] = S[k1 * P + (t ^ colr::swa<P>(k1))];
#pragma unroll
  for (int k1 = 1; k1 < 32; k1++) x[k1] = rows32::twc<+1>(x[k1], __ldg(&twa[k1 * P + t]));
  rows32::dft32<+1>(x);
#pragma unroll
  for (int m = 0; m < 32; m++) __stcs(colg + t + P * m, x[m]);

  // energy: block partial, then the last block sums all partials in order
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  if (lane == 0) red[warp] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sacc = 0.0;
    for (int w = 0; w < nwarp; w++) sacc += red[w];
    epart[blockIdx.x] = sacc;
    __threadfence();
    unsigned prev = atomicAdd(counter, 1u);
    is_last = (prev == gridDim.x - 1) ? 1 : 0;
  }
  __syncthreads();
  if (is_last) {
    __threadfence();
    double sacc = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += NT) sacc += ((volatile double *)epart)[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sacc += __shfl_down_sync(0xffffffffu, sacc, o);
    __syncthreads();
    if (lane == 0) red[warp] = sacc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double tsum = 0.0;
      for (int w = 0; w < nwarp; w++) tsum += red[w];
      *d_epot = 0.5 * tsum;
      *counter = 0u;
    }
  }
}

// Register-transform column kernel (nx = 2^LGN in {1024, 2048}): one
// cluster of CL blocks per ky, launched with its cluster dimension.
template <int D, int CL, int LGN, int MINB, int PAT = 0>
cudaError_t launch_col_r32(gfmd_solver *h, float2 *W, double *d_epot) {
  constexpr int NT = (D / CL) * (1 << LGN) / 32;
  auto kf = k_col_phi_r32<D, CL, LGN, MINB, PAT>;
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

}  // namespace gfmd

#endif
