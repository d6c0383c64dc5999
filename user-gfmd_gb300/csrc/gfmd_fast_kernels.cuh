// Fused force-evaluation kernels for power-of-two grids (the production path).
//
// Three launches per evaluation:
//   k_row_fwd_fast   rows along y: real -> half spectrum; in-place
//                    decimation-in-frequency (DIF) FFT in swizzled shared
//                    memory, then the real-to-complex split, written
//                    transposed into W[ky][dof][x] in chunks of rb
//                    consecutive x;
//   k_col_phi_fast   one block per ky holding all ndof columns along x:
//                    forward DIF FFT (natural -> digit-reversed order),
//                    F = -Phi u with the FP64 energy at the digit-reversed
//                    positions, backward DIT FFT (digit-reversed -> natural),
//                    so the spectrum is never reordered; energy partials are
//                    summed in a fixed order by the last block to finish;
//   k_row_inv_fast   rows: half spectrum gathered and pre-split (complex to
//                    real) straight into digit-reversed slots, DIT backward FFT.
//
// Shared memory holds each transform under the XOR swizzle
// p -> p ^ ((p >> 4) & 15), a bijection on [0, n) for n a power of two that
// keeps the strided butterfly accesses of every stage free of bank conflicts
// (the two-wavefront minimum of a 32-lane float2 access) without padding.
// The Phi phase walks positions in storage order (Phi is packed in the
// digit-reversed wavevector order the forward transform leaves behind), so
// it needs no reordering and has no conflicts either.
//
// Twiddles: one table per DIF stage s with sub-length L_s and radix R_s,
// entry [m][j] = exp(-2 pi i j m / L_s) (j < L_s/R_s, m < R_s), copied into
// shared memory at kernel start, so a twiddle costs one 16-byte shared load
// and the 32 lanes of a warp (consecutive j) read consecutive entries.
// FP32 entries hold (cos_hi, sin_hi, cos_lo, sin_lo) with hi = fl32(v),
// lo = fl32(v - hi) from FP64, and the product multiplies by both, so the
// twiddle representation error drops out ("compensated twiddles").
//
// Global -> shared copies use cp.async (many in flight per thread); the
// Phi stream of the column kernel is laid out in blocks of 32 positions
// ([ky][pos/32][element][pos%32], pos = digit-reversed kx; 18 KB per block
// at ndof 12) and each warp prefetches its next block into L2 with one bulk
// prefetch.
#ifndef GFMD_GB300_FAST_KERNELS_CUH
#define GFMD_GB300_FAST_KERNELS_CUH

#include <cuda_runtime.h>

#include "gfmd_fft.cuh"
#include "gfmd_internal.h"

namespace gfmd {

namespace {

constexpr int kRowThreads = 256;

// Threads of the column kernel: 512 while the per-wavevector product fits in
// 128 registers, else 256.
template <typename T, int D> struct ColThreads {
  static constexpr int value = (sizeof(T) == 4 ? D <= 15 : D <= 6) ? 512 : 256;
};

template <typename T> struct TwE;
template <> struct TwE<float> { using type = float4; };   // (c_hi, s_hi, c_lo, s_lo)
template <> struct TwE<double> { using type = double2; }; // (c, s)

// x * w (sign < 0) or x * conj(w) (sign > 0), w = (c, s) from the table.
__device__ __forceinline__ float2 twmul(float2 x, float4 w, int sign) {
  float sh = sign < 0 ? w.y : -w.y, sl = sign < 0 ? w.w : -w.w;
  float cr = x.x * w.z - x.y * sl;
  float ci = x.x * sl + x.y * w.z;
  return make_float2(fmaf(x.x, w.x, fmaf(-x.y, sh, cr)), fmaf(x.x, sh, fmaf(x.y, w.x, ci)));
}
__device__ __forceinline__ double2 twmul(double2 x, double2 w, int sign) {
  double s = sign < 0 ? w.y : -w.y;
  return make_double2(x.x * w.x - x.y * s, x.x * s + x.y * w.x);
}

__device__ __forceinline__ int swz(int p) { return p ^ ((p >> 4) & 15); }

// Asynchronous global -> shared copies (many in flight per thread, no
// registers held); completed with cp_async_wait_all + a block barrier.
template <int B> __device__ __forceinline__ void cp_async(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  if constexpr (B == 16)
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(B) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// One bulk prefetch of `bytes` (multiple of 16) from global memory into L2.
__device__ __forceinline__ void prefetch_l2(const void *g, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(g), "r"(bytes) : "memory");
}

// Copies `ne` 16-byte table entries into shared memory (asynchronously).
template <typename E>
__device__ __forceinline__ void load_table(E *dst, const E *src, int ne) {
  for (int i = threadIdx.x; i < ne; i += blockDim.x) cp_async<16>(&dst[i], &src[i]);
}

// At most kP2MaxStages stages (n <= 16^3 * 8); loops over stages are unrolled
// to that bound so the plan is indexed statically and stays in registers.
constexpr int kP2MaxStages = 4;

// Position, in the output of the DIF stages, of frequency k.
__device__ __forceinline__ int digit_rev(const P2Plan &p, int k) {
  int pos = 0, lgS = p.lgn;
#pragma unroll
  for (int s = 0; s < kP2MaxStages; s++) {
    if (s < p.nst) {
      lgS -= p.lg[s];
      pos += (k & ((1 << p.lg[s]) - 1)) << lgS;
      k >>= p.lg[s];
    }
  }
  return pos;
}

template <typename T, int R>
__device__ __forceinline__ void dif_task(C<T> *col, int base, int S, int j,
                                         const typename TwE<T>::type *tws) {
  C<T> v[R];
#pragma unroll
  for (int r = 0; r < R; r++) v[r] = col[swz(base + r * S)];
  Dft<T, R>::run(v, -1);
#pragma unroll
  for (int m = 0; m < R; m++) {
    C<T> y = v[m];
    if (m > 0 && j > 0) y = twmul(y, tws[m * S], -1);
    col[swz(base + m * S)] = y;
  }
}

template <typename T, int R>
__device__ __forceinline__ void dit_inv_task(C<T> *col, int base, int S, int j,
                                             const typename TwE<T>::type *tws) {
  C<T> v[R];
#pragma unroll
  for (int m = 0; m < R; m++) {
    C<T> y = col[swz(base + m * S)];
    if (m > 0 && j > 0) y = twmul(y, tws[m * S], +1);
    v[m] = y;
  }
  Dft<T, R>::run(v, +1);
#pragma unroll
  for (int r = 0; r < R; r++) col[swz(base + r * S)] = v[r];
}

// Forward transform of nb columns (stride cs) in place, natural in,
// digit-reversed out; tab holds the stage tables at p.toff[s].  Ends with a
// block barrier.
template <typename T>
__device__ void fft_dif(C<T> *buf, int nb, int cs, const P2Plan &p,
                        const typename TwE<T>::type *tab) {
  int lgL = p.lgn;
#pragma unroll
  for (int s = 0; s < kP2MaxStages; s++) {
    if (s >= p.nst) break;
    const int lgR = p.lg[s], lgS = lgL - lgR, S = 1 << lgS;
    const int lgper = p.lgn - lgR;
    const int total = nb << lgper;
    const typename TwE<T>::type *ts = tab + p.toff[s];  // [m][j]
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int c = t >> lgper, q = t & ((1 << lgper) - 1);
      const int b = q >> lgS, j = q & (S - 1);
      C<T> *col = buf + (size_t)c * cs;
      const int base = (b << lgL) + j;
      switch (lgR) {
        case 4: dif_task<T, 16>(col, base, S, j, ts + j); break;
        case 3: dif_task<T, 8>(col, base, S, j, ts + j); break;
        case 2: dif_task<T, 4>(col, base, S, j, ts + j); break;
        default: dif_task<T, 2>(col, base, S, j, ts + j); break;
      }
    }
    __syncthreads();
    lgL = lgS;
  }
}

// Backward transform in place, digit-reversed in, natural out (unscaled).
// Ends with a block barrier.
template <typename T>
__device__ void fft_dit_inv(C<T> *buf, int nb, int cs, const P2Plan &p,
                            const typename TwE<T>::type *tab) {
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
    const typename TwE<T>::type *ts = tab + p.toff[s];  // [m][j]
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
      const int c = t >> lgper, q = t & ((1 << lgper) - 1);
      const int b = q >> lgS, j = q & (S - 1);
      C<T> *col = buf + (size_t)c * cs;
      const int base = (b << lgL) + j;
      switch (lgR) {
        case 4: dit_inv_task<T, 16>(col, base, S, j, ts + j); break;
        case 3: dit_inv_task<T, 8>(col, base, S, j, ts + j); break;
        case 2: dit_inv_task<T, 4>(col, base, S, j, ts + j); break;
        default: dit_inv_task<T, 2>(col, base, S, j, ts + j); break;
      }
    }
    __syncthreads();
  }
}

// Bytes reserved for the srev lookup (n 16-bit entries, rounded to 16).
__host__ __device__ constexpr size_t srev_bytes(int n) { return ((size_t)n * 2 + 15) / 16 * 16; }

// srev[k] = swz(digit_rev(p, k)) for k < n, computed into shared memory.
__device__ __forceinline__ void make_srev(unsigned short *srev, const P2Plan &p) {
  for (int k = threadIdx.x; k < p.n; k += blockDim.x) srev[k] = (unsigned short)swz(digit_rev(p, k));
}

// Two consecutive reals of the input as one complex value.
template <typename Tin, typename T>
__device__ __forceinline__ C<T> load_pair(const Tin *src) {
  if constexpr (sizeof(Tin) == 4) {
    float2 v = *reinterpret_cast<const float2 *>(src);
    return mk<T>((T)v.x, (T)v.y);
  } else {
    double2 v = *reinterpret_cast<const double2 *>(src);
    return mk<T>((T)v.x, (T)v.y);
  }
}

template <typename Tout, typename T>
__device__ __forceinline__ void store_pair(Tout *dst, C<T> v) {
  if constexpr (sizeof(Tout) == 4) {
    *reinterpret_cast<float2 *>(dst) = make_float2((float)v.x, (float)v.y);
  } else {
    *reinterpret_cast<double2 *>(dst) = make_double2((double)v.x, (double)v.y);
  }
}

// ---------------------------------------------------------------------------
// Rows.  The row table holds the stage tables of the length-n transform
// (n = ny/2) followed, at p.tpost, by e^{-2 pi i k/ny}, k = 0..n.
template <typename T, typename Tin>
__global__ void __launch_bounds__(kRowThreads, sizeof(T) == 4 ? 3 : 2)
    k_row_fwd_fast(const Tin *__restrict__ u, C<T> *__restrict__ W, Geom g, P2Plan p,
                   const typename TwE<T>::type *__restrict__ tab_g, int rb) {
  using E = typename TwE<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = p.n;  // = ny / 2
  E *tab = reinterpret_cast<E *>(smem_raw);
  unsigned short *srev = reinterpret_cast<unsigned short *>(smem_raw + (size_t)p.tsize * sizeof(E));
  C<T> *sm = reinterpret_cast<C<T> *>(smem_raw + (size_t)p.tsize * sizeof(E) + srev_bytes(n));
  load_table(tab, tab_g, p.tsize);
  make_srev(srev, p);
  const int cs = n + 1;  // spare slot n (used by the inverse)
  const int dof = blockIdx.y;
  const int ix0 = blockIdx.x * rb;  // nx is a multiple of rb (both powers of two)
  const int nr = rb, lgrb = __ffs(rb) - 1;
  const Tin *src = u + ((size_t)dof * g.nx + ix0) * g.ny;
  for (int i = threadIdx.x; i < nr * n; i += blockDim.x) {
    const int r = i >> p.lgn, k = i & (n - 1);
    if constexpr (sizeof(Tin) == sizeof(T))
      cp_async<2 * sizeof(T)>(&sm[r * cs + swz(k)], src + (size_t)r * g.ny + 2 * k);
    else
      sm[r * cs + swz(k)] = load_pair<Tin, T>(src + (size_t)r * g.ny + 2 * k);
  }
  cp_async_wait_all();
  __syncthreads();
  fft_dif<T>(sm, nr, cs, p, tab);
  const E *post = tab + p.tpost;
  const int tot = nr * (n + 1);
  for (int i = threadIdx.x; i < tot; i += blockDim.x) {
    const int ky = i >> lgrb, r = i & (nr - 1);
    const C<T> *row = sm + (size_t)r * cs;
    C<T> zk = row[srev[ky == n ? 0 : ky]];
    C<T> zc = cconj<T>(row[srev[ky == 0 ? 0 : n - ky]]);
    C<T> A = cadd<T>(zk, zc), B = csub<T>(zk, zc);
    C<T> wB = twmul(B, post[ky], -1);  // e^{-2 pi i ky/ny} B
    W[((size_t)ky * g.ndof + dof) * g.nxp + ix0 + r] =
        mk<T>((T)0.5 * (A.x + wB.y), (T)0.5 * (A.y - wB.x));
  }
}

// ---------------------------------------------------------------------------
template <typename T, typename Tout>
__global__ void __launch_bounds__(kRowThreads, sizeof(T) == 4 ? 3 : 2)
    k_row_inv_fast(const C<T> *__restrict__ W, Tout *__restrict__ f, Geom g, P2Plan p,
                   const typename TwE<T>::type *__restrict__ tab_g, int rb) {
  using E = typename TwE<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = p.n;
  E *tab = reinterpret_cast<E *>(smem_raw);
  unsigned short *srev = reinterpret_cast<unsigned short *>(smem_raw + (size_t)p.tsize * sizeof(E));
  C<T> *sm = reinterpret_cast<C<T> *>(smem_raw + (size_t)p.tsize * sizeof(E) + srev_bytes(n));
  load_table(tab, tab_g, p.tsize);
  make_srev(srev, p);
  cp_async_wait_all();  // the twiddle table
  __syncthreads();
  const int cs = n + 1;  // row pitch (one spare slot)
  const int dof = blockIdx.y;
  const int ix0 = blockIdx.x * rb;
  const int nr = rb, lgrb = __ffs(rb) - 1;
  // Gather fused with the complex-to-real pre-split, lanes over the block's
  // rows (16 lanes read 128 contiguous bytes of W per wavevector, and their
  // shared-memory stores land in distinct banks):
  //   Z[k] = (X[k] + conj X[n-k]) + i e^{+2 pi i k/ny} (X[k] - conj X[n-k]),
  // each thread owning the pair (k, n-k); imaginary parts of X[0], X[n] dropped.
  const E *post = tab + p.tpost;
  const int half = n / 2 + 1;
  const C<T> *Wd = W + (size_t)dof * g.nxp + ix0;
  const size_t kstride = (size_t)g.ndof * g.nxp;
#pragma unroll 4
  for (int i = threadIdx.x; i < nr * half; i += blockDim.x) {
    const int r = i & (nr - 1), k = i >> lgrb;
    C<T> *row = sm + (size_t)r * cs;
    const C<T> xk = Wd[(size_t)k * kstride + r];
    const C<T> xm = Wd[(size_t)(n - k) * kstride + r];  // k = 0: X[n]
    if (k == 0) {
      row[0] = mk<T>(xk.x + xm.x, xk.x - xm.x);  // slot of k = 0 is 0
    } else {
      const int pk = srev[k], pm = srev[n - k];
      {
        C<T> xc = cconj<T>(xm);
        C<T> A = cadd<T>(xk, xc), B = csub<T>(xk, xc);
        C<T> wB = twmul(B, post[k], +1);
        row[pk] = mk<T>(A.x - wB.y, A.y + wB.x);
      }
      if (pm != pk) {
        C<T> xc = cconj<T>(xk);
        C<T> A = cadd<T>(xm, xc), B = csub<T>(xm, xc);
        C<T> wB = twmul(B, post[n - k], +1);
        row[pm] = mk<T>(A.x - wB.y, A.y + wB.x);
      }
    }
  }
  __syncthreads();
  fft_dit_inv<T>(sm, nr, cs, p, tab);
  Tout *dst = f + ((size_t)dof * g.nx + ix0) * g.ny;
  for (int i = threadIdx.x; i < nr * n; i += blockDim.x) {
    const int r = i >> p.lgn, k = i & (n - 1);
    store_pair<Tout, T>(dst + (size_t)r * g.ny + 2 * k, sm[r * cs + swz(k)]);
  }
}

// ---------------------------------------------------------------------------
// One block per ky; all D columns along x resident in shared memory.
// phi: blocked layout [ky][nxp/32][D*D][32] over digit-reversed positions.
template <typename T, int D>
__global__ void __launch_bounds__(ColThreads<T, D>::value)
    k_col_phi_fast(C<T> *__restrict__ W, const T *__restrict__ phi, Geom g, P2Plan p,
                   const typename TwE<T>::type *__restrict__ tab_g,
                   const double *__restrict__ linf, double *__restrict__ epart,
                   double *__restrict__ scal, unsigned *__restrict__ counter,
                   double *__restrict__ d_epot) {
  using E = typename TwE<T>::type;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ double red[ColThreads<T, D>::value / 32];
  __shared__ int is_last;
  const int n = g.nx;
  const int ky = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarp = blockDim.x >> 5;
  constexpr unsigned kBlk = (unsigned)(D * D * 32 * sizeof(T));  // bytes per 32-wavevector block
  const int nkb = (n + 31) >> 5;
  const T *phik = phi + (size_t)ky * (g.nxp >> 5) * (D * D * 32);

  E *tab = reinterpret_cast<E *>(smem_raw);
  C<T> *sm = reinterpret_cast<C<T> *>(smem_raw + (size_t)p.tsize * sizeof(E));
  load_table(tab, tab_g, p.tsize);
  const int cs = n;
  C<T> *colg = W + (size_t)ky * D * g.nxp;
  for (int i = threadIdx.x; i < D * n; i += blockDim.x) {
    const int c = i >> p.lgn, x = i & (n - 1);
    cp_async<sizeof(C<T>)>(&sm[c * cs + swz(x)], &colg[(size_t)c * g.nxp + x]);
  }
  // The forward transform is compute-bound: start pulling the first round of
  // this block's Phi stream into L2 now, so the DRAM works during it; the
  // loop below keeps one round in flight (measured at 2048^2 ndof 12: one
  // round 0.87 ms per evaluation, two 0.92 ms, none 0.90 ms; deeper rounds
  // of all resident blocks no longer fit in L2).
  constexpr int kPhiAhead = 1;
  if (lane == 0)
    for (int r = 0; r < kPhiAhead; r++) {
      const int kb = warp + r * nwarp;
      if (kb < nkb) prefetch_l2(phik + (size_t)kb * (D * D * 32), kBlk);
    }
  cp_async_wait_all();
  __syncthreads();
  fft_dif<T>(sm, D, cs, p, tab);

  const bool mirror_self = (ky == 0) || (g.ny_even && ky == g.ny / 2);
  const double wgt = mirror_self ? 1.0 : 2.0;
  double e = 0.0;
  for (int kb = warp; kb < nkb; kb += nwarp) {
    if (lane == 0 && kb + kPhiAhead * nwarp < nkb)
      prefetch_l2(phik + (size_t)(kb + kPhiAhead * nwarp) * (D * D * 32), kBlk);
    const int q = (kb << 5) + lane;  // position in the digit-reversed order
    if (q >= n) continue;
    const int pos = swz(q);
    const T *ph = phik + (size_t)kb * (D * D * 32) + lane;
    C<T> uq[D], F[D];
#pragma unroll
    for (int j = 0; j < D; j++) {
      uq[j] = sm[j * cs + pos];
      T h = ph[j * 32];
      F[j] = mk<T>(h * uq[j].x, h * uq[j].y);
    }
    HermPairs<T, D>::run(ph, 32, uq, F);
    // Re(conj(F).u) of this wavevector in the working precision; the sum
    // over wavevectors and blocks is FP64 (FP64 is a slow pipe on GB300)
    T es = 0;
#pragma unroll
    for (int i = 0; i < D; i++) es = fma(F[i].x, uq[i].x, fma(F[i].y, uq[i].y, es));
    e += wgt * (double)es;
    if (ky == 0 && q == 0) {  // kx = 0 sits at position 0
#pragma unroll
      for (int j = 0; j < D; j++) scal[1 + j] = (double)uq[j].x;
#pragma unroll
      for (int l = 0; l < D / 3; l++) {
        e -= 2.0 * linf[l] * (double)uq[3 * l + 2].x;
        F[3 * l + 2].x -= (T)linf[l];
      }
    }
#pragma unroll
    for (int i = 0; i < D; i++) sm[i * cs + pos] = mk<T>(-F[i].x, -F[i].y);
  }
  __syncthreads();
  fft_dit_inv<T>(sm, D, cs, p, tab);
  for (int i = threadIdx.x; i < D * n; i += blockDim.x) {
    const int c = i >> p.lgn, x = i & (n - 1);
    colg[(size_t)c * g.nxp + x] = sm[c * cs + swz(x)];
  }

  // energy: block partial, then the last block sums all partials in order
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  if (lane == 0) red[warp] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < nwarp; w++) s += red[w];
    epart[ky] = s;
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

}  // namespace

}  // namespace gfmd

#endif
