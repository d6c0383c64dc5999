// Row transforms of the FP32 force path for rows of n = 1024 complex points
// (ny = 2048 reals): one warp per row, the transform held in registers.
//
// A row of n = 32 x 32 points is transformed in two register passes (the
// "four-step" factorisation): lane l holds x[l + 32 m], m < 32, and computes
// the 32-point DFT over m in registers; the result is multiplied by the
// compensated twiddle w_n^(l k1) and transposed through the warp's own
// shared-memory row (XOR-swizzled, conflict-free); the second 32-point DFT
// leaves X[l + 32 k2] in lane l, i.e. natural order, strided over lanes.
//
//   k_row_fwd_w32  u rows (global, coalesced 256-byte warp loads) -> row FFT
//                  -> real-to-half-complex split -> W[ky][dof][x] tiles
//                  written by TMA tensor stores from a double-buffered
//                  shared-memory stage (8 consecutive x per ky: 64 bytes);
//   k_row_inv_w32  W tiles loaded by TMA into a double-buffered stage ->
//                  complex-to-real pre-split -> row FFT -> f rows (global,
//                  coalesced stores).
//
// A block owns 8 consecutive rows x = ix0..ix0+7 of one degree of freedom.
// The half spectrum ky = 0..n is processed in mirror pairs (ky, n - ky):
// chunk c covers ky in [c C, (c+1) C) and its mirrors (n - (c+1) C, n - c C],
// both as C x 8 tiles; ky = n/2 is its own mirror and moves through plain
// loads and stores.
#ifndef GFMD_GB300_ROWS_WARP_CUH
#define GFMD_GB300_ROWS_WARP_CUH

#include <cuda.h>
#include <cstdint>
#include <cuda_runtime.h>

#include "gfmd_fft.cuh"
#include "gfmd_internal.h"
#include "gfmd_tma.cuh"

namespace gfmd {

namespace rows32 {

constexpr int kN = 1024;  // complex points per row

// Block shape: RB rows (one warp each) and tiles of C ky x RB x, i.e. RB * 8
// contiguous bytes of W per ky (64 bytes at RB = 8, 128 bytes at RB = 16).
// The row buffer pitch keeps the split's (row, ky) accesses conflict-free.
template <int RB> struct Cfg {
  static constexpr int kRB = RB;
  static constexpr int kThreads = 32 * RB;
  static constexpr int kPitch = RB == 8 ? kN + 2 : kN + 1;
  static constexpr int kChunk = RB == 8 ? 128 : 64;
  static constexpr int kNChunk = kN / 2 / kChunk;
  static constexpr int kTile = kChunk * RB;  // complex per tile
  static constexpr size_t kRowBytes = (size_t)RB * kPitch * 8;
  static constexpr size_t kStageOff = (128 + kRowBytes + 127) / 128 * 128;
  static constexpr size_t kStageBytes = (size_t)2 * 2 * kTile * 8;  // 2 buffers x (lo, hi)
  static constexpr size_t kSmemBytes = kStageOff + kStageBytes;     // + mbarriers at 0
};

// 32-point DFT in registers, natural order in and out:
// X[k] = sum_m x[m] exp(sign 2 pi i m k / 32).  Decimation in time:
// two 16-point DFTs of the even and odd samples, one radix-2 combine.
template <int SIGN> __device__ __forceinline__ void dft32(float2 *x) {
  float2 e[16], o[16];
#pragma unroll
  for (int m = 0; m < 16; m++) {
    e[m] = x[2 * m];
    o[m] = x[2 * m + 1];
  }
  Dft<float, 16>::run(e, SIGN);
  Dft<float, 16>::run(o, SIGN);
  // cos, sin of 2 pi k / 32, k = 0..15
  const float cs[16] = {1.0f, 0.98078528040323044913f, 0.92387953251128675613f, 0.83146961230254523708f,
                        0.70710678118654752440f, 0.55557023301960222474f, 0.38268343236508977173f,
                        0.19509032201612826785f, 0.0f, -0.19509032201612826785f, -0.38268343236508977173f,
                        -0.55557023301960222474f, -0.70710678118654752440f, -0.83146961230254523708f,
                        -0.92387953251128675613f, -0.98078528040323044913f};
  const float sn[16] = {0.0f, 0.19509032201612826785f, 0.38268343236508977173f, 0.55557023301960222474f,
                        0.70710678118654752440f, 0.83146961230254523708f, 0.92387953251128675613f,
                        0.98078528040323044913f, 1.0f, 0.98078528040323044913f, 0.92387953251128675613f,
                        0.83146961230254523708f, 0.70710678118654752440f, 0.55557023301960222474f,
                        0.38268343236508977173f, 0.19509032201612826785f};
#pragma unroll
  for (int k = 0; k < 16; k++) {
    float2 t;
    if (k == 0) {
      t = o[0];
    } else if (k == 8) {
      t = SIGN > 0 ? make_float2(-o[8].y, o[8].x) : make_float2(o[8].y, -o[8].x);
    } else {
      const float c = cs[k], s = SIGN > 0 ? sn[k] : -sn[k];
      t = make_float2(fmaf(o[k].x, c, -o[k].y * s), fmaf(o[k].x, s, o[k].y * c));
    }
    x[k] = make_float2(e[k].x + t.x, e[k].y + t.y);
    x[k + 16] = make_float2(e[k].x - t.x, e[k].y - t.y);
  }
}

// x * w (SIGN < 0) or x * conj(w) (SIGN > 0) with the compensated twiddle
// w = (c_hi + c_lo, s_hi + s_lo).
template <int SIGN> __device__ __forceinline__ float2 twc(float2 x, float4 w) {
  const float sh = SIGN < 0 ? w.y : -w.y, sl = SIGN < 0 ? w.w : -w.w;
  const float cr = x.x * w.z - x.y * sl;
  const float ci = x.x * sl + x.y * w.z;
  return make_float2(fmaf(x.x, w.x, fmaf(-x.y, sh, cr)), fmaf(x.x, sh, fmaf(x.y, w.x, ci)));
}

// Full n-point transform of the warp's row held as x[m] = row[l + 32 m]:
// returns X[l + 32 k2] in x[k2].  tw: [k1][l] table of w_n^(l k1)
// (compensated, n = 1024).  scratch: 1024 complex of this warp's own.
template <int SIGN>
__device__ __forceinline__ void row_fft(float2 *x, const float4 *__restrict__ tw, float2 *scratch, int lane) {
  dft32<SIGN>(x);
#pragma unroll
  for (int k1 = 1; k1 < 32; k1++) x[k1] = twc<SIGN>(x[k1], __ldg(&tw[k1 * 32 + lane]));
  // transpose: element (n2 = lane, k1) to lane k1, register n2
#pragma unroll
  for (int k1 = 0; k1 < 32; k1++) scratch[lane * 32 + (k1 ^ lane)] = x[k1];
  __syncwarp();
#pragma unroll
  for (int n2 = 0; n2 < 32; n2++) x[n2] = scratch[n2 * 32 + (lane ^ n2)];
  __syncwarp();
  dft32<SIGN>(x);
}

// Records a lost wait in the handle's error word.
__device__ __forceinline__ void report_timeout(int *err) { atomicExch(err, (int)GFMD_ETIMEDOUT); }

}  // namespace rows32

// ---------------------------------------------------------------------------
// Split of the forward transform: from X[k], X[n-k] (xk, xm) the half-spectrum
// values W[k] (.x, .y) and W[n-k] (.z, .w); post(k) = e^{-2 pi i k / (2n)}.
__device__ __forceinline__ float2 fwd_split_one(float2 xk, float2 xm, float4 pk) {
  const float2 A = make_float2(xk.x + xm.x, xk.y - xm.y), B = make_float2(xk.x - xm.x, xk.y + xm.y);
  const float2 wB = rows32::twc<-1>(B, pk);
  return make_float2(0.5f * (A.x + wB.y), 0.5f * (A.y - wB.x));
}

// Pre-split of the inverse transform: Z[k] from X[k], X[n-k].
__device__ __forceinline__ float2 inv_split_one(float2 xk, float2 xm, float4 pk) {
  const float2 A = make_float2(xk.x + xm.x, xk.y - xm.y), B = make_float2(xk.x - xm.x, xk.y + xm.y);
  const float2 wB = rows32::twc<+1>(B, pk);
  return make_float2(A.x - wB.y, A.y + wB.x);
}

// Blocks are persistent: block b takes the row sets s = b, b + gridDim.x, ...
// (set s: dof = s / (nx/RB), rows ix0 = RB (s mod nx/RB) .. ix0 + RB - 1).  The
// global loads (forward) or TMA tile loads (inverse) of the next set are
// issued before the current set's split or transform, so they are in flight
// while the block computes.

// Forward: u[dof][x][2n] (Tin) -> W[ky][dof][x] complex FP32, ky = 0..n.
// tmW: 3-D tensor map of W as floats {2 nxp, ndof, nyc}, box {2 RB, 1, C}.
// tw: [k1][l] compensated w_n^(l k1); post: e^{-2 pi i k / (2n)}, k = 0..n.
template <typename Tin, int RB>
__global__ void __launch_bounds__(32 * RB, RB == 8 ? 2 : 1)
    k_row_fwd_w32(const Tin *__restrict__ u, float2 *__restrict__ W, const __grid_constant__ CUtensorMap tmW,
                  Geom g, const float4 *__restrict__ tw, const float4 *__restrict__ post) {
  using namespace rows32;
  using K = Cfg<RB>;
  constexpr int kRB = K::kRB, kPitch = K::kPitch, kChunk = K::kChunk, kNChunk = K::kNChunk, kTile = K::kTile;
  extern __shared__ __align__(128) unsigned char smem_rows[];
  float2 *xs = reinterpret_cast<float2 *>(smem_rows + 128);
  float2 *stage = reinterpret_cast<float2 *>(smem_rows + K::kStageOff);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nxb = g.nx / kRB, nsets = nxb * g.ndof;
  if (threadIdx.x == 0) prefetch_tmap(&tmW);
  const int r = threadIdx.x & (kRB - 1), j0 = threadIdx.x / kRB;

  float2 x[32];
  auto load_rows = [&](int set) {  // this warp's row of the set, into x
    const int dof = set / nxb, ix0 = (set % nxb) * kRB;
    const Tin *src = u + ((size_t)dof * g.nx + ix0 + warp) * (size_t)(2 * kN);
#pragma unroll
    for (int m = 0; m < 32; m++) {
      if constexpr (sizeof(Tin) == 4) {
        x[m] = __ldcs(reinterpret_cast<const float2 *>(src) + lane + 32 * m);
      } else {
        const double2 v = __ldcs(reinterpret_cast<const double2 *>(src) + lane + 32 * m);
        x[m] = make_float2((float)v.x, (float)v.y);
      }
    }
  };
  if ((int)blockIdx.x < nsets) load_rows(blockIdx.x);
  int cc = 0;  // tiles pairs committed by this block so far (stage buffer parity)
  const bool aligned = ((uintptr_t)u & 15) == 0;
  for (int set = blockIdx.x; set < nsets; set += gridDim.x) {
    const int dof = set / nxb, ix0 = (set % nxb) * kRB;
    // the next set's row of this warp streams into L2 during the transform
    // (its loads, issued after it, then hit L2)
    if (lane == 0 && aligned && set + (int)gridDim.x < nsets) {
      const int nset = set + gridDim.x, ndof = nset / nxb, nix0 = (nset % nxb) * kRB;
      bulk_prefetch_l2(u + ((size_t)ndof * g.nx + nix0 + warp) * (size_t)(2 * kN), 2 * kN * sizeof(Tin));
    }
    // ---- row transform (one warp per row) ----
    {
      float2 *row = xs + warp * kPitch;
      row_fft<-1>(x, tw, row, lane);
#pragma unroll
      for (int k2 = 0; k2 < 32; k2++) row[lane + 32 * k2] = x[k2];
    }
    __syncthreads();
    if (set + (int)gridDim.x < nsets) load_rows(set + gridDim.x);  // in flight during the split

    // ---- real-to-half-complex split in mirror pairs of tiles ----
    // thread (r = t % 8, j = t / 8 + 32 i): row r, ky = a + j and n - a - j
    const float2 *row = xs + r * kPitch;
    for (int c = 0; c < kNChunk; c++, cc++) {
      float2 *lo = stage + (cc & 1) * 2 * kTile, *hi = lo + kTile;
      if (cc >= 2) {
        if (threadIdx.x == 0) bulk_wait_read<1>();  // the stores of pair cc - 2 have left this buffer
        __syncthreads();
      }
      const int a = c * kChunk, hbase = kN - a - kChunk + 1;  // hi tile: ky = hbase .. n - a
#pragma unroll 4
      for (int j = j0; j < kChunk; j += K::kThreads / kRB) {
        const int k = a + j;
        const float2 xk = row[k], xm = row[(kN - k) & (kN - 1)];
        lo[j * kRB + r] = fwd_split_one(xk, xm, __ldg(&post[k]));
        hi[(kChunk - 1 - j) * kRB + r] = fwd_split_one(xm, xk, __ldg(&post[kN - k]));
      }
      fence_proxy_async_smem();
      __syncthreads();
      if (threadIdx.x == 0) {
        tma_store_3d(&tmW, 2 * ix0, dof, a, lo);
        tma_store_3d(&tmW, 2 * ix0, dof, hbase, hi);
        bulk_commit();
      }
    }
    // ky = n/2 is its own mirror: plain stores
    if (threadIdx.x < kRB) {
      const float2 xk = xs[threadIdx.x * kPitch + kN / 2];
      W[((size_t)(kN / 2) * g.ndof + dof) * g.nxp + ix0 + threadIdx.x] = fwd_split_one(xk, xk, __ldg(&post[kN / 2]));
    }
    __syncthreads();  // the split's reads of the row buffer are done before the next transform
  }
  if (threadIdx.x == 0) bulk_wait<0>();
}

// ---------------------------------------------------------------------------
// Inverse: W[ky][dof][x] complex FP32 -> f[dof][x][2n] (Tout).  The tiles
// come in by TMA, two mirror pairs in flight (the first two of the next set
// load during the current set's transform); err receives GFMD_ETIMEDOUT if a
// tile never arrives (the block then stops).
template <typename Tout, int RB>
__global__ void __launch_bounds__(32 * RB, RB == 8 ? 2 : 1)
    k_row_inv_w32(const float2 *__restrict__ W, const __grid_constant__ CUtensorMap tmW, Tout *__restrict__ f,
                  Geom g, const float4 *__restrict__ tw, const float4 *__restrict__ post, int *err) {
  using namespace rows32;
  using K = Cfg<RB>;
  constexpr int kRB = K::kRB, kPitch = K::kPitch, kChunk = K::kChunk, kNChunk = K::kNChunk, kTile = K::kTile;
  extern __shared__ __align__(128) unsigned char smem_rows[];
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem_rows);
  float2 *xs = reinterpret_cast<float2 *>(smem_rows + 128);
  float2 *stage = reinterpret_cast<float2 *>(smem_rows + K::kStageOff);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int nxb = g.nx / kRB, nsets = nxb * g.ndof;
  // pair p (global count) of this block: set blockIdx.x + (p / kNChunk) gridDim.x,
  // chunk p % kNChunk, buffer p & 1, mbarrier phase (p >> 1) & 1
  const int npairs = ((int)blockIdx.x < nsets ? (nsets - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0) * kNChunk;
  auto issue = [&](int p) {  // thread 0: both tiles of pair p
    const int set = blockIdx.x + (p / kNChunk) * gridDim.x, c = p % kNChunk;
    const int dof = set / nxb, ix0 = (set % nxb) * kRB;
    float2 *lo = stage + (p & 1) * 2 * kTile, *hi = lo + kTile;
    mbar_arrive_tx(&bar[p & 1], 2 * kTile * 8);
    tma_load_3d(lo, &tmW, 2 * ix0, dof, c * kChunk, &bar[p & 1]);
    tma_load_3d(hi, &tmW, 2 * ix0, dof, kN - c * kChunk - kChunk + 1, &bar[p & 1]);
  };
  if (threadIdx.x == 0) {
    prefetch_tmap(&tmW);
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    if (npairs > 0) issue(0);
    if (npairs > 1) issue(1);
  }
  __syncthreads();  // barrier initialisation visible to all threads
  const int r = threadIdx.x & (kRB - 1), j0 = threadIdx.x / kRB;
  float2 *rowr = xs + r * kPitch;
  int p = 0;
  for (int set = blockIdx.x; set < nsets; set += gridDim.x) {
    const int dof = set / nxb, ix0 = (set % nxb) * kRB;
    // ky = n/2 (its own mirror) with plain loads
    if (threadIdx.x < kRB) {
      const float2 xk = W[((size_t)(kN / 2) * g.ndof + dof) * g.nxp + ix0 + threadIdx.x];
      xs[threadIdx.x * kPitch + kN / 2] = inv_split_one(xk, xk, __ldg(&post[kN / 2]));
    }
    for (int c = 0; c < kNChunk; c++, p++) {
      const float2 *lo = stage + (p & 1) * 2 * kTile, *hi = lo + kTile;
      const bool ok = mbar_wait(&bar[p & 1], (p >> 1) & 1);
      if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) report_timeout(err);
        return;
      }
      const int a = c * kChunk;
#pragma unroll 4
      for (int j = j0; j < kChunk; j += K::kThreads / kRB) {
        const int k = a + j;
        const float2 xk = lo[j * kRB + r], xm = hi[(kChunk - 1 - j) * kRB + r];  // X[k], X[n-k]
        if (k == 0) {
          rowr[0] = make_float2(xk.x + xm.x, xk.x - xm.x);  // imaginary parts of X[0], X[n] dropped
        } else {
          rowr[k] = inv_split_one(xk, xm, __ldg(&post[k]));
          rowr[kN - k] = inv_split_one(xm, xk, __ldg(&post[kN - k]));
        }
      }
      __syncthreads();  // buffer p & 1 consumed
      if (threadIdx.x == 0 && p + 2 < npairs) issue(p + 2);
    }
    // ---- row transform (one warp per row) ----
    float2 *row = xs + warp * kPitch;
    float2 x[32];
#pragma unroll
    for (int m = 0; m < 32; m++) x[m] = row[lane + 32 * m];
    __syncwarp();
    row_fft<+1>(x, tw, row, lane);
    Tout *dst = f + ((size_t)dof * g.nx + ix0 + warp) * (size_t)(2 * kN);
#pragma unroll
    for (int k2 = 0; k2 < 32; k2++) {
      if constexpr (sizeof(Tout) == 4)
        __stcs(reinterpret_cast<float2 *>(dst) + lane + 32 * k2, x[k2]);
      else
        __stcs(reinterpret_cast<double2 *>(dst) + lane + 32 * k2, make_double2((double)x[k2].x, (double)x[k2].y));
    }
    __syncthreads();  // row buffers free before the next set's pre-split
  }
}

}  // namespace gfmd

#endif
