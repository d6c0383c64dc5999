// Deterministic reductions shared by the solver loops: per-thread FP64 or
// compensated FP32 dot products, block partials, and a fixed-order final
// combination by the last block to finish (no second launch, no host
// round trip).
#pragma once
#include <cuda_runtime.h>

namespace gfmd {
namespace red {

constexpr int kT = 256;  // threads per block of the reducing kernels
constexpr int kQ = 10;   // partial slots per block

template <typename T> struct Dot;
template <> struct Dot<double> {
  double s = 0.0;
  __device__ __forceinline__ void add(double a, double b) { s = fma(a, b, s); }
  __device__ __forceinline__ void addsum(double p) { s += p; }
  __device__ __forceinline__ double get() const { return s; }
};
// Compensated FP32 dot product: TwoProd via fmaf, TwoSum on the running sum.
template <> struct Dot<float> {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ void add(float a, float b) {
    const float p = __fmul_rn(a, b);
    const float pe = fmaf(a, b, -p);
    const float s = __fadd_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float se = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = __fadd_rn(lo, __fadd_rn(se, pe));
  }
  // adds a partial sum (TwoSum only)
  __device__ __forceinline__ void addsum(float p) {
    const float s = __fadd_rn(hi, p);
    const float bb = __fsub_rn(s, hi);
    const float se = __fadd_rn(__fsub_rn(hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    hi = s;
    lo = __fadd_rn(lo, se);
  }
  __device__ __forceinline__ double get() const { return (double)hi + (double)lo; }
};

// Block partials of NS sums followed by NM maxima -> part; the block that
// finishes last combines all partials in a fixed order into res[] and
// returns true (all its threads).
template <int NS, int NM>
__device__ bool reduce_last(const double *acc, double *part, unsigned int *counter, double *res) {
  constexpr int NQ = NS + NM;
  static_assert(NQ <= kQ, "too many reduced scalars");
  __shared__ double sh[kT / 32][NQ];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NQ; k++) {
    double v = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double t = __shfl_down_sync(0xffffffffu, v, o);
      v = (k >= NS) ? fmax(v, t) : v + t;
    }
    if (lane == 0) sh[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < NQ) {
    const int k = threadIdx.x;
    double v = sh[0][k];
    for (int w = 1; w < kT / 32; w++) v = (k >= NS) ? fmax(v, sh[w][k]) : v + sh[w][k];
    part[blockIdx.x * kQ + k] = v;
    __threadfence();
  }
  __syncthreads();
  if (threadIdx.x == 0) last = atomicInc(counter, gridDim.x - 1) == gridDim.x - 1;
  __syncthreads();
  if (!last) return false;
#pragma unroll
  for (int k = 0; k < NQ; k++) {
    double v = 0.0;  // sums start at 0; maxima are of |.| >= 0
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kT) {
      const double t = __ldcg(part + (size_t)b * kQ + k);
      v = (k >= NS) ? fmax(v, t) : v + t;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double t = __shfl_down_sync(0xffffffffu, v, o);
      v = (k >= NS) ? fmax(v, t) : v + t;
    }
    if (lane == 0) sh[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < NQ) {
    const int k = threadIdx.x;
    double v = sh[0][k];
    for (int w = 1; w < kT / 32; w++) v = (k >= NS) ? fmax(v, sh[w][k]) : v + sh[w][k];
    res[k] = v;
  }
  __syncthreads();
  return true;
}

}  // namespace red
}  // namespace gfmd
