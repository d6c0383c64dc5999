// Vector loads and stores of the streaming solver kernels.
#pragma once
#include <cuda_runtime.h>

namespace gfmd {

// V consecutive sites per thread: V = 4 with 16-byte loads (two for FP64)
// for grids with nx*ny divisible by 4 (all power-of-two grids), V = 1 else.
// The streaming kernels are bound by the loads each thread keeps in flight.
template <typename T, int V> struct VecN;
template <typename T> struct VecN<T, 1> {
  static __device__ __forceinline__ void ld(const T *p, T o[1]) { o[0] = *p; }
  static __device__ __forceinline__ void st(T *p, const T o[1]) { *p = o[0]; }
};
template <> struct VecN<float, 4> {
  static __device__ __forceinline__ void ld(const float *p, float o[4]) {
    const float4 v = *reinterpret_cast<const float4 *>(p);
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
  }
  static __device__ __forceinline__ void st(float *p, const float o[4]) {
    *reinterpret_cast<float4 *>(p) = make_float4(o[0], o[1], o[2], o[3]);
  }
};
template <> struct VecN<double, 4> {
  static __device__ __forceinline__ void ld(const double *p, double o[4]) {
    const double2 a = *reinterpret_cast<const double2 *>(p), b = *reinterpret_cast<const double2 *>(p + 2);
    o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
  }
  static __device__ __forceinline__ void st(double *p, const double o[4]) {
    *reinterpret_cast<double2 *>(p) = make_double2(o[0], o[1]);
    *reinterpret_cast<double2 *>(p + 2) = make_double2(o[2], o[3]);
  }
};

}  // namespace gfmd
