// Device building blocks for the shared-memory Stockham FFTs of the force
// path: complex arithmetic, compensated twiddle products (FP32 path) and the
// radix-2/3/4/5/8 butterflies.
#ifndef GFMD_GB300_FFT_CUH
#define GFMD_GB300_FFT_CUH

#include <cuda_runtime.h>

#include <utility>

#include "gfmd_internal.h"

namespace gfmd {

template <typename T> struct CT;
template <> struct CT<float> { using type = float2; };
template <> struct CT<double> { using type = double2; };
template <typename T> using C = typename CT<T>::type;

template <typename T> __device__ __forceinline__ C<T> mk(T re, T im) {
  C<T> r;
  r.x = re;
  r.y = im;
  return r;
}
template <typename T> __device__ __forceinline__ C<T> cadd(C<T> a, C<T> b) { return mk<T>(a.x + b.x, a.y + b.y); }
template <typename T> __device__ __forceinline__ C<T> csub(C<T> a, C<T> b) { return mk<T>(a.x - b.x, a.y - b.y); }
template <typename T> __device__ __forceinline__ C<T> cscale(C<T> a, T s) { return mk<T>(a.x * s, a.y * s); }
template <typename T> __device__ __forceinline__ C<T> cconj(C<T> a) { return mk<T>(a.x, -a.y); }
// s * i * a for s = +-1
template <typename T> __device__ __forceinline__ C<T> cmuli(C<T> a, int s) {
  return s > 0 ? mk<T>(-a.y, a.x) : mk<T>(a.y, -a.x);
}
template <typename T> __device__ __forceinline__ C<T> cmul(C<T> a, C<T> b) {
  return mk<T>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// Twiddle table: FP64 keeps the exact double values; FP32 keeps hi + lo with
// hi = float(w), lo = float(w - hi), and multiplies by both, so the twiddle
// representation error (~3e-8) drops out of the transform and only the FP32
// arithmetic roundings remain.
template <typename T> struct Tw;
template <> struct Tw<double> {
  const double2 *hi;
  const void *lo_unused;
  __device__ __forceinline__ double2 get(int i, int sign) const {
    double2 w = hi[i];
    return sign < 0 ? w : make_double2(w.x, -w.y);
  }
  __device__ __forceinline__ double2 mul(double2 x, int i, int sign) const {
    return cmul<double>(x, get(i, sign));
  }
};
template <> struct Tw<float> {
  const float2 *hi;
  const float2 *lo;
  __device__ __forceinline__ float2 mul(float2 x, int i, int sign) const {
    float2 h = hi[i], l = lo[i];
    if (sign > 0) {
      h.y = -h.y;
      l.y = -l.y;
    }
    float cr = x.x * l.x - x.y * l.y;
    float ci = x.x * l.y + x.y * l.x;
    float re = fmaf(x.x, h.x, fmaf(-x.y, h.y, cr));
    float im = fmaf(x.x, h.y, fmaf(x.y, h.x, ci));
    return make_float2(re, im);
  }
};

// ---- butterflies: V[t] = sum_m v[m] exp(sign 2 pi i m t / R) --------------

template <typename T, int R> struct Dft;

template <typename T> struct Dft<T, 2> {
  static __device__ __forceinline__ void run(C<T> *v, int) {
    C<T> a = v[0], b = v[1];
    v[0] = cadd<T>(a, b);
    v[1] = csub<T>(a, b);
  }
};

template <typename T> struct Dft<T, 4> {
  static __device__ __forceinline__ void run(C<T> *v, int s) {
    C<T> s0 = cadd<T>(v[0], v[2]), d0 = csub<T>(v[0], v[2]);
    C<T> s1 = cadd<T>(v[1], v[3]), d1 = cmuli<T>(csub<T>(v[1], v[3]), s);
    v[0] = cadd<T>(s0, s1);
    v[2] = csub<T>(s0, s1);
    v[1] = cadd<T>(d0, d1);
    v[3] = csub<T>(d0, d1);
  }
};

template <typename T> struct Dft<T, 8> {
  static __device__ __forceinline__ void run(C<T> *v, int s) {
    const T h = (T)0.70710678118654752440084436210484904;
    C<T> a[4], b[4];
#pragma unroll
    for (int r = 0; r < 4; r++) {
      a[r] = cadd<T>(v[r], v[r + 4]);
      b[r] = csub<T>(v[r], v[r + 4]);
    }
    // b[r] *= exp(s 2 pi i r / 8)
    {
      C<T> t = b[1];
      b[1] = mk<T>(h * (t.x - s * t.y), h * (t.y + s * t.x));
      b[2] = cmuli<T>(b[2], s);
      t = b[3];
      b[3] = mk<T>(h * (-t.x - s * t.y), h * (-t.y + s * t.x));
    }
    Dft<T, 4>::run(a, s);
    Dft<T, 4>::run(b, s);
#pragma unroll
    for (int t = 0; t < 4; t++) {
      v[2 * t] = a[t];
      v[2 * t + 1] = b[t];
    }
  }
};

template <typename T> struct Dft<T, 3> {
  static __device__ __forceinline__ void run(C<T> *v, int s) {
    const T c = (T)-0.5, sn = (T)0.86602540378443864676372317075293618;
    C<T> t1 = cadd<T>(v[1], v[2]), t2 = csub<T>(v[1], v[2]);
    C<T> a = mk<T>(v[0].x + c * t1.x, v[0].y + c * t1.y);
    C<T> b = cscale<T>(cmuli<T>(t2, s), sn);
    v[0] = cadd<T>(v[0], t1);
    v[1] = cadd<T>(a, b);
    v[2] = csub<T>(a, b);
  }
};

template <typename T> struct Dft<T, 5> {
  static __device__ __forceinline__ void run(C<T> *v, int s) {
    const T c1 = (T)0.30901699437494742410229341718281906;
    const T c2 = (T)-0.80901699437494742410229341718281906;
    const T s1 = (T)0.95105651629515357211643933337938214;
    const T s2 = (T)0.58778525229247312916870595463907277;
    C<T> t1 = cadd<T>(v[1], v[4]), t2 = cadd<T>(v[2], v[3]);
    C<T> t3 = csub<T>(v[1], v[4]), t4 = csub<T>(v[2], v[3]);
    C<T> a1 = mk<T>(v[0].x + c1 * t1.x + c2 * t2.x, v[0].y + c1 * t1.y + c2 * t2.y);
    C<T> a2 = mk<T>(v[0].x + c2 * t1.x + c1 * t2.x, v[0].y + c2 * t1.y + c1 * t2.y);
    C<T> b1 = cmuli<T>(mk<T>(s1 * t3.x + s2 * t4.x, s1 * t3.y + s2 * t4.y), s);
    C<T> b2 = cmuli<T>(mk<T>(s2 * t3.x - s1 * t4.x, s2 * t3.y - s1 * t4.y), s);
    v[0] = cadd<T>(v[0], cadd<T>(t1, t2));
    v[1] = cadd<T>(a1, b1);
    v[4] = csub<T>(a1, b1);
    v[2] = cadd<T>(a2, b2);
    v[3] = csub<T>(a2, b2);
  }
};

// Radix 16 as 4 x 4: X[k1 + 4 k2] = sum_n2 w4^{n2 k2} w16^{n2 k1} sum_n1 x[4 n1 + n2] w4^{n1 k1}.
template <typename T> struct Dft<T, 16> {
  static __device__ __forceinline__ C<T> w16(int e, int s) {
    // exp(s 2 pi i e / 16), e in [0, 9]
    const T c1 = (T)0.92387953251128675612818318939678829;
    const T s1 = (T)0.38268343236508977172845998403039887;
    const T h = (T)0.70710678118654752440084436210484904;
    T cr, ci;
    switch (e) {
      case 0: cr = 1; ci = 0; break;
      case 1: cr = c1; ci = s1; break;
      case 2: cr = h; ci = h; break;
      case 3: cr = s1; ci = c1; break;
      case 4: cr = 0; ci = 1; break;
      case 6: cr = -h; ci = h; break;
      default: cr = -c1; ci = -s1; break;  // e = 9
    }
    return mk<T>(cr, s > 0 ? ci : -ci);
  }
  static __device__ __forceinline__ void run(C<T> *v, int s) {
    C<T> y[16];
#pragma unroll
    for (int n2 = 0; n2 < 4; n2++) {
      C<T> a[4];
#pragma unroll
      for (int n1 = 0; n1 < 4; n1++) a[n1] = v[4 * n1 + n2];
      Dft<T, 4>::run(a, s);
#pragma unroll
      for (int k1 = 0; k1 < 4; k1++)
        y[n2 * 4 + k1] = (n2 * k1 == 0) ? a[k1] : cmul<T>(a[k1], w16(n2 * k1, s));
    }
#pragma unroll
    for (int k1 = 0; k1 < 4; k1++) {
      C<T> b[4];
#pragma unroll
      for (int n2 = 0; n2 < 4; n2++) b[n2] = y[n2 * 4 + k1];
      Dft<T, 4>::run(b, s);
#pragma unroll
      for (int k2 = 0; k2 < 4; k2++) v[k1 + 4 * k2] = b[k2];
    }
  }
};

// F += H u for the off-diagonal part of a packed Hermitian D x D matrix
// (pair (I, J), I < J, at packed index D + 2 (I D - I (I+1)/2 + J - I - 1)
// holding (Re H_IJ, Im H_IJ)), fully unrolled at compile time so that u and F
// stay in registers.  ph points at element 0 of this wavevector; elements
// are ps apart.
template <typename T, int D> struct HermPairs {
  template <int I, int J>
  static __device__ __forceinline__ void pair(const T *__restrict__ ph, size_t ps, const C<T> *uq,
                                              C<T> *F) {
    constexpr int P = D + 2 * (I * D - I * (I + 1) / 2 + (J - I - 1));
    const T hr = ph[P * ps], hi = ph[(P + 1) * ps];
    F[I].x += hr * uq[J].x - hi * uq[J].y;
    F[I].y += hr * uq[J].y + hi * uq[J].x;
    F[J].x += hr * uq[I].x + hi * uq[I].y;
    F[J].y += hr * uq[I].y - hi * uq[I].x;
  }
  template <int I, int... Js>
  static __device__ __forceinline__ void row(const T *__restrict__ ph, size_t ps, const C<T> *uq,
                                             C<T> *F, std::integer_sequence<int, Js...>) {
    (pair<I, I + 1 + Js>(ph, ps, uq, F), ...);
  }
  template <int... Is>
  static __device__ __forceinline__ void rows(const T *__restrict__ ph, size_t ps, const C<T> *uq,
                                              C<T> *F, std::integer_sequence<int, Is...>) {
    (row<Is>(ph, ps, uq, F, std::make_integer_sequence<int, D - 1 - Is>{}), ...);
  }
  static __device__ __forceinline__ void run(const T *__restrict__ ph, size_t ps, const C<T> *uq,
                                             C<T> *F) {
    rows(ph, ps, uq, F, std::make_integer_sequence<int, D - 1>{});
  }
};

// The pairs of a table stored in pattern PAT (pat_keeps): the p-th kept pair
// at elements D + 2p, D + 2p + 1, applied in row-major order like HermPairs.
template <typename T, int D, int PAT> struct HermPairsPat {
  template <int P>
  static __device__ __forceinline__ void pair(const T *__restrict__ ph, size_t ps, const C<T> *uq,
                                              C<T> *F) {
    constexpr int I = pat_pair(D, PAT, P, 0), J = pat_pair(D, PAT, P, 1), E = D + 2 * P;
    const T hr = ph[E * ps], hi = ph[(E + 1) * ps];
    F[I].x += hr * uq[J].x - hi * uq[J].y;
    F[I].y += hr * uq[J].y + hi * uq[J].x;
    F[J].x += hr * uq[I].x + hi * uq[I].y;
    F[J].y += hr * uq[I].y - hi * uq[I].x;
  }
  template <int... Ps>
  static __device__ __forceinline__ void all(const T *__restrict__ ph, size_t ps, const C<T> *uq, C<T> *F,
                                             std::integer_sequence<int, Ps...>) {
    (pair<Ps>(ph, ps, uq, F), ...);
  }
  static __device__ __forceinline__ void run(const T *__restrict__ ph, size_t ps, const C<T> *uq, C<T> *F) {
    all(ph, ps, uq, F, std::make_integer_sequence<int, pat_pairs(D, PAT)>{});
  }
};

// One Stockham stage over `nb` transforms of length n stored with stride
// bstride (complex elements), in -> out:
//   out[(j/Ns)*Ns*R + j%Ns + r*Ns] = DFT_R( in[j + t*n/R] * w^(t*(j%Ns)) )[r].
template <typename T, int R>
__device__ __forceinline__ void stage_r(const C<T> *__restrict__ in, C<T> *__restrict__ out, int n,
                                        int Ns, int nb, int bstride, const Tw<T> &tw, int twoff,
                                        int sign, int tid, int nth) {
  const int m = n / R;
  const int total = m * nb;
  for (int idx = tid; idx < total; idx += nth) {
    const int b = idx / m;
    const int j = idx - b * m;
    const int k = j % Ns;
    const C<T> *ib = in + (size_t)b * bstride;
    C<T> *ob = out + (size_t)b * bstride;
    C<T> v[R];
#pragma unroll
    for (int r = 0; r < R; r++) {
      C<T> x = ib[j + r * m];
      v[r] = (r == 0 || Ns == 1) ? x : tw.mul(x, twoff + k * R + r, sign);
    }
    Dft<T, R>::run(v, sign);
    const int base = (j / Ns) * Ns * R + k;
#pragma unroll
    for (int r = 0; r < R; r++) ob[base + r * Ns] = v[r];
  }
}

// Stage with a radix that has no hand-written butterfly (odd primes > 5):
// a direct O(R^2) DFT per butterfly, roots from the table.
template <typename T>
__device__ void stage_generic(const C<T> *__restrict__ in, C<T> *__restrict__ out, int n, int R,
                              int Ns, int nb, int bstride, const Tw<T> &tw, int twoff, int rootoff,
                              int sign, int tid, int nth) {
  const int m = n / R;
  const int total = m * nb;
  for (int idx = tid; idx < total; idx += nth) {
    const int b = idx / m;
    const int j = idx - b * m;
    const int k = j % Ns;
    const C<T> *ib = in + (size_t)b * bstride;
    C<T> *ob = out + (size_t)b * bstride;
    const int base = (j / Ns) * Ns * R + k;
    for (int t = 0; t < R; t++) {
      C<T> acc = mk<T>(0, 0);
      for (int q = 0; q < R; q++) {
        C<T> x = ib[j + q * m];
        if (q != 0 && Ns != 1) x = tw.mul(x, twoff + k * R + q, sign);
        int e = (q * t) % R;
        acc = cadd<T>(acc, e == 0 ? x : tw.mul(x, rootoff + e, sign));
      }
      ob[base + t * Ns] = acc;
    }
  }
}

// Full transform of nb rows, ping-ponging between a and b.  Returns the
// buffer holding the result.  Every thread of the block must call it.
template <typename T>
__device__ C<T> *fft_block(C<T> *a, C<T> *b, const FftPlan &p, int nb, int bstride,
                           const Tw<T> &tw, int sign) {
  const int tid = threadIdx.x, nth = blockDim.x;
  for (int s = 0; s < p.nst; s++) {
    const int R = p.radix[s], Ns = p.span[s], off = p.twoff[s];
    switch (R) {
      case 2: stage_r<T, 2>(a, b, p.n, Ns, nb, bstride, tw, off, sign, tid, nth); break;
      case 3: stage_r<T, 3>(a, b, p.n, Ns, nb, bstride, tw, off, sign, tid, nth); break;
      case 4: stage_r<T, 4>(a, b, p.n, Ns, nb, bstride, tw, off, sign, tid, nth); break;
      case 5: stage_r<T, 5>(a, b, p.n, Ns, nb, bstride, tw, off, sign, tid, nth); break;
      case 8: stage_r<T, 8>(a, b, p.n, Ns, nb, bstride, tw, off, sign, tid, nth); break;
      default:
        stage_generic<T>(a, b, p.n, R, Ns, nb, bstride, tw, off, p.rootoff[s], sign, tid, nth);
    }
    __syncthreads();
    C<T> *t = a;
    a = b;
    b = t;
  }
  return a;
}

}  // namespace gfmd

#endif
