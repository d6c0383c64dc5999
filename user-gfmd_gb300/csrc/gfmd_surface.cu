// Self-affine rough surfaces by random-phase synthesis on the GPU: the
// half spectrum is written directly into the layout of the FP64 plain-path
// transform, then one inverse column FFT and one c2r row pass (the same
// kernels as the force evaluation) give the real heights, scaled to the
// requested spectral rms slope.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "gfmd_fft.cuh"
#include "gfmd_internal.h"
#include "gfmd_plain_kernels.cuh"

namespace gfmd {

namespace {

constexpr double kTwoPi = 6.283185307179586476925286766559;

struct SurfSpec {
  int nx, ny, nyc, nxp;
  double dqx, dqy;      // 2 pi / (n a)
  double ql2, qs2;      // squared cut-offs
  double expo;          // -(1 + H): C = (q^2 / q_L^2)^expo
  unsigned long long seed;
};

// SplitMix64 output function (Steele, Lea and Flood 2014).
__host__ __device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Uniform [0, 1) for half-spectrum index (i, j).
__device__ __forceinline__ double uniform(const SurfSpec &sp, int i, int j) {
  const unsigned long long key = (unsigned long long)i * (unsigned long long)sp.nyc + (unsigned long long)j;
  const unsigned long long z = mix64(sp.seed ^ mix64(key));
  return (double)(z >> 11) * 0x1.0p-53;
}

// One thread per (kx = i, ky = j): Z into W[j * nxp + i]; block partial of
// w |q|^2 C(q) (w = 1 on the ky = 0 and Nyquist columns, 2 elsewhere).
__global__ void __launch_bounds__(256) k_surface_spectrum(SurfSpec sp, double2 *__restrict__ W,
                                                          double *__restrict__ part) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  double acc = 0.0;
  if (i < sp.nx) {
    const int kx = i <= sp.nx / 2 ? i : i - sp.nx;
    const double qx = sp.dqx * kx, qy = sp.dqy * j;
    const double q2 = qx * qx + qy * qy;
    double amp = 0.0;
    if (q2 > 0.0 && q2 >= sp.ql2 && q2 <= sp.qs2) amp = sqrt(pow(q2 / sp.ql2, sp.expo));
    const bool herm = (j == 0) || (sp.ny % 2 == 0 && j == sp.ny / 2);
    double2 z = make_double2(0.0, 0.0);
    if (amp > 0.0) {
      if (herm) {
        const int ii = i == 0 ? 0 : min(i, sp.nx - i);
        const double u = uniform(sp, ii, j);
        if (i == 0 || 2 * i == sp.nx) {
          z.x = u < 0.5 ? amp : -amp;  // self-conjugate point: real
        } else {
          double sn, cs;
          sincospi(2.0 * u, &sn, &cs);
          z.x = amp * cs;
          z.y = (i == ii) ? amp * sn : -amp * sn;
        }
      } else {
        double sn, cs;
        sincospi(2.0 * uniform(sp, i, j), &sn, &cs);
        z.x = amp * cs;
        z.y = amp * sn;
      }
      acc = (herm ? 1.0 : 2.0) * q2 * amp * amp;
    }
    W[(size_t)j * sp.nxp + i] = z;
  }
  __shared__ double sh[8];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = sh[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) v += sh[w];
    part[(size_t)blockIdx.y * gridDim.x + blockIdx.x] = v;
  }
}

// Fixed-order sum of n partials into out[0].
__global__ void __launch_bounds__(256) k_sum(const double *__restrict__ part, int n, double *__restrict__ out) {
  __shared__ double sh[8];
  double v = 0.0;
  for (int b = threadIdx.x; b < n; b += blockDim.x) v += part[b];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = sh[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    out[0] = t;
  }
}

__global__ void k_scale_to_slope(size_t n, double *__restrict__ h, const double *__restrict__ sum,
                                 double slope) {
  const double s = sum[0] > 0.0 ? slope / sqrt(sum[0]) : 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    h[i] *= s;
}

struct Scratch {
  std::vector<void *> p;
  ~Scratch() {
    for (void *q : p) cudaFree(q);
  }
  cudaError_t alloc(void **out, size_t bytes) {
    cudaError_t e = cudaMalloc(out, bytes);
    if (e == cudaSuccess) p.push_back(*out);
    return e;
  }
};

}  // namespace

}  // namespace gfmd

extern "C" int gfmd_rough_surface(int nx, int ny, const gfmd_surface_params_t *prm, double *d_h,
                                  void *stream_) {
  using namespace gfmd;
  if (!prm || !d_h) return set_error(GFMD_EINVAL, "gfmd_rough_surface: NULL argument");
  if (nx < 2 || ny < 2 || nx > 8192 || ny > 8192)
    return set_error(GFMD_EINVAL, "gfmd_rough_surface: nx, ny must be in [2, 8192]");
  if (!(prm->lattice > 0.0) || !(prm->rms_slope > 0.0) || !(prm->lambda_short > 0.0) ||
      !(prm->lambda_long >= prm->lambda_short) || !std::isfinite(prm->hurst))
    return set_error(GFMD_EINVAL, "gfmd_rough_surface: bad spectrum parameters");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream_);
  Geom g{};
  g.nx = nx;
  g.ny = ny;
  g.ndof = 1;
  g.nyc = ny / 2 + 1;
  g.nxp = (nx + 31) / 32 * 32;
  g.ny_even = ny % 2 == 0 ? 1 : 0;
  g.nrow = g.ny_even ? ny / 2 : ny;
  g.npk = 1;
  int dev = 0, smem = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t cs = sizeof(double2);
  if (2 * (size_t)(g.nrow + 1) * cs > (size_t)smem || 2 * (size_t)nx * cs > (size_t)smem)
    return set_error(GFMD_EINVAL, "gfmd_rough_surface: grid too large");
  std::vector<double> tw;
  const FftPlan prow = make_plan(g.nrow, tw);
  const FftPlan pcol = make_plan(nx, tw);
  g.rpost = (int)(tw.size() / 2);
  for (int k = 0; k <= ny / 2; k++) {
    const double a = -kTwoPi * (double)k / (double)ny;
    tw.push_back(std::cos(a));
    tw.push_back(std::sin(a));
  }
  SurfSpec sp{};
  sp.nx = nx;
  sp.ny = ny;
  sp.nyc = g.nyc;
  sp.nxp = g.nxp;
  sp.dqx = kTwoPi / (nx * prm->lattice);
  sp.dqy = kTwoPi / (ny * prm->lattice);
  const double ql = kTwoPi / prm->lambda_long, qs = kTwoPi / prm->lambda_short;
  sp.ql2 = ql * ql;
  sp.qs2 = qs * qs;
  sp.expo = -(1.0 + prm->hurst);
  sp.seed = prm->seed;

  Scratch sc;
  double2 *d_tw = nullptr, *W = nullptr;
  double *part = nullptr, *sum = nullptr;
  const dim3 grid((nx + 255) / 256, g.nyc);
  const int npart = (int)(grid.x * grid.y);
  cudaError_t e = sc.alloc((void **)&d_tw, tw.size() * sizeof(double));
  if (e == cudaSuccess) e = sc.alloc((void **)&W, (size_t)g.nyc * g.nxp * cs);
  if (e == cudaSuccess) e = sc.alloc((void **)&part, sizeof(double) * npart);
  if (e == cudaSuccess) e = sc.alloc((void **)&sum, sizeof(double));
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_tw, tw.data(), tw.size() * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return set_error(e == cudaErrorMemoryAllocation ? GFMD_ENOMEM : GFMD_ECUDA,
                                         std::string("gfmd_rough_surface: ") + cudaGetErrorString(e));
  Tw<double> twd;
  twd.hi = d_tw;
  twd.lo_unused = nullptr;
  k_surface_spectrum<<<grid, 256, 0, st>>>(sp, W, part);
  k_sum<<<1, 256, 0, st>>>(part, npart, sum);
  // inverse column transforms (one column per ky), then c2r rows
  int cb = 4;
  while (cb > 1 && 2 * (size_t)cb * nx * cs > (size_t)smem) cb /= 2;
  const size_t smc = 2 * (size_t)cb * nx * cs;
  cudaFuncSetAttribute(k_col_fft<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc);
  k_col_fft<double><<<(g.nyc + cb - 1) / cb, kThreads, smc, st>>>(reinterpret_cast<C<double> *>(W), g, pcol,
                                                                    twd, cb, +1);
  int rb = 8;
  while (rb > 1 && 2 * (size_t)rb * (g.nrow + 1) * cs > (size_t)smem) rb /= 2;
  const size_t smr = 2 * (size_t)rb * (g.nrow + 1) * cs;
  auto kr = k_row_inv<double, double>;
  cudaFuncSetAttribute(kr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr);
  kr<<<dim3((nx + rb - 1) / rb, 1), kThreads, smr, st>>>(reinterpret_cast<const C<double> *>(W), d_h, g, prow,
                                                        twd, rb);
  k_scale_to_slope<<<256, 256, 0, st>>>((size_t)nx * ny, d_h, sum, prm->rms_slope);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return set_error(GFMD_ECUDA, std::string("gfmd_rough_surface: ") + cudaGetErrorString(e));
  return GFMD_OK;
}
