// gfmd_post_force_noalloc: the FP64 force evaluation without any device
// allocation.
//
// Who needs it: callers that cannot call cudaMalloc.  Some host programs hand
// the whole device to their own pooling allocator at start-up, so a library
// allocation either fails or fragments the pool behind the host's back; others
// run the force call inside a time-critical loop where cudaMalloc/cudaFree
// (which may synchronize the device) are not acceptable.  gfmd_create cannot
// serve them: it allocates the spectrum, the packed table and the twiddles.
//
// How: the caller passes inputs (u, the half-spectrum Phi table, linf) and
// outputs (f, the energy) in its own device memory.  Everything else the
// pipeline needs — twiddle table, spectrum, energy partials — lives in one
// file-scope __device__ array of kNoallocScratchBytes (16 MiB).  Every GPU on
// which this library's code is loaded holds that array until the process
// exits.  Calls whose scratch would exceed it are rejected.
//
// Sharing: all calls on a device share the one array and it keeps the last
// call's contents.  Each call rewrites every scratch byte it reads (twiddles,
// spectrum, partials), so nothing needs to start at zero.  Calls that overlap
// on the GPU (different streams, or different host threads) race on the
// array and give wrong results; serialize them.
//
// Set-up: the first call on each device looks up the array's device address
// with cudaGetSymbolAddress, with that device current, and caches it; host
// code never passes the array's own name to a kernel (on the host that name
// is only a stand-in, not a device address).  Make the first call on each
// device before any stream capture begins.  Later calls on a stream that is
// not capturing look the address up again (no allocation, no sync), so the
// cache cannot go stale after a cudaDeviceReset reloads the module; a call
// on a capturing stream uses the cached address.
//
// Arguments: every buffer must be reachable from the device (device or
// managed memory, or host memory mapped into the device's address space);
// plain host memory is refused with GFMD_EINVAL before any launch.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>
#include <string>

#include "gfmd_fft.cuh"
#include "gfmd_internal.h"
#include "gfmd_plain_kernels.cuh"

namespace gfmd {

namespace {

constexpr size_t kNoallocScratchBytes = size_t(16) << 20;
constexpr int kNoallocMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoallocScratchBytes];

std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[kNoallocMaxDevices] = {};
int g_noalloc_smem[kNoallocMaxDevices] = {};

size_t align256(size_t b) { return (b + 255) / 256 * 256; }

// Same factorization and table offsets as make_plan (gfmd_capi.cu), without
// building the table; returns the number of complex entries used.
int plan_layout(int n, int base, FftPlan &p) {
  p = FftPlan{};
  p.n = n;
  int m = n, k = 0;
  while (m % 8 == 0) { p.radix[k++] = 8; m /= 8; }
  if (m % 4 == 0) { p.radix[k++] = 4; m /= 4; }
  if (m % 2 == 0) { p.radix[k++] = 2; m /= 2; }
  for (int f = 3; m > 1; f += 2)
    while (m % f == 0) {
      if (k >= kMaxStages) return -1;
      p.radix[k++] = f;
      m /= f;
    }
  p.nst = k;
  int span = 1, off = base;
  for (int s = 0; s < k; s++) {
    const int R = p.radix[s];
    p.span[s] = span;
    p.twoff[s] = off;
    off += span * R;
    p.rootoff[s] = off;
    if (R != 2 && R != 3 && R != 4 && R != 5 && R != 8) off += R;
    span *= R;
  }
  return off - base;
}

__device__ void plan_entry(const FftPlan &p, int i, double2 *tw) {
  for (int s = 0; s < p.nst; s++) {
    const int R = p.radix[s], L = p.span[s] * R;
    int e = i - p.twoff[s];
    if (e >= 0 && e < L) {
      int kk = e / R, r = e - kk * R;
      long mm = ((long)r * kk) % L;
      double sn, cs;
      sincospi(-2.0 * (double)mm / (double)L, &sn, &cs);
      tw[i] = make_double2(cs, sn);
      return;
    }
    e = i - p.rootoff[s];
    if (e >= 0 && e < R && R != 2 && R != 3 && R != 4 && R != 5 && R != 8) {
      double sn, cs;
      sincospi(-2.0 * (double)e / (double)R, &sn, &cs);
      tw[i] = make_double2(cs, sn);
      return;
    }
  }
}

// Twiddles of the row plan, the column plan and exp(-2 pi i k/ny), k <= ny/2.
__global__ void k_noalloc_twiddles(double2 *tw, FftPlan prow, FftPlan pcol, int rpost, int ny,
                                   int ntw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ntw) return;
  if (i >= rpost) {
    double sn, cs;
    sincospi(-2.0 * (double)(i - rpost) / (double)ny, &sn, &cs);
    tw[i] = make_double2(cs, sn);
  } else if (i >= pcol.twoff[0] && pcol.nst > 0) {
    plan_entry(pcol, i, tw);
  } else {
    plan_entry(prow, i, tw);
  }
}

// phi_apply reading the caller's half-spectrum table [nx][ny/2+1][D][D]
// (complex, FP64) directly: Phi_eff = (Phi(k) + conj Phi(-k))/2 on the ky = 0
// and ky = ny/2 columns (both partners stored there), Phi elsewhere.
template <int D>
__global__ void __launch_bounds__(kPhiThreads)
    k_noalloc_phi(double2 *__restrict__ W, const double2 *__restrict__ phi, Geom g,
                  const double *__restrict__ linf, double *__restrict__ epart) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  const int ky = blockIdx.y;
  double e = 0.0;
  if (x < g.nx) {
    const size_t cs = (size_t)g.nxp;
    double2 *col = W + (size_t)ky * D * cs + x;
    const bool mirror_self = (ky == 0) || (g.ny_even && ky == g.ny / 2);
    const int mx = (g.nx - x) % g.nx;
    const double2 *pa = phi + ((size_t)x * g.nyc + ky) * D * D;
    const double2 *pb = phi + ((size_t)mx * g.nyc + ky) * D * D;
    double2 uq[D];
#pragma unroll
    for (int j = 0; j < D; j++) uq[j] = col[j * cs];
    double2 F[D];
#pragma unroll
    for (int i = 0; i < D; i++) {
      double fr = 0.0, fi = 0.0;
#pragma unroll
      for (int j = 0; j < D; j++) {
        double2 a = pa[i * D + j];
        if (mirror_self) {
          double2 b = pb[i * D + j];
          a = make_double2(0.5 * (a.x + b.x), 0.5 * (a.y - b.y));
        }
        fr += a.x * uq[j].x - a.y * uq[j].y;
        fi += a.x * uq[j].y + a.y * uq[j].x;
      }
      F[i] = make_double2(fr, fi);
    }
    double es = 0.0;
#pragma unroll
    for (int i = 0; i < D; i++) es += F[i].x * uq[i].x + F[i].y * uq[i].y;
    e = (mirror_self ? 1.0 : 2.0) * es;
    if (ky == 0 && x == 0 && linf) {
      for (int l = 0; l < D / 3; l++) {
        e -= 2.0 * linf[l] * uq[3 * l + 2].x;
        F[3 * l + 2].x -= linf[l];
      }
    }
#pragma unroll
    for (int i = 0; i < D; i++) col[i * cs] = make_double2(-F[i].x, -F[i].y);
  }
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

int noalloc_fail(int code, const std::string &msg) { return set_error(code, msg); }

// True when the device can dereference p (device, managed, or mapped host
// memory).  cudaPointerGetAttributes allocates nothing.
bool device_reachable(const void *p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // clear the sticky-free error of an unknown pointer
    return false;
  }
  if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged) return true;
  if (a.type == cudaMemoryTypeHost) return a.devicePointer != nullptr;
  return false;
}

}  // namespace

}  // namespace gfmd

extern "C" int gfmd_post_force_noalloc(int nx, int ny, int ndof, const double *d_phi_half,
                                       const double *d_linf, const double *d_u, double *d_f,
                                       double *d_epot, void *cuda_stream) {
  using namespace gfmd;
  const char *who = "gfmd_post_force_noalloc";
  if (nx < 1 || ny < 1 || nx > 8192 || ny > 8192 || ndof < 3 || ndof > kMaxNdof || ndof % 3)
    return noalloc_fail(GFMD_EINVAL, std::string(who) + ": bad grid size or ndof");

  Geom g{};
  g.nx = nx;
  g.ny = ny;
  g.ndof = ndof;
  g.nyc = ny / 2 + 1;
  g.nxp = (nx + 31) / 32 * 32;
  g.ny_even = (ny % 2 == 0) ? 1 : 0;
  g.nrow = g.ny_even ? ny / 2 : ny;
  g.npk = ndof * ndof;
  FftPlan prow, pcol;
  int nrow_tw = plan_layout(g.nrow, 0, prow);
  int ncol_tw = plan_layout(nx, nrow_tw, pcol);
  if (nrow_tw < 0 || ncol_tw < 0) return noalloc_fail(GFMD_EINVAL, std::string(who) + ": too many FFT stages");
  g.rpost = nrow_tw + ncol_tw;
  const int ntw = g.rpost + ny / 2 + 1;
  const int n_epart = ((nx + kPhiThreads - 1) / kPhiThreads) * g.nyc;

  // scratch layout: twiddles | spectrum | energy partials
  const size_t off_w = align256((size_t)ntw * sizeof(double2));
  const size_t off_e = off_w + align256((size_t)g.nyc * ndof * g.nxp * sizeof(double2));
  const size_t need = off_e + align256((size_t)n_epart * sizeof(double));
  if (need > kNoallocScratchBytes)
    return noalloc_fail(GFMD_EINVAL,
                        std::string(who) + ": grid needs " + std::to_string(need) +
                            " bytes of scratch, more than the fixed " +
                            std::to_string(kNoallocScratchBytes) + " bytes (16 MiB)");
  if (!d_phi_half || !d_u || !d_f || !d_epot)
    return noalloc_fail(GFMD_EINVAL, std::string(who) + ": NULL argument");
  if ((const void *)d_u == (const void *)d_f)
    return noalloc_fail(GFMD_EINVAL, std::string(who) + ": u and f must not alias");
  {
    const void *bufs[] = {d_phi_half, d_u, d_f, d_epot, d_linf};
    const char *names[] = {"phi", "u", "f", "epot", "linf"};
    for (int i = 0; i < 5; i++)
      if (bufs[i] && !device_reachable(bufs[i]))
        return noalloc_fail(GFMD_EINVAL, std::string(who) + ": " + names[i] +
                                             " is not device-accessible memory");
  }

  // per-device set-up: device address of the scratch array, shared-memory limit
  int dev = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess)
    return noalloc_fail(GFMD_ECUDA, std::string(who) + ": cudaGetDevice: " + cudaGetErrorString(ce));
  if (dev < 0 || dev >= kNoallocMaxDevices)
    return noalloc_fail(GFMD_EINVAL, std::string(who) + ": device index out of range");
  void *base = nullptr;
  int smem = 0;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  ce = cudaStreamIsCapturing(reinterpret_cast<cudaStream_t>(cuda_stream), &cap);
  if (ce != cudaSuccess)
    return noalloc_fail(GFMD_ECUDA, std::string(who) + ": cudaStreamIsCapturing: " + cudaGetErrorString(ce));
  {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[dev] && cap != cudaStreamCaptureStatusNone)
      return noalloc_fail(GFMD_EINVAL, std::string(who) +
                                           ": the first call on a device must come before stream capture");
    if (g_noalloc_ptr[dev] && cap == cudaStreamCaptureStatusNone) {
      void *p = nullptr;  // refresh: the module may have been reloaded by a device reset
      ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (ce != cudaSuccess || !p)
        return noalloc_fail(GFMD_ECUDA, std::string(who) + ": cudaGetSymbolAddress: " +
                                            cudaGetErrorString(ce));
      g_noalloc_ptr[dev] = p;
    }
    if (!g_noalloc_ptr[dev]) {
      void *p = nullptr;
      ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (ce != cudaSuccess || !p)
        return noalloc_fail(GFMD_ECUDA, std::string(who) + ": cudaGetSymbolAddress: " +
                                            cudaGetErrorString(ce));
      int v = 0;
      ce = cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
      if (ce != cudaSuccess)
        return noalloc_fail(GFMD_ECUDA, std::string(who) + ": cudaDeviceGetAttribute: " +
                                            cudaGetErrorString(ce));
      g_noalloc_smem[dev] = v;
      g_noalloc_ptr[dev] = p;
    }
    base = g_noalloc_ptr[dev];
    smem = g_noalloc_smem[dev];
  }
  if (2 * (size_t)(g.nrow + 1) * sizeof(double2) > (size_t)smem ||
      2 * (size_t)nx * sizeof(double2) > (size_t)smem)
    return noalloc_fail(GFMD_EINVAL, std::string(who) + ": grid too large for one block's shared memory");

  cudaStream_t st = reinterpret_cast<cudaStream_t>(cuda_stream);
  unsigned char *sb = reinterpret_cast<unsigned char *>(base);
  double2 *tw_tab = reinterpret_cast<double2 *>(sb);
  double2 *W = reinterpret_cast<double2 *>(sb + off_w);
  double *epart = reinterpret_cast<double *>(sb + off_e);
  Tw<double> tw;
  tw.hi = tw_tab;
  tw.lo_unused = nullptr;

  k_noalloc_twiddles<<<(ntw + 255) / 256, 256, 0, st>>>(tw_tab, prow, pcol, g.rpost, ny, ntw);

  int rb = 8;
  while (rb > 1 && rb * 2 * (size_t)(g.nrow + 1) * sizeof(double2) > (size_t)smem) rb /= 2;
  size_t smr = 2 * (size_t)rb * (g.nrow + 1) * sizeof(double2);
  dim3 gridr((nx + rb - 1) / rb, ndof);
  cudaFuncSetAttribute(k_row_fwd<double, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr);
  cudaFuncSetAttribute(k_row_inv<double, double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smr);
  k_row_fwd<double, double><<<gridr, kThreads, smr, st>>>(d_u, W, g, prow, tw, rb);

  int cb = 4;
  while (cb > 1 && cb * 2 * (size_t)nx * sizeof(double2) > (size_t)smem) cb /= 2;
  size_t smc = 2 * (size_t)cb * nx * sizeof(double2);
  dim3 gridc((g.nyc * ndof + cb - 1) / cb);
  cudaFuncSetAttribute(k_col_fft<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smc);
  k_col_fft<double><<<gridc, kThreads, smc, st>>>(W, g, pcol, tw, cb, -1);

  dim3 gridp((nx + kPhiThreads - 1) / kPhiThreads, g.nyc);
  const double2 *ph = reinterpret_cast<const double2 *>(d_phi_half);
  switch (ndof) {
    case 3: k_noalloc_phi<3><<<gridp, kPhiThreads, 0, st>>>(W, ph, g, d_linf, epart); break;
    case 6: k_noalloc_phi<6><<<gridp, kPhiThreads, 0, st>>>(W, ph, g, d_linf, epart); break;
    case 9: k_noalloc_phi<9><<<gridp, kPhiThreads, 0, st>>>(W, ph, g, d_linf, epart); break;
    case 12: k_noalloc_phi<12><<<gridp, kPhiThreads, 0, st>>>(W, ph, g, d_linf, epart); break;
    case 15: k_noalloc_phi<15><<<gridp, kPhiThreads, 0, st>>>(W, ph, g, d_linf, epart); break;
    case 18: k_noalloc_phi<18><<<gridp, kPhiThreads, 0, st>>>(W, ph, g, d_linf, epart); break;
    case 21: k_noalloc_phi<21><<<gridp, kPhiThreads, 0, st>>>(W, ph, g, d_linf, epart); break;
    default: k_noalloc_phi<24><<<gridp, kPhiThreads, 0, st>>>(W, ph, g, d_linf, epart); break;
  }
  k_reduce<<<1, 256, 0, st>>>(epart, n_epart, d_epot);
  k_col_fft<double><<<gridc, kThreads, smc, st>>>(W, g, pcol, tw, cb, +1);
  k_row_inv<double, double><<<gridr, kThreads, smr, st>>>(W, d_f, g, prow, tw, rb);
  ce = cudaGetLastError();
  if (ce != cudaSuccess)
    return noalloc_fail(GFMD_ECUDA, std::string(who) + ": launch: " + cudaGetErrorString(ce));
  return GFMD_OK;
}
