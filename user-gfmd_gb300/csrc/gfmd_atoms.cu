// Atom list <-> displacement grid on the GPU, for a fix that keeps its atoms
// on the device.  Restates, for one rank owning the whole grid:
//   FixGFMD::pre_force (src/main/fix_gfmd.cpp:659-858), orthogonal box:
//     grid id (ix - dxshift, iy - dyshift, iu) wrapped into the grid;
//     u = x - xeq with the minimum image in x and y; velocities copied into
//     the grid for the dynamic solvers;
//   FixGFMD::grid_to_list (fix_gfmd.cpp:952-1074): the grid force of every
//     atom, and the sum of the forces over the layer.
// Every grid id is checked in the kernel: an atom with an id outside the
// grid is counted and skipped, never written.  An optional per-slot counter
// reports grid slots filled zero or several times (the reference's check
// that the local atoms and the grid agree, fix_gfmd.cpp:858-870).  The force
// sum is reduced in FP64 in a fixed order.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gfmd_internal.h"

namespace gfmd {
namespace {

__device__ __forceinline__ int wrapi(int i, int n) {
  i %= n;
  return i < 0 ? i + n : i;
}

// Wrap into [-L/2, L/2] like the reference's while loops (fix_gfmd.cpp:770-773),
// which this equals for |d| <= 4 L; larger offsets are first reduced by a
// whole number of periods and non-finite ones returned as they are, so the
// loops run at most once.
__device__ __forceinline__ double min_image(double d, double L) {
  if (!isfinite(d)) return d;
  if (fabs(d) > 4.0 * L) d -= L * rint(d / L);
  const double h = 0.5 * L;
  if (d > h) d -= L;
  if (d < -h) d += L;
  return d;
}

__global__ void k_atoms_to_grid(int natoms, const double *__restrict__ x, const double *__restrict__ xeq,
                                const double *__restrict__ v, const int *__restrict__ gid, int nx, int ny,
                                int nu, double xprd, double yprd, int dxs, int dys, double *__restrict__ u,
                                double *__restrict__ vg, int *__restrict__ slot, int *__restrict__ bad) {
  const size_t N = (size_t)nx * ny;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < natoms; i += gridDim.x * blockDim.x) {
    const int iu = gid[3 * i + 2];
    if (iu < 0 || iu >= nu) {
      atomicAdd(bad, 1);
      continue;
    }
    const int ix = wrapi(gid[3 * i] - dxs, nx), iy = wrapi(gid[3 * i + 1] - dys, ny);
    const size_t s = (size_t)ix * ny + iy;
    const double ux = min_image(x[3 * i] - xeq[3 * i], xprd);
    const double uy = min_image(x[3 * i + 1] - xeq[3 * i + 1], yprd);
    const double uz = x[3 * i + 2] - xeq[3 * i + 2];
    u[(size_t)(3 * iu) * N + s] = ux;
    u[(size_t)(3 * iu + 1) * N + s] = uy;
    u[(size_t)(3 * iu + 2) * N + s] = uz;
    if (v && vg)
      for (int c = 0; c < 3; c++) vg[(size_t)(3 * iu + c) * N + s] = v[3 * i + c];
    if (slot) atomicAdd(&slot[(size_t)iu * N + s], 1);
  }
}

// counts of slots filled 0 times and more than once
__global__ void k_slot_check(size_t n, const int *__restrict__ slot, int *__restrict__ out) {
  int empty = 0, dup = 0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int c = slot[i];
    empty += c == 0;
    dup += c > 1;
  }
  if (empty) atomicAdd(&out[0], empty);
  if (dup) atomicAdd(&out[1], dup);
}

constexpr int kRT = 256;

// f_atoms (+)= grid force of each atom; block partials of the force sum
__global__ void __launch_bounds__(kRT) k_grid_to_atoms(int natoms, const int *__restrict__ gid,
                                                       const double *__restrict__ f, int nx, int ny, int nu,
                                                       double *__restrict__ fa, int accumulate,
                                                       double *__restrict__ part, int *__restrict__ bad) {
  const size_t N = (size_t)nx * ny;
  double acc[3] = {0.0, 0.0, 0.0};
  for (int i = blockIdx.x * kRT + threadIdx.x; i < natoms; i += gridDim.x * kRT) {
    const int ix = gid[3 * i], iy = gid[3 * i + 1], iu = gid[3 * i + 2];
    if (ix < 0 || ix >= nx || iy < 0 || iy >= ny || iu < 0 || iu >= nu) {
      atomicAdd(bad, 1);
      continue;
    }
    const size_t s = (size_t)ix * ny + iy;
    for (int c = 0; c < 3; c++) {
      const double fc = f[(size_t)(3 * iu + c) * N + s];
      fa[3 * i + c] = accumulate ? fa[3 * i + c] + fc : fc;
      acc[c] += fc;
    }
  }
  __shared__ double sh[kRT / 32][3];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int c = 0; c < 3; c++) {
    double v = acc[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[warp][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double v = 0.0;
    for (int w = 0; w < kRT / 32; w++) v += sh[w][threadIdx.x];
    part[blockIdx.x * 3 + threadIdx.x] = v;
  }
}

__global__ void k_sum3(const double *__restrict__ part, int nb, double *__restrict__ out) {
  if (threadIdx.x >= 3) return;
  double v = 0.0;
  for (int b = 0; b < nb; b++) v += part[b * 3 + threadIdx.x];
  out[threadIdx.x] = v;
}

}  // namespace
}  // namespace gfmd

extern "C" {

int gfmd_atoms_to_grid(int natoms, const double *d_x, const double *d_xeq, const double *d_v, const int *d_gid,
                       int nx, int ny, int ndof, double xprd, double yprd, int dxshift, int dyshift,
                       double *d_u, double *d_vgrid, int *d_slot_count, int *status, void *stream) {
  using namespace gfmd;
  if (natoms < 0 || (natoms > 0 && (!d_x || !d_xeq || !d_gid)) || !d_u || nx < 1 || ny < 1 || ndof < 3 ||
      ndof % 3 || !(xprd > 0.0) || !(yprd > 0.0))
    return set_error(GFMD_EINVAL, "gfmd_atoms_to_grid: bad argument");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const size_t nslot = (size_t)(ndof / 3) * nx * ny;
  int *d_cnt = nullptr;
  cudaError_t e = cudaMalloc((void **)&d_cnt, 3 * sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(d_cnt, 0, 3 * sizeof(int), st);
  if (e == cudaSuccess && d_slot_count) e = cudaMemsetAsync(d_slot_count, 0, nslot * sizeof(int), st);
  if (e == cudaSuccess && natoms > 0)
    k_atoms_to_grid<<<std::min(4096, (natoms + 255) / 256), 256, 0, st>>>(
        natoms, d_x, d_xeq, d_v, d_gid, nx, ny, ndof / 3, xprd, yprd, dxshift, dyshift, d_u, d_vgrid, d_slot_count,
        d_cnt);
  if (e == cudaSuccess && d_slot_count)
    k_slot_check<<<std::max<size_t>(1, std::min<size_t>(4096, (nslot + 255) / 256)), 256, 0, st>>>(nslot, d_slot_count,
                                                                                                  d_cnt + 1);
  int h[3] = {0, 0, 0};
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(h, d_cnt, sizeof(h), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (d_cnt) cudaFree(d_cnt);
  if (e != cudaSuccess) return set_error(GFMD_ECUDA, std::string("gfmd_atoms_to_grid: ") + cudaGetErrorString(e));
  // status: [0] atoms with an invalid grid id, [1] empty slots, [2] slots filled twice or more
  if (status) {
    status[0] = h[0];
    status[1] = d_slot_count ? h[1] : -1;
    status[2] = d_slot_count ? h[2] : -1;
  }
  if (h[0]) return set_error(GFMD_EINVAL, "gfmd_atoms_to_grid: atoms with a grid id outside the grid");
  if (d_slot_count && (h[1] || h[2]))
    return set_error(GFMD_EINVAL, "gfmd_atoms_to_grid: atoms and grid slots do not match one to one");
  return GFMD_OK;
}

int gfmd_grid_to_atoms(int natoms, const int *d_gid, const double *d_f, int nx, int ny, int ndof, double *d_fatoms,
                       int accumulate, double *fsum, void *stream) {
  using namespace gfmd;
  if (natoms < 0 || (natoms > 0 && (!d_gid || !d_fatoms)) || !d_f || nx < 1 || ny < 1 || ndof < 3 || ndof % 3)
    return set_error(GFMD_EINVAL, "gfmd_grid_to_atoms: bad argument");
  cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
  const int nb = std::max(1, std::min(1024, (natoms + kRT - 1) / kRT));
  double *d_part = nullptr;
  int *d_bad = nullptr;
  cudaError_t e = cudaMalloc((void **)&d_part, sizeof(double) * (3 * nb + 3));
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_bad, sizeof(int));
  if (e == cudaSuccess) e = cudaMemsetAsync(d_bad, 0, sizeof(int), st);
  if (e == cudaSuccess) {
    k_grid_to_atoms<<<nb, kRT, 0, st>>>(natoms, d_gid, d_f, nx, ny, ndof / 3, d_fatoms, accumulate, d_part, d_bad);
    k_sum3<<<1, 32, 0, st>>>(d_part, nb, d_part + 3 * nb);
    e = cudaGetLastError();
  }
  double hs[3] = {0.0, 0.0, 0.0};
  int bad = 0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(hs, d_part + 3 * nb, sizeof(hs), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (d_part) cudaFree(d_part);
  if (d_bad) cudaFree(d_bad);
  if (e != cudaSuccess) return set_error(GFMD_ECUDA, std::string("gfmd_grid_to_atoms: ") + cudaGetErrorString(e));
  if (fsum)
    for (int c = 0; c < 3; c++) fsum[c] = hs[c];
  if (bad) return set_error(GFMD_EINVAL, "gfmd_grid_to_atoms: atoms with a grid id outside the grid");
  return GFMD_OK;
}

}  // extern "C"
