// gfmd_obstacle_force: the force and energy of a rigid obstacle on the atoms
// of the grid at displacements u, the evaluation FixWallMap::pre_force
// (src/extras/fix_wall_map.cpp:686-817) and FixContactSphere::post_force
// (src/extras/fix_contact_sphere.cpp:207-264) make per atom, for a fix that
// keeps its atoms on the device as a grid.  Same wall code as the solver
// loops (gfmd_obstacle.cuh); every site of the layers the obstacle acts on
// is evaluated (no gating), the energy is summed in a fixed order.
#include <cuda_runtime.h>

#include <string>

#include "gfmd_internal.h"
#include "gfmd_obstacle.cuh"
#include "gfmd_reduce.cuh"

namespace gfmd {

namespace {

using red::kQ;
using red::kT;
using red::reduce_last;

__global__ void __launch_bounds__(kT) k_obstacle_force(Obst o, Geom g, const double *__restrict__ u,
                                                        double *__restrict__ f, double *__restrict__ part,
                                                        unsigned int *counter, double *energy) {
  const size_t N = (size_t)g.nx * g.ny;
  const int nl = g.ndof / 3;
  const double zero[3] = {0.0, 0.0, 0.0};
  double e = 0.0;
  for (size_t s = blockIdx.x * (size_t)kT + threadIdx.x; s < N; s += (size_t)gridDim.x * kT) {
    const int ix = (int)(s / g.ny), iy = (int)(s % g.ny);
    for (int l = 0; l < nl; l++) {
      double fw[3] = {0.0, 0.0, 0.0};
      if (l < o.nlayer && o.kind != GFMD_OBST_NONE) {
        double r[3];
        for (int c = 0; c < 3; c++) r[c] = u[(size_t)(3 * l + c) * N + s] + o.off[l][c];
        r[0] += ix * o.ax;
        r[1] += iy * o.ay;
        const WallOut w = wall_eval<true>(o, ix, iy, s, r, zero);
        e += w.e;
        for (int c = 0; c < 3; c++) fw[c] = w.f[c];
      }
      for (int c = 0; c < 3; c++) f[(size_t)(3 * l + c) * N + s] = fw[c];
    }
  }
  const double acc[1] = {e};
  __shared__ double res[1];
  if (!reduce_last<1, 0>(acc, part, counter, res)) return;
  if (threadIdx.x == 0) {
    *energy = res[0];
    *counter = 0u;
  }
}

}  // namespace

}  // namespace gfmd

extern "C" int gfmd_obstacle_force(int nx, int ny, int ndof, const gfmd_obstacle_t *ob, const double *d_u,
                                   double *d_f, double *d_energy, void *cuda_stream) {
  using namespace gfmd;
  const char *who = "gfmd_obstacle_force";
  if (nx < 1 || ny < 1 || ndof < 3 || ndof > kMaxNdof || ndof % 3)
    return set_error(GFMD_EINVAL, std::string(who) + ": bad grid size or ndof");
  if (!ob || !d_u || !d_f || !d_energy) return set_error(GFMD_EINVAL, std::string(who) + ": NULL argument");
  if (ob->kind < GFMD_OBST_NONE || ob->kind > GFMD_OBST_MAP_BICUBIC)
    return set_error(GFMD_EINVAL, std::string(who) + ": unknown obstacle kind");
  if ((ob->kind == GFMD_OBST_MAP_EXP || ob->kind == GFMD_OBST_MAP_BICUBIC) && !ob->d_map)
    return set_error(GFMD_EINVAL, std::string(who) + ": map obstacle without a map");
  Geom g{};
  g.nx = nx;
  g.ny = ny;
  g.ndof = ndof;
  const Obst o = make_obst(ob, g);
  int dev = 0, sms = 1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const size_t N = (size_t)nx * ny;
  const int blocks = (int)std::max<size_t>(1, std::min<size_t>((size_t)sms * 4, (N + kT - 1) / kT));
  void *scratch = nullptr;  // block partials and the last-block counter
  if (e == cudaSuccess) e = cudaMalloc(&scratch, sizeof(double) * kQ * blocks + 256);
  cudaStream_t st = reinterpret_cast<cudaStream_t>(cuda_stream);
  double *part = reinterpret_cast<double *>(scratch);
  unsigned int *counter = reinterpret_cast<unsigned int *>(part + (size_t)kQ * blocks);
  if (e == cudaSuccess) e = cudaMemsetAsync(counter, 0, sizeof(unsigned int), st);
  if (e == cudaSuccess) {
    k_obstacle_force<<<blocks, kT, 0, st>>>(o, g, d_u, d_f, part, counter, d_energy);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (scratch) cudaFree(scratch);
  if (e != cudaSuccess)
    return set_error(e == cudaErrorMemoryAllocation ? GFMD_ENOMEM : GFMD_ECUDA,
                     std::string(who) + ": " + cudaGetErrorString(e));
  return GFMD_OK;
}
