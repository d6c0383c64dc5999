// Polak-Ribiere conjugate gradients with a Newton line search, resident on
// the GPU with its scalar control on the device.
//
// The minimizer LAMMPS runs on fix gfmd through `minimize` (the reference's
// Hertz tests, tests/TEST_Hertz_*/lammps.in, use min_style cg), restated for
// a grid of displacements u[ndof][nx*ny] with the elastic force from the
// handle's force evaluation and an obstacle force (gfmd_obstacle.cuh).
//
// Layout of one CG iteration (all on one stream, no host round trip):
//   fKh = F_el(h)                  force evaluation of the direction (no
//                                  gamma-point term); F_el is linear, so
//                                  F_el(u + a h) = F_el(u) + a fKh exactly,
//                                  and its energy is h.K.h / 2
//   k_ls_cluster                   FP32 phase with a sphere wall on one atom
//                                  layer: the whole line search in one
//                                  thread-block cluster; for a set too large
//                                  for it, sets the IF node that runs:
//   k_lsinit                       wall curvature and F_w.h along h at a = 0
//                                  over the line-search set, first Newton step
//   k_probe x kLsMax               Newton steps on the line derivative over the
//                                  set, each a no-op once the step has converged
//   k_update                       u += a h, g += a fKh + F_w(u_new) - F_w(u_old),
//                                  Polak-Ribiere beta with the descent check,
//                                  the next line-search set (sites near the
//                                  obstacle) and its bounding box, convergence
//                                  test, loop condition
//   k_dir                          h = g + beta h, max|h|, g.h
// The iteration is the body of a CUDA graph WHILE node; the loop condition is
// set by the last block of k_update, which counts the iterations, so every
// launch of the graph runs at most `recompute` iterations.  Each launch
// starts from a fresh evaluation of F_el(u) (the drift of the incremental
// update is reset) and steepest descent.  Only k_update and k_dir stream the
// vectors; the line-search kernels visit the box of the set.  A batch or
// single solve that qualifies for k_ls_cluster nests the IF node in the
// WHILE body; a runtime that refuses the nested node gets the graph
// without it (probes only).
//
// Precision: the state is held in two types, Tx for u (the quantity that
// accumulates) and Tv for g, h and fKh.  Plain FP64 runs
// <double, double>; the mixed solve runs an FP32 phase <float, float> with
// FP32 force evaluations and then an FP64 refinement <double, float> whose
// restarts use the FP64 force evaluation while the direction forces stay
// FP32 (their error is relative to |h|, which shrinks as the solve
// converges).  Dot products are FP64 (plain) or compensated FP32
// (TwoProd/TwoSum error-free transformations, Ogita, Rump and Oishi 2005; the
// streaming kernels compensate per loop trip rather than per term): on this
// GPU the FP64 ALU rate is below the rate at which HBM streams operands, so
// FP64 arithmetic per element would bound these kernels.  For the same
// reason the FP32 phase evaluates sphere and map walls in FP32.  Per-block
// partials are combined in FP64 in a fixed order by the last block, so
// results are bit-reproducible.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <string>
#include <vector>

#include "gfmd_internal.h"
#include "gfmd_obstacle.cuh"
#include "gfmd_reduce.cuh"
#include "gfmd_vec.cuh"

namespace gfmd {

namespace {

using red::kT;
using red::kQ;
using red::Dot;
using red::reduce_last;
constexpr int kLsMax = 8;   // Newton probes per line search

// Grids whose site count allows the 4-site vector kernels.
inline bool nsite4(const Geom &g) { return ((size_t)g.nx * g.ny) % 4 == 0; }

// Blocks of a grid-stride kernel: the resident blocks of the whole GPU (a
// grid of several partial waves leaves SMs idle at its end), at most one per
// `per_block` elements of work.
template <typename K> int grid_for(K kernel, int sms, size_t work, size_t per_block) {
  static int resident = 0;  // per kernel instance
  if (resident == 0) {
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, kT, 0) != cudaSuccess || nb < 1) nb = 1;
    resident = nb;
  }
  const size_t need = (work + per_block - 1) / per_block;
  return (int)std::max<size_t>(1, std::min<size_t>((size_t)resident * sms, need));
}

#define RT_CHECK(call)                \
  do {                                \
    cudaError_t e_ = (call);          \
    if (e_ != cudaSuccess) return e_; \
  } while (0)

struct CgCtl {
  double a, lo, hi;         // line search: step and bracket
  double gh, hKh;           // g.h of the direction (set with it) and its h.K.h
  double fw0h;              // F_w(u).h over the line-search set
  double gg;                // g.g of the current gradient
  double fmax;              // max |g_i|
  double ew;                // obstacle energy at the last update
  double beta;              // next direction: h = g + beta h (h = z + beta h with a preconditioner)
  double hg;                // h_old . g_new (descent check; g.h of the next direction)
  double ftol;              // tolerance of the running phase
  double ftol_req;          // requested tolerance
  double fmax_restart;      // max |g_i| at the last restart
  double dmax;              // largest move of a component per line-search step (<= 0: none)
  double amax;              // step cap of this line search: dmax / max|h_i|
  double hmax;              // max |h_i| of the direction (set with it)
  int bulk;                 // FP32 phase: tolerance floored at the FP32 noise level
  int parked;               // phase finished: the branch skips its restart and loop
  int it, since, maxit, recompute;
  int ls_it, ls_done;
  int bx0, bx1, by0, by1;   // box of sites (inclusive) holding the line-search set
  int done;                 // 0 running, 1 converged, 2 iteration cap, 3 non-finite
  int obst;
  unsigned int counter;     // last-block detection
};

// Position of atom (site s, layer l) at x + a h, in FP64 and FP32.
template <typename Tx, typename Tv>
__device__ __forceinline__ void atom_pos(const Obst &o, int ix, int iy, int l, const Tx *x, const Tv *h,
                                         size_t N, size_t s, double a, double r[3], double d[3]) {
#pragma unroll
  for (int c = 0; c < 3; c++) {
    const size_t idx = (size_t)(3 * l + c) * N + s;
    const double hv = h ? (double)h[idx] : 0.0;
    d[c] = hv;
    r[c] = (double)x[idx] + a * hv + o.off[l][c];
  }
  r[0] += ix * o.ax;
  r[1] += iy * o.ay;
}

template <typename Tx>
__device__ __forceinline__ float gap_of(const Obst &o, int ix, int iy, int l, const Tx *x, size_t N, size_t s) {
  float r[3];
#pragma unroll
  for (int c = 0; c < 3; c++) r[c] = (float)x[(size_t)(3 * l + c) * N + s] + o.foff[l][c];
  r[0] += (float)ix * o.fax;
  r[1] += (float)iy * o.fay;
  return gap_estimate_f(o, s, r);
}

__device__ __forceinline__ bool wall_near(const Obst &o, float ge) { return ge < o.fgate_wall; }

// The FP32 bulk phase evaluates a map wall in FP32 (its force depends on the
// atom height alone, and every atom under a rough indenter is in range: FP64
// exponentials per atom would bound the phase); FP64 phases use FP64.
template <typename Tx> __device__ __forceinline__ bool map_in_f32(const Obst &o) {
  return sizeof(Tx) == 4 && o.kind == GFMD_OBST_MAP_EXP;
}

__device__ __forceinline__ void set_loop(cudaGraphConditionalHandle hc, int use, unsigned int v) {
  if (use) cudaGraphSetConditional(hc, v);
}

// ---- per-site pieces ----------------------------------------------------------
// Sphere walls in the FP32 phase are evaluated in FP32 (sphere_off keeps the
// gap's rounding relative to the gap; FP64 exponentials and divisions on the
// sites near the obstacle would bound the phase at this GPU's FP64 rate); the
// FP64 phases evaluate them in FP64.
template <typename Tx> __device__ __forceinline__ bool sphere_f32(const Obst &o) {
  return sizeof(Tx) == 4 && (o.kind == GFMD_OBST_SPHERE_EXP || o.kind == GFMD_OBST_SPHERE_LJ);
}

template <typename Tx>
__device__ __forceinline__ float gap_reg(const Obst &o, int ix, int iy, int l, size_t s, const Tx xv[3]) {
  float r[3];
#pragma unroll
  for (int c = 0; c < 3; c++) r[c] = (float)xv[c] + o.foff[l][c];
  r[0] += (float)ix * o.fax;
  r[1] += (float)iy * o.fay;
  return gap_estimate_f(o, s, r);
}

// Gate value of an atom displaced by xd, compared with o.gw (evaluate the
// wall) and o.ga (keep the site in the line-search set): for a sphere
// |d|^2 - R^2 in FP32, for a map the gap estimate (bicubic maps: -1e30).
template <typename Tx>
__device__ __forceinline__ float cg_gate(const Obst &o, const Geom &gm, int ix, int iy, int l, size_t s,
                                         const Tx xd[3]) {
  if (o.kind == GFMD_OBST_SPHERE_EXP || o.kind == GFMD_OBST_SPHERE_LJ)
    return sphere_off(o, gm.nx, gm.ny, ix, iy, l, (float)xd[0], (float)xd[1], (float)xd[2]).s;
  return gap_reg(o, ix, iy, l, s, xd);
}

// Wall on the atom of layer l at site s displaced by xd, with its curvature
// along dir: FP32 in the FP32 phase for spheres and height maps, else FP64.
template <typename Tx, bool BIC>
__device__ __forceinline__ WallOut site_wall(const Obst &o, const Geom &gm, int ix, int iy, int l, size_t s,
                                             const Tx xd[3], const double dir[3]) {
  WallOut w{0.0, {0.0, 0.0, 0.0}, 0.0};
  if (sphere_f32<Tx>(o)) {
    const SphereOff q = sphere_off(o, gm.nx, gm.ny, ix, iy, l, (float)xd[0], (float)xd[1], (float)xd[2]);
    const float df[3] = {(float)dir[0], (float)dir[1], (float)dir[2]};
    float e, f[3], cv;
    if (sphere_wall_f(o, q, df, e, f, cv)) {
      w.e = e;
      w.f[0] = f[0];
      w.f[1] = f[1];
      w.f[2] = f[2];
      w.curv = cv;
    }
    return w;
  }
  if (map_in_f32<Tx>(o)) {
    float e, fz;
    map_wall_f(o, s, (float)xd[2] + o.foff[l][2], e, fz);
    w.e = e;
    w.f[2] = fz;
    w.curv = (double)(fz * o.fnorm * o.finv_sigma) * dir[2] * dir[2];  // d2E/dz2 = F / sigma
    return w;
  }
  double r[3];
#pragma unroll
  for (int c = 0; c < 3; c++) r[c] = (double)xd[c] + o.off[l][c];
  r[0] += ix * o.ax;
  r[1] += iy * o.ay;
  return wall_eval<BIC>(o, ix, iy, s, r, dir);
}

// Box of sites [bx0, bx1] x [by0, by1] holding the line-search set, reduced
// as the maxima of (ix + 1, nx - ix, iy + 1, ny - iy) over its sites (all
// zero: empty box).
struct BoxAcc {
  int a = 0, b = 0, c = 0, d = 0;
  __device__ __forceinline__ void add(int ix, int iy, const Geom &gm) {
    a = max(a, ix + 1);
    b = max(b, gm.nx - ix);
    c = max(c, iy + 1);
    d = max(d, gm.ny - iy);
  }
};
__device__ __forceinline__ void set_box(CgCtl *ctl, const double *r, const Geom &gm, bool full) {
  ctl->bx1 = full ? gm.nx - 1 : (int)r[0] - 1;
  ctl->bx0 = full ? 0 : gm.nx - (int)r[1];
  ctl->by1 = full ? gm.ny - 1 : (int)r[2] - 1;
  ctl->by0 = full ? 0 : gm.ny - (int)r[3];
}

// Sums of the line search over the sites of the box that are in the set, at
// x + a h: F_w(x + a h).h and h^T H_w h.  A set smaller than the grid of
// threads takes one site per thread, consecutive sites on consecutive blocks
// (the wall work then lands on every SM); a larger one is walked in
// coalesced order.
template <typename Tx, typename Tv, bool BIC>
__device__ __forceinline__ void line_walls(const Obst &o, const Geom &gm, const Tx *__restrict__ x,
                                           const Tv *__restrict__ h, const unsigned char *__restrict__ active,
                                           const CgCtl *ctl, double a, double &fh, double &cw) {
  const int N = gm.nx * gm.ny;
  const int w = ctl->by1 - ctl->by0 + 1, ht = ctl->bx1 - ctl->bx0 + 1;
  const int nb = (w > 0 && ht > 0) ? w * ht : 0;
  const int x0 = ctl->bx0, y0 = ctl->by0;
  const int nthr = gridDim.x * kT;
  const Tx at = (Tx)a;
  for (int i = nb <= nthr ? threadIdx.x * gridDim.x + blockIdx.x : blockIdx.x * kT + threadIdx.x; i < nb;
       i += nthr) {
    const int r = i / w;
    const int ix = x0 + r, iy = y0 + (i - r * w);
    const int s = ix * gm.ny + iy;
    if (map_in_f32<Tx>(o)) {
      float fhf = 0.0f, cwf = 0.0f;
      for (int l = 0; l < o.nlayer; l++) {
        const size_t iz = (size_t)(3 * l + 2) * N + s;
        const float hz = (float)h[iz];
        float e, fz;
        map_wall_f(o, s, (float)x[iz] + (float)a * hz + o.foff[l][2], e, fz);
        fhf += fz * hz;
        cwf += fz * o.fnorm * o.finv_sigma * hz * hz;  // d2E/dz2 = F / sigma
      }
      fh += fhf;
      cw += cwf;
      continue;
    }
    if (!active[s]) continue;
    for (int l = 0; l < o.nlayer; l++) {
      Tx xd[3];
      double d[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const size_t idx = (size_t)(3 * l + c) * N + s;
        const Tv hv = h[idx];
        d[c] = (double)hv;
        xd[c] = x[idx] + at * (Tx)hv;
      }
      const WallOut wo = site_wall<Tx, BIC>(o, gm, ix, iy, l, s, xd, d);
      fh += wo.f[0] * d[0] + wo.f[1] * d[1] + wo.f[2] * d[2];
      cw += wo.curv;
    }
  }
}

// ---- restart: g = f_el + F_w(u), h = g; arms the loop ---------------------
template <typename Tx, typename Tv, bool BIC = false>
__global__ void __launch_bounds__(kT, 4) k_restart(const __grid_constant__ Obst o, Geom gm, const Tx *__restrict__ x,
                                                 const Tx *__restrict__ fel, Tv *__restrict__ g,
                                                 Tv *__restrict__ h, unsigned char *__restrict__ active,
                                                 double *__restrict__ part, CgCtl *ctl,
                                                 cudaGraphConditionalHandle hc, int use_hc) {
  const int N = gm.nx * gm.ny;
  const int nl = gm.ndof / 3;
  const bool obst = o.kind != GFMD_OBST_NONE, all = map_in_f32<Tx>(o);
  Dot<Tv> gg;
  double ew = 0.0;
  float fmx = 0.0f, femx = 0.0f;
  const bool has_ext = o.fz_ext != 0.0;
  double fmx_d = 0.0;
  BoxAcc box;
  for (int s = blockIdx.x * kT + threadIdx.x; s < N; s += gridDim.x * kT) {
    const int ix = s / gm.ny, iy = s - ix * gm.ny;
    bool nearflag = false;
    for (int l = 0; l < nl; l++) {
      Tx xd[3];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const size_t idx = (size_t)(3 * l + c) * N + s;
        femx = fmaxf(femx, fabsf((float)fel[idx]));
        xd[c] = x[idx];
      }
      double fw[3] = {0.0, 0.0, 0.0};
      bool hit = false;
      if (obst && l < o.nlayer) {
        const float ge = all ? -1e30f : cg_gate(o, gm, ix, iy, l, s, xd);
        if (ge < o.ga) nearflag = true;
        if (ge < o.gw) {
          const double zero[3] = {0.0, 0.0, 0.0};
          const WallOut w = site_wall<Tx, BIC>(o, gm, ix, iy, l, s, xd, zero);
          fw[0] = w.f[0];
          fw[1] = w.f[1];
          fw[2] = w.f[2];
          ew += w.e;
          hit = true;
        }
      }
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const size_t idx = (size_t)(3 * l + c) * N + s;
        Tv gv;
        const bool ext = has_ext && c == 2 && l < o.nlayer;
        if (hit || ext) gv = (Tv)((double)fel[idx] + (hit ? fw[c] : 0.0) + (ext ? o.fz_ext : 0.0));
        else gv = (Tv)fel[idx];
        g[idx] = gv;
        h[idx] = gv;
        gg.add(gv, gv);
        if constexpr (sizeof(Tv) == 4) fmx = fmaxf(fmx, fabsf(gv));
        else fmx_d = fmax(fmx_d, fabs(gv));
      }
    }
    if (obst) {
      active[s] = nearflag ? 1 : 0;
      if (nearflag && !all) box.add(ix, iy, gm);
    }
  }
  const double acc[8] = {gg.get(), ew, sizeof(Tv) == 4 ? (double)fmx : fmx_d, (double)femx,
                         (double)box.a, (double)box.b, (double)box.c, (double)box.d};
  __shared__ double res[8];
  if (!reduce_last<2, 6>(acc, part, &ctl->counter, res)) return;
  if (threadIdx.x == 0) {
    ctl->gg = res[0];
    ctl->gh = res[0];  // h = g
    ctl->hmax = res[2];
    ctl->ew = res[1];
    ctl->fmax = res[2];
    ctl->fmax_restart = res[2];
    ctl->since = 0;
    ctl->beta = 0.0;
    set_box(ctl, res + 4, gm, all);
    // FP32 state resolves g = f_el + F_w to about eps32 |f_el|: the FP32
    // phase stops at 64 eps32 max|f_el| if that is above the request
    ctl->ftol = ctl->bulk ? fmax(ctl->ftol_req, 64.0 * 5.960464477539063e-8 * res[3]) : ctl->ftol_req;
    if (!isfinite(res[0])) ctl->done = 3;
    else if (res[2] <= ctl->ftol) ctl->done = 1;
    else if (ctl->it >= ctl->maxit) ctl->done = 2;
    else ctl->done = 0;
    set_loop(hc, use_hc, ctl->done == 0 ? 1u : 0u);
  }
}

// Line-search state: step a and its bracket [lo, hi] (hi < 0: none yet).
struct LineState {
  double a, lo, hi, gh, hKh, fw0h, amax;
  int it, done;
};

// Start from the sums at a = 0 (F_w(u).h and the wall curvature along h):
// first Newton step on phi'(a) = -(g.h - a hKh + dF_w(a).h).
__device__ __forceinline__ void ls_init(LineState &L, double fw0h, double cw0, double gh, double hKh, double hmax,
                                        double dmax, bool obst) {
  L.gh = gh;
  L.hKh = hKh;
  L.fw0h = fw0h;
  // LAMMPS min_modify dmax: no component moves more than dmax in one step
  L.amax = (dmax > 0.0 && hmax > 0.0) ? dmax / hmax : 1e300;
  L.lo = 0.0;
  L.it = 0;
  // with the cap, amax is the upper bracket of the step from the start
  L.hi = L.amax < 1e300 ? L.amax : -1.0;
  const double curv = hKh + cw0;
  double a;
  if (curv > 0.0 && gh > 0.0) a = gh / curv;
  else a = gh > 0.0 ? 1e-3 : 0.0;
  if (gh > 0.0 && L.hi >= 0.0 && a >= L.hi) a = 0.5 * L.hi;  // bisect the bracket
  L.a = a;
  L.done = (!obst || gh <= 0.0) ? 1 : 0;
}

// The Newton step of a probe from the reduced F_w(u + a h).h and curvature.
__device__ __forceinline__ void ls_step(LineState &L, double dfh, double cwall) {
  const double a = L.a;
  const double gdir = L.gh - a * L.hKh + (dfh - L.fw0h);
  const double curv = L.hKh + cwall;
  if (gdir > 0.0) L.lo = a;
  else L.hi = a;
  double an = (curv > 0.0) ? a + gdir / curv : -1.0;
  if (L.hi >= 0.0 && (an <= L.lo || an >= L.hi || an < 0.0)) an = 0.5 * (L.lo + L.hi);
  else if (an < 0.0) an = L.lo > 0.0 ? 2.0 * L.lo : 1e-3;
  const double step = fabs(an - a);
  L.a = an;
  L.it += 1;
  // an exact line minimum is not needed: Polak-Ribiere with restarts
  // converges from a step within 1e-6 of it
  if (step <= 1e-6 * fabs(an) || L.it >= kLsMax || !isfinite(an)) L.done = 1;
  if (!isfinite(an)) L.a = 0.0;
}

__device__ __forceinline__ LineState ls_load(const CgCtl *c) {
  LineState L;
  L.a = c->a; L.lo = c->lo; L.hi = c->hi; L.gh = c->gh; L.hKh = c->hKh; L.fw0h = c->fw0h; L.amax = c->amax;
  L.it = c->ls_it; L.done = c->ls_done;
  return L;
}
__device__ __forceinline__ void ls_store(CgCtl *c, const LineState &L) {
  c->a = L.a; c->lo = L.lo; c->hi = L.hi; c->gh = L.gh; c->hKh = L.hKh; c->fw0h = L.fw0h; c->amax = L.amax;
  c->ls_it = L.it; c->ls_done = L.done;
}

// ---- start of the line search: h.K.h from the energy of the direction's
// force evaluation (E(h) = h.K.h / 2 with the gamma-point force off), g.h and
// max|h| from the kernel that formed h, wall terms at a = 0 over the set;
// first Newton step -------------------------------------------------------------
template <typename Tx, typename Tv, bool BIC = false>
__global__ void __launch_bounds__(kT) k_lsinit(const __grid_constant__ Obst o, Geom gm, const Tx *__restrict__ x,
                                                const Tv *__restrict__ h,
                                                const unsigned char *__restrict__ active,
                                                const double *__restrict__ eh, double *__restrict__ part,
                                                CgCtl *ctl) {
  double fh = 0.0, cw = 0.0;
  if (o.kind != GFMD_OBST_NONE) line_walls<Tx, Tv, BIC>(o, gm, x, h, active, ctl, 0.0, fh, cw);
  const double acc[2] = {fh, cw};
  __shared__ double res[2];
  if (!reduce_last<2, 0>(acc, part, &ctl->counter, res)) return;
  if (threadIdx.x == 0) {
    LineState L;
    ls_init(L, res[0], res[1], ctl->gh, 2.0 * (*eh), ctl->hmax, ctl->dmax, o.kind != GFMD_OBST_NONE);
    ls_store(ctl, L);
  }
}

// ---- one Newton probe of the line search at u + a h ------------------------
// gdir(a) = g.h - a hKh + sum F_w(u + a h).h - F_w(u).h   (= -phi'(a))
// curv(a) = hKh + sum h^T H_w(u + a h) h                   (=  phi''(a))
template <typename Tx, typename Tv, bool BIC = false>
__global__ void __launch_bounds__(kT) k_probe(const __grid_constant__ Obst o, Geom gm, const Tx *__restrict__ x,
                                               const Tv *__restrict__ h,
                                               const unsigned char *__restrict__ active,
                                               double *__restrict__ part, CgCtl *ctl) {
  if (ctl->ls_done) return;  // uniform over the grid
  const double a = ctl->a;
  double dfh = 0.0, cw = 0.0;
  line_walls<Tx, Tv, BIC>(o, gm, x, h, active, ctl, a, dfh, cw);
  const double acc[2] = {dfh, cw};
  __shared__ double res[2];
  if (!reduce_last<2, 0>(acc, part, &ctl->counter, res)) return;
  if (threadIdx.x == 0) {
    LineState L = ls_load(ctl);
    ls_step(L, res[0], res[1]);
    ls_store(ctl, L);
  }
}

// ---- the whole line search in one thread-block cluster ---------------------
// FP32 phase, a sphere wall on one atom layer, a set whose box holds at most
// kLsCap sites.  The set's x and h stay in registers for the whole search:
// a Newton step is a pass over registers, a compensated FP32 reduction per
// block and one cluster barrier (every block writes its sums into every
// block's shared memory, double-buffered by step parity, and every block
// reduces them in the same order and takes the same Newton step, so no step
// is broadcast).  One launch replaces k_lsinit
// and up to kLsMax probes, each of which chains a grid-wide reduction
// through global memory.  A larger box leaves the search to those kernels:
// block 0 sets the conditional that runs them.
constexpr int kLsCl = 8;                     // blocks of the cluster (portable size)
constexpr int kLsT = 1024;                   // threads per block
constexpr int kLsS = 3;                      // sites per thread
constexpr int kLsCap = kLsCl * kLsT * kLsS;  // largest box taken (sites)

__host__ __device__ inline int ls_box_sites(const CgCtl &c) {
  const int w = c.by1 - c.by0 + 1, ht = c.bx1 - c.bx0 + 1;
  return (w > 0 && ht > 0) ? w * ht : 0;
}

// Unnormalised FP32 pair hi + lo; the sum adds the rounding error of
// hi_a + hi_b (TwoSum) to the low parts.
struct F2 {
  float hi, lo;
};
__device__ __forceinline__ F2 f2_add(F2 a, F2 b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  return F2{s, __fadd_rn(__fadd_rn(a.lo, b.lo), e)};
}
__device__ __forceinline__ F2 f2_down(F2 v, int off) {
  return F2{__shfl_down_sync(0xffffffffu, v.hi, off), __shfl_down_sync(0xffffffffu, v.lo, off)};
}

template <typename Tx, typename Tv>
__global__ void __cluster_dims__(kLsCl, 1, 1) __launch_bounds__(kLsT, 1)
    k_ls_cluster(const __grid_constant__ Obst o, Geom gm, const Tx *__restrict__ x, const Tv *__restrict__ h,
                 const unsigned char *__restrict__ active, const double *__restrict__ eh, CgCtl *ctl,
                 cudaGraphConditionalHandle hls, int use_hc) {
  static_assert(sizeof(Tx) == 4 && sizeof(Tv) == 4, "the FP32 phase's line search");
  static_assert(kLsT == 32 * 32, "one warp reduces the block's 32 warp sums");
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  const int rank = (int)cl.block_rank();
  const int nb = ls_box_sites(*ctl);
  const bool big = nb > kLsCap;  // uniform over the cluster
  if (rank == 0 && threadIdx.x == 0) set_loop(hls, use_hc, big ? 1u : 0u);
  if (big) return;

  __shared__ F2 ws[kLsT / 32][2];   // warp sums
  __shared__ F2 bs[2][kLsCl][2];    // block sums of a step (by parity), from every block
  __shared__ float pub_a;           // step and flag from this block's thread 0
  __shared__ int pub_done;
  __shared__ LineState L;           // thread 0; the same in every block
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int N = gm.nx * gm.ny;
  const int w = ctl->by1 - ctl->by0 + 1, x0 = ctl->bx0, y0 = ctl->by0;
  // this thread's sites of the set (box positions t, t + nthr, ...) as
  // ix << 16 | iy (nx, ny <= 8192), -1 for none, with their x and h
  int sp[kLsS];
  float xc[kLsS][3], hc[kLsS][3];
#pragma unroll
  for (int k = 0; k < kLsS; k++) {
    const int i = rank * kLsT + (int)threadIdx.x + k * kLsCl * kLsT;
    sp[k] = -1;
#pragma unroll
    for (int c = 0; c < 3; c++) xc[k][c] = hc[k][c] = 0.0f;
    if (i < nb) {
      const int r = i / w;
      const int ix = x0 + r, iy = y0 + (i - r * w);
      const int s = ix * gm.ny + iy;
      if (active[s]) {
        sp[k] = ix << 16 | iy;
#pragma unroll
        for (int c = 0; c < 3; c++) {
          xc[k][c] = (float)x[(size_t)c * N + s];
          hc[k][c] = (float)h[(size_t)c * N + s];
        }
      }
    }
  }
  cl.sync();  // every block has started before shared memory is written across the cluster
  // F_w(x + a h).h and h^T H_w h over this thread's sites
  auto pass = [&](float a, F2 &fh, F2 &cw) {
    fh = F2{0.0f, 0.0f};
    cw = F2{0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < kLsS; k++) {
      if (sp[k] < 0) continue;
      const SphereOff q = sphere_off(o, gm.nx, gm.ny, sp[k] >> 16, sp[k] & 0xffff, 0, xc[k][0] + a * hc[k][0],
                                     xc[k][1] + a * hc[k][1], xc[k][2] + a * hc[k][2]);
      float e, f[3], cv;
      if (sphere_wall_f(o, q, hc[k], e, f, cv)) {
        fh = f2_add(fh, F2{f[0] * hc[k][0] + f[1] * hc[k][1] + f[2] * hc[k][2], 0.0f});
        cw = f2_add(cw, F2{cv, 0.0f});
      }
    }
  };
  // cluster sums of (fa, fb) for the step of parity par, valid in thread 0
  // of every block: each block reduces the kLsCl block sums in rank order,
  // so every block holds the same values (and takes the same Newton step)
  auto cluster_sum = [&](F2 fa, F2 fb, int par, double &sa, double &sb) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      fa = f2_add(fa, f2_down(fa, off));
      fb = f2_add(fb, f2_down(fb, off));
    }
    if (lane == 0) {
      ws[warp][0] = fa;
      ws[warp][1] = fb;
    }
    __syncthreads();
    if (warp == 0) {
      fa = ws[lane][0];
      fb = ws[lane][1];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        fa = f2_add(fa, f2_down(fa, off));
        fb = f2_add(fb, f2_down(fb, off));
      }
      fa = F2{__shfl_sync(0xffffffffu, fa.hi, 0), __shfl_sync(0xffffffffu, fa.lo, 0)};
      fb = F2{__shfl_sync(0xffffffffu, fb.hi, 0), __shfl_sync(0xffffffffu, fb.lo, 0)};
      if (lane < kLsCl) {  // lane q delivers this block's sums to block q
        F2 *dst = cl.map_shared_rank(&bs[par][rank][0], lane);
        dst[0] = fa;
        dst[1] = fb;
      }
    }
    cl.sync();
    if (warp == 0) {
      fa = lane < kLsCl ? bs[par][lane][0] : F2{0.0f, 0.0f};
      fb = lane < kLsCl ? bs[par][lane][1] : F2{0.0f, 0.0f};
#pragma unroll
      for (int off = kLsCl / 2; off > 0; off >>= 1) {
        fa = f2_add(fa, f2_down(fa, off));
        fb = f2_add(fb, f2_down(fb, off));
      }
      sa = (double)fa.hi + (double)fa.lo;
      sb = (double)fb.hi + (double)fb.lo;
    }
  };
  F2 fh, cw;
  double s0 = 0.0, s1 = 0.0;
  int par = 0;
  pass(0.0f, fh, cw);
  cluster_sum(fh, cw, par, s0, s1);
  if (threadIdx.x == 0) {
    ls_init(L, s0, s1, ctl->gh, 2.0 * (*eh), ctl->hmax, ctl->dmax, true);
    pub_a = (float)L.a;
    pub_done = L.done;
  }
  __syncthreads();
  float a = pub_a;
  int done = pub_done;
  while (!done) {  // uniform: every block takes the same steps
    par ^= 1;
    pass(a, fh, cw);
    cluster_sum(fh, cw, par, s0, s1);
    if (threadIdx.x == 0) {
      ls_step(L, s0, s1);
      pub_a = (float)L.a;
      pub_done = L.done;
    }
    __syncthreads();
    a = pub_a;
    done = pub_done;
  }
  // no shared memory is written across the cluster after the last cluster
  // barrier: the blocks may leave in any order
  if (rank == 0 && threadIdx.x == 0) ls_store(ctl, L);
}

// ---- update after the line search ------------------------------------------
// u += a h; g += a fKh + F_w(u_new) - F_w(u_old).  The elastic part of g is
// updated through the linearity of F_el, so f_el itself is not stored, and
// the rounding of the FP32 state is relative to the (small) gradient rather
// than to the elastic force.
template <typename T> struct V3 { T v[3]; };
template <typename Tv> struct WallDelta { double e; Tv g[3]; };

// Near the obstacle: g_new = g_old + a fKh + F_w(x_new) - F_w(x_old), with
// E_w(x_new).  Kept out of line (arguments by value, so the caller's arrays
// stay in registers) so the far-field loop stays small.
template <typename Tx, typename Tv, bool BIC = false>
__device__ __noinline__ WallDelta<Tv> wall_delta(const Obst &o, const Geom &gm, int ix, int iy, int l, int s,
                                                 V3<Tx> xv, V3<Tx> xn, V3<Tv> go, V3<Tv> fk, double a) {
  const double zero[3] = {0.0, 0.0, 0.0};
  const WallOut w1 = site_wall<Tx, BIC>(o, gm, ix, iy, l, s, xn.v, zero);
  const WallOut w0 = site_wall<Tx, BIC>(o, gm, ix, iy, l, s, xv.v, zero);
  WallDelta<Tv> r;
  r.e = w1.e;
  for (int c = 0; c < 3; c++) r.g[c] = (Tv)((double)go.v[c] + a * (double)fk.v[c] + (w1.f[c] - w0.f[c]));
  return r;
}

// Dot products of the streaming kernels: the terms of one loop trip (at most
// V x ndof) are summed in the vector type, each trip sum then enters the
// thread's Dot (FP64, or a compensated FP32 pair): FP32 trip sums round at
// eps32 relative to themselves, below what Polak-Ribiere and the line search
// resolve, at a fraction of the instructions of compensating every term.
template <typename Tx, typename Tv, bool BIC = false, int V = 4>
__global__ void __launch_bounds__(kT, V == 4 ? 2 : 4) k_update(const __grid_constant__ Obst o, Geom gm,
                                                               Tx *__restrict__ x, const Tv *__restrict__ h,
                                                               const Tv *__restrict__ fKh, Tv *__restrict__ g,
                                                               Tv *__restrict__ gp,
                                                               unsigned char *__restrict__ active,
                                                               double *__restrict__ part, CgCtl *ctl,
                                                               cudaGraphConditionalHandle hc, int use_hc) {
  const double ad = ctl->a;
  const Tx a = (Tx)ad;
  const Tv av = (Tv)ad;
  const int N = gm.nx * gm.ny;
  const int nl = gm.ndof / 3;
  const bool obst = o.kind != GFMD_OBST_NONE, all = map_in_f32<Tx>(o);
  Dot<Tv> gg, ggo, hg;
  double ew = 0.0;
  Tv fmx = (Tv)0;
  BoxAcc box;
  for (int s0 = V * (blockIdx.x * kT + threadIdx.x); s0 < N; s0 += V * gridDim.x * kT) {
    bool nearflag[V];
#pragma unroll
    for (int j = 0; j < V; j++) nearflag[j] = false;
    Tv sgg = (Tv)0, sggo = (Tv)0, shg = (Tv)0;
    for (int l = 0; l < nl; l++) {
      Tx xv[3][V], xn[3][V];
      Tv hv[3][V], fk[3][V], go[3][V], gn[3][V];
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const size_t idx = (size_t)(3 * l + c) * N + s0;
        VecN<Tx, V>::ld(x + idx, xv[c]);
        VecN<Tv, V>::ld(h + idx, hv[c]);
        VecN<Tv, V>::ld(fKh + idx, fk[c]);
        VecN<Tv, V>::ld(g + idx, go[c]);
#pragma unroll
        for (int j = 0; j < V; j++) {
          xn[c][j] = xv[c][j] + a * (Tx)hv[c][j];
          gn[c][j] = go[c][j] + av * fk[c][j];
        }
      }
      if (obst && l < o.nlayer) {
#pragma unroll
        for (int j = 0; j < V; j++) {
          const int s = s0 + j;
          if (all) {
            float e1, f1, e0, f0;
            map_wall_f(o, s, (float)xn[2][j] + o.foff[l][2], e1, f1);
            map_wall_f(o, s, (float)xv[2][j] + o.foff[l][2], e0, f0);
            nearflag[j] = true;
            ew += e1;
            gn[2][j] = gn[2][j] + (Tv)(f1 - f0);
          } else {
            const int ix = s / gm.ny, iy = s - ix * gm.ny;
            const Tx xo3[3] = {xv[0][j], xv[1][j], xv[2][j]}, xn3[3] = {xn[0][j], xn[1][j], xn[2][j]};
            const float ge_new = cg_gate(o, gm, ix, iy, l, s, xn3);
            const float ge_old = cg_gate(o, gm, ix, iy, l, s, xo3);
            if (ge_new < o.ga) nearflag[j] = true;
            if (ge_new < o.gw || ge_old < o.gw) {
              const WallDelta<Tv> wd = wall_delta<Tx, Tv, BIC>(
                  o, gm, ix, iy, l, s, V3<Tx>{{xo3[0], xo3[1], xo3[2]}}, V3<Tx>{{xn3[0], xn3[1], xn3[2]}},
                  V3<Tv>{{go[0][j], go[1][j], go[2][j]}}, V3<Tv>{{fk[0][j], fk[1][j], fk[2][j]}}, ad);
              ew += wd.e;
              gn[0][j] = wd.g[0];
              gn[1][j] = wd.g[1];
              gn[2][j] = wd.g[2];
            }
          }
        }
      }
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const size_t idx = (size_t)(3 * l + c) * N + s0;
#pragma unroll
        for (int j = 0; j < V; j++) {
          sgg = fma(gn[c][j], gn[c][j], sgg);
          sggo = fma(gn[c][j], go[c][j], sggo);
          shg = fma(hv[c][j], gn[c][j], shg);
          fmx = fmax(fmx, fabs(gn[c][j]));
        }
        VecN<Tx, V>::st(x + idx, xn[c]);
        VecN<Tv, V>::st(g + idx, gn[c]);
        if (gp) VecN<Tv, V>::st(gp + idx, go[c]);  // previous gradient (preconditioned Polak-Ribiere)
      }
    }
    gg.addsum(sgg);
    ggo.addsum(sggo);
    hg.addsum(shg);
    if (obst) {
#pragma unroll
      for (int j = 0; j < V; j++) {
        active[s0 + j] = nearflag[j] ? 1 : 0;
        if (nearflag[j] && !all) {
          const int ix = (s0 + j) / gm.ny;
          box.add(ix, s0 + j - ix * gm.ny, gm);
        }
      }
    }
  }
  const double acc[9] = {gg.get(), ggo.get(), hg.get(), ew, (double)fmx,
                         (double)box.a, (double)box.b, (double)box.c, (double)box.d};
  __shared__ double res[9];
  if (!reduce_last<4, 5>(acc, part, &ctl->counter, res)) return;
  if (threadIdx.x == 0) {
    const double gg_new = res[0], g_gold = res[1], h_g = res[2];
    if (!gp) {
      const double gg_old = ctl->gg;
      double beta = gg_old > 0.0 ? (gg_new - g_gold) / gg_old : 0.0;  // Polak-Ribiere
      if (beta < 0.0) beta = 0.0;
      // new direction h' = g + beta h must descend: h'.g = gg_new + beta h.g > 0
      if (!(gg_new + beta * h_g > 0.0)) beta = 0.0;
      ctl->beta = beta;
      ctl->gg = gg_new;
    }  // preconditioned: beta follows from the preconditioned gradient (k_pcg_beta)
    ctl->hg = h_g;
    ctl->ew = res[3];
    ctl->fmax = res[4];
    set_box(ctl, res + 5, gm, all);
    ctl->it += 1;
    ctl->since += 1;
    if (!isfinite(gg_new)) ctl->done = 3;
    else if (res[4] <= ctl->ftol) ctl->done = 1;
    else if (ctl->it >= ctl->maxit) ctl->done = 2;
    const bool go_on = ctl->done == 0 && ctl->since < ctl->recompute;
    set_loop(hc, use_hc, go_on ? 1u : 0u);
  }
}

// Direction after an update: h = g + beta h (h = z + beta h with a
// preconditioner, z = -mz), with max|h| for the step cap and
// g.h = g.g + beta h_old.g (g.z + beta h_old.g).
template <typename Tv, int V = 4>
__global__ void __launch_bounds__(kT) k_dir(size_t n, Tv *__restrict__ h, const Tv *__restrict__ g,
                                             const Tv *__restrict__ mz, double *__restrict__ part, CgCtl *ctl) {
  const Tv beta = (Tv)ctl->beta;
  Tv hm = (Tv)0;
  for (size_t i = V * (blockIdx.x * (size_t)kT + threadIdx.x); i < n; i += V * (size_t)gridDim.x * kT) {
    Tv hv[V], gv[V];
    VecN<Tv, V>::ld(h + i, hv);
    VecN<Tv, V>::ld(mz ? mz + i : g + i, gv);
#pragma unroll
    for (int j = 0; j < V; j++) {
      hv[j] = mz ? beta * hv[j] - gv[j] : gv[j] + beta * hv[j];
      hm = fmax(hm, fabs(hv[j]));
    }
    VecN<Tv, V>::st(h + i, hv);
  }
  const double acc[1] = {(double)hm};
  __shared__ double res[1];
  if (!reduce_last<0, 1>(acc, part, &ctl->counter, res)) return;
  if (threadIdx.x == 0) {
    ctl->hmax = res[0];
    ctl->gh = ctl->gg + ctl->beta * ctl->hg;
  }
}

// Preconditioned CG.  The preconditioner handle's force evaluation of g
// returns mz = -z, z = (Phi + c)^{-1} g.
// Restart: h = z; g.z, max|z|.
template <typename Tv>
__global__ void __launch_bounds__(kT) k_pcg_init(size_t n, const Tv *__restrict__ g, const Tv *__restrict__ mz,
                                                  Tv *__restrict__ h, double *__restrict__ part, CgCtl *ctl) {
  Dot<Tv> gz;
  Tv zm = (Tv)0;
  for (size_t i = blockIdx.x * (size_t)kT + threadIdx.x; i < n; i += (size_t)gridDim.x * kT) {
    const Tv z = -mz[i];
    h[i] = z;
    gz.add(g[i], z);
    zm = fmax(zm, fabs(z));
  }
  const double acc[2] = {gz.get(), (double)zm};
  __shared__ double res[2];
  if (!reduce_last<1, 1>(acc, part, &ctl->counter, res)) return;
  if (threadIdx.x == 0) {
    ctl->gg = res[0];
    ctl->gh = res[0];
    ctl->hmax = res[1];
  }
}

// After the update: beta = max(0, z.(g - g_old) / (g_old.z_old)) with the
// descent check h'.g = z.g + beta h.g > 0 (min_cg_gfmd.cpp:172-196).
template <typename Tv, int V = 4>
__global__ void __launch_bounds__(kT) k_pcg_beta(size_t n, const Tv *__restrict__ g, const Tv *__restrict__ gp,
                                                  const Tv *__restrict__ mz, double *__restrict__ part,
                                                  CgCtl *ctl) {
  Dot<Tv> zg, zgo;  // trip sums of V terms, then compensated (as in k_update)
  for (size_t i = V * (blockIdx.x * (size_t)kT + threadIdx.x); i < n; i += V * (size_t)gridDim.x * kT) {
    Tv zv[V], gv[V], pv[V];
    VecN<Tv, V>::ld(mz + i, zv);
    VecN<Tv, V>::ld(g + i, gv);
    VecN<Tv, V>::ld(gp + i, pv);
    Tv s1 = (Tv)0, s2 = (Tv)0;
#pragma unroll
    for (int j = 0; j < V; j++) {
      s1 = fma(-zv[j], gv[j], s1);
      s2 = fma(-zv[j], pv[j], s2);
    }
    zg.addsum(s1);
    zgo.addsum(s2);
  }
  const double acc[2] = {zg.get(), zgo.get()};
  __shared__ double res[2];
  if (!reduce_last<2, 0>(acc, part, &ctl->counter, res)) return;
  if (threadIdx.x == 0) {
    const double old = ctl->gg;
    double beta = old > 0.0 ? (res[0] - res[1]) / old : 0.0;
    if (!(beta > 0.0)) beta = 0.0;
    if (!(res[0] + beta * ctl->hg > 0.0)) beta = 0.0;
    ctl->beta = beta;
    ctl->gg = res[0];
  }
}

__global__ void k_f2d(size_t n, const float *__restrict__ a, double *__restrict__ b) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}
__global__ void k_d2f(size_t n, const double *__restrict__ a, float *__restrict__ b) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// Arms a branch's restart unless the branch is parked.
__global__ void k_gate(const CgCtl *ctl, cudaGraphConditionalHandle hif) {
  if (threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(hif, ctl->parked ? 0u : 1u);
}

// Final report from FP64 elastic forces fel of u: total force
// f = fel + F_w(u) + external; sums: E_w + E_ext, |f|^2; max |f_i|.
template <bool BIC = false>
__global__ void __launch_bounds__(kT) k_report(Obst o, Geom gm, const double *__restrict__ x,
                                                const double *__restrict__ fel, double *__restrict__ part,
                                                CgCtl *ctl, double *__restrict__ out) {
  const int N = gm.nx * gm.ny;
  const int nl = gm.ndof / 3;
  double ew = 0.0, f2 = 0.0, fm = 0.0;
  for (int s = blockIdx.x * kT + threadIdx.x; s < N; s += gridDim.x * kT) {
    const int ix = s / gm.ny, iy = s - ix * gm.ny;
    for (int l = 0; l < nl; l++) {
      double fw[3] = {0.0, 0.0, 0.0};
      if (l < o.nlayer) {
        if (o.kind == GFMD_OBST_MAP_EXP ||
            (o.kind != GFMD_OBST_NONE && wall_near(o, gap_of(o, ix, iy, l, x, N, s)))) {
          double r[3], d[3];
          atom_pos<double, double>(o, ix, iy, l, x, nullptr, N, s, 0.0, r, d);
          const WallOut w = wall_eval<BIC>(o, ix, iy, s, r, d);
          fw[0] = w.f[0];
          fw[1] = w.f[1];
          fw[2] = w.f[2];
          ew += w.e;
        }
        fw[2] += o.fz_ext;
        ew -= o.fz_ext * x[(size_t)(3 * l + 2) * N + s];
      }
      for (int c = 0; c < 3; c++) {
        const double f = fel[(size_t)(3 * l + c) * N + s] + fw[c];
        f2 += f * f;
        fm = fmax(fm, fabs(f));
      }
    }
  }
  const double acc[3] = {ew, f2, fm};
  __shared__ double res[3];
  if (!reduce_last<2, 1>(acc, part, &ctl->counter, res)) return;
  if (threadIdx.x < 3) out[threadIdx.x] = res[threadIdx.x];
}

// ---- host side ---------------------------------------------------------------

// GFMD_TRACE=1 prints the host-side phases of a solve (setup, graph build,
// launches, report) to stderr.
bool trace_on() {
  static const bool on = [] {
    const char *v = std::getenv("GFMD_TRACE");
    return v && v[0] && v[0] != '0';
  }();
  return on;
}
double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

template <typename T> constexpr int io_type() { return sizeof(T) == 8 ? 0 : 1; }

// Device state of one CG problem, carved from the handle's workspace (kept
// between solves, grown when a solve needs more).
struct CgBufs {
  cudaStream_t cs = nullptr;
  int nblk = 0;
  size_t n = 0;
  void *fel = nullptr;      // n doubles: elastic force of a restart (float or double)
  void *g = nullptr, *h = nullptr, *fKh = nullptr;  // n doubles each (Tv)
  void *mz = nullptr, *gp = nullptr;  // preconditioned CG: -z and the previous g (Tv)
  float *u32 = nullptr;     // FP32 displacements of the mixed solve
  float *mapf = nullptr;    // FP32 copy of a map obstacle (gating)
  unsigned char *active = nullptr;
  double *part = nullptr;
  double *d_e = nullptr;    // energy of an evaluation; [1..3] report scalars
  CgCtl *ctl = nullptr;
  CgCtl *hctl = nullptr;    // pinned
  ~CgBufs() {
    if (cs) cudaStreamDestroy(cs);
  }
};

cudaError_t bufs_init(CgBufs &b, gfmd_solver *h, bool mixed, bool map, bool pcg) {
  const Geom &g = h->g;
  b.n = (size_t)g.ndof * g.nx * g.ny;
  const size_t nsite = (size_t)g.nx * g.ny;
  b.nblk = (int)std::max<size_t>(1, std::min<size_t>((size_t)h->sm_count * 4, (nsite + kT - 1) / kT));
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  const size_t vb = up(sizeof(double) * b.n);
  size_t off[12], tot = 0;
  const size_t sz[12] = {vb, vb, vb, vb, mixed ? up(sizeof(float) * b.n) : 0, map ? up(sizeof(float) * nsite) : 0,
                         // partials: room for the most resident 256-thread blocks (8 per SM)
                         up(nsite), up(sizeof(double) * kQ * std::max<size_t>(b.nblk, (size_t)h->sm_count * 8)),
                         up(sizeof(double) * 4), up(sizeof(CgCtl)),
                         pcg ? vb : 0, pcg ? vb : 0};
  for (int k = 0; k < 12; k++) {
    off[k] = tot;
    tot += sz[k];
  }
  cudaError_t e = cudaStreamCreateWithFlags(&b.cs, cudaStreamNonBlocking);
  if (e == cudaSuccess && h->ws_bytes < tot) {
    if (h->ws) cudaFree(h->ws);
    h->ws = nullptr;
    h->ws_bytes = 0;
    e = cudaMalloc(&h->ws, tot);
    if (e == cudaSuccess) h->ws_bytes = tot;
  }
  if (e == cudaSuccess && !h->ws_host) e = cudaMallocHost(&h->ws_host, sizeof(CgCtl));
  if (e != cudaSuccess) return e;
  b.hctl = static_cast<CgCtl *>(h->ws_host);
  char *a = static_cast<char *>(h->ws);
  b.fel = a + off[0];
  b.g = a + off[1];
  b.h = a + off[2];
  b.fKh = a + off[3];
  b.u32 = mixed ? reinterpret_cast<float *>(a + off[4]) : nullptr;
  b.mapf = map ? reinterpret_cast<float *>(a + off[5]) : nullptr;
  b.active = reinterpret_cast<unsigned char *>(a + off[6]);
  b.part = reinterpret_cast<double *>(a + off[7]);
  b.d_e = reinterpret_cast<double *>(a + off[8]);
  b.ctl = reinterpret_cast<CgCtl *>(a + off[9]);
  b.mz = pcg ? a + off[10] : nullptr;
  b.gp = pcg ? a + off[11] : nullptr;
  return cudaSuccess;
}

// Force evaluation on stream st with handle hh.
cudaError_t eval_on(gfmd_solver *hh, cudaStream_t st, const void *in, int in_t, void *out, int out_t,
                    double *d_e, bool with_linf) {
  cudaStream_t keep = hh->stream;
  hh->stream = st;
  cudaError_t e = enqueue_force_opts(hh, in, in_t, out, out_t, d_e, with_linf);
  hh->stream = keep;
  return e;
}

// One CG problem of a batch.
struct Item {
  CgBufs b;
  gfmd_solver *hp = nullptr;    // force handle (FP32 in the mixed solve)
  gfmd_solver *hr64 = nullptr;  // FP64 refinement handle (mixed) or NULL
  gfmd_solver *hpre = nullptr;  // preconditioner handle or NULL
  Obst o{};
  double *u = nullptr;          // caller's FP64 displacements
  bool mixed = false;
  int evals = 0;
  int done = 0;                 // phase result
  int it0 = 0;
  gfmd_min_report_t rep{};
};

// Displacements a phase works on: FP32 copy in the bulk phase, else u.
template <typename Tx> Tx *phase_x(Item &it) {
  if constexpr (sizeof(Tx) == 4) return it.b.u32;
  else return it.u;
}

// The cluster line search: on unless GFMD_LS_CLUSTER=0, the device cannot
// place its cluster, or a graph holding it was refused (then off for the
// process).
std::atomic<int> g_ls_cluster{-1};
bool ls_cluster_on() {
  int v = g_ls_cluster.load();
  if (v < 0) {
    const char *env = std::getenv("GFMD_LS_CLUSTER");
    v = (env && env[0] == '0') ? 0 : 1;
    if (v) {
      cudaLaunchConfig_t cfg = {};
      cfg.gridDim = dim3(kLsCl);
      cfg.blockDim = dim3(kLsT);
      int ncl = 0;
      if (cudaOccupancyMaxActiveClusters(&ncl, k_ls_cluster<float, float>, &cfg) != cudaSuccess || ncl < 1) {
        (void)cudaGetLastError();
        v = 0;
      }
    }
    g_ls_cluster.store(v);
  }
  return v == 1;
}

// Items whose phase <Tx, Tv> runs the cluster line search: the FP32 phase
// with a sphere wall on one atom layer.
template <typename Tx, typename Tv, bool BIC> bool ls_cluster_item(const Item &it) {
  return sizeof(Tx) == 4 && sizeof(Tv) == 4 && !BIC &&
         (it.o.kind == GFMD_OBST_SPHERE_EXP || it.o.kind == GFMD_OBST_SPHERE_LJ) && it.o.nlayer == 1 &&
         ls_cluster_on();
}

// Where the probes of a cluster item go in graph mode: an IF node on hls
// added to the body graph being captured; the caller fills probe_body.
struct LsGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphConditionalHandle hls = 0;
  cudaGraph_t probe_body = nullptr;
};

// Adds a conditional node of the given type after the capture's current
// dependencies on stream st; returns its body graph.
cudaError_t add_cond(cudaStream_t st, cudaGraph_t top, cudaGraphConditionalHandle hc,
                     cudaGraphConditionalNodeType type, cudaGraph_t *body) {
  cudaStreamCaptureStatus cs;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  RT_CHECK(cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd));
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = hc;
  cp.conditional.type = type;
  cp.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  RT_CHECK(cudaGraphAddNode(&node, top, deps, nullptr, nd, &cp));
  *body = cp.conditional.phGraph_out[0];
  return cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

// Restart of one item on stream st: fresh F_el(u), g = f_el + F_w + f_ext,
// h = g; arms the item's loop through hwh when use_hc.
template <typename Tx, typename Tv, bool BIC = false>
cudaError_t enqueue_restart(Item &it, bool refine, cudaStream_t st, cudaGraphConditionalHandle hwh, int use_hc) {
  CgBufs &b = it.b;
  gfmd_solver *hr = refine ? it.hr64 : it.hp;
  Tx *x = phase_x<Tx>(it);
  Tx *fel = reinterpret_cast<Tx *>(b.fel);
  Tv *g = reinterpret_cast<Tv *>(b.g), *h = reinterpret_cast<Tv *>(b.h);
  RT_CHECK(cudaMemsetAsync(&b.ctl->counter, 0, sizeof(unsigned int), st));
  RT_CHECK(eval_on(hr, st, x, io_type<Tx>(), fel, io_type<Tx>(), b.d_e, true));
  k_restart<Tx, Tv, BIC><<<b.nblk, kT, 0, st>>>(it.o, it.hp->g, x, fel, g, h, b.active, b.part, b.ctl, hwh, use_hc);
  if (it.hpre) {
    Tv *mz = reinterpret_cast<Tv *>(b.mz);
    RT_CHECK(eval_on(it.hpre, st, g, io_type<Tv>(), mz, io_type<Tv>(), b.d_e, false));
    k_pcg_init<Tv><<<b.nblk, kT, 0, st>>>(b.n, g, mz, h, b.part, b.ctl);
  }
  return cudaGetLastError();
}

// Line search by the grid-wide kernels: k_lsinit and the probes.
template <typename Tx, typename Tv, bool BIC = false> cudaError_t enqueue_probes(Item &it, cudaStream_t st) {
  CgBufs &b = it.b;
  const Geom &gm = it.hp->g;
  Tx *x = phase_x<Tx>(it);
  Tv *h = reinterpret_cast<Tv *>(b.h);
  const bool obst = it.o.kind != GFMD_OBST_NONE;
  k_lsinit<Tx, Tv, BIC><<<obst ? b.nblk : 1, kT, 0, st>>>(it.o, gm, x, h, b.active, b.d_e, b.part, b.ctl);
  if (obst)
    for (int p = 0; p < kLsMax; p++) k_probe<Tx, Tv, BIC><<<b.nblk, kT, 0, st>>>(it.o, gm, x, h, b.active, b.part, b.ctl);
  return cudaGetLastError();
}

// One CG iteration of one item on stream st.  The line search of a cluster
// item is k_ls_cluster, followed by the probes when its box is too large:
// in graph mode (ls given) inside an IF node that k_ls_cluster sets; with
// direct launches by the same rule, from the host's copy of the control
// block (current: the host reads it back after every iteration).
template <typename Tx, typename Tv, bool BIC = false>
cudaError_t enqueue_iteration(Item &it, cudaStream_t st, cudaGraphConditionalHandle hwh, int use_hc,
                              LsGraph *ls = nullptr) {
  CgBufs &b = it.b;
  gfmd_solver *hd = it.hp;
  const Geom &gm = hd->g;
  Tx *x = phase_x<Tx>(it);
  Tv *g = reinterpret_cast<Tv *>(b.g), *h = reinterpret_cast<Tv *>(b.h), *fKh = reinterpret_cast<Tv *>(b.fKh);
  RT_CHECK(eval_on(hd, st, h, io_type<Tv>(), fKh, io_type<Tv>(), b.d_e, false));
  bool probes = true;
  if constexpr (sizeof(Tx) == 4 && sizeof(Tv) == 4 && !BIC) {
    if (ls_cluster_item<Tx, Tv, BIC>(it)) {
      k_ls_cluster<Tx, Tv><<<kLsCl, kLsT, 0, st>>>(it.o, gm, x, h, b.active, b.d_e, b.ctl, ls ? ls->hls : 0,
                                                   ls ? 1 : 0);
      RT_CHECK(cudaGetLastError());
      if (ls) RT_CHECK(add_cond(st, ls->graph, ls->hls, cudaGraphCondTypeIf, &ls->probe_body));
      probes = !ls && ls_box_sites(*b.hctl) > kLsCap;
    }
  }
  if (probes) RT_CHECK((enqueue_probes<Tx, Tv, BIC>(it, st)));
  auto al16 = [](const void *p) { return p == nullptr || ((uintptr_t)p & 15) == 0; };
  Tv *gp = it.hpre ? reinterpret_cast<Tv *>(b.gp) : nullptr;
  Tv *mz = it.hpre ? reinterpret_cast<Tv *>(b.mz) : nullptr;
  const bool v4 = nsite4(gm) && al16(x) && al16(h) && al16(fKh) && al16(g) && al16(gp) && al16(mz);
  const size_t nsite = (size_t)gm.nx * gm.ny;
  const int sms = it.hp->sm_count;
  if (v4)
    k_update<Tx, Tv, BIC, 4><<<grid_for(k_update<Tx, Tv, BIC, 4>, sms, nsite, 4 * kT), kT, 0, st>>>(
        it.o, gm, x, h, fKh, g, gp, b.active, b.part, b.ctl, hwh, use_hc);
  else
    k_update<Tx, Tv, BIC, 1><<<grid_for(k_update<Tx, Tv, BIC, 1>, sms, nsite, kT), kT, 0, st>>>(
        it.o, gm, x, h, fKh, g, gp, b.active, b.part, b.ctl, hwh, use_hc);
  if (it.hpre) {
    RT_CHECK(eval_on(it.hpre, st, g, io_type<Tv>(), mz, io_type<Tv>(), b.d_e, false));
    if (v4) k_pcg_beta<Tv, 4><<<grid_for(k_pcg_beta<Tv, 4>, sms, b.n, 4 * kT), kT, 0, st>>>(b.n, g, gp, mz, b.part, b.ctl);
    else k_pcg_beta<Tv, 1><<<grid_for(k_pcg_beta<Tv, 1>, sms, b.n, kT), kT, 0, st>>>(b.n, g, gp, mz, b.part, b.ctl);
  }
  if (v4) k_dir<Tv, 4><<<grid_for(k_dir<Tv, 4>, sms, b.n, 4 * kT), kT, 0, st>>>(b.n, h, g, mz, b.part, b.ctl);
  else k_dir<Tv, 1><<<grid_for(k_dir<Tv, 1>, sms, b.n, kT), kT, 0, st>>>(b.n, h, g, mz, b.part, b.ctl);
  return cudaGetLastError();
}

// One phase of a batch as a graph.  Per item, concurrently:
//   k_gate -> IF(not parked) { restart: fresh F_el(u), g, h = g; arms the
//   loop } -> WHILE(armed) { CG iteration }.
template <typename Tx, typename Tv>
cudaError_t build_phase(std::vector<Item *> &its, bool refine, cudaStream_t ms, cudaEvent_t fork,
                        std::vector<cudaEvent_t> &join, cudaGraph_t *graph_out, cudaGraphExec_t *exec_out) {
  const size_t n = its.size();
  cudaGraph_t top = nullptr;
  RT_CHECK(cudaGraphCreate(&top, 0));
  *graph_out = top;
  std::vector<cudaGraphConditionalHandle> hif(n), hwh(n);
  for (size_t i = 0; i < n; i++) {
    RT_CHECK(cudaGraphConditionalHandleCreate(&hif[i], top, 0, cudaGraphCondAssignDefault));
    RT_CHECK(cudaGraphConditionalHandleCreate(&hwh[i], top, 0, cudaGraphCondAssignDefault));
  }
  std::vector<cudaGraph_t> bif(n, nullptr), bwh(n, nullptr);
  RT_CHECK(cudaStreamBeginCaptureToGraph(ms, top, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  cudaError_t e = cudaEventRecord(fork, ms);
  for (size_t i = 0; i < n && e == cudaSuccess; i++) {
    CgBufs &b = its[i]->b;
    e = cudaStreamWaitEvent(b.cs, fork, 0);
    if (e == cudaSuccess) {
      k_gate<<<1, 32, 0, b.cs>>>(b.ctl, hif[i]);
      e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = add_cond(b.cs, top, hif[i], cudaGraphCondTypeIf, &bif[i]);
    if (e == cudaSuccess) e = add_cond(b.cs, top, hwh[i], cudaGraphCondTypeWhile, &bwh[i]);
    if (e == cudaSuccess) e = cudaEventRecord(join[i], b.cs);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ms, join[i], 0);
  }
  cudaGraph_t got = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(ms, &got);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return e;
  for (size_t i = 0; i < n; i++) {
    cudaStream_t st = its[i]->b.cs;
    RT_CHECK(cudaStreamBeginCaptureToGraph(st, bif[i], nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    e = its[i]->o.kind == GFMD_OBST_MAP_BICUBIC ? enqueue_restart<Tx, Tv, true>(*its[i], refine, st, hwh[i], 1)
                                                : enqueue_restart<Tx, Tv>(*its[i], refine, st, hwh[i], 1);
    e2 = cudaStreamEndCapture(st, &got);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return e;
    const bool bic = its[i]->o.kind == GFMD_OBST_MAP_BICUBIC;
    LsGraph lsg;
    lsg.graph = bwh[i];
    const bool lsc = !bic && ls_cluster_item<Tx, Tv, false>(*its[i]);
    if (lsc) RT_CHECK(cudaGraphConditionalHandleCreate(&lsg.hls, bwh[i], 0, cudaGraphCondAssignDefault));
    RT_CHECK(cudaStreamBeginCaptureToGraph(st, bwh[i], nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    e = bic ? enqueue_iteration<Tx, Tv, true>(*its[i], st, hwh[i], 1)
            : enqueue_iteration<Tx, Tv>(*its[i], st, hwh[i], 1, lsc ? &lsg : nullptr);
    e2 = cudaStreamEndCapture(st, &got);
    if (e == cudaSuccess) e = e2;
    if (e != cudaSuccess) return e;
    if (lsg.probe_body) {  // the probes for a box the cluster kernel does not take
      RT_CHECK(cudaStreamBeginCaptureToGraph(st, lsg.probe_body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
      e = enqueue_probes<Tx, Tv>(*its[i], st);
      e2 = cudaStreamEndCapture(st, &got);
      if (e == cudaSuccess) e = e2;
      if (e != cudaSuccess) return e;
    }
  }
  return cudaGraphInstantiate(exec_out, top, 0);
}

// GFMD_NO_GRAPHS=1: the same kernels in the same order, launched directly
// with the loop decisions taken on the host after every restart and
// iteration (one synchronization each).  Results are identical to the graph
// mode; it exists for profilers that do not attribute kernels inside
// conditional graph nodes.
bool no_graphs() {
  static const bool on = [] {
    const char *v = std::getenv("GFMD_NO_GRAPHS");
    return v && v[0] && v[0] != '0';
  }();
  return on;
}

template <typename Tx, typename Tv>
cudaError_t run_launch_direct(std::vector<Item *> &its, bool refine, cudaStream_t ms) {
  const cudaGraphConditionalHandle none = 0;
  for (Item *it : its) {
    CgCtl &c = *it->b.hctl;
    RT_CHECK(cudaMemcpyAsync(&c, it->b.ctl, sizeof(CgCtl), cudaMemcpyDeviceToHost, ms));
    RT_CHECK(cudaStreamSynchronize(ms));
    if (c.parked) continue;
    RT_CHECK((it->o.kind == GFMD_OBST_MAP_BICUBIC ? enqueue_restart<Tx, Tv, true>(*it, refine, ms, none, 0)
                                                  : enqueue_restart<Tx, Tv>(*it, refine, ms, none, 0)));
    RT_CHECK(cudaMemcpyAsync(&c, it->b.ctl, sizeof(CgCtl), cudaMemcpyDeviceToHost, ms));
    RT_CHECK(cudaStreamSynchronize(ms));
    while (c.done == 0 && c.since < c.recompute) {
      RT_CHECK((it->o.kind == GFMD_OBST_MAP_BICUBIC ? enqueue_iteration<Tx, Tv, true>(*it, ms, none, 0)
                                                    : enqueue_iteration<Tx, Tv>(*it, ms, none, 0)));
      RT_CHECK(cudaMemcpyAsync(&c, it->b.ctl, sizeof(CgCtl), cudaMemcpyDeviceToHost, ms));
      RT_CHECK(cudaStreamSynchronize(ms));
    }
  }
  return cudaSuccess;
}

struct GraphHolder {
  cudaGraph_t g = nullptr;
  cudaGraphExec_t x = nullptr;
  void reset() {
    if (x) cudaGraphExecDestroy(x);
    if (g) cudaGraphDestroy(g);
    x = nullptr;
    g = nullptr;
  }
  ~GraphHolder() { reset(); }
};

// Runs one phase of the batch until every item has converged, failed or hit
// the iteration cap; each launch of the graph runs at most `recompute`
// iterations per item, and items that finished are parked (their branches
// do nothing in later launches).  In the FP32 bulk phase an item whose whole
// restart chunk did not halve max|g| is parked as converged: it has reached
// what FP32 state resolves.
template <typename Tx, typename Tv>
cudaError_t run_phase(std::vector<Item *> &its, bool refine, cudaStream_t ms, cudaEvent_t fork,
                      std::vector<cudaEvent_t> &join) {
  GraphHolder gh;
  const double t0 = now_s();
  const bool direct = no_graphs();
  bool lsc = false;
  for (Item *it : its) lsc = lsc || ls_cluster_item<Tx, Tv, false>(*it);
  if (!direct) {
    cudaError_t eb = build_phase<Tx, Tv>(its, refine, ms, fork, join, &gh.g, &gh.x);
    if (eb != cudaSuccess && lsc) {
      // a graph with the cluster line search's nested IF node was refused:
      // the probes alone, for the rest of the process
      (void)cudaGetLastError();
      gh.reset();
      g_ls_cluster.store(0);
      if (trace_on()) std::fprintf(stderr, "gfmd cg: cluster line search off (%s)\n", cudaGetErrorString(eb));
      eb = build_phase<Tx, Tv>(its, refine, ms, fork, join, &gh.g, &gh.x);
    }
    RT_CHECK(eb);
  }
  const double t1 = now_s();
  int launches = 0;
  for (Item *it : its) it->it0 = it->b.hctl->it;
  for (;;) {
    launches++;
    if (direct) RT_CHECK((run_launch_direct<Tx, Tv>(its, refine, ms)));
    else RT_CHECK(cudaGraphLaunch(gh.x, ms));
    for (Item *it : its) RT_CHECK(cudaMemcpyAsync(it->b.hctl, it->b.ctl, sizeof(CgCtl), cudaMemcpyDeviceToHost, ms));
    RT_CHECK(cudaStreamSynchronize(ms));
    bool all = true;
    for (Item *it : its) {
      CgCtl &c = *it->b.hctl;
      if (c.parked) continue;
      it->evals += 1 + (c.it - it->it0);
      const bool ran = c.it != it->it0;
      it->it0 = c.it;
      if (c.done == 0) {
        if (!ran) return cudaErrorUnknown;  // an armed loop always iterates
        if (!(c.bulk && c.since >= c.recompute && !(c.fmax < 0.5 * c.fmax_restart))) {
          all = false;
          continue;
        }
        c.done = 1;  // FP32 stagnation: the bulk phase is over for this item
      }
      it->done = c.done;
      c.parked = 1;
      RT_CHECK(cudaMemcpyAsync(it->b.ctl, &c, sizeof(CgCtl), cudaMemcpyHostToDevice, ms));
    }
    if (all) {
      if (trace_on())
        std::fprintf(stderr, "gfmd cg phase <%s,%s> items %zu: graph build %.3f s, %d launches %.3f s%s\n",
                     sizeof(Tx) == 8 ? "f64" : "f32", sizeof(Tv) == 8 ? "f64" : "f32", its.size(), t1 - t0,
                     launches, now_s() - t1,
                     lsc && g_ls_cluster.load() == 1 ? ", cluster line search" : "");
      return cudaSuccess;
    }
  }
}

// Validates an item and prepares its buffers and control block.
int item_init(Item &it, gfmd_solver *hp, gfmd_solver *hr64, gfmd_solver *hpre, const gfmd_obstacle_t *ob,
              double *u, const gfmd_min_params_t *prm, cudaStream_t ms, std::string &err) {
  it.hp = hp;
  it.hpre = hpre;
  it.hr64 = hp->precision == GFMD_PREC_F32 ? hr64 : nullptr;
  it.u = u;
  it.mixed = hp->precision == GFMD_PREC_F32;
  it.o = make_obst(ob, hp->g);
  const bool map = it.o.kind == GFMD_OBST_MAP_EXP;
  cudaError_t ce = bufs_init(it.b, hp, it.mixed, map, hpre != nullptr);
  if (ce != cudaSuccess) {
    err = cudaGetErrorString(ce);
    return ce == cudaErrorMemoryAllocation ? GFMD_ENOMEM : GFMD_ECUDA;
  }
  const size_t nsite = (size_t)hp->g.nx * hp->g.ny;
  ce = cudaMemsetAsync(it.b.active, 0, nsite, ms);
  if (ce == cudaSuccess && map) {
    k_d2f<<<4 * hp->sm_count, 256, 0, ms>>>(nsite, it.o.map, it.b.mapf);
    it.o.mapf = it.b.mapf;
  }
  CgCtl c{};
  c.ftol = prm->ftol;
  c.ftol_req = prm->ftol;
  c.dmax = prm->dmax > 0.0 && std::isfinite(prm->dmax) ? prm->dmax : 0.0;
  c.bulk = it.mixed ? 1 : 0;
  c.maxit = prm->maxiter > 0 ? prm->maxiter : 100000;
  c.recompute = std::min(10000, prm->recompute > 0 ? prm->recompute : 50);
  c.obst = it.o.kind != GFMD_OBST_NONE;
  *it.b.hctl = c;
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(it.b.ctl, it.b.hctl, sizeof(CgCtl), cudaMemcpyHostToDevice, ms);
  if (ce == cudaSuccess && it.mixed) k_d2f<<<4 * hp->sm_count, 256, 0, ms>>>(it.b.n, u, it.b.u32);
  if (ce == cudaSuccess) ce = cudaGetLastError();
  if (ce != cudaSuccess) {
    err = cudaGetErrorString(ce);
    return GFMD_ECUDA;
  }
  return GFMD_OK;
}

struct StreamSet {
  cudaStream_t ms = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<cudaEvent_t> join;
  ~StreamSet() {
    for (cudaEvent_t e : join) cudaEventDestroy(e);
    if (fork) cudaEventDestroy(fork);
    if (ms) cudaStreamDestroy(ms);
  }
  cudaError_t init(size_t n) {
    cudaError_t e = cudaStreamCreateWithFlags(&ms, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
    join.assign(n, nullptr);
    for (size_t i = 0; i < n && e == cudaSuccess; i++) e = cudaEventCreateWithFlags(&join[i], cudaEventDisableTiming);
    return e;
  }
};

// Solves the items (all plain FP64, or all mixed); fills each item's report.
// Returns GFMD_OK or the first failing item's status.
int solve_batch(std::vector<Item *> &its, const gfmd_min_params_t *prm, cudaStream_t ms,
                cudaEvent_t fork, std::vector<cudaEvent_t> &join, std::string &err) {
  const bool mixed = its[0]->mixed;
  cudaError_t ce;
  if (!mixed) {
    ce = run_phase<double, double>(its, false, ms, fork, join);
  } else {
    ce = run_phase<float, float>(its, false, ms, fork, join);
    std::vector<Item *> ref;
    for (Item *it : its) {
      if (ce != cudaSuccess) break;
      k_f2d<<<4 * it->hp->sm_count, 256, 0, ms>>>(it->b.n, it->b.u32, it->u);
      if (it->done == 1 && it->hr64) {
        CgCtl &c = *it->b.hctl;
        c.done = 0;
        c.bulk = 0;
        c.parked = 0;
        ce = cudaMemcpyAsync(it->b.ctl, &c, sizeof(CgCtl), cudaMemcpyHostToDevice, ms);
        ref.push_back(it);
      }
    }
    if (ce == cudaSuccess) ce = cudaGetLastError();
    // FP64 refinement: FP64 restarts, FP32 direction forces
    if (ce == cudaSuccess && !ref.empty()) ce = run_phase<double, float>(ref, true, ms, fork, join);
  }
  // reports from fresh FP64 (or the item's own precision) evaluations
  const double tr = now_s();
  for (Item *it : its) {
    if (ce != cudaSuccess) break;
    gfmd_solver *hh = it->hr64 ? it->hr64 : it->hp;
    double *fel = reinterpret_cast<double *>(it->b.fel);
    ce = cudaMemsetAsync(&it->b.ctl->counter, 0, sizeof(unsigned int), ms);
    if (ce == cudaSuccess) ce = eval_on(hh, ms, it->u, 0, fel, 0, it->b.d_e, true);
    if (ce == cudaSuccess) {
      if (it->o.kind == GFMD_OBST_MAP_BICUBIC)
        k_report<true><<<it->b.nblk, kT, 0, ms>>>(it->o, hh->g, it->u, fel, it->b.part, it->b.ctl, it->b.d_e + 1);
      else
        k_report<<<it->b.nblk, kT, 0, ms>>>(it->o, hh->g, it->u, fel, it->b.part, it->b.ctl, it->b.d_e + 1);
      ce = cudaGetLastError();
    }
  }
  std::vector<double> sc(4 * its.size());
  for (size_t i = 0; i < its.size() && ce == cudaSuccess; i++)
    ce = cudaMemcpyAsync(&sc[4 * i], its[i]->b.d_e, 4 * sizeof(double), cudaMemcpyDeviceToHost, ms);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(ms);
  if (ce != cudaSuccess) {
    err = cudaGetErrorString(ce);
    cudaStreamSynchronize(ms);
    return GFMD_ECUDA;
  }
  if (trace_on()) std::fprintf(stderr, "gfmd cg reports: %.3f s\n", now_s() - tr);
  int first_bad = GFMD_OK;
  for (size_t i = 0; i < its.size(); i++) {
    Item *it = its[i];
    it->evals++;
    const double fm = sc[4 * i + 3];
    gfmd_min_report_t &r = it->rep;
    r.iterations = it->b.hctl->it;
    r.force_evals = it->evals;
    r.energy = sc[4 * i] + sc[4 * i + 1];
    r.fmax = fm;
    r.fnorm = std::sqrt(sc[4 * i + 2]);
    int status = it->done == 1 ? GFMD_OK : (it->done == 3 ? GFMD_ENONFINITE : GFMD_ENOTCONVERGED);
    if (status == GFMD_OK && !(fm <= prm->ftol * 1.0000001)) status = GFMD_ENOTCONVERGED;
    r.status = status;
    if (status != GFMD_OK && first_bad == GFMD_OK) {
      first_bad = status;
      err = status == GFMD_ENONFINITE ? "non-finite force during CG" : "CG did not reach max|f| <= ftol";
    }
  }
  return first_bad;
}

}  // namespace

int cg_minimize(gfmd_solver *hp, const gfmd_obstacle_t *ob, const gfmd_min_params_t *prm, double *u,
                gfmd_min_report_t *rep, std::string &err) {
  StreamSet ss;
  cudaError_t ce = ss.init(1);
  Item it;
  // order the solve after the caller's stream
  if (ce == cudaSuccess) ce = cudaEventRecord(ss.fork, hp->stream);
  if (ce == cudaSuccess) ce = cudaStreamWaitEvent(ss.ms, ss.fork, 0);
  if (ce != cudaSuccess) {
    err = cudaGetErrorString(ce);
    return GFMD_ECUDA;
  }
  int rc = item_init(it, hp, prm->refine, prm->precond, ob, u, prm, ss.ms, err);
  if (rc != GFMD_OK) return rc;
  std::vector<Item *> its{&it};
  rc = solve_batch(its, prm, ss.ms, ss.fork, ss.join, err);
  if (cudaEventRecord(ss.fork, ss.ms) == cudaSuccess) cudaStreamWaitEvent(hp->stream, ss.fork, 0);
  if (rep) {
    const double secs = rep->seconds;
    *rep = it.rep;
    rep->seconds = secs;
  }
  return rc;
}

}  // namespace gfmd

extern "C" int gfmd_minimize_batch(int n, gfmd_batch_item_t *items, const gfmd_min_params_t *prm) {
  using namespace gfmd;
  if (n < 1 || !items || !prm) return set_error(GFMD_EINVAL, "gfmd_minimize_batch: bad arguments");
  if (prm->method != GFMD_MIN_CG) return set_error(GFMD_EINVAL, "gfmd_minimize_batch: only CG is batched");
  const int prec0 = items[0].handle ? items[0].handle->precision : -1;
  const bool ref0 = items[0].refine != nullptr;
  for (int i = 0; i < n; i++) {
    gfmd_batch_item_t &b = items[i];
    if (!b.handle || !b.d_u) return set_error(GFMD_EINVAL, "gfmd_minimize_batch: NULL handle or d_u");
    for (int j = 0; j < i; j++)  // each handle owns its scratch: one item per handle
      if (items[j].handle == b.handle || (b.refine && items[j].refine == b.refine) ||
          items[j].handle == b.refine || (items[j].refine && items[j].refine == b.handle))
        return set_error(GFMD_EINVAL, "gfmd_minimize_batch: a handle appears in two items");
    if (!b.handle->have_phi) return set_error(GFMD_ENOPHI, "gfmd_minimize_batch: no stiffness table uploaded");
    if (b.handle->precision != prec0 || (b.refine != nullptr) != ref0)
      return set_error(GFMD_EINVAL, "gfmd_minimize_batch: items must share precision and refinement");
    if (b.refine) {
      const Geom &a = b.handle->g, &c = b.refine->g;
      if (a.nx != c.nx || a.ny != c.ny || a.ndof != c.ndof || !b.refine->have_phi ||
          b.refine->precision != GFMD_PREC_F64)
        return set_error(GFMD_EINVAL, "gfmd_minimize_batch: refine handle does not match");
    }
    if (b.precond) {
      const Geom &a = b.handle->g, &c = b.precond->g;
      if (a.nx != c.nx || a.ny != c.ny || a.ndof != c.ndof || !b.precond->have_phi ||
          b.precond->precision != b.handle->precision)
        return set_error(GFMD_EINVAL, "gfmd_minimize_batch: preconditioner does not match");
      for (int j = 0; j < n; j++)
        if (j != i && (items[j].precond == b.precond || items[j].handle == b.precond || items[j].refine == b.precond))
          return set_error(GFMD_EINVAL, "gfmd_minimize_batch: a handle appears in two items");
    }
    if ((b.precond != nullptr) != (items[0].precond != nullptr))
      return set_error(GFMD_EINVAL, "gfmd_minimize_batch: items must share preconditioning");
    const gfmd_obstacle_t *ob = b.obstacle;
    if (ob && (ob->kind < GFMD_OBST_NONE || ob->kind > GFMD_OBST_MAP_BICUBIC))
      return set_error(GFMD_EINVAL, "gfmd_minimize_batch: unknown obstacle kind");
    if (ob && (ob->kind == GFMD_OBST_MAP_EXP || ob->kind == GFMD_OBST_MAP_BICUBIC) && !ob->d_map)
      return set_error(GFMD_EINVAL, "gfmd_minimize_batch: map obstacle without a map");
  }
  const auto t0 = std::chrono::steady_clock::now();
  StreamSet ss;
  cudaError_t ce = ss.init((size_t)n);
  if (ce != cudaSuccess) return set_error(GFMD_ECUDA, std::string("gfmd_minimize_batch: ") + cudaGetErrorString(ce));
  for (int i = 0; i < n && ce == cudaSuccess; i++) {
    ce = cudaEventRecord(ss.join[i], items[i].handle->stream);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(ss.ms, ss.join[i], 0);
  }
  if (ce != cudaSuccess) return set_error(GFMD_ECUDA, std::string("gfmd_minimize_batch: ") + cudaGetErrorString(ce));
  std::vector<Item> store((size_t)n);
  std::vector<Item *> its;
  std::string err;
  const double ti = now_s();
  for (int i = 0; i < n; i++) {
    int rc = item_init(store[i], items[i].handle, items[i].refine, items[i].precond, items[i].obstacle,
                       items[i].d_u, prm, ss.ms, err);
    if (rc != GFMD_OK) return set_error(rc, "gfmd_minimize_batch: " + err);
    its.push_back(&store[i]);
  }
  if (trace_on()) std::fprintf(stderr, "gfmd cg setup of %d items: %.3f s\n", n, now_s() - ti);
  const int rc = solve_batch(its, prm, ss.ms, ss.fork, ss.join, err);
  const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (int i = 0; i < n; i++) {
    items[i].report = store[i].rep;
    items[i].report.seconds = secs;
  }
  if (cudaEventRecord(ss.fork, ss.ms) == cudaSuccess)
    for (int i = 0; i < n; i++) cudaStreamWaitEvent(items[i].handle->stream, ss.fork, 0);
  if (rc != GFMD_OK) return set_error(rc, "gfmd_minimize_batch: " + err);
  return GFMD_OK;
}
