// Solver loops around the force evaluation, resident on the GPU:
//   static  - FIRE (FixFIRE, src/cuda/fix_fire.cpp:117-297) and the trust
//             region (MinTRGFMD, src/extras/min_tr_gfmd.cpp:95-241), each a
//             CUDA graph per phase with its scalar logic on the device;
//             conjugate gradients live in gfmd_cg.cu;
//   dynamic - damped velocity Verlet lives in gfmd_dynamics.cu.
// Obstacles (gfmd_obstacle.cuh) act on every atom of the grid.
//
// State vectors here are FP64 [ndof][nx*ny]; the elastic forces come from the
// handle's force evaluation (FP64 or FP32 arithmetic).  Scalars (dot
// products, maxima, energies) are reduced in FP64 in a fixed order: per-block
// partials, then one block, so runs are bit-reproducible.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <string>
#include <vector>

#include "gfmd_internal.h"
#include "gfmd_obstacle.cuh"
#include "gfmd_reduce.cuh"

namespace gfmd {

namespace {

constexpr int kRedThreads = 256;
constexpr int kMaxRed = 8;  // scalars per reduction

// Per-thread accumulators -> block partials part[blockIdx.x * kMaxRed + k]
// (sums for k < nsum, maximum at k = nsum).
__device__ __forceinline__ void block_reduce(double *acc, int nsum, bool with_max, double *part) {
  __shared__ double sh[kRedThreads / 32][kMaxRed];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nq = nsum + (with_max ? 1 : 0);
  for (int k = 0; k < nq; k++) {
    double v = acc[k];
    for (int o = 16; o > 0; o >>= 1) {
      double t = __shfl_down_sync(0xffffffffu, v, o);
      v = (with_max && k == nsum) ? fmax(v, t) : v + t;
    }
    if (lane == 0) sh[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < nq) {
    const int k = threadIdx.x;
    double v = sh[0][k];
    for (int w = 1; w < (int)(blockDim.x >> 5); w++)
      v = (with_max && k == nsum) ? fmax(v, sh[w][k]) : v + sh[w][k];
    part[blockIdx.x * kMaxRed + k] = v;
  }
}

// Fixed-order combination of nblk partials into out[0..nq): thread t takes
// partials t, t+256, ... in order, then a fixed shuffle tree.
__global__ void __launch_bounds__(kRedThreads) k_finish(const double *__restrict__ part, int nblk, int nsum,
                                                        int with_max, double *__restrict__ out) {
  __shared__ double sh[kRedThreads / 32][kMaxRed];
  const int nq = nsum + with_max;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int k = 0; k < nq; k++) {
    const bool mx = with_max && k == nsum;
    double v = 0.0;
    for (int b = threadIdx.x; b < nblk; b += kRedThreads) {
      const double t = part[b * kMaxRed + k];
      v = mx ? fmax(v, t) : v + t;
    }
    for (int o = 16; o > 0; o >>= 1) {
      const double t = __shfl_down_sync(0xffffffffu, v, o);
      v = mx ? fmax(v, t) : v + t;
    }
    if (lane == 0) sh[warp][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < nq) {
    const int k = threadIdx.x;
    const bool mx = with_max && k == nsum;
    double v = sh[0][k];
    for (int w = 1; w < kRedThreads / 32; w++) v = mx ? fmax(v, sh[w][k]) : v + sh[w][k];
    out[k] = v;
  }
}

__device__ __forceinline__ void site_pos(const Obst &o, const Geom &g, size_t s, int l,
                                         const double *x, size_t N, double a, const double *h,
                                         double r[3], double dir[3]) {
  const int ix = (int)(s / g.ny), iy = (int)(s % g.ny);
  for (int c = 0; c < 3; c++) {
    const size_t idx = (size_t)(3 * l + c) * N + s;
    const double hv = h ? h[idx] : 0.0;
    dir[c] = hv;
    r[c] = x[idx] + a * hv + o.off[l][c];
  }
  r[0] += ix * o.ax;
  r[1] += iy * o.ay;
}

// f_total = f_el + F_w(u); optionally stores it; sums: E_w, |f|^2, and the
// maximum per-atom force component; fw (if not NULL) gets F_w.
__global__ void __launch_bounds__(kRedThreads) k_total_force(Obst o, Geom g, const double *__restrict__ x,
                                                             const double *__restrict__ fel,
                                                             double *__restrict__ ftot,
                                                             double *__restrict__ part,
                                                             unsigned char *__restrict__ active) {
  const size_t N = (size_t)g.nx * g.ny;
  const int nl = g.ndof / 3;
  double acc[3] = {0.0, 0.0, 0.0};
  for (size_t s = blockIdx.x * (size_t)blockDim.x + threadIdx.x; s < N; s += (size_t)gridDim.x * blockDim.x) {
    bool near = false;
    for (int l = 0; l < nl; l++) {
      double fw[3] = {0.0, 0.0, 0.0};
      if (l < o.nlayer && o.kind != GFMD_OBST_NONE) {
        double r[3], dir[3];
        site_pos(o, g, s, l, x, N, 0.0, nullptr, r, dir);
        const float ge = gap_estimate(o, s, r);
        if (ge < (float)(o.gcut + o.margin)) near = true;
        WallOut w{0.0, {0.0, 0.0, 0.0}, 0.0};
        if (ge < (float)o.gcut + 0.01f * (float)o.gcut + 1e-3f)
          w = wall_eval(o, (int)(s / g.ny), (int)(s % g.ny), s, r, dir);
        fw[0] = w.f[0];
        fw[1] = w.f[1];
        fw[2] = w.f[2];
        acc[0] += w.e;
      }
      if (l < o.nlayer && o.fz_ext != 0.0) {
        fw[2] += o.fz_ext;  // load control: constant external force
        acc[0] -= o.fz_ext * x[(size_t)(3 * l + 2) * N + s];
      }
      for (int c = 0; c < 3; c++) {
        const size_t idx = (size_t)(3 * l + c) * N + s;
        const double f = fel[idx] + fw[c];
        if (ftot) ftot[idx] = f;
        acc[1] += f * f;
        acc[2] = fmax(acc[2], fabs(f));
      }
    }
    if (active) active[s] = near ? 1 : 0;
  }
  block_reduce(acc, 2, true, part);
}




// ---------------------------------------------------------------------------
// Host-side driver state.

struct Work {
  gfmd_solver *h;
  cudaStream_t st;
  int nblk;
  double *part = nullptr;  // nblk * kMaxRed
  double *res = nullptr;   // kMaxRed (device)
  double *hres = nullptr;  // pinned host copy
  double *d_e = nullptr;   // energy of a force evaluation
  unsigned char *active = nullptr;  // per site: near the obstacle (line search)
  double *bufs[6] = {};
  size_t n = 0;
  ~Work() {
    if (part) cudaFree(part);
    if (res) cudaFree(res);
    if (hres) cudaFreeHost(hres);
    if (d_e) cudaFree(d_e);
    if (active) cudaFree(active);
    for (double *b : bufs)
      if (b) cudaFree(b);
  }
};

cudaError_t work_init(Work &w, gfmd_solver *h, int nbuf, cudaStream_t st = nullptr, bool use_st = false) {
  w.h = h;
  w.st = use_st ? st : h->stream;
  w.n = (size_t)h->g.ndof * h->g.nx * h->g.ny;
  w.nblk = std::max(1, std::min(h->sm_count * 4, (int)((w.n / 3 + kRedThreads - 1) / kRedThreads)));
  cudaError_t e = cudaMalloc((void **)&w.part, sizeof(double) * w.nblk * kMaxRed);
  if (e == cudaSuccess) e = cudaMalloc((void **)&w.res, sizeof(double) * kMaxRed);
  if (e == cudaSuccess) e = cudaMallocHost((void **)&w.hres, sizeof(double) * kMaxRed);
  if (e == cudaSuccess) e = cudaMalloc((void **)&w.d_e, sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void **)&w.active, (size_t)h->g.nx * h->g.ny);
  for (int i = 0; i < nbuf && e == cudaSuccess; i++) e = cudaMalloc((void **)&w.bufs[i], sizeof(double) * w.n);
  return e;
}

// Reduce the partials and copy nq scalars to w.hres (synchronizes).
cudaError_t fetch(Work &w, int nsum, bool with_max) {
  k_finish<<<1, kRedThreads, 0, w.st>>>(w.part, w.nblk, nsum, with_max ? 1 : 0, w.res);
  cudaError_t e = cudaMemcpyAsync(w.hres, w.res, sizeof(double) * (nsum + (with_max ? 1 : 0)),
                                  cudaMemcpyDeviceToHost, w.st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(w.st);
  return e;
}

// Elastic force of u (f64 in/out) with the handle; returns E_el (synchronizes).
cudaError_t elastic(Work &w, gfmd_solver *hh, const double *u, double *f, bool with_linf, double *eel) {
  cudaStream_t keep = hh->stream;
  hh->stream = w.st;
  cudaError_t e = enqueue_force_opts(hh, u, 0, f, 0, w.d_e, with_linf);
  hh->stream = keep;
  if (e != cudaSuccess) return e;
  if (eel) {
    e = cudaMemcpyAsync(w.hres + kMaxRed - 1, w.d_e, sizeof(double), cudaMemcpyDeviceToHost, w.st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(w.st);
    *eel = w.hres[kMaxRed - 1];
  }
  return e;
}

#define RT(call)                              \
  do {                                        \
    cudaError_t e_ = (call);                  \
    if (e_ != cudaSuccess) return e_;         \
  } while (0)

// Total force f = F_el(u) + F_w(u) into ftot, with E and max|f|, |f|^2.
cudaError_t total_force(Work &w, gfmd_solver *hh, const Obst &o, const double *u, double *fel,
                        double *ftot, double *E, double *fmax, double *f2) {
  double eel = 0.0;
  RT(elastic(w, hh, u, fel, true, &eel));
  k_total_force<<<w.nblk, kRedThreads, 0, w.st>>>(o, hh->g, u, fel, ftot, w.part, w.active);
  RT(fetch(w, 2, true));
  if (E) *E = eel + w.hres[0];
  if (f2) *f2 = w.hres[1];
  if (fmax) *fmax = w.hres[2];
  return cudaSuccess;
}

// ---- static: FIRE -----------------------------------------------------------
// FixFIRE (src/cuda/fix_fire.cpp:117-297) with its scalar logic on the
// device: one CUDA graph per phase, a prologue (v = 0 on the first phase,
// the total force) and a WHILE loop whose body is
//   k_fire_first   v += dt/2 f (|v| per atom limited), u += dt v
//   F_el(u)        the handle's force evaluation
//   k_fire_total   f = F_el + F_w, E_w, |f|^2, max|f_i| (last block)
//   k_fire_second  v += dt/2 f (limited), v.f, v.v, f.f; the last block takes
//                  FIRE's decision (P = v.f < 0: stop, dt *= decfac, mixing
//                  reset; else mix v with f, and after minsteps positive steps
//                  dt = min(incfac dt, dtmax), mixing *= mixdec), counts the
//                  iteration and sets the loop condition
//   k_fire_mix     v = 0, or v = (1 - mix) v + mix |v|/|f| f
// No scalar returns to the host until the phase ends.  With a refine
// handle, the FP32 phase also ends when max|f| has not halved for 500 steps
// (FP32 forces stall at their noise level), and the FP64 phase continues
// with the same velocities, step and mixing.
namespace fire {

using red::reduce_last;
constexpr int kT = red::kT;

struct Ctl {
  double dt, mix, amix, help;  // step, mixing; mixing and |v|/|f| factor of this step
  double fmax, f2, ew, best;   // max|f_i|, |f|^2, wall energy, last halving of max|f|
  int cut, it, best_it;
  int done;    // 0 running, 1 converged, 2 iteration cap, 3 non-finite, 4 stalled
  int zero_v;  // this step's decision: stop (v = 0)
  int evals;
  unsigned int counter;
};

struct Par {
  int minsteps, maxit, stall_check;
  double incfac, decfac, mix_in, mixdec, max_dt, xlimit, ftol;
};

__device__ __forceinline__ double vlimsq(const Par &p, double dt) {
  return p.xlimit > 0.0 ? (p.xlimit / dt) * (p.xlimit / dt) : 0.0;
}

__global__ void __launch_bounds__(kT) k_fire_first(Geom g, double *__restrict__ x, double *__restrict__ v,
                                                    const double *__restrict__ f, Par p, const Ctl *ctl) {
  const double dt = ctl->dt, dtf = 0.5 * dt, vl = vlimsq(p, dt);
  const size_t N = (size_t)g.nx * g.ny;
  const int nl = g.ndof / 3;
  for (size_t s = blockIdx.x * (size_t)kT + threadIdx.x; s < N; s += (size_t)gridDim.x * kT)
    for (int l = 0; l < nl; l++) {
      double vv[3], vsq = 0.0;
      for (int c = 0; c < 3; c++) {
        const size_t idx = (size_t)(3 * l + c) * N + s;
        vv[c] = v[idx] + dtf * f[idx];
        vsq += vv[c] * vv[c];
      }
      const double sc = (vl > 0.0 && vsq > vl) ? sqrt(vl / vsq) : 1.0;
      for (int c = 0; c < 3; c++) {
        const size_t idx = (size_t)(3 * l + c) * N + s;
        v[idx] = vv[c] * sc;
        x[idx] += dt * v[idx];
      }
    }
}

// f = F_el + F_w (+ external load); with `check` (the prologue) the last
// block also tests convergence and arms the loop.
__global__ void __launch_bounds__(kT) k_fire_total(Obst o, Geom g, const double *__restrict__ x,
                                                    const double *__restrict__ fel, double *__restrict__ ftot,
                                                    double *__restrict__ part, Ctl *ctl, Par p, int check,
                                                    cudaGraphConditionalHandle hc) {
  const size_t N = (size_t)g.nx * g.ny;
  const int nl = g.ndof / 3;
  double ew = 0.0, f2 = 0.0, fm = 0.0;
  for (size_t s = blockIdx.x * (size_t)kT + threadIdx.x; s < N; s += (size_t)gridDim.x * kT) {
    for (int l = 0; l < nl; l++) {
      double fw[3] = {0.0, 0.0, 0.0};
      if (l < o.nlayer && o.kind != GFMD_OBST_NONE) {
        double r[3], dir[3];
        site_pos(o, g, s, l, x, N, 0.0, nullptr, r, dir);
        const float ge = gap_estimate(o, s, r);
        if (ge < (float)o.gcut + 0.01f * (float)o.gcut + 1e-3f) {
          const WallOut w = wall_eval(o, (int)(s / g.ny), (int)(s % g.ny), s, r, dir);
          fw[0] = w.f[0];
          fw[1] = w.f[1];
          fw[2] = w.f[2];
          ew += w.e;
        }
      }
      if (l < o.nlayer && o.fz_ext != 0.0) {
        fw[2] += o.fz_ext;
        ew -= o.fz_ext * x[(size_t)(3 * l + 2) * N + s];
      }
      for (int c = 0; c < 3; c++) {
        const size_t idx = (size_t)(3 * l + c) * N + s;
        const double f = fel[idx] + fw[c];
        ftot[idx] = f;
        f2 += f * f;
        fm = fmax(fm, fabs(f));
      }
    }
  }
  const double acc[3] = {ew, f2, fm};
  __shared__ double res[3];
  if (!reduce_last<2, 1>(acc, part, &ctl->counter, res)) return;
  if (threadIdx.x == 0) {
    ctl->ew = res[0];
    ctl->f2 = res[1];
    ctl->fmax = res[2];
    ctl->evals += 1;
    if (check) {
      ctl->best = res[2];
      ctl->best_it = ctl->it;
      if (!isfinite(res[2])) ctl->done = 3;
      else if (res[2] <= p.ftol) ctl->done = 1;
      else if (ctl->it >= p.maxit) ctl->done = 2;
      else ctl->done = 0;
      cudaGraphSetConditional(hc, ctl->done == 0 ? 1u : 0u);
    }
  }
}

__global__ void __launch_bounds__(kT) k_fire_second(Geom g, double *__restrict__ v, const double *__restrict__ f,
                                                     double *__restrict__ part, Ctl *ctl, Par p,
                                                     cudaGraphConditionalHandle hc) {
  const double dt = ctl->dt, dtf = 0.5 * dt, vl = vlimsq(p, dt);
  const size_t N = (size_t)g.nx * g.ny;
  const int nl = g.ndof / 3;
  double vf = 0.0, vv2 = 0.0, ff = 0.0;
  for (size_t s = blockIdx.x * (size_t)kT + threadIdx.x; s < N; s += (size_t)gridDim.x * kT)
    for (int l = 0; l < nl; l++) {
      double vv[3], vsq = 0.0;
      for (int c = 0; c < 3; c++) {
        const size_t idx = (size_t)(3 * l + c) * N + s;
        vv[c] = v[idx] + dtf * f[idx];
        vsq += vv[c] * vv[c];
      }
      const double sc = (vl > 0.0 && vsq > vl) ? sqrt(vl / vsq) : 1.0;
      for (int c = 0; c < 3; c++) {
        const size_t idx = (size_t)(3 * l + c) * N + s;
        const double vn = vv[c] * sc;
        v[idx] = vn;
        vf += vn * f[idx];
        vv2 += vn * vn;
        ff += f[idx] * f[idx];
      }
    }
  const double acc[3] = {vf, vv2, ff};
  __shared__ double res[3];
  if (!reduce_last<3, 0>(acc, part, &ctl->counter, res)) return;
  if (threadIdx.x == 0) {
    const double P = res[0], vvs = res[1], ffs = res[2];
    ctl->help = ffs > 0.0 ? ctl->mix * sqrt(vvs / ffs) : 0.0;
    ctl->amix = ctl->mix;
    if (P < 0.0) {
      ctl->zero_v = 1;
      ctl->cut = p.minsteps;
      ctl->dt *= p.decfac;
      ctl->mix = p.mix_in;
    } else {
      ctl->zero_v = 0;
      if (ctl->cut < 0) {
        ctl->dt = fmin(ctl->dt * p.incfac, p.max_dt);
        ctl->mix *= p.mixdec;
      } else {
        ctl->cut -= 1;
      }
    }
    ctl->it += 1;
    const double fm = ctl->fmax;
    if (fm < 0.5 * ctl->best) {
      ctl->best = fm;
      ctl->best_it = ctl->it;
    }
    if (!isfinite(fm)) ctl->done = 3;
    else if (fm <= p.ftol) ctl->done = 1;
    else if (p.stall_check && ctl->it - ctl->best_it >= 500) ctl->done = 4;
    else if (ctl->it >= p.maxit) ctl->done = 2;
    cudaGraphSetConditional(hc, ctl->done == 0 ? 1u : 0u);
  }
}

__global__ void __launch_bounds__(kT) k_fire_mix(size_t n, double *__restrict__ v, const double *__restrict__ f,
                                                  const Ctl *ctl) {
  const bool stop = ctl->zero_v != 0;
  const double a = 1.0 - ctl->amix, b = ctl->help;
  for (size_t i = blockIdx.x * (size_t)kT + threadIdx.x; i < n; i += (size_t)gridDim.x * kT)
    v[i] = stop ? 0.0 : a * v[i] + b * f[i];
}

}  // namespace fire

// One FIRE phase on handle hh as a graph: prologue (total force, convergence
// test) and WHILE(running) { FIRE step }.  Synchronizes its stream.
cudaError_t fire_phase(gfmd_solver *hh, cudaStream_t st, const Obst &o, const fire::Par &p, double *u, double *v,
                       double *fel, double *f, double *part, double *d_e, fire::Ctl *ctl, int nblk) {
  using namespace fire;
  const Geom &g = hh->g;
  const size_t n = (size_t)g.ndof * g.nx * g.ny;
  cudaGraph_t graph = nullptr, body = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphConditionalHandle hc;
  cudaError_t e = cudaGraphCreate(&graph, 0);
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hc, graph, 0, cudaGraphCondAssignDefault);
  auto eval = [&](cudaStream_t cs) {
    cudaStream_t keep = hh->stream;
    hh->stream = cs;
    cudaError_t ee = enqueue_force_opts(hh, u, 0, fel, 0, d_e, true);
    hh->stream = keep;
    return ee;
  };
  if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(st, graph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    cudaError_t ec = eval(st);
    if (ec == cudaSuccess) {
      k_fire_total<<<nblk, kT, 0, st>>>(o, g, u, fel, f, part, ctl, p, 1, hc);
      ec = cudaGetLastError();
    }
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    if (ec == cudaSuccess) ec = cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd);
    cudaGraphNodeParams cp = {};
    cudaGraphNode_t node = nullptr;
    if (ec == cudaSuccess) {
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = hc;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      ec = cudaGraphAddNode(&node, graph, deps, nullptr, nd, &cp);
    }
    if (ec == cudaSuccess) {
      body = cp.conditional.phGraph_out[0];
      ec = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    }
    cudaGraph_t got = nullptr;
    e = cudaStreamEndCapture(st, &got);
    if (ec != cudaSuccess) e = ec;
  }
  if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    k_fire_first<<<nblk, kT, 0, st>>>(g, u, v, f, p, ctl);
    cudaError_t ec = eval(st);
    if (ec == cudaSuccess) {
      k_fire_total<<<nblk, kT, 0, st>>>(o, g, u, fel, f, part, ctl, p, 0, hc);
      k_fire_second<<<nblk, kT, 0, st>>>(g, v, f, part, ctl, p, hc);
      k_fire_mix<<<nblk * 4, kT, 0, st>>>(n, v, f, ctl);
      ec = cudaGetLastError();
    }
    cudaGraph_t got = nullptr;
    e = cudaStreamEndCapture(st, &got);
    if (ec != cudaSuccess) e = ec;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  return e;
}

int fire_solve(gfmd_solver *hp, const gfmd_obstacle_t *ob, const gfmd_min_params_t *prm,
               double *u, gfmd_min_report_t *rep, std::string &err) {
  Work w;
  cudaError_t ce = work_init(w, hp, 3);  // fel, f, v
  if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return ce == cudaErrorMemoryAllocation ? GFMD_ENOMEM : GFMD_ECUDA; }
  double *fel = w.bufs[0], *f = w.bufs[1], *v = w.bufs[2];
  const Obst o = make_obst(ob, hp->g);
  // FixFIRE defaults (src/cuda/fix_fire.cpp:63-69)
  fire::Par p{};
  p.minsteps = prm->fire_minsteps > 0 ? prm->fire_minsteps : 10;
  p.incfac = prm->fire_incfac > 0 ? prm->fire_incfac : 1.2;
  p.decfac = prm->fire_decfac > 0 ? prm->fire_decfac : 0.5;
  p.mix_in = prm->fire_mix > 0 ? prm->fire_mix : 0.1;
  p.mixdec = prm->fire_mixdec > 0 ? prm->fire_mixdec : 0.99;
  p.max_dt = prm->fire_dtmax > 0 ? prm->fire_dtmax : 0.001;
  p.xlimit = prm->fire_xlimit;
  p.maxit = prm->maxiter > 0 ? prm->maxiter : 100000;
  p.ftol = prm->ftol;
  p.stall_check = prm->refine ? 1 : 0;
  fire::Ctl c{};
  c.dt = prm->fire_dt > 0 ? prm->fire_dt : p.max_dt;
  c.mix = p.mix_in;
  c.cut = p.minsteps;
  fire::Ctl *ctl = nullptr;
  double *part = nullptr;  // last-block partials
  // the phases are captured on a stream of their own (the handle's may be
  // the legacy default stream, which cannot be captured), ordered after it
  cudaStream_t gs = nullptr;
  cudaEvent_t ev = nullptr;
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&gs, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaEventRecord(ev, w.st);
  if (ce == cudaSuccess) ce = cudaStreamWaitEvent(gs, ev, 0);
  w.st = gs;
  if (ce == cudaSuccess) ce = cudaMalloc((void **)&ctl, sizeof(fire::Ctl));
  if (ce == cudaSuccess) ce = cudaMalloc((void **)&part, sizeof(double) * red::kQ * w.nblk);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(ctl, &c, sizeof(c), cudaMemcpyHostToDevice, w.st);
  if (ce == cudaSuccess) ce = cudaMemsetAsync(v, 0, sizeof(double) * w.n, w.st);
  int status = GFMD_ENOTCONVERGED;
  if (ce == cudaSuccess) ce = fire_phase(hp, w.st, o, p, u, v, fel, f, part, w.d_e, ctl, w.nblk);
  if (ce == cudaSuccess) ce = cudaMemcpy(&c, ctl, sizeof(c), cudaMemcpyDeviceToHost);
  if (ce == cudaSuccess && prm->refine && (c.done == 1 || c.done == 4)) {
    // FP64 phase: same velocities, step and mixing
    p.stall_check = 0;
    c.done = 0;
    ce = cudaMemcpyAsync(ctl, &c, sizeof(c), cudaMemcpyHostToDevice, w.st);
    if (ce == cudaSuccess) ce = fire_phase(prm->refine, w.st, o, p, u, v, fel, f, part, w.d_e, ctl, w.nblk);
    if (ce == cudaSuccess) ce = cudaMemcpy(&c, ctl, sizeof(c), cudaMemcpyDeviceToHost);
  }
  double eel = 0.0;
  if (ce == cudaSuccess) ce = cudaMemcpy(&eel, w.d_e, sizeof(double), cudaMemcpyDeviceToHost);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(gs);
  if (part) cudaFree(part);
  if (ctl) cudaFree(ctl);
  if (ev) cudaEventDestroy(ev);
  if (gs) cudaStreamDestroy(gs);
  if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return GFMD_ECUDA; }
  if (c.done == 1) status = GFMD_OK;
  else if (c.done == 3) status = GFMD_ENONFINITE;
  if (rep) {
    rep->iterations = c.it;
    rep->force_evals = c.evals;
    rep->energy = eel + c.ew;
    rep->fmax = c.fmax;
    rep->fnorm = std::sqrt(c.f2);
  }
  if (status == GFMD_ENOTCONVERGED) err = "FIRE reached the iteration cap before max|f| <= ftol";
  if (status == GFMD_ENONFINITE) err = "non-finite force during FIRE";
  return status;
}

// ---- static: trust region ---------------------------------------------------
// MinTRGFMD::iterate (src/extras/min_tr_gfmd.cpp:95-241): a step a*h along
// the preconditioned force h = P f, a = min(1, delta/sqrt(g.h)); the step is
// accepted when the energy drop is at least rho_tol of the model's
// (a - a^2/2) g.h, else undone with the radius halved to a sqrt(g.h)/2; on
// acceptance the radius becomes min(2 delta, max(delta/2,
// 2|dE| / (min(1/2, 1 - delta/(2 sqrt(g.h))) sqrt(g.h)))).  P is the
// preconditioner handle (-(Phi + shift)^{-1} as a force evaluation, so h is
// minus its output) or the identity.  Convergence is max|f_i| <= ftol as for
// the other methods (the reference's loop tests |f|_2 against LAMMPS' ftol,
// and has an energy criterion that the reference's tests switch off with
// etol = 0).
//
// The scalar logic runs on the device: one CUDA graph per phase, a prologue
// (total force, preconditioned direction, radius) and a WHILE loop whose body
// is
//   k_tr_step     u += a h
//   F_el(u)       the handle's force evaluation (with its energy)
//   k_tr_total    f = F_el + F_w, E, max|f_i|; the last block accepts or
//                 rejects the step (rho) and updates the radius
//   k_tr_undo     on a rejection: u -= a h, f = g (the old gradient)
//   P f           the preconditioner's evaluation, every step: after a
//                 rejection it recomputes the same h from the restored f
//   k_tr_dir      h = P f, g = f, g.h; the last block makes the checks that
//                 open the next step (iteration cap, descent, the FP32
//                 phase's hand-over) and sets the loop condition
// With a refine handle the FP32 phase ends when max|f| <= ftol, or when its
// energies can no longer rank a step (the model decrease below 64 FP32 ulp
// of |E|, or 32 rejections in a row); the FP64 handle then restarts.
namespace tr {

using red::reduce_last;
constexpr int kT = red::kT;

struct Ctl {
  double E, Eprev, fmax, f2, ew, gg, delta, a;
  int it, evals, rejects, accept;
  int done;  // 0 running, 1 converged, 2 iteration cap, 3 non-finite, 4 hand over, 5 no descent
  unsigned int counter;
};

struct Par {
  double dmax, rho_tol, ftol, e_noise;
  int maxit, handover;
};

// f = F_el + F_w (+ external load), E_w, |f|^2, max|f_i|; the last block sets
// E = E_el + E_w and, after a step (restart = 0), accepts or rejects it.
__global__ void __launch_bounds__(kT) k_tr_total(Obst o, Geom g, const double *__restrict__ x,
                                                  const double *__restrict__ fel, double *__restrict__ ftot,
                                                  const double *__restrict__ eel, double *__restrict__ part,
                                                  Ctl *ctl, Par p, int restart) {
  const size_t N = (size_t)g.nx * g.ny;
  const int nl = g.ndof / 3;
  double ew = 0.0, f2 = 0.0, fm = 0.0;
  for (size_t s = blockIdx.x * (size_t)kT + threadIdx.x; s < N; s += (size_t)gridDim.x * kT) {
    for (int l = 0; l < nl; l++) {
      double fw[3] = {0.0, 0.0, 0.0};
      if (l < o.nlayer && o.kind != GFMD_OBST_NONE) {
        double r[3], dir[3];
        site_pos(o, g, s, l, x, N, 0.0, nullptr, r, dir);
        const float ge = gap_estimate(o, s, r);
        if (ge < (float)o.gcut + 0.01f * (float)o.gcut + 1e-3f) {
          const WallOut w = wall_eval(o, (int)(s / g.ny), (int)(s % g.ny), s, r, dir);
          fw[0] = w.f[0];
          fw[1] = w.f[1];
          fw[2] = w.f[2];
          ew += w.e;
        }
      }
      if (l < o.nlayer && o.fz_ext != 0.0) {
        fw[2] += o.fz_ext;
        ew -= o.fz_ext * x[(size_t)(3 * l + 2) * N + s];
      }
      for (int c = 0; c < 3; c++) {
        const size_t idx = (size_t)(3 * l + c) * N + s;
        const double f = fel[idx] + fw[c];
        ftot[idx] = f;
        f2 += f * f;
        fm = fmax(fm, fabs(f));
      }
    }
  }
  const double acc[3] = {ew, f2, fm};
  __shared__ double res[3];
  if (!reduce_last<2, 1>(acc, part, &ctl->counter, res)) return;
  if (threadIdx.x == 0) {
    const double E = *eel + res[0];
    ctl->ew = res[0];
    ctl->f2 = res[1];
    ctl->fmax = res[2];
    ctl->E = E;
    ctl->evals += 1;
    ctl->accept = 1;
    if (restart) {
      ctl->Eprev = E;
      if (!isfinite(res[2]) || !isfinite(E)) ctl->done = 3;
      else if (res[2] <= p.ftol) ctl->done = 1;
      return;
    }
    ctl->it += 1;
    if (!isfinite(res[2])) {  // (a non-finite E alone fails rho and is declined)
      ctl->done = 3;
      return;
    }
    if (res[2] <= p.ftol) {  // converged at the new point
      ctl->done = 1;
      return;
    }
    const double a = ctl->a, gg = ctl->gg, sg = sqrt(gg), delta = ctl->delta;
    const double rho = (ctl->Eprev - E) / ((a - 0.5 * a * a) * gg);
    if (!(rho >= p.rho_tol)) {
      // declined: the step is undone (k_tr_undo), the old gradient kept
      ctl->delta = 0.5 * a * sg;
      ctl->E = ctl->Eprev;
      ctl->rejects += 1;
      ctl->accept = 0;
    } else {
      ctl->rejects = 0;
      const double fac = 2.0 * fabs(E - ctl->Eprev) / (fmin(0.5, 1.0 - delta / (2.0 * sg)) * sg);
      ctl->delta = fmin(2.0 * delta, fmax(0.5 * delta, fac));
      ctl->Eprev = E;
    }
  }
}

// u += a h
__global__ void __launch_bounds__(kT) k_tr_step(size_t n, double *__restrict__ u, const double *__restrict__ h,
                                                 const Ctl *ctl) {
  const double a = ctl->a;
  for (size_t i = blockIdx.x * (size_t)kT + threadIdx.x; i < n; i += (size_t)gridDim.x * kT)
    u[i] = 1.0 * u[i] + a * h[i];
}

// after a rejected step: u -= a h, f = g
__global__ void __launch_bounds__(kT) k_tr_undo(size_t n, double *__restrict__ u, double *__restrict__ f,
                                                 const double *__restrict__ g, const double *__restrict__ h,
                                                 const Ctl *ctl) {
  if (ctl->accept || ctl->done) return;  // uniform over the grid
  const double a = -ctl->a;
  for (size_t i = blockIdx.x * (size_t)kT + threadIdx.x; i < n; i += (size_t)gridDim.x * kT) {
    u[i] = 1.0 * u[i] + a * h[i];
    f[i] = g[i];
  }
}

// h = P f (-pf with a preconditioner, else f), g = f, g.h; the last block
// opens the next step or ends the phase.
__global__ void __launch_bounds__(kT) k_tr_dir(size_t n, const double *__restrict__ f,
                                                const double *__restrict__ pf, double *__restrict__ g,
                                                double *__restrict__ h, double *__restrict__ part, Ctl *ctl,
                                                Par p, int restart, cudaGraphConditionalHandle hc) {
  double gh = 0.0;
  for (size_t i = blockIdx.x * (size_t)kT + threadIdx.x; i < n; i += (size_t)gridDim.x * kT) {
    const double fv = f[i], hv = pf ? -pf[i] : fv;
    g[i] = fv;
    h[i] = hv;
    gh += fv * hv;
  }
  const double acc[1] = {gh};
  __shared__ double res[1];
  if (!reduce_last<1, 0>(acc, part, &ctl->counter, res)) return;
  if (threadIdx.x == 0) {
    const double gg = res[0];
    ctl->gg = gg;
    // preconditioner applications that the step needed (after a restart or
    // an accepted step of an unfinished phase)
    if (pf && ctl->done == 0 && ctl->accept) ctl->evals += 1;
    if (restart && ctl->done == 0) ctl->delta = fmin(p.dmax, sqrt(gg));
    if (ctl->done == 0) {
      if (ctl->it >= p.maxit) ctl->done = 2;
      else if (!(gg > 0.0)) ctl->done = 5;
      else {
        const double a = fmin(1.0, ctl->delta / sqrt(gg));
        ctl->a = a;
        if (p.handover && ((a - 0.5 * a * a) * gg <= p.e_noise * fabs(ctl->E) || ctl->rejects >= 32))
          ctl->done = 4;
      }
    }
    if (hc) cudaGraphSetConditional(hc, ctl->done == 0 ? 1u : 0u);
  }
}

}  // namespace tr

// One trust-region phase on handle hh as a graph: the prologue (restart) and
// WHILE(running) { step }.  Synchronizes its stream.
cudaError_t tr_phase(gfmd_solver *hh, gfmd_solver *pre, cudaStream_t st, const Obst &o, const tr::Par &p,
                     double *u, double *fel, double *f, double *gv, double *h, double *pf, double *part,
                     double *d_e, double *d_e_pre, tr::Ctl *ctl, int nblk) {
  using namespace tr;
  const Geom &g = hh->g;
  const size_t n = (size_t)g.ndof * g.nx * g.ny;
  cudaGraph_t graph = nullptr, body = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphConditionalHandle hc;
  cudaError_t e = cudaGraphCreate(&graph, 0);
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&hc, graph, 0, cudaGraphCondAssignDefault);
  auto eval = [&](gfmd_solver *hx, cudaStream_t cs, const double *in, double *out, double *de, bool linf) {
    cudaStream_t keep = hx->stream;
    hx->stream = cs;
    cudaError_t ee = enqueue_force_opts(hx, in, 0, out, 0, de, linf);
    hx->stream = keep;
    return ee;
  };
  // total force of u, the preconditioned direction and its checks
  auto tail = [&](cudaStream_t cs, int restart, cudaGraphConditionalHandle hset) {
    cudaError_t ee = cudaSuccess;
    if (pre) ee = eval(pre, cs, f, pf, d_e_pre, false);
    if (ee == cudaSuccess) {
      k_tr_dir<<<nblk, kT, 0, cs>>>(n, f, pre ? pf : nullptr, gv, h, part, ctl, p, restart, hset);
      ee = cudaGetLastError();
    }
    return ee;
  };
  if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(st, graph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    cudaError_t ec = eval(hh, st, u, fel, d_e, true);
    if (ec == cudaSuccess) {
      k_tr_total<<<nblk, kT, 0, st>>>(o, g, u, fel, f, d_e, part, ctl, p, 1);
      ec = cudaGetLastError();
    }
    if (ec == cudaSuccess) ec = tail(st, 1, hc);
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    if (ec == cudaSuccess) ec = cudaStreamGetCaptureInfo(st, &cs, nullptr, nullptr, &deps, nullptr, &nd);
    cudaGraphNodeParams cp = {};
    cudaGraphNode_t node = nullptr;
    if (ec == cudaSuccess) {
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = hc;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      ec = cudaGraphAddNode(&node, graph, deps, nullptr, nd, &cp);
    }
    if (ec == cudaSuccess) {
      body = cp.conditional.phGraph_out[0];
      ec = cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    }
    cudaGraph_t got = nullptr;
    e = cudaStreamEndCapture(st, &got);
    if (ec != cudaSuccess) e = ec;
  }
  if (e == cudaSuccess) e = cudaStreamBeginCaptureToGraph(st, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
  if (e == cudaSuccess) {
    k_tr_step<<<nblk * 4, kT, 0, st>>>(n, u, h, ctl);
    cudaError_t ec = cudaGetLastError();
    if (ec == cudaSuccess) ec = eval(hh, st, u, fel, d_e, true);
    if (ec == cudaSuccess) {
      k_tr_total<<<nblk, kT, 0, st>>>(o, g, u, fel, f, d_e, part, ctl, p, 0);
      k_tr_undo<<<nblk * 4, kT, 0, st>>>(n, u, f, gv, h, ctl);
      ec = cudaGetLastError();
    }
    if (ec == cudaSuccess) ec = tail(st, 0, hc);
    cudaGraph_t got = nullptr;
    e = cudaStreamEndCapture(st, &got);
    if (ec != cudaSuccess) e = ec;
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, graph, 0);
  if (e == cudaSuccess) e = cudaGraphLaunch(exec, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (exec) cudaGraphExecDestroy(exec);
  if (graph) cudaGraphDestroy(graph);
  return e;
}

int tr_solve(gfmd_solver *hp, const gfmd_obstacle_t *ob, const gfmd_min_params_t *prm,
             double *u, gfmd_min_report_t *rep, std::string &err) {
  Work w;
  cudaError_t ce = work_init(w, hp, 5);  // fel, f, g, h, Pf
  if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return ce == cudaErrorMemoryAllocation ? GFMD_ENOMEM : GFMD_ECUDA; }
  double *fel = w.bufs[0], *f = w.bufs[1], *gv = w.bufs[2], *h = w.bufs[3], *pf = w.bufs[4];
  const Obst o = make_obst(ob, hp->g);
  tr::Par p{};
  p.dmax = prm->tr_dmax > 0 ? prm->tr_dmax : 0.1;
  p.rho_tol = prm->tr_rho_tol > 0 ? prm->tr_rho_tol : 0.01;
  p.maxit = prm->maxiter > 0 ? prm->maxiter : 100000;
  p.ftol = prm->ftol;
  p.handover = prm->refine ? 1 : 0;
  p.e_noise = hp->precision == GFMD_PREC_F32 ? 64.0 * 5.960464477539063e-8 : 0.0;
  tr::Ctl c{};
  tr::Ctl *ctl = nullptr;
  double *part = nullptr, *d_e_pre = nullptr;
  // phases captured on a stream of their own, ordered after the handle's
  cudaStream_t gs = nullptr;
  cudaEvent_t ev = nullptr;
  if (ce == cudaSuccess) ce = cudaStreamCreateWithFlags(&gs, cudaStreamNonBlocking);
  if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  if (ce == cudaSuccess) ce = cudaEventRecord(ev, w.st);
  if (ce == cudaSuccess) ce = cudaStreamWaitEvent(gs, ev, 0);
  w.st = gs;
  if (ce == cudaSuccess) ce = cudaMalloc((void **)&ctl, sizeof(tr::Ctl));
  if (ce == cudaSuccess) ce = cudaMalloc((void **)&d_e_pre, sizeof(double));
  if (ce == cudaSuccess) ce = cudaMalloc((void **)&part, sizeof(double) * red::kQ * w.nblk);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(ctl, &c, sizeof(c), cudaMemcpyHostToDevice, w.st);
  if (ce == cudaSuccess)
    ce = tr_phase(hp, prm->precond, w.st, o, p, u, fel, f, gv, h, pf, part, w.d_e, d_e_pre, ctl, w.nblk);
  if (ce == cudaSuccess) ce = cudaMemcpy(&c, ctl, sizeof(c), cudaMemcpyDeviceToHost);
  gfmd_solver *hh = hp;
  if (ce == cudaSuccess && prm->refine && (c.done == 1 || c.done == 4)) {
    // FP64 phase: restart with the refine handle
    hh = prm->refine;
    p.handover = 0;
    p.e_noise = 0.0;
    c.done = 0;
    c.rejects = 0;
    ce = cudaMemcpyAsync(ctl, &c, sizeof(c), cudaMemcpyHostToDevice, w.st);
    if (ce == cudaSuccess)
      ce = tr_phase(hh, prm->precond, w.st, o, p, u, fel, f, gv, h, pf, part, w.d_e, d_e_pre, ctl, w.nblk);
    if (ce == cudaSuccess) ce = cudaMemcpy(&c, ctl, sizeof(c), cudaMemcpyDeviceToHost);
  }
  double E = 0.0, fmax = 0.0, f2 = 0.0;
  if (ce == cudaSuccess && c.done != 3 && c.done != 5)
    ce = total_force(w, hh, o, u, fel, f, &E, &fmax, &f2);  // fresh forces at the end point
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(gs);
  if (part) cudaFree(part);
  if (d_e_pre) cudaFree(d_e_pre);
  if (ctl) cudaFree(ctl);
  if (ev) cudaEventDestroy(ev);
  if (gs) cudaStreamDestroy(gs);
  if (ce != cudaSuccess) { err = cudaGetErrorString(ce); return GFMD_ECUDA; }
  int status = GFMD_ENOTCONVERGED;
  if (c.done == 1) status = GFMD_OK;
  else if (c.done == 3 || c.done == 5) status = GFMD_ENONFINITE;
  if (c.done == 3 || c.done == 5) {
    E = c.E;
    fmax = c.fmax;
    f2 = c.f2;
  }
  if (rep) {
    rep->iterations = c.it;
    rep->force_evals = c.evals;
    rep->energy = E;
    rep->fmax = fmax;
    rep->fnorm = std::sqrt(f2);
  }
  if (status == GFMD_ENOTCONVERGED) err = "trust region reached the iteration cap before max|f| <= ftol";
  if (c.done == 5) err = "the preconditioned gradient is not a descent direction";
  else if (status == GFMD_ENONFINITE) err = "non-finite force during the trust-region solve";
  return status;
}

}  // namespace

cudaError_t report_total_force(gfmd_solver *hh, cudaStream_t st, const Obst &o, const double *u,
                               double *E, double *fmax, double *f2) {
  Work w;
  RT(work_init(w, hh, 1, st, true));
  return total_force(w, hh, o, u, w.bufs[0], nullptr, E, fmax, f2);
}

}  // namespace gfmd

extern "C" {

int gfmd_minimize(gfmd_handle_t h, const gfmd_obstacle_t *obst, const gfmd_min_params_t *prm,
                  double *d_u, gfmd_min_report_t *rep) {
  if (!h || !prm || !d_u) return gfmd::set_error(GFMD_EINVAL, "gfmd_minimize: NULL argument");
  if (!h->have_phi) return gfmd::set_error(GFMD_ENOPHI, "gfmd_minimize: no stiffness table uploaded");
  if (prm->refine) {
    const gfmd::Geom &a = h->g, &b = prm->refine->g;
    if (a.nx != b.nx || a.ny != b.ny || a.ndof != b.ndof || !prm->refine->have_phi)
      return gfmd::set_error(GFMD_EINVAL, "gfmd_minimize: refine handle does not match");
  }
  if (prm->precond) {
    const gfmd::Geom &a = h->g, &b = prm->precond->g;
    if (a.nx != b.nx || a.ny != b.ny || a.ndof != b.ndof || !prm->precond->have_phi ||
        prm->precond->precision != h->precision || prm->precond == h || prm->precond == prm->refine)
      return gfmd::set_error(GFMD_EINVAL, "gfmd_minimize: preconditioner does not match");
  }
  if (obst && (obst->kind == GFMD_OBST_MAP_EXP || obst->kind == GFMD_OBST_MAP_BICUBIC) && !obst->d_map)
    return gfmd::set_error(GFMD_EINVAL, "gfmd_minimize: map obstacle without a map");
  if (obst && (obst->kind < GFMD_OBST_NONE || obst->kind > GFMD_OBST_MAP_BICUBIC))
    return gfmd::set_error(GFMD_EINVAL, "gfmd_minimize: unknown obstacle kind");
  if (obst && obst->kind == GFMD_OBST_MAP_BICUBIC && prm && prm->method != GFMD_MIN_CG)
    return gfmd::set_error(GFMD_EINVAL, "gfmd_minimize: the bicubic map wall runs with GFMD_MIN_CG");
  std::string err;
  auto t0 = std::chrono::steady_clock::now();
  int rc;
  if (prm->method == GFMD_MIN_CG) rc = gfmd::cg_minimize(h, obst, prm, d_u, rep, err);
  else if (prm->method == GFMD_MIN_FIRE) rc = gfmd::fire_solve(h, obst, prm, d_u, rep, err);
  else if (prm->method == GFMD_MIN_TR) rc = gfmd::tr_solve(h, obst, prm, d_u, rep, err);
  else return gfmd::set_error(GFMD_EINVAL, "gfmd_minimize: unknown method");
  if (rep) {
    rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    rep->status = rc;
  }
  if (rc != GFMD_OK) return gfmd::set_error(rc, "gfmd_minimize: " + err);
  return GFMD_OK;
}

}  // extern "C"
