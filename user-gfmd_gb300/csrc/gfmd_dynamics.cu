// Damped velocity Verlet (fix nve with linear damping; gamma = 0 is fix nve)
// on the GPU, all steps in one CUDA graph:
//   prologue   f_el = F_el(u); k_second (no kick): f = f_el + F_w(u) + f_ext,
//              E(0) = E_el + E_w + E_ext + |v|^2 / 2, then the first half
//              of step 1: v_h = v + dt/2 (f - gamma v); u += dt v_h
//   WHILE(step < nsteps) {
//     f_el = F_el(u)                 (the handle's force evaluation)
//     k_second   f = f_el + F_w(u) + f_ext (not stored); v = (v_h + dt/2 f) / (1 + dt gamma/2);
//                E(step) in FP64 by the last block, which also advances the
//                step and sets the loop condition; then, unless this was the
//                last step, the first half of the next one in the same pass
//   }
// The state is held in the handle's precision: FP32 handles run FP32 u, v, f
// with FP32 forces and FP64 energy reductions (kinetic energy as a
// compensated FP32 dot product); FP64 handles run FP64 throughout.  Unit
// masses.  Restates the time integration the reference's dynamics tests run
// on fix gfmd (tests/TEST_energy_conservation_*/lammps.in: fix nve).
#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <cmath>
#include <string>
#include <vector>

#include "gfmd_internal.h"
#include "gfmd_obstacle.cuh"
#include "gfmd_reduce.cuh"
#include "gfmd_vec.cuh"

namespace gfmd {

namespace {

using red::Dot;
using red::kQ;
using red::kT;
using red::reduce_last;

struct DynCtl {
  int step, nsteps;
  int status;  // 0 running/ok, 3 non-finite energy
  unsigned int counter;
};

// Obstacle force on atom (site s, layer l) into fw, energy into e.
template <typename T>
__device__ __forceinline__ bool atom_wall(const Obst &o, int ix, int iy, int l, int s, int N, const T *u,
                                          double fw[3], double &e) {
  fw[0] = fw[1] = fw[2] = 0.0;
  if (l >= o.nlayer) return false;
  bool hit = false;
  const size_t iz = (size_t)(3 * l + 2) * N + s;
  if (o.kind == GFMD_OBST_MAP_EXP && sizeof(T) == 4) {
    float ef, fz;
    map_wall_f(o, s, (float)u[iz] + o.foff[l][2], ef, fz);
    fw[2] = fz;
    e += ef;
    hit = true;
  } else if (o.kind != GFMD_OBST_NONE) {
    float r[3];
    for (int c = 0; c < 3; c++) r[c] = (float)u[(size_t)(3 * l + c) * N + s] + o.foff[l][c];
    r[0] += (float)ix * o.fax;
    r[1] += (float)iy * o.fay;
    if (gap_estimate_f(o, s, r) < o.fgate_wall) {
      double rd[3];
      const double zero[3] = {0.0, 0.0, 0.0};
      for (int c = 0; c < 3; c++) rd[c] = (double)u[(size_t)(3 * l + c) * N + s] + o.off[l][c];
      rd[0] += ix * o.ax;
      rd[1] += iy * o.ay;
      const WallOut w = wall_eval(o, ix, iy, s, rd, zero);
      fw[0] = w.f[0];
      fw[1] = w.f[1];
      fw[2] = w.f[2];
      e += w.e;
      hit = true;
    }
  }
  if (o.fz_ext != 0.0) {
    fw[2] += o.fz_ext;
    e -= o.fz_ext * (double)u[iz];
    hit = true;
  }
  return hit;
}

// f = f_el + F_w(u) + f_ext; with kick, v = (v + dt/2 f) / (1 + dt gamma/2);
// energy of the state into energies[step] (advancing step first with kick).
// Unless this was the last step, the first half of the next step follows in
// the same pass (v_h = v + dt/2 (f - gamma v), u += dt v_h), so a step costs
// one evaluation and one pass over the state: read f_el, v, u, write v, u
// (the total force itself is not stored).  V consecutive sites per thread
// (V = 4: 16-byte loads); OBST = false compiles the pass without the wall
// code.  |v|^2 and |f|^2 are summed per loop trip in T, each trip sum then
// entering the thread's Dot (FP64, or a compensated FP32 pair).
template <typename T, int V, bool OBST>
__global__ void __launch_bounds__(kT) k_second(Obst o, Geom gm, T *__restrict__ u, T *__restrict__ v,
                                                const T *__restrict__ fel, T dt, T gamma, int kick,
                                                const double *__restrict__ d_eel, double *__restrict__ energies,
                                                double *__restrict__ part, DynCtl *ctl, double *__restrict__ last,
                                                cudaGraphConditionalHandle hc, int use_hc) {
  const int N = gm.nx * gm.ny;
  const int nl = gm.ndof / 3;
  const T hdt = (T)0.5 * dt;
  const T den = (T)1 / ((T)1 + hdt * gamma);
  // read before the last block advances the step: is there a next step?
  const bool next = (ctl->step + (kick ? 1 : 0)) < ctl->nsteps;
  Dot<T> vv, ff;
  double ew = 0.0;
  float fm = 0.0f;
  for (int s0 = V * (blockIdx.x * kT + threadIdx.x); s0 < N; s0 += V * gridDim.x * kT) {
    int six[V], siy[V];
    if constexpr (OBST) {
      int ix = s0 / gm.ny, iy = s0 - ix * gm.ny;  // one division per trip
#pragma unroll
      for (int j = 0; j < V; j++) {
        six[j] = ix;
        siy[j] = iy;
        if (++iy == gm.ny) {
          iy = 0;
          ix++;
        }
      }
    }
    T svv = (T)0, sff = (T)0;
    for (int l = 0; l < nl; l++) {
      double fw[V][3];
      bool hit[V];
      if constexpr (OBST) {
#pragma unroll
        for (int j = 0; j < V; j++) hit[j] = atom_wall<T>(o, six[j], siy[j], l, s0 + j, N, u, fw[j], ew);
      }
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const size_t idx = (size_t)(3 * l + c) * N + s0;
        T fv[V], vn[V], uu[V];
        VecN<T, V>::ld(fel + idx, fv);
        VecN<T, V>::ld(v + idx, vn);
        if (next) VecN<T, V>::ld(u + idx, uu);
#pragma unroll
        for (int j = 0; j < V; j++) {
          if constexpr (OBST) {
            if (hit[j]) fv[j] = (T)((double)fv[j] + fw[j][c]);
          }
          if (kick) vn[j] = (vn[j] + hdt * fv[j]) * den;
          svv = fma(vn[j], vn[j], svv);
          sff = fma(fv[j], fv[j], sff);
          fm = fmaxf(fm, fabsf((float)fv[j]));
          if (next) {
            vn[j] = vn[j] + hdt * (fv[j] - gamma * vn[j]);
            uu[j] = uu[j] + dt * vn[j];
          }
        }
        if (next) {
          VecN<T, V>::st(v + idx, vn);
          VecN<T, V>::st(u + idx, uu);
        } else if (kick) {
          VecN<T, V>::st(v + idx, vn);
        }
      }
    }
    vv.addsum(svv);
    ff.addsum(sff);
  }
  const double acc[4] = {vv.get(), ew, ff.get(), (double)fm};
  __shared__ double res[4];
  if (!reduce_last<3, 1>(acc, part, &ctl->counter, res)) return;
  if (threadIdx.x == 0) {
    if (kick) ctl->step += 1;
    const double E = d_eel[0] + res[1] + 0.5 * res[0];
    energies[ctl->step] = E;
    last[0] = E;
    last[1] = res[2];
    last[2] = res[3];
    if (!isfinite(E)) ctl->status = 3;
    const bool go_on = ctl->status == 0 && ctl->step < ctl->nsteps;
    if (use_hc) cudaGraphSetConditional(hc, go_on ? 1u : 0u);
  }
}

// One launch of the pass in the variant that fits the grid and the buffers.
template <typename T>
cudaError_t launch_second(int nblk, cudaStream_t st, const Obst &o, const Geom &gm, T *u, T *v, const T *fel, T dt,
                          T gamma, int kick, const double *d_eel, double *en, double *part, DynCtl *ctl,
                          double *last, cudaGraphConditionalHandle hc) {
  const bool obst = o.kind != GFMD_OBST_NONE || o.fz_ext != 0.0;
  auto al16 = [](const void *p) { return ((uintptr_t)p & 15) == 0; };
  const bool v4 = ((size_t)gm.nx * gm.ny) % 4 == 0 && al16(u) && al16(v) && al16(fel);
  if (v4 && obst)
    k_second<T, 4, true><<<nblk, kT, 0, st>>>(o, gm, u, v, fel, dt, gamma, kick, d_eel, en, part, ctl, last, hc, 1);
  else if (v4)
    k_second<T, 4, false><<<nblk, kT, 0, st>>>(o, gm, u, v, fel, dt, gamma, kick, d_eel, en, part, ctl, last, hc, 1);
  else if (obst)
    k_second<T, 1, true><<<nblk, kT, 0, st>>>(o, gm, u, v, fel, dt, gamma, kick, d_eel, en, part, ctl, last, hc, 1);
  else
    k_second<T, 1, false><<<nblk, kT, 0, st>>>(o, gm, u, v, fel, dt, gamma, kick, d_eel, en, part, ctl, last, hc, 1);
  return cudaGetLastError();
}

__global__ void k_cvt_f(size_t n, const double *__restrict__ a, float *__restrict__ b) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}
__global__ void k_cvt_d(size_t n, const float *__restrict__ a, double *__restrict__ b) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}

struct DynBufs {
  cudaStream_t cs = nullptr;
  cudaEvent_t ev = nullptr;
  void *arena = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  ~DynBufs() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    if (arena) cudaFree(arena);
    if (ev) cudaEventDestroy(ev);
    if (cs) cudaStreamDestroy(cs);
  }
};

cudaError_t eval_dyn(gfmd_solver *hh, cudaStream_t st, const void *in, void *out, int t, double *d_e) {
  cudaStream_t keep = hh->stream;
  hh->stream = st;
  cudaError_t e = enqueue_force_opts(hh, in, t, out, t, d_e, true);
  hh->stream = keep;
  return e;
}

#define DT_CHECK(call)                \
  do {                                \
    cudaError_t e_ = (call);          \
    if (e_ != cudaSuccess) return e_; \
  } while (0)

template <typename T>
cudaError_t run_t(gfmd_solver *h, const Obst &o0, double dt, double gamma, int nsteps, double *d_u, double *d_v,
                  double *energies, double *last_host) {
  const Geom &gm = h->g;
  const size_t n = (size_t)gm.ndof * gm.nx * gm.ny, nsite = (size_t)gm.nx * gm.ny;
  const int nblk = (int)std::max<size_t>(1, std::min<size_t>((size_t)h->sm_count * 4, (nsite + kT - 1) / kT));
  const bool f32 = sizeof(T) == 4;
  Obst o = o0;
  DynBufs b;
  DT_CHECK(cudaStreamCreateWithFlags(&b.cs, cudaStreamNonBlocking));
  DT_CHECK(cudaEventCreateWithFlags(&b.ev, cudaEventDisableTiming));
  auto up = [](size_t x) { return (x + 255) / 256 * 256; };
  const bool map = o.kind == GFMD_OBST_MAP_EXP && f32;
  const size_t sz[8] = {up(sizeof(T) * n), 0, f32 ? up(sizeof(T) * n) : 0, f32 ? up(sizeof(T) * n) : 0,
                        up(sizeof(double) * (nsteps + 1)), up(sizeof(double) * kQ * nblk), up(sizeof(double) * 4 + sizeof(DynCtl)),
                        map ? up(sizeof(float) * nsite) : 0};
  size_t off[8], tot = 0;
  for (int k = 0; k < 8; k++) {
    off[k] = tot;
    tot += sz[k];
  }
  DT_CHECK(cudaMalloc(&b.arena, tot));
  char *a = static_cast<char *>(b.arena);
  T *fel = reinterpret_cast<T *>(a + off[0]);
  T *u = f32 ? reinterpret_cast<T *>(a + off[2]) : reinterpret_cast<T *>(d_u);
  T *v = f32 ? reinterpret_cast<T *>(a + off[3]) : reinterpret_cast<T *>(d_v);
  double *en = reinterpret_cast<double *>(a + off[4]);
  double *part = reinterpret_cast<double *>(a + off[5]);
  double *scal = reinterpret_cast<double *>(a + off[6]);  // [0] E_el of an evaluation, [1..3] last
  DynCtl *ctl = reinterpret_cast<DynCtl *>(a + off[6] + sizeof(double) * 4);
  const int eb = 4 * h->sm_count;
  // order after the caller's stream
  DT_CHECK(cudaEventRecord(b.ev, h->stream));
  DT_CHECK(cudaStreamWaitEvent(b.cs, b.ev, 0));
  if (map) {
    float *mapf = reinterpret_cast<float *>(a + off[7]);
    k_cvt_f<<<eb, 256, 0, b.cs>>>(nsite, o.map, mapf);
    o.mapf = mapf;
  }
  if (f32) {
    k_cvt_f<<<eb, 256, 0, b.cs>>>(n, d_u, reinterpret_cast<float *>(u));
    k_cvt_f<<<eb, 256, 0, b.cs>>>(n, d_v, reinterpret_cast<float *>(v));
  }
  DynCtl c{0, nsteps, 0, 0};
  DT_CHECK(cudaMemcpyAsync(ctl, &c, sizeof(DynCtl), cudaMemcpyHostToDevice, b.cs));
  const int t = f32 ? 1 : 0;
  // graph: prologue + WHILE(step < nsteps)
  DT_CHECK(cudaGraphCreate(&b.graph, 0));
  cudaGraphConditionalHandle hc;
  DT_CHECK(cudaGraphConditionalHandleCreate(&hc, b.graph, 0, cudaGraphCondAssignDefault));
  DT_CHECK(cudaStreamBeginCaptureToGraph(b.cs, b.graph, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  cudaError_t e = eval_dyn(h, b.cs, u, fel, t, scal);
  if (e == cudaSuccess)
    e = launch_second<T>(nblk, b.cs, o, gm, u, v, fel, (T)dt, (T)gamma, 0, scal, en, part, ctl, scal + 1, hc);
  cudaGraph_t body = nullptr;
  if (e == cudaSuccess) {
    cudaStreamCaptureStatus cs;
    const cudaGraphNode_t *deps = nullptr;
    size_t nd = 0;
    e = cudaStreamGetCaptureInfo(b.cs, &cs, nullptr, nullptr, &deps, nullptr, &nd);
    cudaGraphNodeParams cp = {};
    cudaGraphNode_t node = nullptr;
    if (e == cudaSuccess) {
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = hc;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      e = cudaGraphAddNode(&node, b.graph, deps, nullptr, nd, &cp);
    }
    if (e == cudaSuccess) {
      body = cp.conditional.phGraph_out[0];
      e = cudaStreamUpdateCaptureDependencies(b.cs, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
    }
  }
  cudaGraph_t got = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(b.cs, &got);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return e;
  DT_CHECK(cudaStreamBeginCaptureToGraph(b.cs, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
  e = eval_dyn(h, b.cs, u, fel, t, scal);
  if (e == cudaSuccess)
    e = launch_second<T>(nblk, b.cs, o, gm, u, v, fel, (T)dt, (T)gamma, 1, scal, en, part, ctl, scal + 1, hc);
  e2 = cudaStreamEndCapture(b.cs, &got);
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return e;
  DT_CHECK(cudaGraphInstantiate(&b.exec, b.graph, 0));
  DT_CHECK(cudaMemsetAsync(&ctl->counter, 0, sizeof(unsigned int), b.cs));
  DT_CHECK(cudaGraphLaunch(b.exec, b.cs));
  if (f32) {
    k_cvt_d<<<eb, 256, 0, b.cs>>>(n, reinterpret_cast<const float *>(u), d_u);
    k_cvt_d<<<eb, 256, 0, b.cs>>>(n, reinterpret_cast<const float *>(v), d_v);
  }
  std::vector<double> hl(3);
  DT_CHECK(cudaMemcpyAsync(hl.data(), scal + 1, 3 * sizeof(double), cudaMemcpyDeviceToHost, b.cs));
  DT_CHECK(cudaMemcpyAsync(&c, ctl, sizeof(DynCtl), cudaMemcpyDeviceToHost, b.cs));
  if (energies) DT_CHECK(cudaMemcpyAsync(energies, en, sizeof(double) * (nsteps + 1), cudaMemcpyDeviceToHost, b.cs));
  DT_CHECK(cudaStreamSynchronize(b.cs));
  DT_CHECK(cudaEventRecord(b.ev, b.cs));
  DT_CHECK(cudaStreamWaitEvent(h->stream, b.ev, 0));
  last_host[0] = hl[0];
  last_host[1] = hl[1];
  last_host[2] = hl[2];
  last_host[3] = c.status;
  last_host[4] = c.step;
  return cudaSuccess;
}

}  // namespace

}  // namespace gfmd

extern "C" int gfmd_run_dynamics(gfmd_handle_t h, const gfmd_obstacle_t *obst, double dt, double gamma,
                                 int nsteps, double *d_u, double *d_v, double *energies,
                                 gfmd_min_report_t *rep) {
  using namespace gfmd;
  if (!h || !d_u || !d_v || nsteps < 0 || !(dt > 0.0) || gamma < 0.0)
    return set_error(GFMD_EINVAL, "gfmd_run_dynamics: bad argument");
  if (!h->have_phi) return set_error(GFMD_ENOPHI, "gfmd_run_dynamics: no stiffness table uploaded");
  if (obst && (obst->kind == GFMD_OBST_MAP_EXP || obst->kind == GFMD_OBST_MAP_BICUBIC) && !obst->d_map)
    return set_error(GFMD_EINVAL, "gfmd_run_dynamics: map obstacle without a map");
  if (obst && (obst->kind < GFMD_OBST_NONE || obst->kind > GFMD_OBST_MAP_BICUBIC))
    return set_error(GFMD_EINVAL, "gfmd_run_dynamics: unknown obstacle kind");
  if (obst && obst->kind == GFMD_OBST_MAP_BICUBIC)
    return set_error(GFMD_EINVAL, "gfmd_run_dynamics: the bicubic map wall is offered by gfmd_minimize (CG) "
                                  "and gfmd_obstacle_force; use GFMD_OBST_MAP_EXP here");
  const auto t0 = std::chrono::steady_clock::now();
  const Obst o = make_obst(obst, h->g);
  double last[5] = {0, 0, 0, 0, 0};
  cudaError_t e = h->precision == GFMD_PREC_F32 ? run_t<float>(h, o, dt, gamma, nsteps, d_u, d_v, energies, last)
                                                 : run_t<double>(h, o, dt, gamma, nsteps, d_u, d_v, energies, last);
  if (e != cudaSuccess)
    return set_error(e == cudaErrorMemoryAllocation ? GFMD_ENOMEM : GFMD_ECUDA,
                     std::string("gfmd_run_dynamics: ") + cudaGetErrorString(e));
  const int status = (int)last[3] == 0 ? GFMD_OK : GFMD_ENONFINITE;
  if (rep) {
    rep->iterations = (int)last[4];
    rep->force_evals = (int)last[4] + 1;
    rep->energy = last[0];
    rep->fmax = last[2];
    rep->fnorm = std::sqrt(last[1]);
    rep->status = status;
    rep->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
  if (status != GFMD_OK) return set_error(status, "gfmd_run_dynamics: non-finite energy");
  return GFMD_OK;
}
