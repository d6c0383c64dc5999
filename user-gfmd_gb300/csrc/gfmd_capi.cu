// C ABI of gfmd_gb300 (declared in include/gfmd_gb300.h): solver handles,
// FFT plans and twiddle tables, stiffness-table packing and upload, and the
// host-side stiffness-kernel tables.
#include <cuda_runtime.h>

#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <algorithm>
#include <atomic>
#include <tuple>
#include <mutex>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include "gfmd_internal.h"
#include "stiffness.h"

struct gfmd_kernel {
  std::unique_ptr<gfmd::StiffnessKernel> k;
};

namespace {

thread_local std::string g_err;

int fail(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(e == cudaErrorMemoryAllocation ? GFMD_ENOMEM : GFMD_ECUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call, what)                        \
  do {                                        \
    cudaError_t e_ = (call);                  \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

constexpr double kPi = 3.14159265358979323846264338327950288;

void release(gfmd_solver *h) {
  if (!h) return;
  void *ptrs[] = {h->d_zero,  h->d_tw_hi, h->d_tw_lo,  h->d_W,     h->d_phi,     h->d_linf,
                  h->d_epart, h->d_scal,   h->d_io,    h->d_ftw,
                  h->d_counter, h->d_tw32, h->d_err, h->d_twc};
  for (void *p : ptrs)
    if (p) cudaFree(p);
  if (h->ws) cudaFree(h->ws);
  if (h->ws_host) cudaFreeHost(h->ws_host);
  release(h->prec_grad);
  delete h;
}

// Runs fn(i0, i1) over [0, n) on all host cores.
template <typename F> void parallel_for(long n, F fn) {
  int nt = (int)std::max(1u, std::thread::hardware_concurrency());
  if (n < 4096) nt = 1;
  std::vector<std::thread> th;
  long chunk = (n + nt - 1) / nt;
  for (int t = 0; t < nt; t++) {
    long a = t * chunk, b = std::min(n, a + chunk);
    if (a >= b) break;
    if (t == nt - 1 || nt == 1) fn(a, b);
    else th.emplace_back(fn, a, b);
  }
  for (auto &t : th) t.join();
}

bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// Position of frequency k after the in-place DIF stages of plan p.
int p2_digit_rev(const gfmd::P2Plan &p, int k) {
  int pos = 0, lgS = p.lgn;
  for (int s = 0; s < p.nst; s++) {
    lgS -= p.lg[s];
    pos += (k & ((1 << p.lg[s]) - 1)) << lgS;
    k >>= p.lg[s];
  }
  return pos;
}

gfmd::P2Plan make_p2(int n) {
  gfmd::P2Plan p{};
  p.n = n;
  while ((1 << p.lgn) < n) p.lgn++;
  int m = n;
  while (m % 16 == 0) { p.radix[p.nst] = 16; p.lg[p.nst++] = 4; m /= 16; }
  if (m > 1) {
    p.radix[p.nst] = m;
    p.lg[p.nst++] = m == 8 ? 3 : (m == 4 ? 2 : 1);
  }
  return p;
}

// Appends the per-stage twiddle tables of plan p (entry [m][j] =
// exp(-2 pi i j m / L_s), so consecutive j sit in consecutive entries) as (c, s) doubles to d and (c_hi, s_hi, c_lo, s_lo)
// floats to f, setting p.toff relative to the start of this plan's table.
void push_stage_tables(gfmd::P2Plan &p, std::vector<double> &d, std::vector<float> &f) {
  auto push = [&](double c, double sn) {
    d.push_back(c);
    d.push_back(sn);
    float ch = (float)c, sh = (float)sn;
    f.push_back(ch);
    f.push_back(sh);
    f.push_back((float)(c - (double)ch));
    f.push_back((float)(sn - (double)sh));
  };
  const size_t base = d.size() / 2;
  int L = p.n;
  for (int s = 0; s < p.nst; s++) {
    const int R = p.radix[s], S = L / R;
    p.toff[s] = (int)(d.size() / 2 - base);
    for (int m = 0; m < R; m++)
      for (int j = 0; j < S; j++) {
        long e = ((long)j * m) % L;
        double a = -2.0 * kPi * (double)e / (double)L;
        push(std::cos(a), std::sin(a));
      }
    L = S;
  }
  p.tsize = (int)(d.size() / 2 - base);
}

// Compensated FP32 table entry (c_hi, s_hi, c_lo, s_lo) of exp(-2 pi i e / L).
void push_c4(std::vector<float> &f, long e, long L) {
  const double a = -2.0 * kPi * (double)(e % L) / (double)L;
  const double c = std::cos(a), sn = std::sin(a);
  const float ch = (float)c, sh = (float)sn;
  f.push_back(ch);
  f.push_back(sh);
  f.push_back((float)(c - (double)ch));
  f.push_back((float)(sn - (double)sh));
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no
// link-time dependency on the driver library).
using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiled encode_tiled() {
  static EncodeTiled fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiled>(p);
  });
  return fn;
}

// Column-kernel cluster size for D columns of length nx: the fewest blocks
// per ky whose share of the columns fits in 100 KB of shared memory (two
// blocks per SM); 0 if the cluster kernel has no instance for D.
int pick_col_cluster(int D, int nx) {
  if (D != 3 && D != 6 && D != 12) return 0;
  for (int cl : {1, 2, 4})
    if (D % cl == 0 && (size_t)(D / cl) * nx * 8 <= 100 * 1024 && !(D == 3 && cl > 1)) return cl;
  return 0;
}

// FP32 kernels of the fused path: the warp-per-row row kernels with TMA
// tiles when ny = 2048 (rows of 1024 complex points), and the cluster
// column kernel.  Tables and the tensor map of W are built here; a grid
// these kernels do not cover keeps the earlier fused kernels.
cudaError_t setup_fp32_kernels(gfmd_solver *h) {
  const gfmd::Geom &g = h->g;
  cudaError_t e = cudaMalloc((void **)&h->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemset(h->d_err, 0, sizeof(int));
  if (e != cudaSuccess) return e;
  const int D = g.ndof;
  const char *r32env = getenv("GFMD_COL_R32");  // 0: keep the shared-memory-stage column kernel
  const bool r32_ok = !(r32env && r32env[0] == '0');
  if (r32_ok && (g.nx == 1024 || g.nx == 2048) && (D == 3 || D == 6 || D == 12)) {
    // register-transform column kernel: DL = D / CL columns of nx / 32
    // threads each, at most 256 threads and 100 KB of shared memory a block
    const int P = g.nx / 32;
    int cl = 0;
    for (int c : {1, 2, 3, 4, 6})
      if (D % c == 0 && (D / c) * P <= 256 && (size_t)(D / c) * g.nx * 8 <= 100 * 1024) {
        cl = c;
        break;
      }
    // ndof 12 at nx = 2048: a 6-block cluster of 2 columns (128 threads) per
    // block, 4 blocks per SM, measured faster than the 3-block one (its
    // smaller blocks let the column transforms of one block overlap the
    // Phi stream of another): 0.442 against 0.450 ms per evaluation
    if (D == 12 && g.nx == 2048) cl = 6;
    if (cl > 0 && g.nyc * cl <= h->n_epart) {
      std::vector<float> f;
      for (int k1 = 0; k1 < 32; k1++)
        for (int t = 0; t < P; t++) push_c4(f, (long)t * k1, g.nx);
      e = cudaMalloc(&h->d_twc, f.size() * sizeof(float));
      if (e == cudaSuccess) e = cudaMemcpy(h->d_twc, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return e;
      h->col_r32 = true;
      h->col_cl = cl;
      h->col_minb = (D == 12 && g.nx == 2048) ? 4 : (D == 12 ? 2 : 3);  // compiled residency of the default instance
      h->phi_v = (D * D) % 4 == 0 ? 4 : 1;
      h->bytes += (double)f.size() * sizeof(float);
    }
  }
  const int cl = h->col_r32 ? 0 : pick_col_cluster(g.ndof, g.nx);
  int nepart_needed = g.nyc * std::max(cl, 1);
  if (cl > 0 && nepart_needed <= h->n_epart) {
    h->col_cl = cl;
    h->phi_v = (g.ndof * g.ndof) % 4 == 0 ? 4 : 1;
  }
  if (g.ny == 2048 && g.nx % 16 == 0 && encode_tiled() != nullptr) {
    std::vector<float> f;
    for (int k1 = 0; k1 < 32; k1++)
      for (int l = 0; l < 32; l++) push_c4(f, (long)l * k1, 1024);
    for (int k = 0; k <= 1024; k++) push_c4(f, k, 2048);
    e = cudaMalloc(&h->d_tw32, f.size() * sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(h->d_tw32, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    const cuuint64_t dims[3] = {(cuuint64_t)2 * g.nxp, (cuuint64_t)g.ndof, (cuuint64_t)g.nyc};
    const cuuint64_t strides[2] = {(cuuint64_t)2 * g.nxp * 4, (cuuint64_t)g.ndof * 2 * g.nxp * 4};
    const cuuint32_t box8[3] = {16, 1, 128}, box16[3] = {32, 1, 64}, estr[3] = {1, 1, 1};
    CUresult r = encode_tiled()(&h->tm_w[0], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, h->d_W, dims, strides, box8,
                                estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r == CUDA_SUCCESS)
      r = encode_tiled()(&h->tm_w[1], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, h->d_W, dims, strides, box16, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r == CUDA_SUCCESS) {
      h->rows32 = true;
      h->bytes += (double)f.size() * sizeof(float);
    }
  }
  return cudaSuccess;
}

// Sets up the fused power-of-two path when the grid allows it.
cudaError_t setup_fast(gfmd_solver *h) {
  const gfmd::Geom &g = h->g;
  const size_t cs = h->precision == GFMD_PREC_F64 ? 16 : 8;
  if (!is_pow2(g.nx) || g.nx < 16 || !g.ny_even || !is_pow2(g.nrow) || g.nrow < 16) return cudaSuccess;
  if (g.nx > 8192 || g.nrow > 8192) return cudaSuccess;
  gfmd::P2Plan pr = make_p2(g.nrow), pc = make_p2(g.nx);
  std::vector<double> d;
  std::vector<float> f;
  push_stage_tables(pr, d, f);
  pr.tpost = pr.tsize;
  for (int k = 0; k <= g.ny / 2; k++) {
    double a = -2.0 * kPi * (double)k / (double)g.ny;
    double c = std::cos(a), sn = std::sin(a);
    d.push_back(c);
    d.push_back(sn);
    float ch = (float)c, sh = (float)sn;
    f.push_back(ch);
    f.push_back(sh);
    f.push_back((float)(c - (double)ch));
    f.push_back((float)(sn - (double)sh));
  }
  pr.tsize += g.ny / 2 + 1;
  const int col_off = pr.tsize;
  push_stage_tables(pc, d, f);
  // shared-memory budgets (static shared memory of the kernels < 256 bytes):
  // the single-block column kernel holds all ndof columns and its twiddles;
  // the FP32 cluster column kernel spreads the columns over 1-4 blocks
  const size_t slack = 256;
  const char *v1env = getenv("GFMD_FAST_V1");  // 1: only the earlier fused kernels
  const bool v1 = v1env && v1env[0] == '1';
  const bool col_fits = (size_t)pc.tsize * 16 + (size_t)g.ndof * g.nx * cs + slack <= h->smem_optin;
  const bool cl_fits = h->precision == GFMD_PREC_F32 && !v1 && pick_col_cluster(g.ndof, g.nx) > 0;
  if (!col_fits && !cl_fits) return cudaSuccess;
  const size_t row_bytes = (size_t)(g.nrow + 1) * cs;
  const size_t row_fixed = (size_t)pr.tsize * 16 + ((size_t)g.nrow * 2 + 15) / 16 * 16;
  int rb = 16;
  while (rb > 1 && (rb > g.nx || row_fixed + rb * row_bytes > 72 * 1024)) rb /= 2;
  if (row_fixed + rb * row_bytes + slack > h->smem_optin) return cudaSuccess;
  const size_t nent = (size_t)col_off + pc.tsize;
  cudaError_t e = cudaMalloc(&h->d_ftw, nent * 16);
  if (e == cudaSuccess) {
    const void *src = h->precision == GFMD_PREC_F64 ? (const void *)d.data() : (const void *)f.data();
    e = cudaMemcpy(h->d_ftw, src, nent * 16, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) e = cudaMalloc((void **)&h->d_counter, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(h->d_counter, 0, sizeof(unsigned));
  if (e != cudaSuccess) return e;
  h->p2_row = pr;
  h->p2_col = pc;
  h->ftw_col_off = col_off;
  h->fast_rb = rb;
  h->fast_rb_max = rb;
  h->bytes += (double)nent * 16 + sizeof(unsigned);
  h->fast = true;
  if (h->precision == GFMD_PREC_F32 && !v1) {
    e = setup_fp32_kernels(h);
    if (e != cudaSuccess) return e;
  }
  if (!col_fits && h->col_cl == 0) h->fast = false;  // no column kernel fits: general path
  return cudaSuccess;
}

}  // namespace

namespace gfmd {

int set_error(int code, const std::string &msg) { return fail(code, msg); }

size_t phi_index(const gfmd_solver *h, int ky, int pos, int e) {
  const Geom &g = h->g;
  size_t D2 = (size_t)g.npk;
  if (!h->fast) {  // [ky][e][nxp]
    if (h->phi_pat != 0) {  // elements of the storage pattern only
      if (h->phi_slot[e] < 0) return kPhiAbsent;
      e = h->phi_slot[e];
      D2 = (size_t)(g.ndof + 2 * pat_pairs(g.ndof, h->phi_pat));
    }
    return ((size_t)ky * D2 + e) * g.nxp + pos;
  }
  const size_t blk = (size_t)ky * (g.nxp / 32) + pos / 32;
  if (h->col_cl > 0 && h->phi_v == 4) {  // [ky][x/32][e/4][32][4]
    if (h->phi_pat != 0) {  // elements of the storage pattern only
      if (h->phi_slot[e] < 0) return kPhiAbsent;
      e = h->phi_slot[e];
      D2 = (size_t)pat_floats(g.ndof, h->phi_pat);
    }
    return (blk * (D2 / 4) + e / 4) * 128 + (size_t)(pos % 32) * 4 + e % 4;
  }
  return (blk * D2 + e) * 32 + pos % 32;  // [ky][x/32][e][32]
}

int phi_reals(const gfmd_solver *h) {
  const int D = h->g.ndof;
  if (h->phi_pat == 0) return h->g.npk;
  return h->fast ? pat_floats(D, h->phi_pat) : D + 2 * pat_pairs(D, h->phi_pat);
}

FftPlan make_plan(int n, std::vector<double> &tw) {
  FftPlan p{};
  p.n = n;
  int m = n, k = 0;
  while (m % 8 == 0) { p.radix[k++] = 8; m /= 8; }
  if (m % 4 == 0) { p.radix[k++] = 4; m /= 4; }
  if (m % 2 == 0) { p.radix[k++] = 2; m /= 2; }
  for (int f = 3; m > 1; f += 2)
    while (m % f == 0) { p.radix[k++] = f; m /= f; }
  p.nst = k;
  int span = 1;
  for (int s = 0; s < k; s++) {
    const int R = p.radix[s], L = span * R;
    p.span[s] = span;
    p.twoff[s] = (int)(tw.size() / 2);
    for (int kk = 0; kk < span; kk++)
      for (int r = 0; r < R; r++) {
        long e = ((long)r * kk) % L;
        double a = -2.0 * kPi * (double)e / (double)L;
        tw.push_back(std::cos(a));
        tw.push_back(std::sin(a));
      }
    p.rootoff[s] = (int)(tw.size() / 2);
    if (R != 2 && R != 3 && R != 4 && R != 5 && R != 8)
      for (int mm = 0; mm < R; mm++) {
        double a = -2.0 * kPi * (double)mm / (double)R;
        tw.push_back(std::cos(a));
        tw.push_back(std::sin(a));
      }
    span = L;
  }
  return p;
}

}  // namespace gfmd

extern "C" {

const char *gfmd_last_error(void) { return g_err.c_str(); }

const char *gfmd_version(void) { return "gfmd_gb300 0.1 (sm_103a)"; }

int gfmd_create(int nx, int ny, int ndof, int precision, gfmd_handle_t *out) {
  if (!out) return fail(GFMD_EINVAL, "gfmd_create: out is NULL");
  *out = nullptr;
  if (nx < 1 || ny < 1 || nx > 8192 || ny > 8192)
    return fail(GFMD_EINVAL, "gfmd_create: nx, ny must be in [1, 8192]");
  if (ndof < 3 || ndof > gfmd::kMaxNdof || ndof % 3 != 0)
    return fail(GFMD_EINVAL, "gfmd_create: ndof must be 3, 6, ..., 24");
  if (precision != GFMD_PREC_F64 && precision != GFMD_PREC_F32)
    return fail(GFMD_EINVAL, "gfmd_create: unknown precision");

  auto *h = new gfmd_solver();
  h->precision = precision;
  gfmd::Geom &g = h->g;
  g.nx = nx;
  g.ny = ny;
  g.ndof = ndof;
  g.nyc = ny / 2 + 1;
  g.nxp = (nx + 31) / 32 * 32;
  g.ny_even = (ny % 2 == 0) ? 1 : 0;
  g.nrow = g.ny_even ? ny / 2 : ny;
  g.npk = ndof * ndof;

  cudaError_t e = cudaGetDevice(&h->device);
  if (e != cudaSuccess) { release(h); return cuda_fail(e, "gfmd_create: cudaGetDevice"); }
  int v = 0;
  cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, h->device);
  h->sm_count = v;
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device);
  h->smem_optin = (size_t)v;

  const size_t cs = precision == GFMD_PREC_F64 ? 16 : 8;
  if (2 * (size_t)(g.nrow + 1) * cs > h->smem_optin || 2 * (size_t)nx * cs > h->smem_optin) {
    release(h);
    return fail(GFMD_EINVAL, "gfmd_create: grid too large for this precision");
  }

  // plans and twiddles: row plan, column plan, r2c post-twiddles
  std::vector<double> tw;
  h->plan_row = gfmd::make_plan(g.nrow, tw);
  h->plan_col = gfmd::make_plan(nx, tw);
  g.rpost = (int)(tw.size() / 2);
  for (int k = 0; k <= ny / 2; k++) {
    double a = -2.0 * kPi * (double)k / (double)ny;
    tw.push_back(std::cos(a));
    tw.push_back(std::sin(a));
  }
  const size_t ntw = tw.size() / 2;
  if (precision == GFMD_PREC_F64) {
    e = cudaMalloc(&h->d_tw_hi, ntw * sizeof(double2));
    if (e == cudaSuccess) e = cudaMemcpy(h->d_tw_hi, tw.data(), ntw * sizeof(double2), cudaMemcpyHostToDevice);
  } else {
    std::vector<float> hi(2 * ntw), lo(2 * ntw);
    for (size_t i = 0; i < 2 * ntw; i++) {
      hi[i] = (float)tw[i];
      lo[i] = (float)(tw[i] - (double)hi[i]);
    }
    e = cudaMalloc(&h->d_tw_hi, ntw * sizeof(float2));
    if (e == cudaSuccess) e = cudaMalloc(&h->d_tw_lo, ntw * sizeof(float2));
    if (e == cudaSuccess) e = cudaMemcpy(h->d_tw_hi, hi.data(), ntw * sizeof(float2), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(h->d_tw_lo, lo.data(), ntw * sizeof(float2), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) { release(h); return cuda_fail(e, "gfmd_create: twiddles"); }

  size_t wb, pb;
  gfmd::force_layout(g, precision, &wb, &pb, &h->n_epart);
  e = cudaMalloc(&h->d_W, wb);
  if (e == cudaSuccess) e = cudaMalloc(&h->d_phi, pb);
  if (e == cudaSuccess) e = cudaMalloc((void **)&h->d_linf, sizeof(double) * (ndof / 3));
  if (e == cudaSuccess) e = cudaMalloc((void **)&h->d_epart, sizeof(double) * h->n_epart);
  if (e == cudaSuccess) e = cudaMalloc((void **)&h->d_scal, sizeof(double) * (1 + gfmd::kMaxNdof));
  if (e == cudaSuccess) e = cudaMalloc((void **)&h->d_zero, sizeof(double) * gfmd::kMaxNdof);
  if (e == cudaSuccess) e = cudaMemset(h->d_zero, 0, sizeof(double) * gfmd::kMaxNdof);
  if (e == cudaSuccess) e = cudaMemset(h->d_linf, 0, sizeof(double) * (ndof / 3));
  if (e == cudaSuccess) e = cudaMemset(h->d_scal, 0, sizeof(double) * (1 + gfmd::kMaxNdof));
  if (e != cudaSuccess) { release(h); return cuda_fail(e, "gfmd_create: device buffers"); }
  h->bytes = (double)wb + (double)pb + 8.0 * (h->n_epart + ndof / 3 + 1 + gfmd::kMaxNdof) +
             (double)ntw * cs * (precision == GFMD_PREC_F64 ? 1 : 2);
  if (getenv("GFMD_PLAIN_PATH") == nullptr || getenv("GFMD_PLAIN_PATH")[0] == '0') {
    e = setup_fast(h);
    if (e != cudaSuccess) { release(h); return cuda_fail(e, "gfmd_create: fused-path tables"); }
  }
  *out = h;
  return GFMD_OK;
}

int gfmd_destroy(gfmd_handle_t h) {
  if (!h) return fail(GFMD_EINVAL, "gfmd_destroy: NULL handle");
  release(h);
  return GFMD_OK;
}

int gfmd_set_stream(gfmd_handle_t h, void *stream) {
  if (!h) return fail(GFMD_EINVAL, "gfmd_set_stream: NULL handle");
  h->stream = reinterpret_cast<cudaStream_t>(stream);
  return GFMD_OK;
}

int gfmd_solver_info(gfmd_handle_t h, int *launches_per_eval, int *fused) {
  if (!h) return fail(GFMD_EINVAL, "gfmd_solver_info: NULL handle");
  if (launches_per_eval) *launches_per_eval = gfmd::force_launches(h);
  if (fused) *fused = h->fast ? 1 : 0;
  return GFMD_OK;
}

int gfmd_memory_usage(gfmd_handle_t h, double *bytes) {
  if (!h || !bytes) return fail(GFMD_EINVAL, "gfmd_memory_usage: NULL argument");
  *bytes = h->bytes + (h->prec_grad ? h->prec_grad->bytes : 0.0);  // + gfmd_prec_gradient's handle
  return GFMD_OK;
}

// Pack the table into [nyc][npk][nxp] reals of the handle's precision:
// Phi_eff(k) = (Phi(k) + conj Phi(-k)) / 2 on the stored half spectrum, then
// its Hermitian part H; p < D holds Re H_pp, then (Re H_ij, Im H_ij) for
// i < j in row-major order.  With Phi_eff the half-spectrum real transforms
// reproduce the real part of the reference's full complex transforms.
// ---- plan autotuner -----------------------------------------------------
// The fused path's launch plan has free parameters that change no
// arithmetic: the rows per block of the shared-memory row kernels (1/4 to 1
// of the largest that fits the shared-memory budget) and, for the
// register-transform column kernel, the rounds of its Phi stream prefetched
// into L2 ahead of use (1-3) and the resident blocks per SM it is compiled
// for (2-4 for the 3-column kernel at nx = 2048), plus the rows per block of
// the warp-row kernels.  With the table
// uploaded, each candidate is timed (CUDA events, best of 3 runs of 4
// evaluations after a warm-up, each evaluation after a write of 1.25x the L2
// size) on scratch inputs and the fastest is kept; results are cached per grid,
// precision and kernel selection for the process.  GFMD_AUTOTUNE=0 keeps the
// rule-based defaults.
namespace {
struct PlanKey {
  int nx, ny, ndof, prec, kernels;
  bool operator<(const PlanKey &o) const {
    return std::tie(nx, ny, ndof, prec, kernels) < std::tie(o.nx, o.ny, o.ndof, o.prec, o.kernels);
  }
};
struct Plan {
  int rb, col_pf, col_minb, row_rb;
};
std::mutex g_plan_mu;
std::map<PlanKey, Plan> g_plans;

cudaError_t autotune(gfmd_solver *h) {
  if (!h->fast || h->tuned) return cudaSuccess;
  const char *env = getenv("GFMD_AUTOTUNE");
  if (env && env[0] == '0') return cudaSuccess;
  const PlanKey key{h->g.nx, h->g.ny, h->g.ndof, h->precision,
                    (h->rows32 ? 1 : 0) | (h->col_r32 ? 2 : 0) | (h->col_cl << 2) | (h->phi_pat << 8)};
  {
    std::lock_guard<std::mutex> lk(g_plan_mu);
    auto it = g_plans.find(key);
    if (it != g_plans.end()) {
      h->fast_rb = it->second.rb;
      h->col_pf = it->second.col_pf;
      h->col_minb = it->second.col_minb;
      h->row_rb = it->second.row_rb;
      h->tuned = true;
      return cudaSuccess;
    }
  }
  const size_t n = (size_t)h->g.ndof * h->g.nx * h->g.ny;
  const size_t es = h->precision == GFMD_PREC_F64 ? 8 : 4;
  void *u = nullptr, *f = nullptr;
  double *ep = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaError_t e = cudaMalloc(&u, n * es);
  if (e == cudaSuccess) e = cudaMalloc(&f, n * es);
  if (e == cudaSuccess) e = cudaMalloc((void **)&ep, sizeof(double));
  if (e == cudaSuccess) e = cudaMemset(u, 0, n * es);
  int dev = 0, l2 = 0;
  if (e == cudaSuccess) e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
  const size_t flush_bytes = std::max<size_t>((size_t)l2 * 5 / 4, 1 << 20);
  void *flush = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&flush, flush_bytes);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  const int t = h->precision == GFMD_PREC_F64 ? 0 : 1;
  const char *tr = getenv("GFMD_TRACE");
  const bool trace = tr && tr[0] && tr[0] != '0';
  cudaStream_t keep = h->stream;
  const Plan p0{h->fast_rb, h->col_pf, h->col_minb, h->row_rb};
  std::vector<Plan> cand;
  std::vector<int> rbs, pfs{h->col_pf}, minbs{h->col_minb}, rrbs{h->row_rb};
  if (h->rows32) rrbs = {8, 16};
  if (h->rows32 && h->precision == GFMD_PREC_F32) rbs.push_back(h->fast_rb);  // not used by those kernels
  else
    for (int rb = h->fast_rb_max; rb >= 1 && rb * 4 >= h->fast_rb_max; rb /= 2) rbs.push_back(rb);
  if (h->col_r32) {
    pfs = {1, 2, 3};
    if (h->g.ndof == 3 && h->g.nx == 2048) minbs = {2, 3, 4};
  }
  for (int rb : rbs)
    for (int pf : pfs)
      for (int mb : minbs)
        for (int rr : rrbs) cand.push_back({rb, pf, mb, rr});
  Plan best_p = p0;
  float best = 1e30f;
  h->stream = st;
  for (const Plan &c : cand) {
    if (e != cudaSuccess) break;
    h->fast_rb = c.rb;
    h->col_pf = c.col_pf;
    h->col_minb = c.col_minb;
    h->row_rb = c.row_rb;
    e = gfmd::enqueue_force(h, u, t, f, t, ep);  // warm-up
    float ms = 1e30f;
    for (int r = 0; r < 3 && e == cudaSuccess; r++) {
      float tot = 0.0f;
      for (int k = 0; k < 4 && e == cudaSuccess; k++) {
        // each evaluation starts from an L2 holding other data, as in a
        // solver loop whose vector kernels stream between evaluations
        e = cudaMemsetAsync(flush, k, flush_bytes, st);
        if (e == cudaSuccess) e = cudaEventRecord(e0, st);
        if (e == cudaSuccess) e = gfmd::enqueue_force(h, u, t, f, t, ep);
        if (e == cudaSuccess) e = cudaEventRecord(e1, st);
        if (e == cudaSuccess) e = cudaEventSynchronize(e1);
        float x = 0.0f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&x, e0, e1);
        tot += x;
      }
      ms = std::min(ms, tot);
    }
    if (trace)
      fprintf(stderr,
              "gfmd autotune %dx%d ndof %d: rows/block %d (warp rows %d), column Phi prefetch %d, blocks/SM %d: "
              "%.4f ms\n",
              h->g.nx, h->g.ny, h->g.ndof, c.rb, c.row_rb, c.col_pf, c.col_minb, ms);
    if (e == cudaSuccess && ms < best) {
      best = ms;
      best_p = c;
    }
  }
  h->stream = keep;
  const Plan &use = e == cudaSuccess ? best_p : p0;
  h->fast_rb = use.rb;
  h->col_pf = use.col_pf;
  h->col_minb = use.col_minb;
  h->row_rb = use.row_rb;
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  for (void *p : {u, f, (void *)ep, flush})
    if (p) cudaFree(p);
  if (e != cudaSuccess) return e;
  h->tuned = true;
  std::lock_guard<std::mutex> lk(g_plan_mu);
  g_plans[key] = use;
  return cudaSuccess;
}
}  // namespace

int gfmd_set_phi(gfmd_handle_t h, const double *phi, int layout, const double *linf) {
  if (!h || !phi) return fail(GFMD_EINVAL, "gfmd_set_phi: NULL argument");
  release(h->prec_grad);  // built from the previous table
  h->prec_grad = nullptr;
  h->prec_cavg.clear();
  if (layout != GFMD_PHI_FULL && layout != GFMD_PHI_HALF)
    return fail(GFMD_EINVAL, "gfmd_set_phi: unknown layout");
  const gfmd::Geom &g = h->g;
  const int D = g.ndof, D2 = D * D;
  const size_t nq = (size_t)g.nyc * g.nxp;
  const bool f64 = h->precision == GFMD_PREC_F64;
  const bool fused = h->fast;
  std::vector<double> packd;
  std::vector<float> packf;
  if (f64) packd.assign(nq * D2, 0.0);
  else packf.assign(nq * D2, 0.0f);
  bool finite = true;

  auto src = [&](int kx, int ky) -> const double * {
    if (layout == GFMD_PHI_FULL) return phi + 2 * ((size_t)kx * g.ny + ky) * D2;
    return phi + 2 * ((size_t)kx * g.nyc + ky) * D2;
  };
  // storage pattern: the register-transform column kernel at ndof 12 skips
  // the pairs that are exactly zero at every wavevector of the table
  // (GFMD_PHI_DENSE=1: always every pair)
  const int old_pat = h->phi_pat;
  h->phi_pat = 0;
  h->phi_slot.clear();
  const char *dense_env = getenv("GFMD_PHI_DENSE");
  const bool pat_kernel = (h->col_r32 && !f64 && h->phi_v == 4) || !h->fast;  // kernels with pattern instances
  if (pat_kernel && D == 12 && !(dense_env && dense_env[0] == '1')) {
    const size_t nsrc = layout == GFMD_PHI_FULL ? (size_t)g.nx * g.ny : (size_t)g.nx * g.nyc;
    std::mutex mu;
    std::vector<char> nz(D2, 0);
    parallel_for((long)nsrc, [&](long a, long b) {
      std::vector<char> loc(D2, 0);
      for (long t = a; t < b; t++) {
        const double *pe = phi + 2 * (size_t)t * D2;
        for (int e = 0; e < D2; e++) loc[e] |= (pe[2 * e] != 0.0 || pe[2 * e + 1] != 0.0) ? 1 : 0;
      }
      std::lock_guard<std::mutex> lk(mu);
      for (int e = 0; e < D2; e++) nz[e] |= loc[e];
    });
    for (int pat : {2, 1}) {
      bool fits = true;
      for (int i = 0; i < D && fits; i++)
        for (int j = i + 1; j < D; j++)
          if (!gfmd::pat_keeps(D, pat, i, j) && (nz[i * D + j] || nz[j * D + i])) {
            fits = false;
            break;
          }
      if (!fits) continue;
      h->phi_pat = pat;
      h->phi_slot.assign(D2, -1);
      for (int i = 0; i < D; i++) h->phi_slot[i] = i;
      int pd = D, ps = D;  // dense and pattern positions, pairs in row-major order
      for (int i = 0; i < D; i++)
        for (int j = i + 1; j < D; j++, pd += 2)
          if (gfmd::pat_keeps(D, pat, i, j)) {
            h->phi_slot[pd] = ps;
            h->phi_slot[pd + 1] = ps + 1;
            ps += 2;
          }
      break;
    }
  }
  if (h->phi_pat != old_pat) h->tuned = false;  // another column kernel: plan it again
  parallel_for((long)g.nyc * g.nx, [&](long a, long b) {
    std::vector<double> eff(2 * D2);
    bool ok = true;
    for (long t = a; t < b; t++) {
      int ky = (int)(t / g.nx), kx = (int)(t % g.nx);
      int mx = (g.nx - kx) % g.nx, my = (g.ny - ky) % g.ny;
      const double *pa = src(kx, ky);
      const double *pb = nullptr;
      if (layout == GFMD_PHI_FULL) pb = src(mx, my);
      else if (my == ky) pb = src(mx, ky);  // ky = 0 or ny/2: mirror stored
      for (int e = 0; e < D2; e++) {
        if (pb) {
          eff[2 * e] = 0.5 * (pa[2 * e] + pb[2 * e]);
          eff[2 * e + 1] = 0.5 * (pa[2 * e + 1] - pb[2 * e + 1]);
        } else {
          eff[2 * e] = pa[2 * e];
          eff[2 * e + 1] = pa[2 * e + 1];
        }
      }
      // storage position: the digit-reversed position of kx on the fused
      // path (the order its forward FFT leaves), kx otherwise
      const int xs = !fused ? kx
                     : h->col_r32 ? (g.nx / 32) * (kx & 31) + (kx >> 5)
                                  : p2_digit_rev(h->p2_col, kx);
      auto put = [&](int p, double v) {
        if (!std::isfinite(v)) ok = false;
        const size_t at = gfmd::phi_index(h, ky, xs, p);
        if (at == gfmd::kPhiAbsent) return;  // zero at every wavevector
        if (f64) packd[at] = v;
        else packf[at] = (float)v;
      };
      for (int i = 0; i < D; i++) put(i, eff[2 * (i * D + i)]);
      int p = D;
      for (int i = 0; i < D; i++)
        for (int j = i + 1; j < D; j++) {
          double re = 0.5 * (eff[2 * (i * D + j)] + eff[2 * (j * D + i)]);
          double im = 0.5 * (eff[2 * (i * D + j) + 1] - eff[2 * (j * D + i) + 1]);
          put(p++, re);
          put(p++, im);
        }
    }
    if (!ok) finite = false;
  });
  if (!finite) return fail(GFMD_ENONFINITE, "gfmd_set_phi: table holds NaN or Inf");
  const void *hp = f64 ? (const void *)packd.data() : (const void *)packf.data();
  const size_t per_q = (size_t)gfmd::phi_reals(h);
  size_t bytes = nq * per_q * (f64 ? 8 : 4);
  CK(cudaMemcpy(h->d_phi, hp, bytes, cudaMemcpyHostToDevice), "gfmd_set_phi: upload");
  std::vector<double> lf(D / 3, 0.0);
  if (linf)
    for (int i = 0; i < D / 3; i++) lf[i] = linf[i];
  CK(cudaMemcpy(h->d_linf, lf.data(), sizeof(double) * lf.size(), cudaMemcpyHostToDevice),
     "gfmd_set_phi: linf");
  h->have_phi = true;
  CK(autotune(h), "gfmd_set_phi: plan autotuning");
  return GFMD_OK;
}

int gfmd_plan_info(gfmd_handle_t h, int *rows_per_block, int *phi_prefetch) {
  if (!h) return fail(GFMD_EINVAL, "gfmd_plan_info: NULL handle");
  if (rows_per_block) *rows_per_block = h->fast ? h->fast_rb : 0;
  if (phi_prefetch) *phi_prefetch = h->fast ? (h->col_r32 ? h->col_pf : h->fast_pf) : 0;
  return GFMD_OK;
}

}  // extern "C"

// dst[i] = s * src[i], grid-stride
__global__ void k_scaled_copy(const double *__restrict__ src, double *__restrict__ dst, size_t n, double s) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = s * src[i];
}

// A new handle on h's grid and precision whose force evaluation applies
// -scale * A(q)^{-1}, A(q) = block(Phi table entry of h) built by `fill`
// (which receives the Hermitian block of h's table as uploaded, i.e. already
// divided by nx*ny, and may change it in place).  The inverse is Gauss-Jordan
// without pivoting (A Hermitian positive definite); its Hermitian part is
// packed.  Returns a GFMD status; `who` prefixes messages.
template <typename Fill>
static int inverse_table_handle(gfmd_handle_t h, const char *who, double scale, Fill fill,
                                gfmd_handle_t *out) {
  *out = nullptr;
  const std::string w(who);
  if (!h->have_phi) return fail(GFMD_ENOPHI, w + ": no stiffness table uploaded");
  const gfmd::Geom &g = h->g;
  gfmd_handle_t p = nullptr;
  int rc = gfmd_create(g.nx, g.ny, g.ndof, h->precision, &p);
  if (rc != GFMD_OK) return rc;
  if (p->fast != h->fast || p->col_cl != h->col_cl || p->phi_v != h->phi_v ||
      p->col_r32 != h->col_r32) {  // same parameters, same path
    release(p);
    return fail(GFMD_ECUDA, w + ": path mismatch");
  }
  const int D = g.ndof, D2 = D * D;
  const size_t nslot = (size_t)g.nyc * g.nxp, nel = nslot * D2;
  const bool f64 = h->precision == GFMD_PREC_F64;
  std::vector<double> tab(nel);
  {
    std::vector<float> tf;
    cudaError_t e;
    if (f64) {
      e = cudaMemcpy(tab.data(), h->d_phi, nel * 8, cudaMemcpyDeviceToHost);
    } else {
      tf.resize(nel);
      e = cudaMemcpy(tf.data(), h->d_phi, nel * 4, cudaMemcpyDeviceToHost);
      for (size_t i = 0; i < nel; i++) tab[i] = tf[i];
    }
    if (e != cudaSuccess) {
      release(p);
      return cuda_fail(e, (w + ": download").c_str());
    }
  }
  std::vector<double> inv(nel, 0.0);  // p's table (every pair: the inverse is dense)
  std::atomic<bool> ok(true);
  parallel_for((long)nslot, [&](long a, long b) {
    std::vector<std::complex<double>> A(D2), I(D2);
    for (long t = a; t < b; t++) {
      const int ky = (int)(t / g.nxp), xs = (int)(t % g.nxp);
      // h's table (pairs outside its storage pattern are zero); p's table
      auto rd = [&](int e) {
        const size_t i = gfmd::phi_index(h, ky, xs, e);
        return i == gfmd::kPhiAbsent ? 0.0 : tab[i];
      };
      auto at = [&](int e) { return gfmd::phi_index(p, ky, xs, e); };
      // Hermitian block of the uploaded table
      for (int i = 0; i < D; i++) A[i * D + i] = rd(i);
      int q = D;
      for (int i = 0; i < D; i++)
        for (int j = i + 1; j < D; j++) {
          const std::complex<double> v(rd(q), rd(q + 1));
          A[i * D + j] = v;
          A[j * D + i] = std::conj(v);
          q += 2;
        }
      fill(A.data());
      // Gauss-Jordan inverse (Hermitian positive definite: no pivoting)
      for (int i = 0; i < D2; i++) I[i] = 0.0;
      for (int i = 0; i < D; i++) I[i * D + i] = 1.0;
      for (int c = 0; c < D; c++) {
        const std::complex<double> piv = A[c * D + c];
        if (!(std::abs(piv) > 0.0) || !std::isfinite(std::abs(piv))) {
          ok = false;
          break;
        }
        const std::complex<double> ip = 1.0 / piv;
        for (int k = 0; k < D; k++) {
          A[c * D + k] *= ip;
          I[c * D + k] *= ip;
        }
        for (int r = 0; r < D; r++) {
          if (r == c) continue;
          const std::complex<double> f = A[r * D + c];
          if (f == 0.0) continue;
          for (int k = 0; k < D; k++) {
            A[r * D + k] -= f * A[c * D + k];
            I[r * D + k] -= f * I[c * D + k];
          }
        }
      }
      // pack scale * inverse (Hermitian part)
      for (int i = 0; i < D; i++) inv[at(i)] = scale * I[i * D + i].real();
      q = D;
      for (int i = 0; i < D; i++)
        for (int j = i + 1; j < D; j++) {
          const std::complex<double> v = 0.5 * scale * (I[i * D + j] + std::conj(I[j * D + i]));
          inv[at(q)] = v.real();
          inv[at(q + 1)] = v.imag();
          q += 2;
        }
    }
  });
  if (!ok) {
    release(p);
    return fail(GFMD_ENONFINITE, w + ": singular block");
  }
  cudaError_t e;
  if (f64) {
    e = cudaMemcpy(p->d_phi, inv.data(), nel * 8, cudaMemcpyHostToDevice);
  } else {
    std::vector<float> tf(nel);
    for (size_t i = 0; i < nel; i++) tf[i] = (float)inv[i];
    e = cudaMemcpy(p->d_phi, tf.data(), nel * 4, cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    release(p);
    return cuda_fail(e, (w + ": upload").c_str());
  }
  p->have_phi = true;
  e = autotune(p);
  if (e != cudaSuccess) {
    release(p);
    return cuda_fail(e, (w + ": plan autotuning").c_str());
  }
  *out = p;
  return GFMD_OK;
}

extern "C" {

int gfmd_make_preconditioner(gfmd_handle_t h, double shift, gfmd_handle_t *out) {
  if (!h || !out) return fail(GFMD_EINVAL, "gfmd_make_preconditioner: NULL argument");
  *out = nullptr;
  if (!(shift > 0.0) || !std::isfinite(shift)) return fail(GFMD_EINVAL, "gfmd_make_preconditioner: shift must be > 0");
  // (Phi + shift)^{-1} / N with Phi = N * table: the force path's unscaled
  // transform pair then applies -(Phi + shift)^{-1}
  const double N = (double)h->g.nx * (double)h->g.ny;
  const int D = h->g.ndof;
  return inverse_table_handle(h, "gfmd_make_preconditioner", 1.0 / N,
                              [&](std::complex<double> *A) {
                                for (int i = 0; i < D * D; i++) A[i] *= N;
                                for (int i = 0; i < D; i++) A[i * D + i] += shift;
                              },
                              out);
}

int gfmd_prec_gradient(gfmd_handle_t h, const double *cavg, const double *d_g, double *d_gP) {
  if (!h || !cavg || !d_g || !d_gP) return fail(GFMD_EINVAL, "gfmd_prec_gradient: NULL argument");
  if (d_g == d_gP) return fail(GFMD_EINVAL, "gfmd_prec_gradient: g and gP must not alias");
  const int D = h->g.ndof;
  for (int i = 0; i < D; i++)
    for (int j = 0; j < D; j++) {
      const double a = cavg[i * D + j], b = cavg[j * D + i];
      if (!std::isfinite(a)) return fail(GFMD_EINVAL, "gfmd_prec_gradient: Cavg holds NaN or Inf");
      if (std::fabs(a - b) > 1e-12 * (std::fabs(a) + std::fabs(b)))
        return fail(GFMD_EINVAL, "gfmd_prec_gradient: Cavg must be symmetric");
    }
  std::vector<double> c(cavg, cavg + (size_t)D * D);
  if (!h->prec_grad || h->prec_cavg != c) {
    release(h->prec_grad);
    h->prec_grad = nullptr;
    h->prec_cavg.clear();
    gfmd_handle_t p = nullptr;
    // the reference's operator (Phi(q)/N + Cavg)^{-1} between unscaled
    // transforms; the force path applies -table, so the table is -M
    int rc = inverse_table_handle(h, "gfmd_prec_gradient", -1.0,
                                  [&](std::complex<double> *A) {
                                    for (int i = 0; i < D * D; i++) A[i] += c[i];
                                  },
                                  &p);
    if (rc != GFMD_OK) return rc;
    h->prec_grad = p;
    h->prec_cavg = c;
  }
  h->prec_grad->stream = h->stream;
  cudaError_t e = gfmd::enqueue_force_opts(h->prec_grad, d_g, 0, d_gP, 0, h->prec_grad->d_scal, false);
  if (e != cudaSuccess) return cuda_fail(e, "gfmd_prec_gradient");
  if (D > 3) {
    // precondition_gradient<DEF_G> writes back only three components for
    // ndof > 3 (gfmd_misc.h:121-124); the others leave the unscaled
    // transform pair as nx*ny*g
    const size_t nxy = (size_t)h->g.nx * h->g.ny, n = (size_t)(D - 3) * nxy;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)std::max(1, h->sm_count) * 8);
    k_scaled_copy<<<blocks, 256, 0, h->stream>>>(d_g + 3 * nxy, d_gP + 3 * nxy, n,
                                                  (double)h->g.nx * (double)h->g.ny);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(e, "gfmd_prec_gradient");
  }
  return GFMD_OK;
}

static int force_common(gfmd_handle_t h, const void *d_u, int in_t, void *d_f, int out_t,
                        double *d_epot, const char *who) {
  if (!h || !d_u || !d_f) return fail(GFMD_EINVAL, std::string(who) + ": NULL argument");
  if (d_u == d_f) return fail(GFMD_EINVAL, std::string(who) + ": u and f must not alias");
  if (!h->have_phi) return fail(GFMD_ENOPHI, std::string(who) + ": no stiffness table uploaded");
  cudaError_t e = gfmd::enqueue_force(h, d_u, in_t, d_f, out_t, d_epot ? d_epot : h->d_scal);
  if (e != cudaSuccess) return cuda_fail(e, who);
  return GFMD_OK;
}

int gfmd_force_f64(gfmd_handle_t h, const double *d_u, double *d_f, double *d_epot) {
  if (h && h->precision != GFMD_PREC_F64)
    return fail(GFMD_EINVAL, "gfmd_force_f64: handle is not FP64");
  return force_common(h, d_u, 0, d_f, 0, d_epot, "gfmd_force_f64");
}

int gfmd_force_f32(gfmd_handle_t h, const float *d_u, float *d_f, double *d_epot) {
  if (h && h->precision != GFMD_PREC_F32)
    return fail(GFMD_EINVAL, "gfmd_force_f32: handle is not FP32");
  return force_common(h, d_u, 1, d_f, 1, d_epot, "gfmd_force_f32");
}

// After a synchronisation: a bounded device wait that gave up (recorded in
// the handle's error word by the TMA row kernels) becomes GFMD_ETIMEDOUT.
static int check_device_error(gfmd_handle_t h, const char *who) {
  if (!h->d_err) return GFMD_OK;
  int v = 0;
  CK(cudaMemcpy(&v, h->d_err, sizeof(int), cudaMemcpyDeviceToHost), who);
  if (v == 0) return GFMD_OK;
  CK(cudaMemset(h->d_err, 0, sizeof(int)), who);
  return fail(GFMD_ETIMEDOUT, std::string(who) + ": a device wait for a tile timed out");
}

int gfmd_post_force(gfmd_handle_t h, const double *d_u, double *d_f, double *epot) {
  int rc = force_common(h, d_u, 0, d_f, 0, h ? h->d_scal : nullptr, "gfmd_post_force");
  if (rc) return rc;
  double e = 0.0;
  CK(cudaMemcpyAsync(&e, h->d_scal, sizeof(double), cudaMemcpyDeviceToHost, h->stream),
     "gfmd_post_force: energy");
  CK(cudaStreamSynchronize(h->stream), "gfmd_post_force");
  if ((rc = check_device_error(h, "gfmd_post_force"))) return rc;
  if (!std::isfinite(e)) return fail(GFMD_ENONFINITE, "gfmd_post_force: energy is not finite");
  if (epot) *epot = e;
  return GFMD_OK;
}

int gfmd_post_force_host(gfmd_handle_t h, const double *u, double *f, double *epot) {
  if (!h || !u || !f) return fail(GFMD_EINVAL, "gfmd_post_force_host: NULL argument");
  const size_t n = (size_t)h->g.ndof * h->g.nx * h->g.ny;
  if (!h->d_io) CK(cudaMalloc(&h->d_io, 2 * n * sizeof(double)), "gfmd_post_force_host: staging");
  double *du = reinterpret_cast<double *>(h->d_io), *df = du + n;
  CK(cudaMemcpyAsync(du, u, n * sizeof(double), cudaMemcpyHostToDevice, h->stream),
     "gfmd_post_force_host: copy in");
  int rc = force_common(h, du, 0, df, 0, h->d_scal, "gfmd_post_force_host");
  if (rc) return rc;
  double e = 0.0;
  CK(cudaMemcpyAsync(f, df, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
     "gfmd_post_force_host: copy out");
  CK(cudaMemcpyAsync(&e, h->d_scal, sizeof(double), cudaMemcpyDeviceToHost, h->stream),
     "gfmd_post_force_host: energy");
  CK(cudaStreamSynchronize(h->stream), "gfmd_post_force_host");
  if ((rc = check_device_error(h, "gfmd_post_force_host"))) return rc;
  if (!std::isfinite(e)) return fail(GFMD_ENONFINITE, "gfmd_post_force_host: energy is not finite");
  if (epot) *epot = e;
  return GFMD_OK;
}

int gfmd_prec_gradient_host(gfmd_handle_t h, const double *cavg, const double *g, double *gP) {
  if (!h || !cavg || !g || !gP) return fail(GFMD_EINVAL, "gfmd_prec_gradient_host: NULL argument");
  const size_t n = (size_t)h->g.ndof * h->g.nx * h->g.ny;
  if (!h->d_io) CK(cudaMalloc(&h->d_io, 2 * n * sizeof(double)), "gfmd_prec_gradient_host: staging");
  double *dg = reinterpret_cast<double *>(h->d_io), *dp = dg + n;
  CK(cudaMemcpyAsync(dg, g, n * sizeof(double), cudaMemcpyHostToDevice, h->stream),
     "gfmd_prec_gradient_host: copy in");
  int rc = gfmd_prec_gradient(h, cavg, dg, dp);
  if (rc) return rc;
  CK(cudaMemcpyAsync(gP, dp, n * sizeof(double), cudaMemcpyDeviceToHost, h->stream),
     "gfmd_prec_gradient_host: copy out");
  CK(cudaStreamSynchronize(h->stream), "gfmd_prec_gradient_host");
  return GFMD_OK;
}

int gfmd_force_kernel_times(gfmd_handle_t h, const void *d_u, void *d_f, double *d_epot, float *ms, int nmax,
                            int *nk) {
  if (!h || !d_u || !d_f || !d_epot || !ms || !nk)
    return fail(GFMD_EINVAL, "gfmd_force_kernel_times: NULL argument");
  if (d_u == d_f) return fail(GFMD_EINVAL, "gfmd_force_kernel_times: u and f must not alias");
  if (!h->have_phi) return fail(GFMD_ENOPHI, "gfmd_force_kernel_times: no stiffness table uploaded");
  const int nl = gfmd::force_launches(h);
  if (nmax < nl) return fail(GFMD_EINVAL, "gfmd_force_kernel_times: ms holds fewer entries than launches");
  std::vector<cudaEvent_t> ev(nl + 1, nullptr);
  cudaError_t e = cudaSuccess;
  for (auto &x : ev)
    if (e == cudaSuccess) e = cudaEventCreate(&x);
  if (e == cudaSuccess) {
    h->mark = ev.data();
    h->nmark = nl + 1;
    const int t = h->precision == GFMD_PREC_F64 ? 0 : 1;
    e = gfmd::enqueue_force(h, d_u, t, d_f, t, d_epot);
    h->mark = nullptr;
    h->nmark = 0;
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
  for (int i = 0; i < nl && e == cudaSuccess; i++) e = cudaEventElapsedTime(&ms[i], ev[i], ev[i + 1]);
  for (auto &x : ev)
    if (x) cudaEventDestroy(x);
  if (e != cudaSuccess) return cuda_fail(e, "gfmd_force_kernel_times");
  *nk = nl;
  return check_device_error(h, "gfmd_force_kernel_times");
}

int gfmd_kernel_plan(gfmd_handle_t h, int *row_warp_tma, int *col_cluster, int *phi_vector) {
  if (!h) return fail(GFMD_EINVAL, "gfmd_kernel_plan: NULL handle");
  if (row_warp_tma) *row_warp_tma = h->rows32 ? 1 : 0;
  if (col_cluster) *col_cluster = h->col_cl;
  if (phi_vector) *phi_vector = h->phi_v;
  return GFMD_OK;
}

int gfmd_phi_pattern(gfmd_handle_t h, int *pattern, int *reals_per_wavevector) {
  if (!h) return fail(GFMD_EINVAL, "gfmd_phi_pattern: NULL handle");
  if (pattern) *pattern = h->phi_pat;
  if (reals_per_wavevector) *reals_per_wavevector = gfmd::phi_reals(h);
  return GFMD_OK;
}

int gfmd_get_u0(gfmd_handle_t h, double *u0) {
  if (!h || !u0) return fail(GFMD_EINVAL, "gfmd_get_u0: NULL argument");
  CK(cudaMemcpyAsync(u0, h->d_scal + 1, sizeof(double) * h->g.ndof, cudaMemcpyDeviceToHost,
                     h->stream),
     "gfmd_get_u0");
  CK(cudaStreamSynchronize(h->stream), "gfmd_get_u0");
  return GFMD_OK;
}

// ---- stiffness-kernel tables ----------------------------------------------

int gfmd_kernel_create(const char *args, gfmd_kernel_t *out) {
  if (!args || !out) return fail(GFMD_EINVAL, "gfmd_kernel_create: NULL argument");
  *out = nullptr;
  std::istringstream is(args);
  std::vector<std::string> tok;
  std::string t;
  while (is >> t) tok.push_back(t);
  try {
    size_t pos = 0;
    std::unique_ptr<gfmd::StiffnessKernel> k(gfmd::StiffnessKernel::create(tok, pos));
    if (pos != tok.size())
      return fail(GFMD_EINVAL, "gfmd_kernel_create: unexpected argument '" + tok[pos] + "'");
    *out = new gfmd_kernel{std::move(k)};
  } catch (const std::exception &ex) {
    return fail(GFMD_EINVAL, std::string("gfmd_kernel_create: ") + ex.what());
  }
  return GFMD_OK;
}

int gfmd_kernel_destroy(gfmd_kernel_t k) {
  if (!k) return fail(GFMD_EINVAL, "gfmd_kernel_destroy: NULL kernel");
  delete k;
  return GFMD_OK;
}

int gfmd_kernel_info(gfmd_kernel_t k, int *ndof, int *height) {
  if (!k) return fail(GFMD_EINVAL, "gfmd_kernel_info: NULL kernel");
  if (ndof) *ndof = k->k->ndof();
  if (height) *height = k->k->height();
  return GFMD_OK;
}

int gfmd_kernel_set_box(gfmd_kernel_t k, double xprd, double yprd) {
  if (!k) return fail(GFMD_EINVAL, "gfmd_kernel_set_box: NULL kernel");
  if (!(xprd >= 0.0) || !(yprd >= 0.0) || !std::isfinite(xprd) || !std::isfinite(yprd))
    return fail(GFMD_EINVAL, "gfmd_kernel_set_box: box lengths must be finite and >= 0");
  k->k->set_box(xprd, yprd);
  return GFMD_OK;
}

int gfmd_kernel_phi(gfmd_kernel_t k, int nx, int ny, int layout, double *phi, double *linf,
                    int nthreads) {
  if (!k || !phi) return fail(GFMD_EINVAL, "gfmd_kernel_phi: NULL argument");
  std::string err = gfmd::fill_phi_table(*k->k, nx, ny, layout, phi, nthreads);
  if (!err.empty()) return fail(GFMD_EINVAL, "gfmd_kernel_phi: " + err);
  if (linf) {
    std::vector<double> l = k->k->linf();
    for (size_t i = 0; i < l.size(); i++) linf[i] = l[i];
  }
  return GFMD_OK;
}

}  // extern "C"
