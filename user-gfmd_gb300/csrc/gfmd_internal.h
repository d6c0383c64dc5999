// Internal declarations shared by the CUDA translation units of gfmd_gb300.
#ifndef GFMD_GB300_INTERNAL_H
#define GFMD_GB300_INTERNAL_H

#include <cuda.h>
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/gfmd_gb300.h"

namespace gfmd {

constexpr int kMaxStages = 24;
constexpr int kMaxNdof = 24;

// Mixed-radix Stockham plan of a length-n complex transform.  Stage s has
// radix radix[s] and span (product of earlier radices) span[s]; its forward
// twiddles exp(-2 pi i r k / (span*radix)) sit at twoff[s] + k*radix + r of
// the handle's twiddle table, and for radices without a hand-written
// butterfly the roots exp(-2 pi i m / radix) sit at rootoff[s] + m.
struct FftPlan {
  int n;
  int nst;
  int radix[kMaxStages];
  int span[kMaxStages];
  int twoff[kMaxStages];
  int rootoff[kMaxStages];
};

// Builds the plan and appends its twiddles (FP64) to `tw`.
FftPlan make_plan(int n, std::vector<double> &tw);

// Power-of-two plan of the fused kernels: in-place decimation-in-frequency
// stages with radices radix[0..nst) (16s, then one 8, 4 or 2); twiddles
// w_n^k, k = 0..n-1, at table offset twoff.
struct P2Plan {
  int n, lgn;
  int nst;
  int radix[4];
  int lg[4];     // log2 radix
  int toff[4];   // table entry offset of each stage's [j][m] twiddles
  int tpost;     // entry offset of the real-to-complex post-twiddles (rows)
  int tsize;     // table entries (16 bytes each)
};

// Geometry of one solver handle.
struct Geom {
  int nx, ny, ndof;
  int nyc;      // ny/2 + 1 stored wavevectors along y
  int nxp;      // padded row pitch (elements) of the spectrum and Phi arrays
  int ny_even;  // ny even: real rows go through a half-length complex FFT
  int nrow;     // length of the complex row transform (ny/2 or ny)
  int rpost;    // table offset of exp(-2 pi i k/ny), k = 0..ny/2
  int npk;      // packed Phi reals per wavevector (= ndof*ndof)
};

struct Launch;  // per-precision launch parameters (force_kernels.cu)

}  // namespace gfmd

struct gfmd_solver {
  gfmd::Geom g;
  int precision;
  cudaStream_t stream = nullptr;
  int device = 0;
  int sm_count = 0;
  size_t smem_optin = 0;

  gfmd::FftPlan plan_row{}, plan_col{};
  void *d_tw_hi = nullptr;   // double2 (FP64) or float2 (FP32) twiddles
  void *d_tw_lo = nullptr;   // float2 residuals (FP32 only)
  void *d_W = nullptr;       // spectrum [nyc][ndof][nxp] complex
  void *d_phi = nullptr;     // packed Phi [nyc][npk][nxp] real
  double *d_linf = nullptr;  // [ndof/3]
  double *d_zero = nullptr;  // [kMaxNdof] zeros (linf switched off)
  double *d_epart = nullptr; // per-block energy partials
  double *d_scal = nullptr;  // [0] energy, [1..ndof] u(q=0)
  void *d_io = nullptr;      // staging for host-buffer calls: u then f, FP64
  int n_epart = 0;
  bool have_phi = false;

  // fused power-of-two path (see gfmd_fast_kernels.cuh)
  bool fast = false;
  gfmd::P2Plan p2_row{}, p2_col{};
  int fast_rb = 8;           // rows per block of the row kernels (tuned)
  int fast_rb_max = 8;       // largest that fits the shared-memory budget
  int fast_pf = 1;           // Phi prefetch depth of the column kernel (rounds)
  bool tuned = false;
  void *d_ftw = nullptr;     // octant tables of w_ny and w_nx (see gfmd_fast_kernels.cuh)
  int ftw_col_off = 0;       // entry offset of the w_nx table
  unsigned *d_counter = nullptr;  // blocks finished in the column kernel
  int fast_rpost = 0;
  double bytes = 0.0;

  // FP32 kernels of the fused path (gfmd_rows_warp.cuh, gfmd_col_cluster.cuh)
  bool rows32 = false;       // warp-per-row row kernels with TMA tiles (ny = 2048)
  int col_cl = 0;            // blocks per ky of the cluster column kernel (0: not used)
  int phi_v = 1;             // packed-Phi vector width of that kernel (1 or 4)
  int phi_pat = 0;           // storage pattern of the packed table (pat_keeps), chosen at upload
  std::vector<int> phi_slot; // pattern != 0: float slot of each dense element (-1: structural zero)
  bool col_r32 = false;      // register-transform column kernel (nx = 1024, 2048): positions
                             // q = (nx/32) (kx mod 32) + kx/32; else digit-reversed kx
  void *d_twc = nullptr;     // float4 [k1][t] w_nx^(t k1) of that kernel
  int col_pf = 1;            // Phi rounds prefetched into L2 ahead (tuned)
  int col_minb = 2;          // resident blocks per SM the kernel is compiled for (tuned: 2-4)
  void *d_tw32 = nullptr;    // float4: [k1][l] w_1024^(l k1), then e^{-2 pi i k/2048}, k = 0..1024
  CUtensorMap tm_w[2];       // W as floats {2 nxp, ndof, nyc}, boxes {16, 1, 128} and {32, 1, 64}
  int row_rb = 8;            // rows per block of those kernels (8 or 16, tuned)
  int *d_err = nullptr;      // device error word: GFMD_ETIMEDOUT from a bounded wait
  cudaEvent_t *mark = nullptr;  // when set: events recorded around each launch
  int nmark = 0;

  // solver workspace, kept between solves (gfmd_cg.cu)
  void *ws = nullptr;
  size_t ws_bytes = 0;
  void *ws_host = nullptr;   // pinned control block

  // handle applying (Phi/(nx ny) + Cavg)^{-1}, built by gfmd_prec_gradient for
  // the Cavg it holds; dropped when the table changes
  gfmd_solver *prec_grad = nullptr;
  std::vector<double> prec_cavg;
};

namespace gfmd {
// Storage patterns of the packed table (register-transform column kernel).
// PAT 0: every pair.  PAT 1 (layer-tridiagonal): the pairs inside a layer's
// 3x3 block and between adjacent layers; blocks of layers two or more apart
// are zero.  PAT 2: as 1, and the 3x3 blocks of all layers but the last are
// diagonal (the table of a slab with nearest-neighbour interactions whose
// last layer carries the substrate below).  The kept pairs stay in row-major
// order, so every force component sums the same nonzero terms in the same
// order as with PAT 0; an element of a pattern is D diagonal reals followed
// by the (Re, Im) of the kept pairs, padded to a multiple of 4 floats.
constexpr bool pat_keeps(int D, int PAT, int i, int j) {
  const int li = i / 3, lj = j / 3;
  if (PAT == 0) return true;
  if (lj - li >= 2) return false;
  if (PAT == 2 && li == lj && li < D / 3 - 1) return false;
  return true;
}
constexpr int pat_pairs(int D, int PAT) {
  int n = 0;
  for (int i = 0; i < D; i++)
    for (int j = i + 1; j < D; j++) n += pat_keeps(D, PAT, i, j) ? 1 : 0;
  return n;
}
// row (which = 0) or column (1) of the p-th kept pair
constexpr int pat_pair(int D, int PAT, int p, int which) {
  for (int i = 0; i < D; i++)
    for (int j = i + 1; j < D; j++)
      if (pat_keeps(D, PAT, i, j)) {
        if (p == 0) return which == 0 ? i : j;
        p--;
      }
  return -1;
}
constexpr int pat_floats(int D, int PAT) { return (D + 2 * pat_pairs(D, PAT) + 3) / 4 * 4; }
// phi_index of an element outside the handle's storage pattern
constexpr size_t kPhiAbsent = ~(size_t)0;

// Enqueue one force evaluation.  u/f are [ndof][nx*ny] of type in_t/out_t
// (0 = double, 1 = float); energy -> d_epot (device double).
cudaError_t enqueue_force(gfmd_solver *h, const void *d_u, int in_t, void *d_f, int out_t,
                          double *d_epot);
// The same with the gamma-point linear force switched off (with_linf = false),
// for the force of a search direction.
cudaError_t enqueue_force_opts(gfmd_solver *h, const void *d_u, int in_t, void *d_f, int out_t,
                               double *d_epot, bool with_linf);
// Polak-Ribiere CG with device-side control (gfmd_cg.cu).
int cg_minimize(gfmd_solver *hp, const gfmd_obstacle_t *ob, const gfmd_min_params_t *prm, double *u,
                gfmd_min_report_t *rep, std::string &err);
// Records msg as the calling thread's gfmd_last_error() and returns code.
int set_error(int code, const std::string &msg);
// The register-transform column kernel of h on W (gfmd_col_r32.cu), and its
// instances for structured ndof-12 tables (gfmd_col_r32_pat.cu).
cudaError_t enqueue_col_r32(gfmd_solver *h, float2 *W, double *d_epot);
cudaError_t enqueue_col_r32_pat(gfmd_solver *h, float2 *W, double *d_epot);
// The fused shared-memory column kernel of h on W (C<float> / C<double>)
// with dynamic shared memory smem (gfmd_col_fast_f32.cu, gfmd_col_fast_f64.cu).
cudaError_t enqueue_col_fast_f32(gfmd_solver *h, void *W, size_t smem, double *d_epot);
cudaError_t enqueue_col_fast_f64(gfmd_solver *h, void *W, size_t smem, double *d_epot);
// The thread-block-cluster column kernel of h on W (gfmd_col_cl.cu).
cudaError_t enqueue_col_cl(gfmd_solver *h, float2 *W, double *d_epot);
// Warp-per-row TMA row transforms: u (in_t) -> W, W -> f (out_t) (gfmd_rows32.cu).
cudaError_t enqueue_row_fwd32(gfmd_solver *h, const void *d_u, int in_t);
cudaError_t enqueue_row_inv32(gfmd_solver *h, void *d_f, int out_t);
// Phi application of the general-size path on the grid `grid` of
// wavevector blocks (gfmd_phi_plain_f32.cu, gfmd_phi_plain_f64.cu).
cudaError_t enqueue_phi_plain_f32(gfmd_solver *h, dim3 grid);
cudaError_t enqueue_phi_plain_f64(gfmd_solver *h, dim3 grid);
// Kernel launches one force evaluation makes.
int force_launches(const gfmd_solver *h);
// Index (in reals) of packed element e of the wavevector at storage position
// pos (digit-reversed kx on the fused path, kx otherwise) of row ky.
size_t phi_index(const gfmd_solver *h, int ky, int pos, int e);
// Reals per wavevector of h's packed table (every pair, or its storage pattern's).
int phi_reals(const gfmd_solver *h);
// Device bytes of the spectrum/Phi arrays and the number of energy partials.
void force_layout(const Geom &g, int precision, size_t *w_bytes, size_t *phi_bytes, int *n_epart);
}  // namespace gfmd

#endif
