// Learned warm start: a BF16 convolutional encoder-decoder that maps
// (indenter height map, load) to a displacement field, trained and run with
// hand-written tensor-core kernels.  No counterpart in the reference.
//
// Network (periodic 3x3 convolutions, C base channels, 4 levels):
//   a1 = relu(conv1(x))      C    H        a5 = relu(conv5(pool(a4)))  2C  H/8
//   a2 = relu(conv2(a1))     C    H        s2 = up(a5) + a4             2C  H/4
//   a3 = relu(conv3(pool a2)) 2C  H/2      a6 = relu(conv6(s2))         2C  H/4
//   a4 = relu(conv4(pool a3)) 2C  H/4      s1 = up(a6) + a3             2C  H/2
//                                          a7 = relu(conv7(s1))         C   H/2
//                                          s0 = up(a7) + a2             C   H
//                                          a8 = relu(conv8(s0))         C   H
//                                          y  = conv9(a8)               out H
// pool = 2x2 average, up = nearest 2x.  Tensors are NHWC FP32 in HBM; the
// convolutions are implicit GEMMs on the tensor cores (mma.sync m16n8k16,
// BF16 operands converted while staging tiles in shared memory, FP32
// accumulation): forward and data gradient share one kernel (the data
// gradient is the convolution of the output gradient with the flipped,
// transposed filter); the weight gradient is a split-K GEMM over pixels with
// a fixed-order reduction of the per-chunk partials (deterministic).  Master
// weights and Adam moments are FP32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "gfmd_internal.h"

struct gfmd_ws_net;

namespace gfmd {
namespace {

constexpr int kConvThreads = 128;  // 4 warps, 16 pixels each
constexpr int kTileM = 64;         // pixels per block
constexpr int kPitch = 24;         // bf16 row pitch of the staged tiles (16 + 8)
constexpr int kDwChunks = 64;      // pixel chunks of the weight gradient

__device__ __forceinline__ int nbr_pixel(int p, int t, int H, int W, int flip) {
  const int HW = H * W;
  const int n = p / HW, r = p - n * HW;
  const int y = r / W, x = r - y * W;
  int dy = t / 3 - 1, dx = t % 3 - 1;
  if (flip) {
    dy = -dy;
    dx = -dx;
  }
  int yy = y + dy, xx = x + dx;
  yy = yy < 0 ? yy + H : (yy >= H ? yy - H : yy);
  xx = xx < 0 ? xx + W : (xx >= W ? xx - W : xx);
  return n * HW + yy * W + xx;
}

__device__ __forceinline__ void mma_bf16(float d[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// Y[p][co] = act(sum_{t, k} X[nbr(p, t)][k] * B[t][k][co] + bias[co]) for
// co < Cy.  B is packed BF16 [9][nkc][NT][16] (k within a 16-chunk
// innermost); X has Cx channels (k >= Cx read as zero).
template <int NT>
__global__ void __launch_bounds__(kConvThreads) k_conv(const float *__restrict__ X, int Cx, int P, int H, int W,
                                                       const __nv_bfloat16 *__restrict__ B, int nkc,
                                                       const float *__restrict__ bias, float *__restrict__ Y,
                                                       int Cy, int relu, int flip) {
  __shared__ __align__(16) __nv_bfloat16 As[kTileM][kPitch];
  __shared__ __align__(16) __nv_bfloat16 Bt[NT][kPitch];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int p0 = blockIdx.x * kTileM;
  float acc[NT / 8][4];
#pragma unroll
  for (int j = 0; j < NT / 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
  // this thread's staging slot of the A tile: pixel tid/2, channels (tid&1)*8..+8
  const int ap = tid >> 1, ac = (tid & 1) * 8;
  const int pix = p0 + ap;
  for (int t = 0; t < 9; t++) {
    const int q = pix < P ? nbr_pixel(pix, t, H, W, flip) : -1;
    for (int kc = 0; kc < nkc; kc++) {
      // A: 8 consecutive channels of pixel q
      __nv_bfloat162 v[4];
#pragma unroll
      for (int e = 0; e < 4; e++) {
        const int c0 = kc * 16 + ac + 2 * e;
        float lo = 0.0f, hi = 0.0f;
        if (q >= 0) {
          if (c0 < Cx) lo = X[(size_t)q * Cx + c0];
          if (c0 + 1 < Cx) hi = X[(size_t)q * Cx + c0 + 1];
        }
        v[e] = __floats2bfloat162_rn(lo, hi);
      }
      *reinterpret_cast<uint4 *>(&As[ap][ac]) = *reinterpret_cast<uint4 *>(v);
      // B: NT x 16 bf16, contiguous; one 16-byte chunk per thread
      const __nv_bfloat16 *bsrc = B + ((size_t)(t * nkc + kc) * NT) * 16;
      for (int ch = tid; ch < NT * 2; ch += kConvThreads) {
        const int n = ch >> 1, h8 = (ch & 1) * 8;
        *reinterpret_cast<uint4 *>(&Bt[n][h8]) = *reinterpret_cast<const uint4 *>(bsrc + n * 16 + h8);
      }
      __syncthreads();
      const int r = warp * 16 + (lane >> 2), c = (lane & 3) * 2;
      uint32_t a[4];
      a[0] = *reinterpret_cast<const uint32_t *>(&As[r][c]);
      a[1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][c]);
      a[2] = *reinterpret_cast<const uint32_t *>(&As[r][c + 8]);
      a[3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][c + 8]);
#pragma unroll
      for (int j = 0; j < NT / 8; j++) {
        const int n = j * 8 + (lane >> 2);
        uint32_t b[2];
        b[0] = *reinterpret_cast<const uint32_t *>(&Bt[n][c]);
        b[1] = *reinterpret_cast<const uint32_t *>(&Bt[n][c + 8]);
        mma_bf16(acc[j], a, b);
      }
      __syncthreads();
    }
  }
  // epilogue
  const int r0 = p0 + warp * 16 + (lane >> 2);
#pragma unroll
  for (int j = 0; j < NT / 8; j++) {
    const int co = j * 8 + (lane & 3) * 2;
#pragma unroll
    for (int h = 0; h < 2; h++) {
      const int p = r0 + h * 8;
      if (p >= P) continue;
#pragma unroll
      for (int e = 0; e < 2; e++) {
        const int cc = co + e;
        if (cc >= Cy) continue;
        float v = acc[j][2 * h + e] + (bias ? bias[cc] : 0.0f);
        if (relu) v = fmaxf(v, 0.0f);
        Y[(size_t)p * Cy + cc] = v;
      }
    }
  }
}

// Weight gradient partials: part[chunk][t][k][co] = sum over the chunk's
// pixels p of X[nbr(p, t)][k] * G[p][co]  (k < KP, co < NT).  Grid
// (kDwChunks, 9); warp w handles k in [16 w, 16 w + 16).
template <int NT>
__global__ void __launch_bounds__(kConvThreads) k_conv_dw(const float *__restrict__ X, int Cx, const float *__restrict__ G,
                                                          int Cg, int P, int H, int W, int KP,
                                                          float *__restrict__ part) {
  __shared__ __align__(16) __nv_bfloat16 As[64][kPitch];   // [k][pixel]
  __shared__ __align__(16) __nv_bfloat16 Bt[NT][kPitch];   // [co][pixel]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int chunk = blockIdx.x, t = blockIdx.y;
  const int per = (P + kDwChunks - 1) / kDwChunks;
  const int pa = chunk * per, pb = min(P, pa + per);
  float acc[NT / 8][4];
#pragma unroll
  for (int j = 0; j < NT / 8; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.0f;
  for (int p0 = pa; p0 < pb; p0 += 16) {
    // stage X (transposed: [k][px]) and G ([co][px]); zero beyond the chunk
    for (int i = tid; i < KP * 16; i += kConvThreads) {
      const int px = i % 16, k = i / 16;
      const int p = p0 + px;
      float v = 0.0f;
      if (p < pb && k < Cx) v = X[(size_t)nbr_pixel(p, t, H, W, 0) * Cx + k];
      As[k][px] = __float2bfloat16_rn(v);
    }
    for (int i = tid; i < NT * 16; i += kConvThreads) {
      const int px = i % 16, co = i / 16;
      const int p = p0 + px;
      float v = 0.0f;
      if (p < pb && co < Cg) v = G[(size_t)p * Cg + co];
      Bt[co][px] = __float2bfloat16_rn(v);
    }
    __syncthreads();
    if (warp * 16 < KP) {
      const int r = warp * 16 + (lane >> 2), c = (lane & 3) * 2;
      uint32_t a[4];
      a[0] = *reinterpret_cast<const uint32_t *>(&As[r][c]);
      a[1] = *reinterpret_cast<const uint32_t *>(&As[r + 8][c]);
      a[2] = *reinterpret_cast<const uint32_t *>(&As[r][c + 8]);
      a[3] = *reinterpret_cast<const uint32_t *>(&As[r + 8][c + 8]);
#pragma unroll
      for (int j = 0; j < NT / 8; j++) {
        const int n = j * 8 + (lane >> 2);
        uint32_t b[2];
        b[0] = *reinterpret_cast<const uint32_t *>(&Bt[n][c]);
        b[1] = *reinterpret_cast<const uint32_t *>(&Bt[n][c + 8]);
        mma_bf16(acc[j], a, b);
      }
    }
    __syncthreads();
  }
  if (warp * 16 >= KP) return;
  const int k0 = warp * 16 + (lane >> 2);
  float *out = part + ((size_t)(chunk * 9 + t) * KP) * NT;
#pragma unroll
  for (int j = 0; j < NT / 8; j++) {
    const int co = j * 8 + (lane & 3) * 2;
    out[(size_t)k0 * NT + co] = acc[j][0];
    out[(size_t)k0 * NT + co + 1] = acc[j][1];
    out[(size_t)(k0 + 8) * NT + co] = acc[j][2];
    out[(size_t)(k0 + 8) * NT + co + 1] = acc[j][3];
  }
}

// dW[co][t][k] = sum over chunks (fixed order) of part[chunk][t][k][co].
__global__ void k_dw_reduce(const float *__restrict__ part, int KP, int NT, int Cx, int Cy,
                            float *__restrict__ dW) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int total = Cy * 9 * Cx;
  if (i >= total) return;
  const int k = i % Cx, t = (i / Cx) % 9, co = i / (9 * Cx);
  float s = 0.0f;
  for (int c = 0; c < kDwChunks; c++) s += part[((size_t)(c * 9 + t) * KP + k) * NT + co];
  dW[i] = s;
}

// Bias gradient partials and reduction: db[co] = sum_p G[p][co].
__global__ void k_db_part(const float *__restrict__ G, int Cg, int P, float *__restrict__ part) {
  const int co = threadIdx.x;  // blockDim = Cg
  const int per = (P + gridDim.x - 1) / gridDim.x;
  const int pa = blockIdx.x * per, pb = min(P, pa + per);
  float s = 0.0f;
  for (int p = pa; p < pb; p++) s += G[(size_t)p * Cg + co];
  part[blockIdx.x * Cg + co] = s;
}
__global__ void k_db_reduce(const float *__restrict__ part, int nb, int Cg, float *__restrict__ db) {
  const int co = threadIdx.x;
  if (co >= Cg) return;
  float s = 0.0f;
  for (int b = 0; b < nb; b++) s += part[b * Cg + co];
  db[co] = s;
}

// Pack master weights W[co][t][k] (FP32) into the B operands:
//   forward  Bf[t][kc][NTf][16]: Bf(t, k, n = co)
//   backward Bb[t'][kc][NTb][16]: Bb(t', k = co, n = ci) = W[co][8 - t'][ci]
__global__ void k_pack(const float *__restrict__ Wm, int Cout, int Cin, __nv_bfloat16 *__restrict__ Bf, int nkcf,
                       int NTf, __nv_bfloat16 *__restrict__ Bb, int nkcb, int NTb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nf = 9 * nkcf * NTf * 16, nbk = 9 * nkcb * NTb * 16;
  if (i < nf) {
    const int kk = i % 16, n = (i / 16) % NTf, kc = (i / (16 * NTf)) % nkcf, t = i / (16 * NTf * nkcf);
    const int k = kc * 16 + kk;
    float v = (n < Cout && k < Cin) ? Wm[((size_t)n * 9 + t) * Cin + k] : 0.0f;
    Bf[i] = __float2bfloat16_rn(v);
  } else if (i < nf + nbk) {
    const int j = i - nf;
    const int kk = j % 16, n = (j / 16) % NTb, kc = (j / (16 * NTb)) % nkcb, t = j / (16 * NTb * nkcb);
    const int co = kc * 16 + kk, ci = n;
    float v = (co < Cout && ci < Cin) ? Wm[((size_t)co * 9 + (8 - t)) * Cin + ci] : 0.0f;
    Bb[j] = __float2bfloat16_rn(v);
  }
}

__global__ void k_pool(const float *__restrict__ X, int C, int Pb, int H, int W, float *__restrict__ Y) {
  // Y has H/2 x W/2 pixels per image; Pb = batch * H/2 * W/2
  const int Ho = H / 2, Wo = W / 2;
  const size_t total = (size_t)Pb * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = i % C;
    const int p = (int)(i / C);
    const int n = p / (Ho * Wo), r = p % (Ho * Wo), y = r / Wo, x = r % Wo;
    const size_t b = ((size_t)n * H + 2 * y) * W + 2 * x;
    Y[i] = 0.25f * (X[b * C + c] + X[(b + 1) * C + c] + X[(b + W) * C + c] + X[(b + W + 1) * C + c]);
  }
}

// G_in[fine] (+)= 0.25 G[coarse] (pool backward); acc = 1 adds, 0 assigns.
__global__ void k_pool_bwd(const float *__restrict__ G, int C, int Pf, int H, int W, float *__restrict__ Gin, int acc) {
  const size_t total = (size_t)Pf * C;
  const int Wo = W / 2, Ho = H / 2;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = i % C;
    const int p = (int)(i / C);
    const int n = p / (H * W), r = p % (H * W), y = r / W, x = r % W;
    const float v = 0.25f * G[(((size_t)n * Ho + y / 2) * Wo + x / 2) * C + c];
    Gin[i] = acc ? Gin[i] + v : v;
  }
}

// S[fine] = A[coarse(p)] + skip[fine]
__global__ void k_up_add(const float *__restrict__ A, const float *__restrict__ skip, int C, int Pf, int H, int W,
                         float *__restrict__ S) {
  const size_t total = (size_t)Pf * C;
  const int Wo = W / 2, Ho = H / 2;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = i % C;
    const int p = (int)(i / C);
    const int n = p / (H * W), r = p % (H * W), y = r / W, x = r % W;
    S[i] = A[(((size_t)n * Ho + y / 2) * Wo + x / 2) * C + c] + skip[i];
  }
}

// G_coarse[q] = sum of the 4 fine gradients (up backward)
__global__ void k_up_bwd(const float *__restrict__ G, int C, int Pc, int H, int W, float *__restrict__ Gc) {
  // H, W fine sizes; Pc = batch * H/2 * W/2
  const size_t total = (size_t)Pc * C;
  const int Ho = H / 2, Wo = W / 2;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = i % C;
    const int p = (int)(i / C);
    const int n = p / (Ho * Wo), r = p % (Ho * Wo), y = r / Wo, x = r % Wo;
    const size_t b = ((size_t)n * H + 2 * y) * W + 2 * x;
    Gc[i] = G[b * C + c] + G[(b + 1) * C + c] + G[(b + W) * C + c] + G[(b + W + 1) * C + c];
  }
}

// G *= (A > 0)   (relu backward on the layer output A)
__global__ void k_relu_mask(float *__restrict__ G, const float *__restrict__ A, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    if (!(A[i] > 0.0f)) G[i] = 0.0f;
}

// MSE loss L = mean((Y - T)^2) over n; G = 2 (Y - T) / n; block partials of
// the squared error in FP64, summed in a fixed order by k_sum_d.
__global__ void k_mse(const float *__restrict__ Y, const float *__restrict__ T, size_t n, float *__restrict__ G,
                      double *__restrict__ part) {
  __shared__ double sh[8];
  double s = 0.0;
  const float sc = 2.0f / (float)n;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float d = Y[i] - T[i];
    G[i] = sc * d;
    s += (double)d * (double)d;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += sh[w];
    part[blockIdx.x] = t;
  }
}
__global__ void k_sum_d(const double *__restrict__ part, int nb, double scale, double *__restrict__ out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double s = 0.0;
  for (int b = 0; b < nb; b++) s += part[b];
  out[0] = s * scale;
}

// Adam (Kingma and Ba 2015) on FP32 master parameters.
__global__ void k_adam(float *__restrict__ w, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, size_t n, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

// Solver layout [ndof][H*W] (per image, FP64) <-> NHWC FP32.
__global__ void k_to_nhwc(const double *__restrict__ u, int C, int HW, float scale, float *__restrict__ out) {
  const size_t total = (size_t)HW * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = i % C, p = (int)(i / C);
    out[i] = (float)(u[(size_t)c * HW + p] * scale);
  }
}
__global__ void k_from_nhwc(const float *__restrict__ in, int C, int HW, double scale, double *__restrict__ u) {
  const size_t total = (size_t)HW * C;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int c = i % C, p = (int)(i / C);
    u[(size_t)c * HW + p] = (double)in[i] * scale;
  }
}

int pad8(int c) { return (c + 7) / 8 * 8; }
int pad16(int c) { return (c + 15) / 16 * 16; }

struct Conv {
  int cin, cout;
  size_t w_off, b_off;      // into the parameter array
  int nkcf, ntf, nkcb, ntb;  // packed operand shapes
  __nv_bfloat16 *bf = nullptr, *bb = nullptr;
};

}  // namespace
}  // namespace gfmd

struct gfmd_ws_net {
  int in_ch, out_ch, base;
  std::vector<gfmd::Conv> conv;  // 9 layers
  size_t nparam = 0;
  float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16 *packed = nullptr;
  size_t packed_n = 0;
  bool packed_valid = false;
  long step = 0;
  cudaStream_t stream = nullptr;
  // activations for the current (batch, H, W)
  int batch = 0, H = 0, W = 0;
  void *act = nullptr;
  size_t act_bytes = 0;
  float *dw_part = nullptr;
  double *d_red = nullptr;   // reduction scratch
  float *db_part = nullptr;
};

namespace gfmd {
namespace {

struct Acts {
  float *x, *a1, *a2, *p1, *a3, *p2, *a4, *p3, *a5, *s2, *a6, *s1, *a7, *s0, *a8, *y;
  float *g0, *g1, *g2, *g3;  // gradient scratch: two at full size, two at half size
};

size_t up256(size_t x) { return (x + 255) / 256 * 256; }

cudaError_t ensure_acts(gfmd_ws_net *n, int batch, int H, int W, Acts &A) {
  const int C = n->base, C2 = 2 * n->base;
  const size_t P0 = (size_t)batch * H * W, P1 = P0 / 4, P2 = P0 / 16, P3 = P0 / 64;
  const size_t sz[] = {P0 * n->in_ch, P0 * C, P0 * C, P1 * C, P1 * C2, P2 * C2, P2 * C2, P3 * C2, P3 * C2,
                       P2 * C2, P2 * C2, P1 * C2, P1 * C, P0 * C, P0 * C, P0 * n->out_ch,
                       P0 * std::max(C2, n->out_ch), P0 * C2, P1 * C2, P1 * C2};
  const int nb = (int)(sizeof(sz) / sizeof(sz[0]));
  size_t tot = 0;
  for (int i = 0; i < nb; i++) tot += up256(sz[i] * sizeof(float));
  if (tot > n->act_bytes) {
    if (n->act) cudaFree(n->act);
    n->act = nullptr;
    n->act_bytes = 0;
    cudaError_t e = cudaMalloc(&n->act, tot);
    if (e != cudaSuccess) return e;
    n->act_bytes = tot;
  }
  char *a = static_cast<char *>(n->act);
  float **dst[] = {&A.x, &A.a1, &A.a2, &A.p1, &A.a3, &A.p2, &A.a4, &A.p3, &A.a5, &A.s2, &A.a6, &A.s1, &A.a7, &A.s0,
                   &A.a8, &A.y, &A.g0, &A.g1, &A.g2, &A.g3};
  for (int i = 0; i < nb; i++) {
    *dst[i] = reinterpret_cast<float *>(a);
    a += up256(sz[i] * sizeof(float));
  }
  n->batch = batch;
  n->H = H;
  n->W = W;
  return cudaSuccess;
}

cudaError_t pack_weights(gfmd_ws_net *n) {
  if (n->packed_valid) return cudaSuccess;
  for (Conv &c : n->conv) {
    const int tot = 9 * c.nkcf * c.ntf * 16 + 9 * c.nkcb * c.ntb * 16;
    k_pack<<<(tot + 255) / 256, 256, 0, n->stream>>>(n->w + c.w_off, c.cout, c.cin, c.bf, c.nkcf, c.ntf, c.bb, c.nkcb,
                                                     c.ntb);
  }
  n->packed_valid = true;
  return cudaGetLastError();
}

template <int NT>
void launch_conv_t(cudaStream_t st, const float *X, int Cx, int P, int H, int W, const __nv_bfloat16 *B, int nkc,
                   const float *bias, float *Y, int Cy, int relu, int flip) {
  k_conv<NT><<<(P + kTileM - 1) / kTileM, kConvThreads, 0, st>>>(X, Cx, P, H, W, B, nkc, bias, Y, Cy, relu, flip);
}

void launch_conv(cudaStream_t st, int NT, const float *X, int Cx, int P, int H, int W, const __nv_bfloat16 *B, int nkc,
                 const float *bias, float *Y, int Cy, int relu, int flip) {
  switch (NT) {
    case 8: launch_conv_t<8>(st, X, Cx, P, H, W, B, nkc, bias, Y, Cy, relu, flip); break;
    case 16: launch_conv_t<16>(st, X, Cx, P, H, W, B, nkc, bias, Y, Cy, relu, flip); break;
    case 32: launch_conv_t<32>(st, X, Cx, P, H, W, B, nkc, bias, Y, Cy, relu, flip); break;
    default: launch_conv_t<64>(st, X, Cx, P, H, W, B, nkc, bias, Y, Cy, relu, flip); break;
  }
}

template <int NT>
void launch_dw_t(cudaStream_t st, const float *X, int Cx, const float *G, int Cg, int P, int H, int W, int KP,
                 float *part) {
  k_conv_dw<NT><<<dim3(kDwChunks, 9), kConvThreads, 0, st>>>(X, Cx, G, Cg, P, H, W, KP, part);
}

// Weight and bias gradients of conv c with input X (Cx channels) and output
// gradient G (already masked), at P pixels of size H x W.
void conv_grads(gfmd_ws_net *n, const Conv &c, const float *X, const float *G, int P, int H, int W) {
  cudaStream_t st = n->stream;
  const int KP = pad16(c.cin), NT = pad8(c.cout);
  switch (NT) {
    case 8: launch_dw_t<8>(st, X, c.cin, G, c.cout, P, H, W, KP, n->dw_part); break;
    case 16: launch_dw_t<16>(st, X, c.cin, G, c.cout, P, H, W, KP, n->dw_part); break;
    case 32: launch_dw_t<32>(st, X, c.cin, G, c.cout, P, H, W, KP, n->dw_part); break;
    default: launch_dw_t<64>(st, X, c.cin, G, c.cout, P, H, W, KP, n->dw_part); break;
  }
  const int tot = c.cout * 9 * c.cin;
  k_dw_reduce<<<(tot + 255) / 256, 256, 0, st>>>(n->dw_part, KP, NT, c.cin, c.cout, n->g + c.w_off);
  k_db_part<<<64, c.cout, 0, st>>>(G, c.cout, P, n->db_part);
  k_db_reduce<<<1, 64, 0, st>>>(n->db_part, 64, c.cout, n->g + c.b_off);
}

void conv_fwd(gfmd_ws_net *n, const Conv &c, const float *X, float *Y, int P, int H, int W, int relu) {
  launch_conv(n->stream, c.ntf, X, c.cin, P, H, W, c.bf, c.nkcf, n->w + c.b_off, Y, c.cout, relu, 0);
}
// data gradient: Gin[q] = sum_t G[q - off(t)] W[t] = sum_t' G[q + off(t')] W[8 - t'],
// the forward convolution of G with the tap-flipped, transposed filter Bb
void conv_bwd_data(gfmd_ws_net *n, const Conv &c, const float *G, float *Gin, int P, int H, int W) {
  launch_conv(n->stream, c.ntb, G, c.cout, P, H, W, c.bb, c.nkcb, nullptr, Gin, c.cin, 0, 0);
}

int grid_for(size_t n) { return (int)std::min<size_t>(4096, (n + 255) / 256); }

void forward(gfmd_ws_net *n, Acts &A) {
  const int B = n->batch, H = n->H, W = n->W;
  const int P0 = B * H * W, P1 = P0 / 4, P2 = P0 / 16, P3 = P0 / 64;
  const int C = n->base, C2 = 2 * C;
  cudaStream_t st = n->stream;
  std::vector<Conv> &cv = n->conv;
  conv_fwd(n, cv[0], A.x, A.a1, P0, H, W, 1);
  conv_fwd(n, cv[1], A.a1, A.a2, P0, H, W, 1);
  k_pool<<<grid_for((size_t)P1 * C), 256, 0, st>>>(A.a2, C, P1, H, W, A.p1);
  conv_fwd(n, cv[2], A.p1, A.a3, P1, H / 2, W / 2, 1);
  k_pool<<<grid_for((size_t)P2 * C2), 256, 0, st>>>(A.a3, C2, P2, H / 2, W / 2, A.p2);
  conv_fwd(n, cv[3], A.p2, A.a4, P2, H / 4, W / 4, 1);
  k_pool<<<grid_for((size_t)P3 * C2), 256, 0, st>>>(A.a4, C2, P3, H / 4, W / 4, A.p3);
  conv_fwd(n, cv[4], A.p3, A.a5, P3, H / 8, W / 8, 1);
  k_up_add<<<grid_for((size_t)P2 * C2), 256, 0, st>>>(A.a5, A.a4, C2, P2, H / 4, W / 4, A.s2);
  conv_fwd(n, cv[5], A.s2, A.a6, P2, H / 4, W / 4, 1);
  k_up_add<<<grid_for((size_t)P1 * C2), 256, 0, st>>>(A.a6, A.a3, C2, P1, H / 2, W / 2, A.s1);
  conv_fwd(n, cv[6], A.s1, A.a7, P1, H / 2, W / 2, 1);
  k_up_add<<<grid_for((size_t)P0 * C), 256, 0, st>>>(A.a7, A.a2, C, P0, H, W, A.s0);
  conv_fwd(n, cv[7], A.s0, A.a8, P0, H, W, 1);
  conv_fwd(n, cv[8], A.a8, A.y, P0, H, W, 0);
}

// Backward from dL/dy in A.g0 (full size, out_ch channels).
void backward(gfmd_ws_net *n, Acts &A) {
  const int B = n->batch, H = n->H, W = n->W;
  const int P0 = B * H * W, P1 = P0 / 4, P2 = P0 / 16, P3 = P0 / 64;
  const int C = n->base, C2 = 2 * C;
  cudaStream_t st = n->stream;
  std::vector<Conv> &cv = n->conv;
  // conv9 (input a8)
  conv_grads(n, cv[8], A.a8, A.g0, P0, H, W);
  conv_bwd_data(n, cv[8], A.g0, A.g1, P0, H, W);                       // g1 = dL/da8
  k_relu_mask<<<grid_for((size_t)P0 * C), 256, 0, st>>>(A.g1, A.a8, (size_t)P0 * C);
  conv_grads(n, cv[7], A.s0, A.g1, P0, H, W);
  conv_bwd_data(n, cv[7], A.g1, A.g0, P0, H, W);                       // g0 = dL/ds0 (C)
  k_up_bwd<<<grid_for((size_t)P1 * C), 256, 0, st>>>(A.g0, C, P1, H, W, A.g2);  // g2 = dL/da7
  k_relu_mask<<<grid_for((size_t)P1 * C), 256, 0, st>>>(A.g2, A.a7, (size_t)P1 * C);
  conv_grads(n, cv[6], A.s1, A.g2, P1, H / 2, W / 2);
  conv_bwd_data(n, cv[6], A.g2, A.g3, P1, H / 2, W / 2);               // g3 = dL/ds1 (2C)
  // dL/da6 (quarter size) into g1's storage
  float *ga6 = A.g1;
  k_up_bwd<<<grid_for((size_t)P2 * C2), 256, 0, st>>>(A.g3, C2, P2, H / 2, W / 2, ga6);
  k_relu_mask<<<grid_for((size_t)P2 * C2), 256, 0, st>>>(ga6, A.a6, (size_t)P2 * C2);
  conv_grads(n, cv[5], A.s2, ga6, P2, H / 4, W / 4);
  float *gs2 = A.g1 + (size_t)P2 * C2;                                  // dL/ds2 (2C, quarter)
  conv_bwd_data(n, cv[5], ga6, gs2, P2, H / 4, W / 4);
  float *ga5 = A.g2;                                                    // eighth size
  k_up_bwd<<<grid_for((size_t)P3 * C2), 256, 0, st>>>(gs2, C2, P3, H / 4, W / 4, ga5);
  k_relu_mask<<<grid_for((size_t)P3 * C2), 256, 0, st>>>(ga5, A.a5, (size_t)P3 * C2);
  conv_grads(n, cv[4], A.p3, ga5, P3, H / 8, W / 8);
  float *gp3 = A.g2 + (size_t)P3 * C2;
  conv_bwd_data(n, cv[4], ga5, gp3, P3, H / 8, W / 8);
  // dL/da4 = pool^T(gp3) + gs2 (skip)
  float *ga4 = A.g1 + 2 * (size_t)P2 * C2;
  cudaMemcpyAsync(ga4, gs2, sizeof(float) * (size_t)P2 * C2, cudaMemcpyDeviceToDevice, st);
  k_pool_bwd<<<grid_for((size_t)P2 * C2), 256, 0, st>>>(gp3, C2, P2, H / 4, W / 4, ga4, 1);
  k_relu_mask<<<grid_for((size_t)P2 * C2), 256, 0, st>>>(ga4, A.a4, (size_t)P2 * C2);
  conv_grads(n, cv[3], A.p2, ga4, P2, H / 4, W / 4);
  float *gp2 = A.g1 + 3 * (size_t)P2 * C2;
  conv_bwd_data(n, cv[3], ga4, gp2, P2, H / 4, W / 4);
  // dL/da3 = pool^T(gp2) + g3 (skip dL/ds1)
  k_pool_bwd<<<grid_for((size_t)P1 * C2), 256, 0, st>>>(gp2, C2, P1, H / 2, W / 2, A.g3, 1);
  k_relu_mask<<<grid_for((size_t)P1 * C2), 256, 0, st>>>(A.g3, A.a3, (size_t)P1 * C2);
  conv_grads(n, cv[2], A.p1, A.g3, P1, H / 2, W / 2);
  conv_bwd_data(n, cv[2], A.g3, A.g2, P1, H / 2, W / 2);               // g2 = dL/dp1 (C, half)
  // dL/da2 = pool^T(gp1) + g0 (skip dL/ds0)
  k_pool_bwd<<<grid_for((size_t)P0 * C), 256, 0, st>>>(A.g2, C, P0, H, W, A.g0, 1);
  k_relu_mask<<<grid_for((size_t)P0 * C), 256, 0, st>>>(A.g0, A.a2, (size_t)P0 * C);
  conv_grads(n, cv[1], A.a1, A.g0, P0, H, W);
  conv_bwd_data(n, cv[1], A.g0, A.g1, P0, H, W);                       // g1 = dL/da1
  k_relu_mask<<<grid_for((size_t)P0 * C), 256, 0, st>>>(A.g1, A.a1, (size_t)P0 * C);
  conv_grads(n, cv[0], A.x, A.g1, P0, H, W);
}

// Reproducible initial weights: He-uniform from a SplitMix64 stream.
unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int check_shape(int batch, int H, int W) {
  return batch >= 1 && H >= 8 && W >= 8 && H % 8 == 0 && W % 8 == 0 && (long long)batch * H * W <= (1LL << 30);
}

}  // namespace
}  // namespace gfmd

extern "C" {

int gfmd_ws_create(int in_ch, int out_ch, int base_ch, unsigned long long seed, gfmd_ws_handle_t *out) {
  using namespace gfmd;
  if (!out) return set_error(GFMD_EINVAL, "gfmd_ws_create: out is NULL");
  *out = nullptr;
  if (in_ch < 1 || in_ch > 64 || out_ch < 1 || out_ch > 64 || base_ch < 8 || base_ch > 32 || base_ch % 8)
    return set_error(GFMD_EINVAL, "gfmd_ws_create: channels out of range (in, out <= 64; base 8..32, multiple of 8)");
  auto *n = new gfmd_ws_net();
  n->in_ch = in_ch;
  n->out_ch = out_ch;
  n->base = base_ch;
  const int C = base_ch, C2 = 2 * base_ch;
  const int io[9][2] = {{in_ch, C}, {C, C}, {C, C2}, {C2, C2}, {C2, C2}, {C2, C2}, {C2, C}, {C, C}, {C, out_ch}};
  size_t off = 0, poff = 0;
  for (auto &p : io) {
    Conv c{};
    c.cin = p[0];
    c.cout = p[1];
    c.w_off = off;
    off += (size_t)c.cout * 9 * c.cin;
    c.b_off = off;
    off += c.cout;
    c.nkcf = pad16(c.cin) / 16;
    c.ntf = pad8(c.cout) <= 8 ? 8 : (pad8(c.cout) <= 16 ? 16 : (pad8(c.cout) <= 32 ? 32 : 64));
    c.nkcb = pad16(c.cout) / 16;
    c.ntb = pad8(c.cin) <= 8 ? 8 : (pad8(c.cin) <= 16 ? 16 : (pad8(c.cin) <= 32 ? 32 : 64));
    n->conv.push_back(c);
    poff += (size_t)9 * c.nkcf * c.ntf * 16 + (size_t)9 * c.nkcb * c.ntb * 16;
  }
  n->nparam = off;
  n->packed_n = poff;
  cudaError_t e = cudaMalloc((void **)&n->w, sizeof(float) * off * 4);
  if (e == cudaSuccess) e = cudaMalloc((void **)&n->packed, sizeof(__nv_bfloat16) * poff);
  if (e == cudaSuccess) e = cudaMalloc((void **)&n->dw_part, sizeof(float) * kDwChunks * 9 * 64 * 64);
  if (e == cudaSuccess) e = cudaMalloc((void **)&n->db_part, sizeof(float) * 64 * 64);
  if (e == cudaSuccess) e = cudaMalloc((void **)&n->d_red, sizeof(double) * 4200);
  if (e != cudaSuccess) {
    gfmd_ws_destroy(n);
    return set_error(GFMD_ENOMEM, "gfmd_ws_create: device memory");
  }
  n->g = n->w + off;
  n->m = n->g + off;
  n->v = n->m + off;
  size_t q = 0;
  for (Conv &c : n->conv) {
    c.bf = n->packed + q;
    q += (size_t)9 * c.nkcf * c.ntf * 16;
    c.bb = n->packed + q;
    q += (size_t)9 * c.nkcb * c.ntb * 16;
  }
  std::vector<float> h(off, 0.0f);
  unsigned long long st = seed;
  for (const Conv &c : n->conv) {
    const float lim = std::sqrt(6.0f / (9.0f * c.cin));
    for (size_t i = 0; i < (size_t)c.cout * 9 * c.cin; i++) {
      st = mix64(st);
      const double u = (double)(st >> 11) * 0x1.0p-53;
      h[c.w_off + i] = (float)((2.0 * u - 1.0) * lim);
    }
  }
  e = cudaMemcpy(n->w, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(n->g, 0, sizeof(float) * off * 3);  // g, m, v
  if (e != cudaSuccess) {
    gfmd_ws_destroy(n);
    return set_error(GFMD_ECUDA, "gfmd_ws_create: upload");
  }
  *out = n;
  return GFMD_OK;
}

int gfmd_ws_destroy(gfmd_ws_handle_t n) {
  if (!n) return gfmd::set_error(GFMD_EINVAL, "gfmd_ws_destroy: NULL handle");
  for (void *p : {(void *)n->w, (void *)n->packed, (void *)n->dw_part, (void *)n->db_part, (void *)n->d_red, n->act})
    if (p) cudaFree(p);
  delete n;
  return GFMD_OK;
}

int gfmd_ws_set_stream(gfmd_ws_handle_t n, void *stream) {
  if (!n) return gfmd::set_error(GFMD_EINVAL, "gfmd_ws_set_stream: NULL handle");
  n->stream = reinterpret_cast<cudaStream_t>(stream);
  return GFMD_OK;
}

int gfmd_ws_num_params(gfmd_ws_handle_t n, long long *count) {
  if (!n || !count) return gfmd::set_error(GFMD_EINVAL, "gfmd_ws_num_params: NULL argument");
  *count = (long long)n->nparam;
  return GFMD_OK;
}

int gfmd_ws_get_params(gfmd_ws_handle_t n, float *host_w, float *host_grad) {
  if (!n) return gfmd::set_error(GFMD_EINVAL, "gfmd_ws_get_params: NULL handle");
  cudaError_t e = cudaStreamSynchronize(n->stream);
  if (e == cudaSuccess && host_w) e = cudaMemcpy(host_w, n->w, sizeof(float) * n->nparam, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && host_grad) e = cudaMemcpy(host_grad, n->g, sizeof(float) * n->nparam, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return gfmd::set_error(GFMD_ECUDA, std::string("gfmd_ws_get_params: ") + cudaGetErrorString(e));
  return GFMD_OK;
}

int gfmd_ws_set_params(gfmd_ws_handle_t n, const float *host_w) {
  if (!n || !host_w) return gfmd::set_error(GFMD_EINVAL, "gfmd_ws_set_params: NULL argument");
  cudaError_t e = cudaStreamSynchronize(n->stream);
  if (e == cudaSuccess) e = cudaMemcpy(n->w, host_w, sizeof(float) * n->nparam, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return gfmd::set_error(GFMD_ECUDA, std::string("gfmd_ws_set_params: ") + cudaGetErrorString(e));
  n->packed_valid = false;
  return GFMD_OK;
}

int gfmd_ws_forward(gfmd_ws_handle_t n, int batch, int H, int W, const float *d_in, float *d_out) {
  using namespace gfmd;
  if (!n || !d_in || !d_out) return set_error(GFMD_EINVAL, "gfmd_ws_forward: NULL argument");
  if (!check_shape(batch, H, W)) return set_error(GFMD_EINVAL, "gfmd_ws_forward: H, W must be multiples of 8");
  Acts A;
  cudaError_t e = ensure_acts(n, batch, H, W, A);
  if (e == cudaSuccess) e = pack_weights(n);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(A.x, d_in, sizeof(float) * (size_t)batch * H * W * n->in_ch, cudaMemcpyDeviceToDevice,
                        n->stream);
  if (e == cudaSuccess) {
    forward(n, A);
    e = cudaMemcpyAsync(d_out, A.y, sizeof(float) * (size_t)batch * H * W * n->out_ch, cudaMemcpyDeviceToDevice,
                        n->stream);
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(GFMD_ECUDA, std::string("gfmd_ws_forward: ") + cudaGetErrorString(e));
  return GFMD_OK;
}

int gfmd_ws_loss_grad(gfmd_ws_handle_t n, int batch, int H, int W, const float *d_in, const float *d_target,
                      double *loss) {
  using namespace gfmd;
  if (!n || !d_in || !d_target) return set_error(GFMD_EINVAL, "gfmd_ws_loss_grad: NULL argument");
  if (!check_shape(batch, H, W)) return set_error(GFMD_EINVAL, "gfmd_ws_loss_grad: H, W must be multiples of 8");
  Acts A;
  cudaError_t e = ensure_acts(n, batch, H, W, A);
  if (e == cudaSuccess) e = pack_weights(n);
  const size_t ny = (size_t)batch * H * W * n->out_ch;
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(A.x, d_in, sizeof(float) * (size_t)batch * H * W * n->in_ch, cudaMemcpyDeviceToDevice,
                        n->stream);
  if (e == cudaSuccess) {
    forward(n, A);
    const int nb = 1024;
    k_mse<<<nb, 256, 0, n->stream>>>(A.y, d_target, ny, A.g0, n->d_red);
    k_sum_d<<<1, 32, 0, n->stream>>>(n->d_red, nb, 1.0 / (double)ny, n->d_red + 4096);
    backward(n, A);
    if (loss) {
      e = cudaMemcpyAsync(loss, n->d_red + 4096, sizeof(double), cudaMemcpyDeviceToHost, n->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(n->stream);
    }
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(GFMD_ECUDA, std::string("gfmd_ws_loss_grad: ") + cudaGetErrorString(e));
  return GFMD_OK;
}

int gfmd_ws_adam_step(gfmd_ws_handle_t n, float lr, float beta1, float beta2, float eps) {
  using namespace gfmd;
  if (!n || !(lr > 0.0f)) return set_error(GFMD_EINVAL, "gfmd_ws_adam_step: bad argument");
  n->step++;
  const float c1 = 1.0f - std::pow(beta1, (float)n->step), c2 = 1.0f - std::pow(beta2, (float)n->step);
  k_adam<<<grid_for(n->nparam), 256, 0, n->stream>>>(n->w, n->g, n->m, n->v, n->nparam, lr, beta1, beta2, eps, c1, c2);
  n->packed_valid = false;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_error(GFMD_ECUDA, std::string("gfmd_ws_adam_step: ") + cudaGetErrorString(e));
  return GFMD_OK;
}

int gfmd_ws_to_nhwc(const double *d_u, int channels, int nsite, float scale, float *d_out, void *stream) {
  if (!d_u || !d_out || channels < 1 || nsite < 1) return gfmd::set_error(GFMD_EINVAL, "gfmd_ws_to_nhwc: bad argument");
  gfmd::k_to_nhwc<<<gfmd::grid_for((size_t)nsite * channels), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      d_u, channels, nsite, scale, d_out);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GFMD_OK : gfmd::set_error(GFMD_ECUDA, cudaGetErrorString(e));
}

int gfmd_ws_from_nhwc(const float *d_in, int channels, int nsite, double scale, double *d_u, void *stream) {
  if (!d_u || !d_in || channels < 1 || nsite < 1) return gfmd::set_error(GFMD_EINVAL, "gfmd_ws_from_nhwc: bad argument");
  gfmd::k_from_nhwc<<<gfmd::grid_for((size_t)nsite * channels), 256, 0, reinterpret_cast<cudaStream_t>(stream)>>>(
      d_in, channels, nsite, scale, d_u);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GFMD_OK : gfmd::set_error(GFMD_ECUDA, cudaGetErrorString(e));
}

}  // extern "C"
