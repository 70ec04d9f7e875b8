// Training of the potential-surrogate MLP on the GPU.
//
// One call, gal_mlp_train_step, runs for a batch of B points: the forward pass,
// the input-gradient (backward) pass, the loss on potential and gradient
// targets, the exact parameter gradient of that loss (backpropagation through
// the backward pass, which needs SiLU'' terms), and an Adam update. Weights and
// the activations that enter the 256x256 products are rounded to bfloat16 in
// the forward and backward passes, as the tensor-core inference kernel does, so
// the trained network is the one that will be run (gradients pass the rounding
// straight through). gal_mlp_loss_grads returns the loss and gradient without
// updating (checked against a NumPy restatement).
//
// Every product with 256 output columns and K >= 64 (the 256 x 256 layers of
// the forward and backward passes, and the weight gradients with K = batch)
// runs on the tensor cores (tc_gemm.cuh): operands the quantised passes round
// to bf16 enter as one bf16 part, all others as two (hi + lo), so the
// gradients keep FP32-level accuracy. The elementwise step after each product
// runs in its store phase; in the quantised passes the weights, and the
// activations passed from product to product, travel as bf16 operand images
// fed by bulk copies. The first layer (K = 3) is one fused kernel, the
// 1-column and 3-column products are warp row sums, the column sums of the
// bias and first-layer gradients go through per-chunk partials finished in
// one launch, and the weight gradients and column sums run on a second
// stream beside the chain of input-gradient products. Every reduction adds in
// a fixed order, so training is deterministic. The FP32 tiled kernel and the
// grid-stride elementwise kernels remain as the path for products the tensor
// cores do not take.
#include <cuda_runtime.h>

#include <atomic>
#include <string>

#include "handle.h"
#include "mlp.cuh"
#include "tc_gemm.cuh"

namespace gal {
namespace mlp {

// C[M,N] = alpha * op(A)[M,K] op(B)[K,N] + beta * C + bias[n], row-major storage.
// op(A)(m,k) = TA ? A[k*lda+m] : A[m*lda+k]; op(B)(k,n) = TB ? B[n*ldb+k] : B[k*ldb+n].
// qa / qb round the loaded operand to bfloat16.
// With gridDim.z > 1 the K range is split across blockIdx.z and every block adds
// alpha * (its partial product) into C with atomics (C prepared by the caller).
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) k_gemm(int M, int N, int K, const float* __restrict__ A, int lda,
                                              const float* __restrict__ B, int ldb, float* __restrict__ C, int ldc,
                                              float alpha, float beta, const float* __restrict__ bias, int qa,
                                              int qb) {
  __shared__ float As[16][64 + 1];
  __shared__ float Bs[16][64 + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int m0 = blockIdx.y * 64, n0 = blockIdx.x * 64;
  const bool split = gridDim.z > 1;
  const int kchunk = split ? ((K + gridDim.z - 1) / gridDim.z + 15) / 16 * 16 : K;
  const int kbeg = split ? (int)blockIdx.z * kchunk : 0;
  const int kend = split ? min(K, kbeg + kchunk) : K;
  float acc[4][4] = {};
  for (int k0 = kbeg; k0 < kend; k0 += 16) {
    for (int i = threadIdx.x; i < 1024; i += 256) {
      int mm, kk;
      if (TA) { kk = i / 64; mm = i % 64; } else { mm = i / 16; kk = i % 16; }
      const int m = m0 + mm, k = k0 + kk;
      float v = 0.0f;
      if (m < M && k < kend) v = TA ? A[(int64_t)k * lda + m] : A[(int64_t)m * lda + k];
      As[kk][mm] = qa ? bf16r(v) : v;
      int nn, kb;
      if (TB) { nn = i / 16; kb = i % 16; } else { kb = i / 64; nn = i % 64; }
      const int n = n0 + nn, kq = k0 + kb;
      float w = 0.0f;
      if (n < N && kq < kend) w = TB ? B[(int64_t)n * ldb + kq] : B[(int64_t)kq * ldb + n];
      Bs[kb][nn] = qb ? bf16r(w) : w;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 16; ++kk) {
      float a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][ty * 4 + r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[kk][tx * 4 + c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r) {
    const int m = m0 + ty * 4 + r;
    if (m >= M) continue;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int n = n0 + tx * 4 + c;
      if (n >= N) continue;
      if (split) {
        atomicAdd(&C[(int64_t)m * ldc + n], alpha * acc[r][c]);
        continue;
      }
      float v = alpha * acc[r][c];
      if (beta != 0.0f) v += beta * C[(int64_t)m * ldc + n];
      if (bias) v += bias[n];
      C[(int64_t)m * ldc + n] = v;
    }
  }
}

#define GRID_STRIDE(i, n) for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

// H = silu(Z), optionally rounded to bfloat16
__global__ void k_silu(const float* Z, float* Hout, int64_t n, int q) {
  GRID_STRIDE(i, n) {
    const float h = silu(Z[i]);
    Hout[i] = q ? bf16r(h) : h;
  }
}

// D = s(Z) * U with s = silu' (optionally bf16-rounded, as stored by the inference kernel), D optionally rounded
__global__ void k_dmul(const float* Z, const float* U, float* D, int64_t n, int qs, int qd) {
  GRID_STRIDE(i, n) {
    float s = dsilu(Z[i]);
    if (qs) s = bf16r(s);
    const float d = s * U[i];
    D[i] = qd ? bf16r(d) : d;
  }
}

// D4[b, c] = silu'(Z4[b, c]) * w5[c]
__global__ void k_d4(const float* Z, const float* w5, float* D, int64_t n, int q) {
  GRID_STRIDE(i, n) {
    const float d = dsilu(Z[i]) * w5[i % H];
    D[i] = q ? bf16r(d) : d;
  }
}

// Ub = s(Z) * Db;  Zb = silu''(Z) * U * Db   (the z-dependence of the backward pass)
__global__ void k_dd(const float* Z, const float* U, const float* Db, float* Ub, float* Zb, int64_t n, int qs) {
  GRID_STRIDE(i, n) {
    const float z = Z[i];
    float s = dsilu(z);
    if (qs) s = bf16r(s);
    Ub[i] = s * Db[i];
    Zb[i] = d2silu(z) * U[i] * Db[i];
  }
}

// Zb4 = silu''(Z4) * w5 * Db4 + silu'(Z4) * Pb[b] * w5
__global__ void k_zb4(const float* Z, const float* Db, const float* Pb, const float* w5, float* Zb, int64_t n) {
  GRID_STRIDE(i, n) {
    const float z = Z[i];
    const float w = w5[i % H];
    Zb[i] = d2silu(z) * w * Db[i] + dsilu(z) * Pb[i / H] * w;
  }
}

// Zb += silu'(Z) * Hb
__global__ void k_zb_acc(const float* Z, const float* Hb, float* Zb, int64_t n) {
  GRID_STRIDE(i, n) { Zb[i] += dsilu(Z[i]) * Hb[i]; }
}

// Column sums over the B rows of a [B][H] array in two deterministic passes:
// k_colpart sums f(b, c) over 64-row chunks, k_colfinal_all adds the chunks in
// order. f: mode 0 X[b,c]; 1 X[b,c] v[b]; 2 silu'(X[b,c]) Y[b,c];
// 3 X[b,c] V[b][j] for j = 0..2, out[c][3] (the first layer's weight gradient);
// 4 both mode 3 (into part) and mode 0 (into part2) from one read of X.
// In k_colpart warp w sums rows w*8 .. w*8+7 of the chunk, lane l columns
// 4l..4l+3 and 128+4l..128+4l+3 (two float4 per row: a warp reads whole
// rows); the eight loads of each operand are issued together, and the eight
// warps' sums are added in warp order through shared memory.
constexpr int kColRows = 64;

template <int mode>
__global__ void __launch_bounds__(256) k_colpart(const float* X, const float* Y, const float* v, const float* V,
                                                 int64_t rows, float* part, float* part2) {
  tc::pdl_wait();
  tc::pdl_trigger();
  __shared__ float red[4][8][H];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int64_t b0 = (int64_t)blockIdx.x * kColRows + wp * 8;
  float s[4][8];
#pragma unroll
  for (int j = 0; j < 4; ++j)
#pragma unroll
    for (int e = 0; e < 8; ++e) s[j][e] = 0.0f;
  // all of the thread's loads first, then the sums
  const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float4 xa[8], xb[8], ya[8], yb[8];
  float sc[8][3];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int64_t b = b0 + i;
    const bool in = b < rows;
    const float4* xr = reinterpret_cast<const float4*>(X + b * H);
    xa[i] = in ? xr[lane] : z4;
    xb[i] = in ? xr[32 + lane] : z4;
    if constexpr (mode == 2) {
      const float4* yr = reinterpret_cast<const float4*>(Y + b * H);
      ya[i] = in ? yr[lane] : z4;
      yb[i] = in ? yr[32 + lane] : z4;
    }
    if constexpr (mode == 1) sc[i][0] = in ? v[b] : 0.0f;
    if constexpr (mode >= 3)
#pragma unroll
      for (int j = 0; j < 3; ++j) sc[i][j] = in ? V[b * 3 + j] : 0.0f;
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const float x[8] = {xa[i].x, xa[i].y, xa[i].z, xa[i].w, xb[i].x, xb[i].y, xb[i].z, xb[i].w};
    if constexpr (mode == 0) {
#pragma unroll
      for (int e = 0; e < 8; ++e) s[0][e] += x[e];
    } else if constexpr (mode == 1) {
#pragma unroll
      for (int e = 0; e < 8; ++e) s[0][e] += x[e] * sc[i][0];
    } else if constexpr (mode == 2) {
      const float y[8] = {ya[i].x, ya[i].y, ya[i].z, ya[i].w, yb[i].x, yb[i].y, yb[i].z, yb[i].w};
#pragma unroll
      for (int e = 0; e < 8; ++e) s[0][e] += dsilu(x[e]) * y[e];
    } else {
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int e = 0; e < 8; ++e) s[j][e] = fmaf(x[e], sc[i][j], s[j][e]);
      if constexpr (mode == 4)
#pragma unroll
        for (int e = 0; e < 8; ++e) s[3][e] += x[e];
    }
  }
  constexpr int nj = mode >= 3 ? 3 : 1, nr = mode == 4 ? 4 : nj;
#pragma unroll
  for (int j = 0; j < nr; ++j)
#pragma unroll
    for (int e = 0; e < 8; ++e) red[j][wp][(e < 4 ? 0 : 128) + 4 * lane + (e & 3)] = s[j][e];
  __syncthreads();
  const int c = threadIdx.x;
  float* p = part + ((int64_t)blockIdx.x * H + c) * 3;
  for (int j = 0; j < 3; ++j) {
    float t = 0.0f;
    if (j < nj)
#pragma unroll
      for (int q = 0; q < 8; ++q) t += red[j][q][c];
    p[j] = t;
  }
  if constexpr (mode == 4) {
    float t = 0.0f;
#pragma unroll
    for (int q = 0; q < 8; ++q) t += red[3][q][c];
    float* p2 = part2 + ((int64_t)blockIdx.x * H + c) * 3;
    p2[0] = t;
    p2[1] = 0.0f;
    p2[2] = 0.0f;
  }
}

// The column sums of one training step, finished in one launch. Job j adds
// the chunks of part[j][0] (and then those of part[j][1], when set) for each
// of its H * nj outputs and stores the total (first + second) to out[j];
// a job with nj = 0 is the sum of n0 scalars part[j][0][0..n0) (the output
// bias gradient and the loss from the loss kernel's per-block sums).
constexpr int kColJobs = 8;
struct ColJobs {
  const float* part[kColJobs][2];
  float* out[kColJobs];
  int nj[kColJobs];
  int64_t chunks;
  int n0;
};

// grid (H / 32, jobs): 32 columns per block; the 8 warps sum interleaved
// chunks, then one warp adds the 8 partial sums in a fixed order.
__global__ void __launch_bounds__(256) k_colfinal_all(ColJobs J) {
  tc::pdl_wait();
  tc::pdl_trigger();
  __shared__ float red[8][32][3];
  const int job = blockIdx.y;
  const int cl = threadIdx.x & 31, g = threadIdx.x >> 5;
  const int c = blockIdx.x * 32 + cl;
  const int nj = J.nj[job];
  if (nj == 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      float t = 0.0f;
      for (int i = 0; i < J.n0; ++i) t += J.part[job][0][i];
      *J.out[job] = t;
    }
    return;
  }
  float tot[3] = {0.0f, 0.0f, 0.0f};
  for (int src = 0; src < 2; ++src) {
    const float* part = J.part[job][src];
    if (!part) break;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      if (j >= nj) break;
      float s = 0.0f;
#pragma unroll 16
      for (int64_t k = g; k < J.chunks; k += 8) s += part[(k * H + c) * 3 + j];
      red[g][cl][j] = s;
    }
    __syncthreads();
    if (g == 0) {
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        if (j >= nj) break;
        float s = 0.0f;
#pragma unroll
        for (int q = 0; q < 8; ++q) s += red[q][cl][j];
        tot[j] = src == 0 ? s : tot[j] + s;
      }
    }
    __syncthreads();
  }
  if (g == 0) {
#pragma unroll
    for (int j = 0; j < 3; ++j)
      if (j < nj) J.out[job][(int64_t)c * nj + j] = tot[j];
  }
}

// out[b][j] = sum_c X[b][c] W[c * ncol + j] (+ bias[j]) for ncol = 1 or 3: the
// products with one or three output columns (the last layer's output and the
// first layer's input gradient). One warp per row, lanes over columns
// (coalesced), a fixed-order shuffle reduction.
__global__ void __launch_bounds__(256) k_rowdot(const float* X, const float* W, const float* bias, int64_t rows,
                                                int ncol, float* out) {
  tc::pdl_wait();
  tc::pdl_trigger();
  const int lane = threadIdx.x & 31;
  const int64_t b = (int64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
  if (b >= rows) return;
  float x[H / 32];
#pragma unroll
  for (int i = 0; i < H / 32; ++i) x[i] = X[b * H + lane + 32 * i];
  for (int j = 0; j < ncol; ++j) {
    float acc = 0.0f;
#pragma unroll
    for (int i = 0; i < H / 32; ++i) acc = fmaf(x[i], W[(lane + 32 * i) * ncol + j], acc);
#pragma unroll
    for (int m = 16; m >= 1; m >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, m);
    if (lane == 0) out[b * ncol + j] = bias ? acc + bias[j] : acc;
  }
}

// residuals, their loss weights and the loss value
// (optional per-point weights wt[b] multiply both terms of point b)
// lpart[block] = the block's share of the loss and pbsum[block] its sum of Pb
// (the output bias gradient), both added up in a fixed order afterwards
__global__ void k_loss(const float* out, const float* G, const float* phi_t, const float* g_t, const float* wt,
                       int64_t B, float alpha, float beta, float* Pb, float* Eb, float* lpart, float* pbsum) {
  tc::pdl_wait();
  tc::pdl_trigger();
  float s = 0.0f, ps = 0.0f;
  GRID_STRIDE(b, B) {
    const float w = wt ? wt[b] : 1.0f;
    const float r = out[b] - phi_t[b];
    Pb[b] = 2.0f * alpha * w * r / (float)B;
    ps += Pb[b];
    s += alpha * w * r * r;
#pragma unroll
    for (int j = 0; j < 3; ++j) {
      const float e = G[b * 3 + j] - g_t[b * 3 + j];
      Eb[b * 3 + j] = 2.0f * beta * w * e / (float)B;
      s += beta * w * e * e;
    }
  }
  __shared__ float red[2][256];
  red[0][threadIdx.x] = s;
  red[1][threadIdx.x] = ps;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) {
      red[0][threadIdx.x] += red[0][threadIdx.x + w];
      red[1][threadIdx.x] += red[1][threadIdx.x + w];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    lpart[blockIdx.x] = red[0][0] / (float)B;
    pbsum[blockIdx.x] = red[1][0];
  }
}

__global__ void k_adam(float* p, const float* g, float* m, float* v, int64_t n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
  tc::pdl_wait();
  tc::pdl_trigger();
  GRID_STRIDE(i, n) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

struct Ws {
  float *Z[5], *Hh[5], *D[5], *U[4], *Zb[5], *Db, *Ub, *Ub2, *Ub3, *Hb, *out, *G, *Pb, *Eb;  // Ub1, Ub2, Ub3
  float* colpart;  // [kColSlots][chunks][H][3] partial column sums, one slot per column sum of a step
  float* pbsum;    // [kLossBlocks] per-block sums of Pb
  float* lpart;    // [kLossBlocks] per-block shares of the loss
  float* splitk;   // [kMaxSplits][H][H] partial tiles of the tensor-core weight gradients
  uint8_t* wimg;   // bf16 images of W2, W3, W4 as a product's B operand, both orientations (wimg_of())
  uint8_t* aimg[2];  // bf16 A-operand images passed between the quantised forward / input-gradient products
  int* err;  // set by a tensor-core product that gave up waiting (gal_mlp_workspace_error)
};

static int64_t col_chunks(int64_t B) { return (B + kColRows - 1) / kColRows; }
constexpr int kMaxSplits = 32;
constexpr int kColSlots = 8;      // column sums per training step
// B-operand images of the three 256 x 256 layers: per matrix two orientations
// (B(n, k) = W[n][k] for the forward products, W[k][n] for the backward ones)
// of two 64 KB column blocks
constexpr size_t kWimgOne = 2 * tcg::BIMG_BYTES;  // one orientation of one matrix
constexpr size_t kWimgBytes = 3 * 2 * kWimgOne;
constexpr int kLossBlocks = 4096;  // k_loss's largest grid (ew_grid)

// The bf16 B-operand images of W2, W3, W4, rounded to nearest as put() rounds
// a quantised operand: image (matrix m, orientation o) at wimg + (2 m + o) *
// kWimgOne, column block nb at + nb * BIMG_BYTES, laid out by tc::sw128_offset
// for 128 rows (n) x 256 K; o = 0: B(n, k) = W[n][k], o = 1: B(n, k) = W[k][n].
// One thread per 16-byte chunk (8 consecutive k).
__device__ __forceinline__ void wimg_chunk(const float* P, uint8_t* wimg, int i) {
  const int chunk = i & 31, row = (i >> 5) & 127, nb = (i >> 12) & 1, o = (i >> 13) & 1, m = i >> 14;
  if (m >= 3) return;
  const float* W = P + (m == 0 ? OFF_W2 : (m == 1 ? OFF_W3 : OFF_W4));
  const int n = nb * 128 + row, k0 = chunk * 8;
  uint32_t h[4];
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int k = k0 + 2 * j;
    const float v0 = o ? W[k * H + n] : W[n * H + k];
    const float v1 = o ? W[(k + 1) * H + n] : W[n * H + k + 1];
    h[j] = (uint32_t)tcg::bf16_bits(v0) | ((uint32_t)tcg::bf16_bits(v1) << 16);
  }
  *reinterpret_cast<uint4*>(wimg + (size_t)(2 * m + o) * kWimgOne + (size_t)nb * tcg::BIMG_BYTES +
                            tc::sw128_offset(128, row, k0)) = make_uint4(h[0], h[1], h[2], h[3]);
}
constexpr int kWimgBlocks = 3 * 2 * 2 * 128 * 32 / 256;

// The first layer's 3-wide products with the elementwise step that follows:
//   MODE 0: Z1 = X W1^T + b1 and H1 = silu(Z1) (bf16-rounded when q) -> o1 = Z1, o2 = H1
//   MODE 1: Db1 = X W1^T (X = the gradient residual weights), then
//           o1 = Ub = silu'(Z1) Db1, o2 = Zb1 = silu''(Z1) U1 Db1 (Db1 itself is not stored)
// Thread c owns column c (row c of W1 in registers); a block takes kL1Rows rows,
// all of whose loads are issued before the first store.
// The sum is fma(w0, x0, fma(w1, x1, fma(w2, x2, b1))), the inference
// kernel's order, so both compute the same first layer.
constexpr int kL1Rows = 8;

// MODE 0 with wimg set: blocks from nrow_blocks on build the layers' weight
// images instead (wimg_chunk), in the same launch.
template <int MODE>
__global__ void __launch_bounds__(256) k_layer1(const float* __restrict__ X, const float* __restrict__ W1,
                                                const float* __restrict__ b1, const float* __restrict__ Z,
                                                const float* __restrict__ U, float* __restrict__ o1,
                                                float* __restrict__ o2, int64_t rows, int q, const float* P,
                                                uint8_t* wimg, unsigned nrow_blocks) {
  tc::pdl_wait();
  tc::pdl_trigger();
  if (MODE == 0 && wimg && blockIdx.x >= nrow_blocks) {
    wimg_chunk(P, wimg, (int)(blockIdx.x - nrow_blocks) * 256 + threadIdx.x);
    return;
  }
  const int c = threadIdx.x;
  const float w0 = W1[3 * c], w1 = W1[3 * c + 1], w2 = W1[3 * c + 2];
  const float bc = MODE == 0 ? b1[c] : 0.0f;
  const int64_t b0 = (int64_t)blockIdx.x * kL1Rows;
  float v[kL1Rows], z[kL1Rows], u[kL1Rows];
#pragma unroll
  for (int i = 0; i < kL1Rows; ++i) {
    const int64_t b = b0 + i < rows ? b0 + i : rows - 1;  // rows past the end repeat the last (not stored)
    v[i] = fmaf(w0, X[3 * b], fmaf(w1, X[3 * b + 1], fmaf(w2, X[3 * b + 2], bc)));
    if constexpr (MODE == 1) {
      z[i] = Z[b * H + c];
      u[i] = U[b * H + c];
    }
  }
#pragma unroll
  for (int i = 0; i < kL1Rows; ++i) {
    const int64_t b = b0 + i;
    if (b >= rows) break;
    const int64_t idx = b * H + c;
    if constexpr (MODE == 0) {
      const float h = silu(v[i]);
      o1[idx] = v[i];
      o2[idx] = q ? bf16r(h) : h;
    } else {
      o1[idx] = dsilu(z[i]) * v[i];
      o2[idx] = d2silu(z[i]) * u[i] * v[i];
    }
  }
}

// an A-operand image of a [B][256] activation: 64 KB per 128-row block
static size_t aimg_bytes(int64_t B) { return (size_t)((B + 127) / 128) * tcg::BIMG_BYTES; }

static size_t ws_bytes(int64_t B) {
  const size_t big = sizeof(float) * (size_t)B * H;
  return big * (4 + 4 + 4 + 3 + 4 + 5) + sizeof(float) * (size_t)B * (1 + 3 + 1 + 3) +
         sizeof(float) * (size_t)kColSlots * col_chunks(B) * H * 3 + sizeof(float) * 2 * kLossBlocks +
         sizeof(float) * (size_t)kMaxSplits * H * H + kWimgBytes + 2 * aimg_bytes(B) + 64 * 256;
}

static Ws carve(void* ws, int64_t B) {
  Ws w{};
  // 256-byte aligned whatever the caller's pointer (the size has the slack):
  // the column sums read rows as float4
  char* p = reinterpret_cast<char*>((reinterpret_cast<uintptr_t>(ws) + 255) & ~(uintptr_t)255);
  const size_t big = sizeof(float) * (size_t)B * H;
  auto take = [&](size_t bytes) {
    float* r = reinterpret_cast<float*>(p);
    p += (bytes + 255) & ~(size_t)255;
    return r;
  };
  for (int k = 1; k <= 4; ++k) w.Z[k] = take(big);
  for (int k = 1; k <= 4; ++k) w.Hh[k] = take(big);
  for (int k = 1; k <= 4; ++k) w.D[k] = take(big);
  for (int k = 1; k <= 3; ++k) w.U[k] = take(big);
  for (int k = 1; k <= 4; ++k) w.Zb[k] = take(big);
  w.Db = take(big);
  w.Ub = take(big);
  w.Ub2 = take(big);
  w.Ub3 = take(big);
  w.Hb = take(big);
  w.out = take(sizeof(float) * B);
  w.G = take(sizeof(float) * B * 3);
  w.Pb = take(sizeof(float) * B);
  w.Eb = take(sizeof(float) * B * 3);
  w.err = reinterpret_cast<int*>(take(256));
  w.colpart = take(sizeof(float) * (size_t)kColSlots * col_chunks(B) * H * 3);
  w.pbsum = take(sizeof(float) * kLossBlocks);
  w.lpart = take(sizeof(float) * kLossBlocks);
  w.splitk = take(sizeof(float) * (size_t)kMaxSplits * H * H);
  w.wimg = reinterpret_cast<uint8_t*>(take(kWimgBytes));
  for (auto& im : w.aimg) im = reinterpret_cast<uint8_t*>(take(aimg_bytes(B)));
  return w;
}

// Tensor-core product C = op(A) op(B) (+ beta C) (+ bias) with op as in
// gemm() below; split_a / split_b as in tc_gemm.cuh. Returns false when the
// kernel cannot be configured (then the caller uses the FP32 kernel).
// The elementwise step fused into a product's store (tcg::EPI_*); the FP32
// fallback runs the same step as a kernel of its own.
struct Epi {
  int mode = tcg::EPI_NONE;
  const float* e1 = nullptr;
  const float* e2 = nullptr;
  float* o1 = nullptr;
  float* o2 = nullptr;
  const float* cvec = nullptr;
  const float* rvec = nullptr;
  int q1 = 0, q2 = 0;
  uint8_t* img = nullptr;  // also write a bf16 A-operand image of o1 (img_src 1) or o2 (2)
  int img_src = 0;
};

// Launch with programmatic stream serialization (the kernel calls
// tc::pdl_wait() before touching global memory): its blocks may be scheduled,
// and run their set-up, while the kernel before it in the stream finishes.
template <typename... KArgs, typename... Args>
static void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                       Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// the image of layer `layer` (2..4) as B operand: orientation 0 for B(n, k) =
// W[n][k] (forward and second-order passes), 1 for W[k][n] (input gradient)
static const uint8_t* wimg_of(const Ws& w, int layer, int orient) {
  return w.wimg + (size_t)(2 * (layer - 2) + orient) * kWimgOne;
}

// the tensor-core product kernels' shared-memory opt-in, once per device
static bool tc_configure() {
  static std::atomic<int> configured[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return false;
  if (!configured[dev].load()) {
    const void* fns[] = {(const void*)tcg::k_tc_gemm<tcg::EPI_NONE>, (const void*)tcg::k_tc_gemm<tcg::EPI_SILU>,
                         (const void*)tcg::k_tc_gemm<tcg::EPI_DMUL>, (const void*)tcg::k_tc_gemm<tcg::EPI_DD>,
                         (const void*)tcg::k_tc_gemm<tcg::EPI_ZBACC>, (const void*)tcg::k_tc_gemm<tcg::EPI_SILU_D4>,
                         (const void*)tcg::k_tc_gemm<tcg::EPI_ZB4>};
    for (const void* f : fns)
      if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)tcg::SMEM_MAX) != cudaSuccess)
        return false;
    configured[dev].store(1);
  }
  return true;
}

// C[H][H] = A1^T B1 + A2^T B2 with A_i, B_i of [K][H] (row-major): both terms
// of a weight gradient in one split-K launch (slices 0..z-1 the first term,
// z..2z-1 the second, one wave of CTAs) and one ordered sum of the slices.
static bool tc_wgrad2(cudaStream_t s, int K, const float* A1, const float* B1, int split_a1, int split_b1,
                      const float* A2, const float* B2, int split_a2, int split_b2, float* C, int* err,
                      float* part) {
  if (K < tcg::BK || !tc_configure()) return false;
  const int tiles = (H / tcg::BN) * (H / tcg::BM);
  int per = device_sm_count() / (2 * tiles);
  if (per > K / (4 * tcg::BK)) per = K / (4 * tcg::BK);
  if (per > kMaxSplits / 2) per = kMaxSplits / 2;
  if (per < 1) per = 1;
  tcg::Args a{};
  a.M = H;
  a.N = H;
  a.K = K;
  a.A = A1;
  a.sam = 1;
  a.sak = H;
  a.B = B1;
  a.sbn = 1;
  a.sbk = H;
  a.split_a = split_a1;
  a.split_b = split_b1;
  a.A2 = A2;
  a.sam2 = 1;
  a.sak2 = H;
  a.B2 = B2;
  a.sbn2 = 1;
  a.sbk2 = H;
  a.split_a2 = split_a2;
  a.split_b2 = split_b2;
  a.C = C;
  a.ldc = H;
  a.err = err;
  a.part = part;
  a.kchunk = ((K + per - 1) / per + tcg::BK - 1) / tcg::BK * tcg::BK;
  const int z = (K + a.kchunk - 1) / a.kchunk;
  a.z2 = z;
  const dim3 grid(H / tcg::BN, H / tcg::BM, 2 * z);
  const uint32_t st1 = tcg::stage_bytes(split_a1, split_b1), st2 = tcg::stage_bytes(split_a2, split_b2);
  a.stage = st1 > st2 ? st1 : st2;
  a.bar_off = tcg::bar_offset(a.stage);
  launch_pdl(tcg::k_tc_gemm<tcg::EPI_NONE>, grid, tcg::NTHREADS, tcg::smem_alloc_at(a.bar_off), s, a);
  launch_pdl(tcg::k_splitk_sum, dim3((H * H + 255) / 256), 256, 0, s, (const float*)part, 2 * z, (int)H, (int)H, C,
             (int64_t)H, 0.0f);
  return true;
}

static bool tc_gemm(cudaStream_t s, bool TA, bool TB, int M, int N, int K, const float* A, int lda, const float* B,
                    int ldb, float* C, int ldc, float beta, const float* bias, int split_a, int split_b, int* err,
                    float* part, const Epi& epi, const uint8_t* bimg, const uint8_t* aimg) {
  if (!tc_configure()) return false;
  tcg::Args a{};
  a.M = M;
  a.N = N;
  a.K = K;
  a.A = A;
  a.sam = TA ? 1 : lda;
  a.sak = TA ? lda : 1;
  a.B = B;
  a.sbn = TB ? ldb : 1;
  a.sbk = TB ? 1 : ldb;
  a.C = C;
  a.ldc = ldc;
  a.beta = beta;
  a.bias = bias;
  a.split_a = split_a;
  a.split_b = split_b;
  a.err = err;
  a.epi = epi.mode;
  a.e1 = epi.e1;
  a.e2 = epi.e2;
  a.o1 = epi.o1;
  a.o2 = epi.o2;
  a.cvec = epi.cvec;
  a.rvec = epi.rvec;
  a.q1 = epi.q1;
  a.q2 = epi.q2;
  a.img_out = epi.img;
  a.img_src = epi.img_src;
  dim3 grid((N + tcg::BN - 1) / tcg::BN, (M + tcg::BM - 1) / tcg::BM, 1);
  a.kchunk = ((K + tcg::BK - 1) / tcg::BK) * tcg::BK;
  // few output tiles and a long K (the weight gradients, K = batch): split K
  // over enough CTAs to fill the GPU; each stores its partial tile, and the
  // slices are added in a fixed order (deterministic, unlike atomics)
  const int tiles = (int)(grid.x * grid.y);
  const int sms = device_sm_count();
  if (!bias && part && epi.mode == tcg::EPI_NONE && (int64_t)M * N <= (int64_t)H * H && tiles < sms &&
      K >= 4 * tcg::BK) {
    int splits = sms / tiles;
    if (splits > K / (4 * tcg::BK)) splits = K / (4 * tcg::BK);
    if (splits > kMaxSplits) splits = kMaxSplits;
    if (splits > 1) {
      a.kchunk = ((K + splits - 1) / splits + tcg::BK - 1) / tcg::BK * tcg::BK;
      grid.z = (K + a.kchunk - 1) / a.kchunk;
      a.part = part;
    }
  }
  if (bimg && !split_b && N == H && K == H && grid.z == 1) {
    // B from its bf16 image: the stages hold A only; with A's image too, A's
    // four K blocks take the place of the two stages
    a.bimg = bimg;
    a.aimg = aimg && !split_a ? aimg : nullptr;
    a.stage = a.aimg ? 2 * tcg::A_BLK : tcg::stage_bytes(split_a, 0) - tcg::B_BLK;
    a.bar_off = tcg::bar_offset_img(a.stage);
  } else {
    a.stage = tcg::stage_bytes(split_a, split_b);
    a.bar_off = tcg::bar_offset(a.stage);
  }
  const uint32_t smem = tcg::smem_alloc_at(a.bar_off);
  switch (epi.mode) {
    case tcg::EPI_SILU: launch_pdl(tcg::k_tc_gemm<tcg::EPI_SILU>, grid, tcg::NTHREADS, smem, s, a); break;
    case tcg::EPI_DMUL: launch_pdl(tcg::k_tc_gemm<tcg::EPI_DMUL>, grid, tcg::NTHREADS, smem, s, a); break;
    case tcg::EPI_DD: launch_pdl(tcg::k_tc_gemm<tcg::EPI_DD>, grid, tcg::NTHREADS, smem, s, a); break;
    case tcg::EPI_ZBACC: launch_pdl(tcg::k_tc_gemm<tcg::EPI_ZBACC>, grid, tcg::NTHREADS, smem, s, a); break;
    case tcg::EPI_SILU_D4: launch_pdl(tcg::k_tc_gemm<tcg::EPI_SILU_D4>, grid, tcg::NTHREADS, smem, s, a); break;
    case tcg::EPI_ZB4: launch_pdl(tcg::k_tc_gemm<tcg::EPI_ZB4>, grid, tcg::NTHREADS, smem, s, a); break;
    default: launch_pdl(tcg::k_tc_gemm<tcg::EPI_NONE>, grid, tcg::NTHREADS, smem, s, a); break;
  }
  if (grid.z > 1) {
    const int64_t mn = (int64_t)M * N;
    launch_pdl(tcg::k_splitk_sum, dim3((unsigned)((mn + 255) / 256)), 256, 0, s, (const float*)part, (int)grid.z, M,
               N, C, (int64_t)ldc, beta);
  }
  return true;
}

// Products run on the tensor cores when they have 256 output columns and
// K >= 64, else on the FP32 kernel. qa / qb: the operand is rounded to bf16
// (one bf16 part on the tensor cores); otherwise it enters unrounded (two parts).
// bimg: B's bf16 image (wimg_of()), used when B is rounded (qb); aimg: A's, the
// image a previous product wrote (Epi::img), used with bimg when A is rounded (qa).
static void epi_fallback(cudaStream_t s, const Epi& e, const float* C, int64_t n);

template <bool TA, bool TB>
static void gemm(cudaStream_t s, const Ws& w, int M, int N, int K, const float* A, int lda, const float* B, int ldb,
                 float* C, int ldc, float beta = 0.0f, const float* bias = nullptr, int qa = 0, int qb = 0,
                 const Epi& epi = Epi(), const uint8_t* bimg = nullptr, const uint8_t* aimg = nullptr) {
  if (N == H && K >= tcg::BK &&
      tc_gemm(s, TA, TB, M, N, K, A, lda, B, ldb, C, ldc, beta, bias, qa ? 0 : 1, qb ? 0 : 1, w.err, w.splitk, epi,
              qb ? bimg : nullptr, qa ? aimg : nullptr))
    return;
  if (epi.img) {  // the consumer's A image is not written on this path: it falls back to the array
    Epi e = epi;
    e.img = nullptr;
    gemm<TA, TB>(s, w, M, N, K, A, lda, B, ldb, C, ldc, beta, bias, qa, qb, e);
    return;
  }
  if (epi.mode != tcg::EPI_NONE) {  // FP32 product, then the elementwise step on its own
    gemm<TA, TB>(s, w, M, N, K, A, lda, B, ldb, C, ldc, beta, bias, qa, qb);
    epi_fallback(s, epi, C, (int64_t)M * N);
    return;
  }
  dim3 grid((N + 63) / 64, (M + 63) / 64);
  // few output tiles and a long K (the weight gradients, K = batch): split K over
  // enough blocks to fill the GPU and accumulate with atomics
  const int tiles = (int)(grid.x * grid.y);
  if (!bias && (beta == 0.0f || beta == 1.0f) && tiles < 2 * device_sm_count() && K >= 1024) {
    int splits = 4 * device_sm_count() / tiles;
    if (splits > K / 256) splits = K / 256;
    if (splits > 1) {
      if (beta == 0.0f && ldc == N) cudaMemsetAsync(C, 0, sizeof(float) * (size_t)M * N, s);
      if (beta == 0.0f && ldc != N) {
        k_gemm<TA, TB><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, 1.0f, beta, bias, qa, qb);
        return;
      }
      grid.z = splits;
    }
  }
  k_gemm<TA, TB><<<grid, 256, 0, s>>>(M, N, K, A, lda, B, ldb, C, ldc, 1.0f, beta, bias, qa, qb);
}

// gW = A1^T B1 + A2^T B2 over the batch (the two terms of a weight gradient);
// qa / qb as in gemm()
static void wgrad2(cudaStream_t s, const Ws& w, int B, const float* A1, const float* B1, int qa1, int qb1,
                   const float* A2, const float* B2, int qa2, int qb2, float* C) {
  if (tc_wgrad2(s, B, A1, B1, qa1 ? 0 : 1, qb1 ? 0 : 1, A2, B2, qa2 ? 0 : 1, qb2 ? 0 : 1, C, w.err, w.splitk)) return;
  gemm<true, false>(s, w, H, H, B, A1, H, B1, H, C, H, 0.0f, nullptr, qa1, qb1);
  gemm<true, false>(s, w, H, H, B, A2, H, B2, H, C, H, 1.0f, nullptr, qa2, qb2);
}

static float* col_slot(const Ws& w, int64_t B, int slot) {
  return w.colpart + (size_t)slot * col_chunks(B) * H * 3;
}

// the chunk sums of one column sum into its slot (finished by k_colfinal_all);
// mode 4 also writes mode 0's sums into slot2
static void colpart(cudaStream_t s, const Ws& w, const float* X, const float* Y, const float* v, const float* V,
                    int64_t B, int mode, int slot, int slot2 = -1) {
  const unsigned g = (unsigned)col_chunks(B);
  float* part = col_slot(w, B, slot);
  float* part2 = slot2 >= 0 ? col_slot(w, B, slot2) : nullptr;
  switch (mode) {
    case 0: launch_pdl(k_colpart<0>, g, H, 0, s, X, Y, v, V, B, part, part2); break;
    case 1: launch_pdl(k_colpart<1>, g, H, 0, s, X, Y, v, V, B, part, part2); break;
    case 2: launch_pdl(k_colpart<2>, g, H, 0, s, X, Y, v, V, B, part, part2); break;
    case 3: launch_pdl(k_colpart<3>, g, H, 0, s, X, Y, v, V, B, part, part2); break;
    default: launch_pdl(k_colpart<4>, g, H, 0, s, X, Y, v, V, B, part, part2); break;
  }
}

static unsigned ew_grid(int64_t n) {
  int64_t g = (n + 255) / 256;
  return (unsigned)(g > 4096 ? 4096 : (g < 1 ? 1 : g));
}

static void epi_fallback(cudaStream_t s, const Epi& e, const float* C, int64_t n) {
  switch (e.mode) {
    case tcg::EPI_SILU: k_silu<<<ew_grid(n), 256, 0, s>>>(C, e.o1, n, e.q1); break;
    case tcg::EPI_DMUL: k_dmul<<<ew_grid(n), 256, 0, s>>>(e.e1, C, e.o1, n, e.q1, e.q2); break;
    case tcg::EPI_DD: k_dd<<<ew_grid(n), 256, 0, s>>>(e.e1, e.e2, C, e.o1, e.o2, n, e.q1); break;
    case tcg::EPI_ZBACC: k_zb_acc<<<ew_grid(n), 256, 0, s>>>(e.e1, C, e.o1, n); break;
    case tcg::EPI_SILU_D4:
      k_silu<<<ew_grid(n), 256, 0, s>>>(C, e.o1, n, e.q1);
      k_d4<<<ew_grid(n), 256, 0, s>>>(C, e.cvec, e.o2, n, e.q2);
      break;
    case tcg::EPI_ZB4: k_zb4<<<ew_grid(n), 256, 0, s>>>(e.e1, C, e.rvec, e.cvec, e.o1, n); break;
    default: break;
  }
}

static Epi epi_silu(float* h, int q) {
  Epi e;
  e.mode = tcg::EPI_SILU;
  e.o1 = h;
  e.q1 = q;
  return e;
}
static Epi epi_dmul(const float* z, float* d, int qs, int qd) {
  Epi e;
  e.mode = tcg::EPI_DMUL;
  e.e1 = z;
  e.o1 = d;
  e.q1 = qs;
  e.q2 = qd;
  return e;
}
static Epi epi_dd(const float* z, const float* u, float* ub, float* zb, int qs) {
  Epi e;
  e.mode = tcg::EPI_DD;
  e.e1 = z;
  e.e2 = u;
  e.o1 = ub;
  e.o2 = zb;
  e.q1 = qs;
  return e;
}
static Epi epi_zbacc(const float* z, float* zb) {
  Epi e;
  e.mode = tcg::EPI_ZBACC;
  e.e1 = z;
  e.o1 = zb;
  return e;
}
// H4 = silu(Z4) (qh: rounded) and D4 = silu'(Z4) w5 (qd: rounded)
static Epi epi_silu_d4(float* h, int qh, const float* w5, float* d, int qd) {
  Epi e;
  e.mode = tcg::EPI_SILU_D4;
  e.o1 = h;
  e.o2 = d;
  e.cvec = w5;
  e.q1 = qh;
  e.q2 = qd;
  return e;
}
// Zb4 = silu''(Z4) w5 Db4 + silu'(Z4) Pb w5 (C = Db4)
static Epi epi_zb4(const float* z, const float* w5, const float* pb, float* zb) {
  Epi e;
  e.mode = tcg::EPI_ZB4;
  e.e1 = z;
  e.cvec = w5;
  e.rvec = pb;
  e.o1 = zb;
  return e;
}

static Epi with_img(Epi e, uint8_t* img, int src) {
  e.img = img;
  e.img_src = src;
  return e;
}

// forward and input-gradient pass; leaves Z, H, D, U, out, G in the workspace
static void forward_backward(cudaStream_t s, const float* P, const float* x, int64_t B, const Ws& w, int q) {
  const int Bi = (int)B;
  const unsigned l1_blocks = (unsigned)((B + kL1Rows - 1) / kL1Rows);
  // quantised: the layers' weights enter every product rounded to bf16, from their images (built by
  // extra blocks of the first-layer launch)
  launch_pdl(k_layer1<0>, dim3(l1_blocks + (q ? kWimgBlocks : 0)), H, 0, s, x, P + OFF_W1, P + OFF_B1,
             (const float*)nullptr, (const float*)nullptr, w.Z[1], w.Hh[1], B, q, P, q ? w.wimg : nullptr, l1_blocks);
  // quantised, each product's A image is written by the product before it (im0 / im1 alternate)
  uint8_t* const im0 = q ? w.aimg[0] : nullptr;
  uint8_t* const im1 = q ? w.aimg[1] : nullptr;
  gemm<false, true>(s, w, Bi, H, H, w.Hh[1], H, P + OFF_W2, H, w.Z[2], H, 0.0f, P + OFF_B2, q, q,
                    with_img(epi_silu(w.Hh[2], q), im0, 1), wimg_of(w, 2, 0));                    // H2
  gemm<false, true>(s, w, Bi, H, H, w.Hh[2], H, P + OFF_W3, H, w.Z[3], H, 0.0f, P + OFF_B3, q, q,
                    with_img(epi_silu(w.Hh[3], q), im1, 1), wimg_of(w, 3, 0), im0);               // H3
  gemm<false, true>(s, w, Bi, H, H, w.Hh[3], H, P + OFF_W4, H, w.Z[4], H, 0.0f, P + OFF_B4, q, q,
                    with_img(epi_silu_d4(w.Hh[4], 0, P + OFF_W5, w.D[4], q), im0, 2), wimg_of(w, 4, 0),
                    im1);  // H4 and D4 = silu'(Z4) w5
  launch_pdl(k_rowdot, dim3((unsigned)((B + 7) / 8)), 256, 0, s, (const float*)w.Hh[4], P + OFF_W5, P + OFF_B5, B, 1,
             w.out);
  // input gradient
  gemm<false, false>(s, w, Bi, H, H, w.D[4], H, P + OFF_W4, H, w.U[3], H, 0.0f, nullptr, q, q,
                     with_img(epi_dmul(w.Z[3], w.D[3], q, q), im1, 1), wimg_of(w, 4, 1), im0);   // D3
  gemm<false, false>(s, w, Bi, H, H, w.D[3], H, P + OFF_W3, H, w.U[2], H, 0.0f, nullptr, q, q,
                     with_img(epi_dmul(w.Z[2], w.D[2], q, q), im0, 1), wimg_of(w, 3, 1), im1);   // D2
  gemm<false, false>(s, w, Bi, H, H, w.D[2], H, P + OFF_W2, H, w.U[1], H, 0.0f, nullptr, q, q,
                     epi_dmul(w.Z[1], w.D[1], 0, 0), wimg_of(w, 2, 1), im0);                    // D1
  launch_pdl(k_rowdot, dim3((unsigned)((B + 7) / 8)), 256, 0, s, (const float*)w.D[1], P + OFF_W1,
             (const float*)nullptr, B, 3, w.G);
}

// A second stream for the work of a training step that is off its critical
// path: the weight gradients and column sums run beside the chain of
// input-gradient products, on SMs and shared memory those leave free. Stream
// and fork/join events are created once per thread and device and reused (an
// event is re-recorded by every step, and a wait takes the record current at
// the time of the wait, so a set is never shared between threads). Without
// them everything runs on the caller's stream, in the same order.
constexpr int kSideEvents = 5;
struct SideStream {
  cudaStream_t st[64] = {};
  cudaEvent_t ev[64][kSideEvents] = {};
  ~SideStream() {
    for (int d = 0; d < 64; ++d) {
      for (cudaEvent_t e : ev[d])
        if (e) cudaEventDestroy(e);
      if (st[d]) cudaStreamDestroy(st[d]);
    }
  }
};

struct Side {
  cudaStream_t main, side;  // side == main when no second stream could be made
  cudaEvent_t* ev;
  void fork(int k) const {
    if (side == main) return;
    cudaEventRecord(ev[k], main);
    cudaStreamWaitEvent(side, ev[k], 0);
  }
  void join(int k) const {
    if (side == main) return;
    cudaEventRecord(ev[k], side);
    cudaStreamWaitEvent(main, ev[k], 0);
  }
};

static Side side_of(cudaStream_t s) {
  thread_local SideStream cache;
  Side r{s, s, nullptr};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return r;
  if (!cache.st[dev]) {
    cudaStream_t st = nullptr;
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return r;
    for (int k = 0; k < kSideEvents; ++k)
      if (cudaEventCreateWithFlags(&cache.ev[dev][k], cudaEventDisableTiming) != cudaSuccess) {
        for (int j = 0; j <= k; ++j)
          if (cache.ev[dev][j]) cudaEventDestroy(cache.ev[dev][j]), cache.ev[dev][j] = nullptr;
        cudaStreamDestroy(st);
        return r;
      }
    cache.st[dev] = st;
  }
  r.side = cache.st[dev];
  r.ev = cache.ev[dev];
  return r;
}

static void loss_grads(cudaStream_t s, const float* P, const float* x, const float* phi_t, const float* g_t,
                       const float* wt, int64_t B, float alpha, float beta, float* grad, float* loss, const Ws& w,
                       int q) {
  const int Bi = (int)B;
  forward_backward(s, P, x, B, w, q);
  const unsigned loss_blocks = ew_grid(B);
  launch_pdl(k_loss, loss_blocks, 256, 0, s, (const float*)w.out, (const float*)w.G, phi_t, g_t, wt, B, alpha, beta,
             w.Pb, w.Eb, w.lpart, w.pbsum);
  // Column sums go to slots of their own; one launch at the end finishes them all:
  //   0 + 6: gW1 = D1^T Eb + Zb1^T X   1 + 2: gw5 = sum silu'(Z4) Db4 + H4^T Pb
  //   3, 4, 5, 7: gb4, gb3, gb2, gb1   gb5 = sum Pb from k_loss's block sums
  // The weight gradients and column sums go to the side stream (t), forked
  // after the products whose results they read; the caller's stream (s)
  // carries the chain of input-gradient products.
  const Side sd = side_of(s);
  const cudaStream_t t = sd.side;
  sd.fork(0);
  colpart(t, w, w.D[1], nullptr, nullptr, w.Eb, B, 3, 0);                                     // gW1 = D1^T Eb
  colpart(t, w, w.Hh[4], nullptr, w.Pb, nullptr, B, 1, 2);                                 // gw5 += H4^T Pb
  // ---- through the input-gradient graph, layer 1 up to 4
  launch_pdl(k_layer1<1>, dim3((unsigned)((B + kL1Rows - 1) / kL1Rows)), H, 0, s, (const float*)w.Eb, P + OFF_W1,
             (const float*)nullptr, (const float*)w.Z[1], (const float*)w.U[1], w.Ub, w.Zb[1], B, 0,
             (const float*)nullptr, (uint8_t*)nullptr, 0u);  // Db1 = Eb W1^T
  // Ub1, Ub2, Ub3 in buffers of their own: each stays until the weight gradient
  // that pairs it with a forward-graph term (gWk = Dk^T Ub(k-1) + Zbk^T H(k-1))
  gemm<false, true>(s, w, Bi, H, H, w.Ub, H, P + OFF_W2, H, w.Db, H, 0.0f, nullptr, 0, q,
                    epi_dd(w.Z[2], w.U[2], w.Ub2, w.Zb[2], q), wimg_of(w, 2, 0));             // Db2 = Ub1 W2^T
  gemm<false, true>(s, w, Bi, H, H, w.Ub2, H, P + OFF_W3, H, w.Db, H, 0.0f, nullptr, 0, q,
                    epi_dd(w.Z[3], w.U[3], w.Ub3, w.Zb[3], q), wimg_of(w, 3, 0));             // Db3 = Ub2 W3^T
  gemm<false, true>(s, w, Bi, H, H, w.Ub3, H, P + OFF_W4, H, w.Db, H, 0.0f, nullptr, 0, q,
                    epi_zb4(w.Z[4], P + OFF_W5, w.Pb, w.Zb[4]), wimg_of(w, 4, 0));            // Db4 = Ub3 W4^T, Zb4
  sd.fork(1);
  colpart(t, w, w.Z[4], w.Db, nullptr, nullptr, B, 2, 1);                                 // gw5 = sum silu'(Z4) Db4
  // ---- potential term and the forward graph, layer 4 down to 1
  wgrad2(t, w, Bi, w.D[4], w.Ub3, q, 0, w.Zb[4], w.Hh[3], 0, q, grad + OFF_W4);           // gW4 = D4^T Ub3 + Zb4^T H3
  colpart(t, w, w.Zb[4], nullptr, nullptr, nullptr, B, 0, 3);
  gemm<false, false>(s, w, Bi, H, H, w.Zb[4], H, P + OFF_W4, H, w.Hb, H, 0.0f, nullptr, 0, q,
                     epi_zbacc(w.Z[3], w.Zb[3]), wimg_of(w, 4, 1));                            // Hb3 = Zb4 W4
  sd.fork(2);
  wgrad2(t, w, Bi, w.D[3], w.Ub2, q, 0, w.Zb[3], w.Hh[2], 0, q, grad + OFF_W3);           // gW3 = D3^T Ub2 + Zb3^T H2
  colpart(t, w, w.Zb[3], nullptr, nullptr, nullptr, B, 0, 4);
  gemm<false, false>(s, w, Bi, H, H, w.Zb[3], H, P + OFF_W3, H, w.Hb, H, 0.0f, nullptr, 0, q,
                     epi_zbacc(w.Z[2], w.Zb[2]), wimg_of(w, 3, 1));
  sd.fork(3);
  wgrad2(t, w, Bi, w.D[2], w.Ub, q, 0, w.Zb[2], w.Hh[1], 0, q, grad + OFF_W2);            // gW2 = D2^T Ub1 + Zb2^T H1
  colpart(t, w, w.Zb[2], nullptr, nullptr, nullptr, B, 0, 5);
  gemm<false, false>(s, w, Bi, H, H, w.Zb[2], H, P + OFF_W2, H, w.Hb, H, 0.0f, nullptr, 0, q,
                     epi_zbacc(w.Z[1], w.Zb[1]), wimg_of(w, 2, 1));
  colpart(s, w, w.Zb[1], nullptr, nullptr, x, B, 4, 6, 7);                                  // gW1 += Zb1^T X; gb1
  ColJobs J{};
  const int slot_a[kColJobs - 2] = {0, 1, 3, 4, 5, 7}, slot_b[kColJobs - 2] = {6, 2, -1, -1, -1, -1};
  const int64_t outs[kColJobs - 2] = {OFF_W1, OFF_W5, OFF_B4, OFF_B3, OFF_B2, OFF_B1};
  for (int j = 0; j < kColJobs - 2; ++j) {
    J.part[j][0] = col_slot(w, B, slot_a[j]);
    J.part[j][1] = slot_b[j] >= 0 ? col_slot(w, B, slot_b[j]) : nullptr;
    J.out[j] = grad + outs[j];
    J.nj[j] = j == 0 ? 3 : 1;
  }
  J.part[6][0] = w.pbsum;  // gb5
  J.out[6] = grad + OFF_B5;
  J.part[7][0] = w.lpart;  // the loss
  J.out[7] = loss;
  J.chunks = col_chunks(B);
  J.n0 = (int)loss_blocks;
  sd.join(4);
  launch_pdl(k_colfinal_all, dim3(H / 32, kColJobs), 256, 0, s, J);
}

// ---------------------------------------------------------------- device-driven training
// gal_mlp_train runs whole epochs without the host in the loop: every step
// gathers its batch on the device through a pseudo-random permutation of the
// samples, reads the step number from device memory for the learning-rate
// schedule and Adam's bias corrections, and advances it; so one step has no
// host-side arguments, is captured once as a CUDA graph and replayed.

// MurmurHash3's 32-bit finaliser (Appleby, public domain): a bijective mixer.
__device__ __forceinline__ uint32_t fmix32(uint32_t h) {
  h ^= h >> 16;
  h *= 0x85ebca6bu;
  h ^= h >> 13;
  h *= 0xc2b2ae35u;
  h ^= h >> 16;
  return h;
}

// A keyed permutation of [0, n): a four-round balanced Feistel network on
// 2 hb bits (round function fmix32 of the right half and a round key), with
// cycle-walking past n (Black & Rogaway, "Ciphers with arbitrary finite
// domains", 2002). The domain 2^(2 hb) is below 4 n, so a walk of more than a
// few steps is rare; after 64 the index maps to itself (a repeated sample,
// harmless to stochastic gradient descent).
__device__ __forceinline__ int64_t permute(int64_t i, int64_t n, int hb, uint32_t key) {
  const uint64_t mask = (1ull << hb) - 1ull;
  uint64_t x = (uint64_t)i;
  for (int walk = 0; walk < 64; ++walk) {
    uint64_t L = (x >> hb) & mask, R = x & mask;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const uint64_t F = fmix32((uint32_t)R ^ (key + 0x9e3779b9u * (uint32_t)(r + 1))) & mask;
      const uint64_t t = L ^ F;
      L = R;
      R = t;
    }
    x = (L << hb) | R;
    if ((int64_t)x < n) return (int64_t)x;
  }
  return i;
}

struct TrainRun {
  const float *u, *phi_t, *g_t, *wt;  // the whole training set
  int64_t n, batch, steps_per_epoch, total;
  int hb;
  uint64_t seed;
  float *ub, *pb, *gb, *wb;  // this step's batch
  long long* step;           // device step counter (0-based)
  const float* loss;         // this step's loss (written by k_colfinal_all)
  float* loss_per_epoch;
};

__global__ void k_gather(TrainRun r) {
  tc::pdl_wait();
  tc::pdl_trigger();
  const long long s = *r.step;
  const int64_t e = s / r.steps_per_epoch, b = s % r.steps_per_epoch;
  const uint32_t key = fmix32((uint32_t)r.seed ^ fmix32((uint32_t)e + 0x632be5abu + (uint32_t)(r.seed >> 32)));
  GRID_STRIDE(j, r.batch) {
    const int64_t i = permute(b * r.batch + j, r.n, r.hb, key);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      r.ub[j * 3 + c] = r.u[i * 3 + c];
      r.gb[j * 3 + c] = r.g_t[i * 3 + c];
    }
    r.pb[j] = r.phi_t[i];
    if (r.wt) r.wb[j] = r.wt[i];
  }
}

// Adam with the step's cosine learning rate and bias corrections (step t = s + 1).
__global__ void k_adam_run(float* p, const float* g, float* m, float* v, int64_t np, const long long* step,
                           int64_t total, float lr, float lr_final, float b1, float b2, float eps) {
  tc::pdl_wait();
  tc::pdl_trigger();
  const float t = (float)(*step + 1);
  const float lr_t = lr_final + 0.5f * (lr - lr_final) * (1.0f + cosf(3.14159265358979f * t / (float)total));
  const float c1 = 1.0f - powf(b1, t), c2 = 1.0f - powf(b2, t);
  GRID_STRIDE(i, np) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr_t * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

__global__ void k_step_end(TrainRun r) {
  tc::pdl_wait();
  tc::pdl_trigger();
  const long long s = *r.step;
  if (r.loss_per_epoch) r.loss_per_epoch[s / r.steps_per_epoch] += *r.loss / (float)r.steps_per_epoch;
  *r.step = s + 1;
}

struct RunLayout {
  size_t ub, pb, gb, wb, grad, state, total;
};

static RunLayout run_layout(int64_t B) {
  RunLayout L{};
  size_t off = (ws_bytes(B) + 255) & ~(size_t)255;  // gal_mlp_loss_grads's workspace comes first
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += (bytes + 255) & ~(size_t)255;
    return o;
  };
  L.ub = take(sizeof(float) * 3 * B);
  L.pb = take(sizeof(float) * B);
  L.gb = take(sizeof(float) * 3 * B);
  L.wb = take(sizeof(float) * B);
  L.grad = take(sizeof(float) * NPARAM);
  L.state = take(256);  // step counter, loss
  L.total = off;
  return L;
}

}  // namespace mlp
}  // namespace gal

using namespace gal;
using namespace gal::mlp;

extern "C" {

int64_t gal_mlp_num_params(void) { return NPARAM; }

gal_status gal_mlp_workspace_error(void* workspace, int64_t batch, int32_t* code, gal_stream_t stream) {
  if (!workspace || !code || batch < 1) return fail(GAL_ERR_INVALID_ARGUMENT, "bad arguments");
  int* flag = carve(workspace, batch).err;
  int v = 0;
  cudaError_t e = cudaMemcpyAsync(&v, flag, sizeof(int), cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(flag, 0, sizeof(int), (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "reading the training error flag");
  *code = v;
  return GAL_OK;
}

gal_status gal_mlp_workspace_size(int64_t batch, size_t* bytes) {
  if (!bytes || batch < 1) return fail(GAL_ERR_INVALID_ARGUMENT, "batch >= 1 required");
  if (batch > (int64_t)1 << 24) return fail(GAL_ERR_TOO_LARGE, "batch above 2^24 points");
  *bytes = ws_bytes(batch);
  return GAL_OK;
}

gal_status gal_mlp_forward_f32(const float* params, const float* x, int64_t batch, float* phi, float* grad,
                               int32_t quantize, void* workspace, size_t workspace_bytes, gal_stream_t stream) {
  if (!params || !x || batch < 1) return fail(GAL_ERR_INVALID_ARGUMENT, "bad MLP arguments");
  if (batch > (int64_t)1 << 24) return fail(GAL_ERR_TOO_LARGE, "batch above 2^24 points");
  if (!workspace || workspace_bytes < ws_bytes(batch)) return fail(GAL_ERR_WORKSPACE, "workspace too small");
  cudaStream_t s = (cudaStream_t)stream;
  const Ws w = carve(workspace, batch);
  forward_backward(s, params, x, batch, w, quantize ? 1 : 0);
  cudaError_t e = cudaSuccess;
  if (phi) e = cudaMemcpyAsync(phi, w.out, sizeof(float) * batch, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess && grad) e = cudaMemcpyAsync(grad, w.G, sizeof(float) * batch * 3, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "MLP forward");
}

gal_status gal_mlp_loss_grads(const float* params, const float* x, const float* phi_t, const float* g_t,
                              const float* weights, int64_t batch, float alpha, float beta, int32_t quantize,
                              float* grad, float* loss, void* workspace, size_t workspace_bytes, gal_stream_t stream) {
  if (!params || !x || !phi_t || !g_t || !grad || !loss || batch < 1)
    return fail(GAL_ERR_INVALID_ARGUMENT, "bad MLP arguments");
  if (batch > (int64_t)1 << 24) return fail(GAL_ERR_TOO_LARGE, "batch above 2^24 points");
  if (!workspace || workspace_bytes < ws_bytes(batch)) return fail(GAL_ERR_WORKSPACE, "workspace too small");
  cudaStream_t s = (cudaStream_t)stream;
  loss_grads(s, params, x, phi_t, g_t, weights, batch, alpha, beta, grad, loss, carve(workspace, batch),
             quantize ? 1 : 0);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "MLP loss/gradient");
}

gal_status gal_mlp_train_step(float* params, float* grad, float* adam_m, float* adam_v, const float* x,
                              const float* phi_t, const float* g_t, const float* weights, int64_t batch, float alpha,
                              float beta, float lr, float beta1, float beta2, float eps, int32_t step,
                              int32_t quantize, float* loss, void* workspace, size_t workspace_bytes,
                              gal_stream_t stream) {
  gal_status st = gal_mlp_loss_grads(params, x, phi_t, g_t, weights, batch, alpha, beta, quantize, grad, loss,
                                     workspace, workspace_bytes, stream);
  if (st != GAL_OK) return st;
  if (!adam_m || !adam_v || step < 1) return fail(GAL_ERR_INVALID_ARGUMENT, "Adam state and step >= 1 required");
  const float c1 = 1.0f - powf(beta1, (float)step), c2 = 1.0f - powf(beta2, (float)step);
  launch_pdl(k_adam, ew_grid(NPARAM), 256, 0, (cudaStream_t)stream, params, (const float*)grad, adam_m, adam_v,
             NPARAM, lr, beta1, beta2, eps, c1, c2);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "MLP Adam update");
}

gal_status gal_mlp_train_workspace_size(int64_t batch, size_t* bytes) {
  if (!bytes || batch < 1) return fail(GAL_ERR_INVALID_ARGUMENT, "batch >= 1 required");
  if (batch > (int64_t)1 << 24) return fail(GAL_ERR_TOO_LARGE, "batch above 2^24 points");
  *bytes = run_layout(batch).total;
  return GAL_OK;
}

gal_status gal_mlp_train(float* params, float* adam_m, float* adam_v, const float* u, const float* phi_t,
                         const float* g_t, const float* weights, int64_t n, int64_t batch, int32_t epochs, float alpha,
                         float beta, float lr, float lr_final, float beta1, float beta2, float eps, uint64_t seed,
                         int32_t quantize, float* loss_per_epoch, void* workspace, size_t workspace_bytes,
                         gal_stream_t stream) {
  if (!params || !adam_m || !adam_v || !u || !phi_t || !g_t || batch < 1 || epochs < 0 || n < batch)
    return fail(GAL_ERR_INVALID_ARGUMENT, "bad gal_mlp_train arguments (n >= batch >= 1, epochs >= 0)");
  if (batch > (int64_t)1 << 24 || n > ((int64_t)1 << 40)) return fail(GAL_ERR_TOO_LARGE, "batch or n too large");
  const RunLayout RL = run_layout(batch);
  if (!workspace || workspace_bytes < RL.total) return fail(GAL_ERR_WORKSPACE, "workspace too small");
  if (epochs == 0) return GAL_OK;
  char* ws = static_cast<char*>(workspace);
  TrainRun r{};
  r.u = u;
  r.phi_t = phi_t;
  r.g_t = g_t;
  r.wt = weights;
  r.n = n;
  r.batch = batch;
  r.steps_per_epoch = n / batch;
  r.total = r.steps_per_epoch * epochs;
  int bits = 1;
  while (bits < 62 && ((int64_t)1 << bits) < n) ++bits;
  r.hb = (bits + 1) / 2;
  r.seed = seed;
  r.ub = reinterpret_cast<float*>(ws + RL.ub);
  r.pb = reinterpret_cast<float*>(ws + RL.pb);
  r.gb = reinterpret_cast<float*>(ws + RL.gb);
  r.wb = reinterpret_cast<float*>(ws + RL.wb);
  r.step = reinterpret_cast<long long*>(ws + RL.state);
  float* loss = reinterpret_cast<float*>(ws + RL.state + 8);
  r.loss = loss;
  r.loss_per_epoch = loss_per_epoch;
  float* grad = reinterpret_cast<float*>(ws + RL.grad);
  const Ws w = carve(workspace, batch);
  const int q = quantize ? 1 : 0;
  cudaStream_t caller = (cudaStream_t)stream;
  // one step is captured on a private stream (the legacy default stream cannot
  // be captured), ordered after and before the caller's stream
  cudaStream_t s = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_in, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev_out, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(ev_in, caller);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev_in, 0);
  if (e == cudaSuccess) e = cudaMemsetAsync(ws + RL.state, 0, 256, s);
  if (e == cudaSuccess && loss_per_epoch) e = cudaMemsetAsync(loss_per_epoch, 0, sizeof(float) * epochs, s);
  auto one_step = [&]() {
    launch_pdl(k_gather, ew_grid(batch), 256, 0, s, r);
    loss_grads(s, params, r.ub, r.pb, r.gb, weights ? r.wb : nullptr, batch, alpha, beta, grad, loss, w, q);
    launch_pdl(k_adam_run, ew_grid(NPARAM), 256, 0, s, params, (const float*)grad, adam_m, adam_v, NPARAM,
               (const long long*)r.step, r.total, lr, lr_final, beta1, beta2, eps);
    launch_pdl(k_step_end, 1, 1, 0, s, r);
  };
  if (e == cudaSuccess) {
    // the first step runs uncaptured: it configures the tensor-core kernel
    one_step();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && r.total > 1) {
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
      one_step();
      const cudaError_t e2 = cudaStreamEndCapture(s, &g);
      e = e2 != cudaSuccess ? e2 : cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&exec, g, 0);
    for (int64_t k = 1; k < r.total && e == cudaSuccess; ++k) e = cudaGraphLaunch(exec, s);
  }
  if (ev_out && s) {
    cudaEventRecord(ev_out, s);
    cudaStreamWaitEvent(caller, ev_out, 0);
  }
  if (exec) cudaGraphExecDestroy(exec);
  if (g) cudaGraphDestroy(g);
  if (ev_in) cudaEventDestroy(ev_in);
  if (ev_out) cudaEventDestroy(ev_out);
  if (s) cudaStreamDestroy(s);  // returns at once; queued work still completes
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "gal_mlp_train");
}

}  // extern "C"
