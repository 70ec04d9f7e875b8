// Tensor-core inference of the potential-surrogate MLP: potential and its
// gradient (the acceleration) at n positions, one fused kernel.
//
// One CTA per SM, persistent over tiles of 128 points, 256 threads (two per
// point: each handles 128 of the 256 hidden units). Per tile:
//   layer 1 (3 -> 256) on CUDA cores -> h1 (bf16) into the shared-memory
//   operand tile; then six 128x256x256 products on the tensor cores
//   (tcgen05.mma kind::f16, bf16 x bf16 -> f32 accumulator in TMEM):
//     z2 = h1 W2^T, z3 = h2 W3^T, z4 = h3 W4^T           (forward)
//     u3 = d4 W4,   u2 = d3 W3,   u1 = d2 W2              (input gradient)
//   with d4 = silu'(z4) w5, d3 = silu'(z3) u3, d2 = silu'(z2) u2 (bf16), and
//   grad_u out = (silu'(z1) u1) W1 on CUDA cores. silu'(z2), silu'(z3) wait in
//   TMEM as packed bf16 pairs; every operand tile is rewritten in place.
// Weights stream through a three-stage ring of 32 KB K-blocks (bulk copies from
// pre-swizzled global images) overlapping the products. The numerics are those
// of the training kernels' quantised forward/backward (mlp_train.cu).
//
// Every mbarrier wait is bounded: on timeout the kernel records an error code,
// releases its TMEM and returns.
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "handle.h"
#include "mlp.cuh"
#include "tc.cuh"

namespace gal {
namespace mlp {

constexpr int TILE = 128;
constexpr int NTHREADS = 256;
constexpr int STAGES = 3;
constexpr uint32_t KBLOCK_BYTES = 256 * 128;           // 256 rows x 64 bf16
constexpr int KBLOCKS_PER_GEMM = 4;
constexpr int GEMMS = 6;
constexpr int KBLOCKS_PER_TILE = GEMMS * KBLOCKS_PER_GEMM;  // 24
constexpr uint32_t A_BYTES = TILE * 256 * 2;            // 64 KB
constexpr uint32_t SMEM_A = 0;
constexpr uint32_t SMEM_RING = A_BYTES;
constexpr uint32_t SMEM_SMALL = SMEM_RING + STAGES * KBLOCK_BYTES;  // 160 KB
constexpr int SMALL_FLOATS = H * 3 + 5 * H + 1;         // W1, b1, b2, b3, b4, w5, b5
constexpr uint32_t SMEM_PART = SMEM_SMALL + ((SMALL_FLOATS * 4 + 255) / 256) * 256;
constexpr uint32_t SMEM_BAR = SMEM_PART + TILE * 4 * 4;
constexpr uint32_t SMEM_TOTAL = SMEM_BAR + 256;
constexpr uint32_t SMEM_ALLOC = SMEM_TOTAL + 1024;      // room to align the base to 1024
constexpr uint32_t WAIT_LIMIT = 1u << 24;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t COL_S2 = 256, COL_S3 = 384;          // packed silu'(z2), silu'(z3)

struct InferArgs {
  const double* x;       // [3][n]
  int64_t n;
  double inv_length;     // network input u = x * inv_length
  double gscale;         // physical gradient = gscale * grad_u out
  double pscale;         // physical potential = pscale * out
  double* grad;          // [3][n] or NULL
  int32_t accumulate;    // grad += (1) or = (0)
  double* phi;           // [n] or NULL
  const float* small;    // W1, b1, b2, b3, b4, w5, b5 (SMALL_FLOATS)
  const uint8_t* wimg;   // 24 pre-swizzled 32 KB K-blocks
  int* err;
};

struct Ring {
  uint64_t* full;
  uint64_t* empty;
  uint8_t* buf;
  const uint8_t* wimg;
  int64_t total;  // K-blocks this CTA will consume
};

// issue the bulk copy of K-block jj (thread 0 only)
__device__ __forceinline__ bool produce(const Ring& r, int64_t jj) {
  if (jj >= r.total) return true;
  const int s = (int)(jj % STAGES);
  const int64_t use = jj / STAGES;
  if (use > 0 && !tc::mbar_wait(&r.empty[s], (uint32_t)((use - 1) & 1), WAIT_LIMIT)) return false;
  tc::mbar_expect_tx(&r.full[s], KBLOCK_BYTES);
  tc::bulk_g2s(r.buf + (size_t)s * KBLOCK_BYTES, r.wimg + (size_t)(jj % KBLOCKS_PER_TILE) * KBLOCK_BYTES,
               KBLOCK_BYTES, &r.full[s]);
  return true;
}

// one 128x256x256 product: D[tmem] = A[smem tile] x (K-blocks j0..j0+3)^T
__device__ __forceinline__ bool issue_gemm(const Ring& r, int64_t j0, uint32_t a_base, uint32_t tmem,
                                           uint64_t* mma_bar) {
  constexpr uint32_t idesc = tc::idesc_bf16(TILE, 256);
  for (int kb = 0; kb < KBLOCKS_PER_GEMM; ++kb) {
    const int64_t j = j0 + kb;
    const int s = (int)(j % STAGES);
    if (!tc::mbar_wait(&r.full[s], (uint32_t)((j / STAGES) & 1), WAIT_LIMIT)) return false;
    tc::tc_fence_after();
    const uint32_t b_base = tc::smem_u32(r.buf + (size_t)s * KBLOCK_BYTES);
#pragma unroll
    for (int ks = 0; ks < 4; ++ks) {
      const uint64_t ad = tc::desc_sw128(a_base + kb * (TILE * 128) + ks * 32);
      const uint64_t bd = tc::desc_sw128(b_base + ks * 32);
      tc::mma_bf16(tmem, ad, bd, idesc, (kb | ks) != 0);
    }
    tc::mma_commit(&r.empty[s]);       // stage free once these products complete
    if (!produce(r, j + 2)) return false;
  }
  tc::mma_commit(mma_bar);
  return true;
}

__device__ __forceinline__ float sig(float z) { return tc::rcp_approx(1.0f + __expf(-z)); }

// write 32 consecutive hidden units [c, c+32) of row `row` into the operand tile
__device__ __forceinline__ void store_row32(uint8_t* tile, int row, int c, const float (&v)[32]) {
#pragma unroll
  for (int q = 0; q < 4; ++q) {  // four 16-byte chunks of 8 values
    uint4 w;
    w.x = tc::pack_bf16x2(v[8 * q + 0], v[8 * q + 1]);
    w.y = tc::pack_bf16x2(v[8 * q + 2], v[8 * q + 3]);
    w.z = tc::pack_bf16x2(v[8 * q + 4], v[8 * q + 5]);
    w.w = tc::pack_bf16x2(v[8 * q + 6], v[8 * q + 7]);
    *reinterpret_cast<uint4*>(tile + tc::sw128_offset(TILE, row, c + 8 * q)) = w;
  }
}

__global__ void __launch_bounds__(NTHREADS, 1) k_mlp_infer(InferArgs a) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  uint8_t* tileA = smem + SMEM_A;
  float* sm = reinterpret_cast<float*>(smem + SMEM_SMALL);
  const float* sW1 = sm;
  const float* sb1 = sm + 3 * H;
  const float* sb2 = sb1 + H;
  const float* sb3 = sb2 + H;
  const float* sb4 = sb3 + H;
  const float* sw5 = sb4 + H;
  float* part = reinterpret_cast<float*>(smem + SMEM_PART);  // [TILE][4]
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + SMEM_BAR);
  uint64_t* full = bars;
  uint64_t* empty = bars + STAGES;
  uint64_t* mma_bar = bars + 2 * STAGES;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(bars + 2 * STAGES + 1);
  __shared__ int abort_flag;

  const int t = threadIdx.x;
  const int row = t & (TILE - 1);
  const int half = t >> 7;
  const int c0 = half * 128;
  const int warp = t >> 5;

  for (int i = t; i < SMALL_FLOATS; i += NTHREADS) sm[i] = a.small[i];
  if (t == 0) {
    abort_flag = 0;
    for (int s = 0; s < STAGES; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    tc::mbar_init(mma_bar, 1);
    tc::fence_barrier_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tmem_holder, TMEM_COLS);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;  // this warp's TMEM lanes

  const int64_t ntiles = (a.n + TILE - 1) / TILE;
  const int64_t my_tiles = ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;
  Ring ring{full, empty, smem + SMEM_RING, a.wimg, my_tiles * KBLOCKS_PER_TILE};
  const uint32_t a_base = tc::smem_u32(tileA);
  if (t == 0) {
    if (!produce(ring, 0) || !produce(ring, 1)) abort_flag = 1;
  }
  __syncthreads();
  int64_t gemm_count = 0;   // products waited for
  int64_t gemm_issued = 0;  // products issued (thread 0)

  for (int64_t it = 0; it < my_tiles && !abort_flag; ++it) {
    const int64_t tile = blockIdx.x + it * gridDim.x;
    const int64_t gi = tile * TILE + row;
    const bool valid = gi < a.n;
    float u[3] = {0.f, 0.f, 0.f};
    if (valid) {
#pragma unroll
      for (int j = 0; j < 3; ++j) u[j] = (float)(a.x[j * a.n + gi] * a.inv_length);
    }
    // layer 1 on CUDA cores: h1 = silu(W1 u + b1) -> operand tile
    for (int c = c0; c < c0 + 128; c += 32) {
      float v[32];
#pragma unroll
      for (int q = 0; q < 32; ++q) {
        const int cc = c + q;
        const float z = fmaf(sW1[3 * cc], u[0], fmaf(sW1[3 * cc + 1], u[1], fmaf(sW1[3 * cc + 2], u[2], sb1[cc])));
        v[q] = z * sig(z);
      }
      store_row32(tileA, row, c, v);
    }
    float gpart[3] = {0.f, 0.f, 0.f};
    float ppart = 0.f;
    for (int g = 0; g < GEMMS; ++g) {
      tc::fence_proxy_async_smem();
      tc::tc_fence_before();
      __syncthreads();
      if (abort_flag) break;
      if (t == 0) {
        tc::tc_fence_after();
        if (!issue_gemm(ring, (it * GEMMS + g) * KBLOCKS_PER_GEMM, a_base, tmem, mma_bar)) {
          abort_flag = 1;
          if (a.err) atomicExch(a.err, 1);
        } else {
          ++gemm_issued;
        }
      }
      if (!tc::mbar_wait(mma_bar, (uint32_t)(gemm_count & 1), WAIT_LIMIT)) {
        abort_flag = 1;
        if (a.err) atomicExch(a.err, 2);
      }
      ++gemm_count;
      __syncthreads();
      if (abort_flag) break;
      tc::tc_fence_after();
      // epilogue over this thread's 128 columns, 32 at a time
      for (int c = c0; c < c0 + 128; c += 32) {
        uint32_t acc[32];
        tc::tmem_ld32(tmem + lane_base + (uint32_t)c, acc);
        uint32_t sp[16];
        if (g == 3 || g == 4) tc::tmem_ld16(tmem + lane_base + (uint32_t)((g == 3 ? COL_S3 : COL_S2) + c / 2), sp);
        tc::tmem_wait_ld();
        float v[32];
        if (g <= 1) {  // z2 / z3: h = silu(z) -> tile, silu'(z) -> TMEM
          const float* bb = g == 0 ? sb2 : sb3;
          uint32_t spk[16];
#pragma unroll
          for (int q = 0; q < 32; q += 2) {
            const float z0 = __uint_as_float(acc[q]) + bb[c + q];
            const float z1 = __uint_as_float(acc[q + 1]) + bb[c + q + 1];
            const float s0 = sig(z0), s1 = sig(z1);
            v[q] = z0 * s0;
            v[q + 1] = z1 * s1;
            spk[q / 2] = tc::pack_bf16x2(s0 * (1.f + z0 * (1.f - s0)), s1 * (1.f + z1 * (1.f - s1)));
          }
          tc::tmem_st16(tmem + lane_base + (uint32_t)((g == 0 ? COL_S2 : COL_S3) + c / 2), spk);
          store_row32(tileA, row, c, v);
        } else if (g == 2) {  // z4: d4 = silu'(z4) w5 -> tile; out = w5 . silu(z4)
#pragma unroll
          for (int q = 0; q < 32; ++q) {
            const float z = __uint_as_float(acc[q]) + sb4[c + q];
            const float s = sig(z);
            ppart = fmaf(z * s, sw5[c + q], ppart);
            v[q] = s * (1.f + z * (1.f - s)) * sw5[c + q];
          }
          store_row32(tileA, row, c, v);
        } else if (g <= 4) {  // u3 / u2: d = silu'(z) u -> tile
#pragma unroll
          for (int q = 0; q < 32; q += 2) {
            v[q] = tc::bf16_lo(sp[q / 2]) * __uint_as_float(acc[q]);
            v[q + 1] = tc::bf16_hi(sp[q / 2]) * __uint_as_float(acc[q + 1]);
          }
          store_row32(tileA, row, c, v);
        } else {  // u1: grad_u out = sum_c silu'(z1_c) u1_c W1[c]
#pragma unroll
          for (int q = 0; q < 32; ++q) {
            const int cc = c + q;
            const float z = fmaf(sW1[3 * cc], u[0], fmaf(sW1[3 * cc + 1], u[1], fmaf(sW1[3 * cc + 2], u[2], sb1[cc])));
            const float s = sig(z);
            const float d1 = s * (1.f + z * (1.f - s)) * __uint_as_float(acc[q]);
            gpart[0] = fmaf(d1, sW1[3 * cc], gpart[0]);
            gpart[1] = fmaf(d1, sW1[3 * cc + 1], gpart[1]);
            gpart[2] = fmaf(d1, sW1[3 * cc + 2], gpart[2]);
          }
        }
      }
      if (g <= 1) tc::tmem_wait_st();
    }
    if (abort_flag) break;
    // combine the two halves of each row and write the outputs
    if (half == 1) {
      part[row * 4 + 0] = gpart[0];
      part[row * 4 + 1] = gpart[1];
      part[row * 4 + 2] = gpart[2];
      part[row * 4 + 3] = ppart;
    }
    __syncthreads();
    if (half == 0 && valid) {
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const double gj = a.gscale * (double)(gpart[j] + part[row * 4 + j]);
        if (a.grad) a.grad[j * a.n + gi] = a.accumulate ? a.grad[j * a.n + gi] + gj : gj;
      }
      if (a.phi) a.phi[gi] = a.pscale * (double)(ppart + part[row * 4 + 3] + sw5[H]);
    }
  }
  // release TMEM, making sure no product is still running on it
  if (abort_flag && t == 0 && gemm_issued > gemm_count)
    tc::mbar_wait(mma_bar, (uint32_t)((gemm_issued - 1) & 1), WAIT_LIMIT);
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, TMEM_COLS);
}

}  // namespace mlp
}  // namespace gal

using namespace gal;
using namespace gal::mlp;

struct gal_mlp {
  float* d_small;      // W1, b1, b2, b3, b4, w5, b5
  uint8_t* d_wimg;     // 24 x 32 KB pre-swizzled bf16 K-blocks
  int* d_err;
  double length_scale, phi_scale;
};

namespace {
uint16_t to_bf16(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  u += 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
}  // namespace

extern "C" {

gal_status gal_mlp_create(const float* params_host, double length_scale, double phi_scale, gal_mlp** out) {
  if (!params_host || !out || !(length_scale > 0) || !(phi_scale != 0))
    return fail(GAL_ERR_INVALID_ARGUMENT, "bad gal_mlp_create arguments");
  *out = nullptr;
  const float* P = params_host;
  std::vector<float> small(SMALL_FLOATS);
  std::memcpy(small.data(), P + OFF_W1, sizeof(float) * 3 * H);
  std::memcpy(small.data() + 3 * H, P + OFF_B1, sizeof(float) * H);
  std::memcpy(small.data() + 4 * H, P + OFF_B2, sizeof(float) * H);
  std::memcpy(small.data() + 5 * H, P + OFF_B3, sizeof(float) * H);
  std::memcpy(small.data() + 6 * H, P + OFF_B4, sizeof(float) * H);
  std::memcpy(small.data() + 7 * H, P + OFF_W5, sizeof(float) * H);
  small[8 * H] = P[OFF_B5];
  // B operands, K-major: product "A x B^T" with B[n][k]. Forward z = h W^T uses
  // B = W (n = output unit, k = input unit); backward u = d W uses B = W^T.
  std::vector<uint8_t> img((size_t)KBLOCKS_PER_TILE * KBLOCK_BYTES, 0);
  const int64_t offs[3] = {OFF_W2, OFF_W3, OFF_W4};
  const int order[6][2] = {{0, 0}, {1, 0}, {2, 0}, {2, 1}, {1, 1}, {0, 1}};  // (matrix, transposed)
  for (int g = 0; g < GEMMS; ++g) {
    const float* W = P + offs[order[g][0]];
    const bool tr = order[g][1] != 0;
    for (int n = 0; n < H; ++n)
      for (int k = 0; k < H; ++k) {
        const float v = tr ? W[(size_t)k * H + n] : W[(size_t)n * H + k];
        const uint32_t kb = k >> 6;
        const uint32_t off = tc::sw128_offset(256, n, k & 63);  // within the K-block
        const uint16_t b = to_bf16(v);
        std::memcpy(&img[((size_t)g * KBLOCKS_PER_GEMM + kb) * KBLOCK_BYTES + off], &b, 2);
      }
  }
  gal_mlp* m = new gal_mlp();
  m->length_scale = length_scale;
  m->phi_scale = phi_scale;
  cudaError_t e = cudaMalloc(&m->d_small, sizeof(float) * small.size());
  if (e == cudaSuccess) e = cudaMalloc(&m->d_wimg, img.size());
  if (e == cudaSuccess) e = cudaMalloc(&m->d_err, sizeof(int));
  if (e == cudaSuccess) e = cudaMemcpy(m->d_small, small.data(), sizeof(float) * small.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(m->d_wimg, img.data(), img.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(m->d_err, 0, sizeof(int));
  if (e != cudaSuccess) {
    cudaFree(m->d_small);
    cudaFree(m->d_wimg);
    cudaFree(m->d_err);
    delete m;
    return cuda_fail(e, "gal_mlp_create");
  }
  *out = m;
  return GAL_OK;
}

gal_status gal_mlp_destroy(gal_mlp* m) {
  if (!m) return GAL_OK;
  cudaFree(m->d_small);
  cudaFree(m->d_wimg);
  cudaFree(m->d_err);
  delete m;
  return GAL_OK;
}

gal_status gal_mlp_eval(const gal_mlp* m, const double* x, int64_t n, double* grad, int32_t accumulate,
                        double grad_sign, double* phi, gal_stream_t stream) {
  if (!m || (!x && n) || n < 0) return fail(GAL_ERR_INVALID_ARGUMENT, "bad gal_mlp_eval arguments");
  if (n == 0) return GAL_OK;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_ALLOC);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_mlp_infer)");
    attr = true;
  }
  InferArgs a{};
  a.x = x;
  a.n = n;
  a.inv_length = 1.0 / m->length_scale;
  a.gscale = grad_sign * m->phi_scale / m->length_scale;
  a.pscale = m->phi_scale;
  a.grad = grad;
  a.accumulate = accumulate;
  a.phi = phi;
  a.small = m->d_small;
  a.wimg = m->d_wimg;
  a.err = m->d_err;
  const int64_t ntiles = (n + TILE - 1) / TILE;
  int64_t grid = device_sm_count();
  if (grid > ntiles) grid = ntiles;
  k_mlp_infer<<<(unsigned)grid, NTHREADS, SMEM_ALLOC, (cudaStream_t)stream>>>(a);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GAL_OK : cuda_fail(e, "MLP inference launch");
}

gal_status gal_mlp_error(const gal_mlp* m, int32_t* code) {
  if (!m || !code) return fail(GAL_ERR_INVALID_ARGUMENT, "bad arguments");
  int v = 0;
  cudaError_t e = cudaMemcpy(&v, m->d_err, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "reading the MLP error flag");
  *code = v;
  return GAL_OK;
}

}  // extern "C"
