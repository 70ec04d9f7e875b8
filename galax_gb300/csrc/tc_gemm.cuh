// Tensor-core GEMM for the surrogate's training products (tcgen05.mma,
// kind::f16: bf16 operands, f32 accumulation in TMEM):
//
//   C[m][n] = sum_k A(m, k) B(n, k) (+ beta C[m][n]) (+ bias[n])
//
// with A(m, k) = A[m sam + k sak] and B(n, k) = B[n sbn + k sbk] read from FP32
// arrays of any layout (row- or column-major), so the transposed products of
// backpropagation need no transposes in memory. Every operand block is rounded
// to bf16 on its way into shared memory; an operand may instead be split into
// two bf16 parts, v = hi + lo with hi = bf16(v), lo = bf16(v - hi), and the
// product formed as hi*hi + hi*lo + lo*hi (the bf16x3 scheme of Henry, Tang &
// Heinecke, "Leveraging the bfloat16 artificial intelligence datatype for
// higher-precision computations", ARITH 2019), which carries ~16 significant
// bits per operand: the FP32 reference gradients of the loss need that, the
// quantised forward pass does not.
//
// One CTA of 256 threads computes a 128 x 128 tile of C (so the 8192 x 256
// products of a training batch spread over 128 CTAs); K runs in blocks of 64
// through two shared-memory stages (A and B hi, and lo for split operands:
// 32-64 KB; 128 x 64, K-major, 128-byte swizzle, the layout of the inference
// kernel's operands).
// All threads load and convert; thread 0 issues the products and commits them
// to the stage's mbarrier, which frees the stage for the block after next. The
// accumulator (128 TMEM columns) drains through shared memory so that C is
// read and written row-contiguously. With gridDim.z > 1 each z takes a K
// range and stores its partial tile into its own slice of `part` ([z][M][N]),
// which k_splitk_sum then adds into C in z order, so results do not depend on
// the order in which CTAs finish.
//
// Every mbarrier wait is bounded; on timeout the kernel records an error code,
// waits (bounded) for its products, releases TMEM and returns.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "mlp.cuh"
#include "tc.cuh"

namespace gal {
namespace tcg {

constexpr int BM = 128, BN = 128, BK = 64;
constexpr int NTHREADS = 256;
constexpr uint32_t A_BLK = BM * 128;  // 16 KB: 128 rows x 64 bf16
constexpr uint32_t B_BLK = BN * 128;  // 16 KB
constexpr int OUT_STRIDE = BN + 4;  // floats per staged output row: rows 16-byte aligned, float4 access conflict-free
constexpr uint32_t OUT_BYTES = (uint32_t)BM * OUT_STRIDE * 4;  // the staged output tile (reuses the stages)
constexpr uint32_t WAIT_LIMIT = 1u << 24;
// A stage holds A hi [, A lo], B hi [, B lo] (the lo parts only for split
// operands), so products without split operands need half the shared memory
// and several CTAs (of this or a concurrent product) fit on an SM.
__host__ __device__ constexpr uint32_t stage_bytes(int split_a, int split_b) {
  return A_BLK * (1 + (split_a ? 1 : 0)) + B_BLK * (1 + (split_b ? 1 : 0));
}
__host__ __device__ constexpr uint32_t bar_offset(uint32_t stage) {
  return 2 * stage > OUT_BYTES ? 2 * stage : (OUT_BYTES + 1023) / 1024 * 1024;
}
constexpr uint32_t BIMG_BYTES = 4 * B_BLK;  // the B image of one column block (K = 256)
// image mode: the two A stages, then B whole
__host__ __device__ constexpr uint32_t bar_offset_img(uint32_t stage) {
  return 2 * stage + BIMG_BYTES > OUT_BYTES ? 2 * stage + BIMG_BYTES : (OUT_BYTES + 1023) / 1024 * 1024;
}
__host__ __device__ constexpr uint32_t smem_alloc_at(uint32_t bar_off) {
  return bar_off + 64 + 1024;  // barriers, TMEM address, alignment slack
}
__host__ __device__ constexpr uint32_t smem_alloc(uint32_t stage) { return smem_alloc_at(bar_offset(stage)); }
constexpr uint32_t SMEM_MAX = smem_alloc(stage_bytes(1, 1));
static_assert(SMEM_MAX <= 227 * 1024, "shared memory budget");

struct Args {
  int M, N, K;
  const float* A;
  int64_t sam, sak;
  const float* B;
  int64_t sbn, sbk;
  float* C;
  int64_t ldc;
  float beta;
  const float* bias;
  int split_a, split_b;
  uint32_t stage;    // bytes per pipeline stage: stage_bytes() of the launch's most split source
  uint32_t bar_off;  // shared-memory offset of the barriers (bar_offset())
  // Optional: B as a pre-swizzled bf16 image (K = 256, B not split, one K
  // range): for CTA column block nb the 64 KB at bimg + nb * 64 KB, the four
  // 16 KB K blocks exactly as put() would lay them out; bulk-copied into
  // shared memory at the start instead of staged through registers.
  const uint8_t* bimg;
  // Optional, with bimg: A as a bf16 image of the same layout (row block mb
  // of 128 rows at aimg + mb * 64 KB); then the product is fed by bulk copies
  // alone (split_a = 0, K = 256).
  const uint8_t* aimg;
  // Optional: the store phase also writes a bf16 image (the layout of aimg)
  // of o1 (img_src = 1) or o2 (img_src = 2), for the next product's A.
  uint8_t* img_out;
  int img_src;
  int kchunk;  // K per blockIdx.z, a multiple of BK
  float* part;  // gridDim.z > 1: partial tiles [z][M][N]
  int* err;
  // Optional second product of the same shape and K, added into the same C:
  // slices blockIdx.z >= z2 compute A2(m, k) B2(n, k) over their K range
  // (slice z - z2); only with gridDim.z > 1 (partial tiles)
  const float* A2;
  int64_t sam2, sak2;
  const float* B2;
  int64_t sbn2, sbk2;
  int split_a2, split_b2;
  int z2;
  // Elementwise work of the next training step fused into the store of C
  // (same layout as C, v = the stored value of C[m][n]):
  //   EPI_SILU : o1 = silu(v)                                  (q1: rounded to bf16)
  //   EPI_DMUL : o1 = silu'(e1) v                              (q1: silu' rounded, q2: o1 rounded)
  //   EPI_DD   : o1 = silu'(e1) v (q1: silu' rounded), o2 = silu''(e1) e2 v; C not stored
  //   EPI_ZBACC: o1 += silu'(e1) v; C not stored
  //   EPI_SILU_D4: o1 = silu(v) (q1: rounded), o2 = silu'(v) cvec[n] (q2: rounded)
  //   EPI_ZB4  : o1 = silu''(e1) cvec[n] v + silu'(e1) rvec[m] cvec[n]
  int epi;
  const float *e1, *e2;
  float *o1, *o2;
  const float* cvec;  // per column n
  const float* rvec;  // per row m
  int q1, q2;
};

enum { EPI_NONE = 0, EPI_SILU = 1, EPI_DMUL = 2, EPI_DD = 3, EPI_ZBACC = 4, EPI_SILU_D4 = 5, EPI_ZB4 = 6 };

template <int EPI>
constexpr bool epi_stores_c() {
  return EPI != EPI_DD && EPI != EPI_ZBACC;
}
template <int EPI>
constexpr bool epi_reads_e1() {
  return EPI == EPI_DMUL || EPI == EPI_DD || EPI == EPI_ZBACC || EPI == EPI_ZB4;
}
template <int EPI>
constexpr bool epi_writes_o2() {
  return EPI == EPI_DD || EPI == EPI_SILU_D4;
}

// The fused step for one element: v = C[m][n] (beta and bias applied), x1 =
// e1, x2 = e2, xo = o1 at the same place, cv = cvec[n], rv = rvec[m].
template <int EPI>
__device__ __forceinline__ void fused_step(const Args& a, float v, float x1, float x2, float xo, float cv, float rv,
                                           float& r1, float& r2) {
  if constexpr (EPI == EPI_SILU || EPI == EPI_SILU_D4) {
    const float h = mlp::silu(v);
    r1 = a.q1 ? mlp::bf16r(h) : h;
    if constexpr (EPI == EPI_SILU_D4) {
      const float d = mlp::dsilu(v) * cv;
      r2 = a.q2 ? mlp::bf16r(d) : d;
    }
  } else if constexpr (EPI == EPI_DMUL) {
    float sd = mlp::dsilu(x1);
    if (a.q1) sd = mlp::bf16r(sd);
    const float d = sd * v;
    r1 = a.q2 ? mlp::bf16r(d) : d;
  } else if constexpr (EPI == EPI_DD) {
    float sd = mlp::dsilu(x1);
    if (a.q1) sd = mlp::bf16r(sd);
    r1 = sd * v;
    r2 = mlp::d2silu(x1) * x2 * v;
  } else if constexpr (EPI == EPI_ZBACC) {
    r1 = xo + mlp::dsilu(x1) * v;
  } else if constexpr (EPI == EPI_ZB4) {
    r1 = mlp::d2silu(x1) * cv * v + mlp::dsilu(x1) * rv * cv;
  }
}

__device__ __forceinline__ uint16_t bf16_bits(float f) {
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(0.0f), "f"(f));
  return (uint16_t)(r & 0xffffu);
}

// One thread's share of an operand block, rows [r0, r0+R) x k [k0, k0+64):
// PER chunks of 8 consecutive k. Consecutive threads take consecutive chunks
// along the contiguous dimension of the source, so global reads coalesce.
// fetch() issues all of a thread's loads; put() converts them to bf16 (hi,
// and lo when split) and stores them into the 128-byte-swizzled stage. The
// main loop fetches block kb + 1 before the barrier and product issue of
// block kb, so the load latency overlaps them.
template <int R>
struct Frag {
  static constexpr int PER = R * 8 / NTHREADS;
  float v[PER][8];
};

template <int R>
__device__ __forceinline__ void chunk_of(int u, bool kmajor, int& row, int& c) {
  const int i = threadIdx.x + u * NTHREADS;
  row = kmajor ? (i >> 3) : (i % R);
  c = kmajor ? (i & 7) : (i / R);
}

template <int R>
__device__ __forceinline__ void fetch(Frag<R>& f, const float* src, int64_t s_row, int64_t s_k, int r0, int rlim,
                                      int k0, int klim) {
  const bool kmajor = s_k == 1;
#pragma unroll
  for (int u = 0; u < Frag<R>::PER; ++u) {
    int row, c;
    chunk_of<R>(u, kmajor, row, c);
    const int gr = r0 + row, k = k0 + 8 * c;
    if (kmajor && gr < rlim && k + 8 <= klim && ((reinterpret_cast<uintptr_t>(src + gr * s_row + k) & 15) == 0)) {
      const float4 a = __ldg(reinterpret_cast<const float4*>(src + gr * s_row + k));
      const float4 b = __ldg(reinterpret_cast<const float4*>(src + gr * s_row + k + 4));
      f.v[u][0] = a.x; f.v[u][1] = a.y; f.v[u][2] = a.z; f.v[u][3] = a.w;
      f.v[u][4] = b.x; f.v[u][5] = b.y; f.v[u][6] = b.z; f.v[u][7] = b.w;
    } else {
#pragma unroll
      for (int j = 0; j < 8; ++j)
        f.v[u][j] = (gr < rlim && k + j < klim) ? __ldg(src + gr * s_row + (int64_t)(k + j) * s_k) : 0.0f;
    }
  }
}

template <int R>
__device__ __forceinline__ void put(const Frag<R>& f, uint8_t* hi, uint8_t* lo, bool kmajor, int split) {
#pragma unroll
  for (int u = 0; u < Frag<R>::PER; ++u) {
    int row, c;
    chunk_of<R>(u, kmajor, row, c);
    uint32_t h[4], l[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint16_t h0 = bf16_bits(f.v[u][2 * j]), h1 = bf16_bits(f.v[u][2 * j + 1]);
      h[j] = (uint32_t)h0 | ((uint32_t)h1 << 16);
      if (split) {
        const uint16_t l0 = bf16_bits(f.v[u][2 * j] - __uint_as_float((uint32_t)h0 << 16));
        const uint16_t l1 = bf16_bits(f.v[u][2 * j + 1] - __uint_as_float((uint32_t)h1 << 16));
        l[j] = (uint32_t)l0 | ((uint32_t)l1 << 16);
      }
    }
    const uint32_t off = tc::sw128_offset(R, row, 8 * c);
    *reinterpret_cast<uint4*>(hi + off) = make_uint4(h[0], h[1], h[2], h[3]);
    if (split) *reinterpret_cast<uint4*>(lo + off) = make_uint4(l[0], l[1], l[2], l[3]);
  }
}

__device__ __forceinline__ void prefetch_l2(const float* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// The operands of the fused step do not depend on the product: ask L2 for the
// tile's lines while the tensor cores work, so that the store phase finds them
// there.
template <int EPI>
__device__ __forceinline__ void prefetch_epilogue(const Args& a, int m0, int n0) {
  if constexpr (epi_reads_e1<EPI>()) {
    for (int i = threadIdx.x; i < BM * (BN / 32); i += NTHREADS) {
      const int m = m0 + (i >> 2), n = n0 + (i & 3) * 32;
      if (m >= a.M || n >= a.N) continue;
      const int64_t idx = (int64_t)m * a.ldc + n;
      prefetch_l2(a.e1 + idx);
      if constexpr (EPI == EPI_DD) prefetch_l2(a.e2 + idx);
      if constexpr (EPI == EPI_ZBACC) prefetch_l2(a.o1 + idx);
    }
  }
}

__device__ __forceinline__ void ld4(const float* p, float (&x)[4]) {
  const float4 v = *reinterpret_cast<const float4*>(p);
  x[0] = v.x; x[1] = v.y; x[2] = v.z; x[3] = v.w;
}

// Store phase: the staged tile `out` (rows of OUT_STRIDE floats) into C and
// the fused step's outputs. vec: every array 16-byte aligned, ldc and N
// multiples of 4; then warp w takes rows w, w + 8, ... and lane l columns
// 4l..4l+3 as float4, in groups of four rows whose loads (the fused step's
// operands, C when beta != 0) are all issued before the group's first store
// (the stores may alias them as far as the compiler knows, so interleaved
// loads would each wait a full memory latency). Otherwise one element at a
// time.
template <int EPI>
__device__ __forceinline__ void store_tile(const Args& a, const float* out, int m0, int n0, bool vec) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int WARPS = NTHREADS / 32, RG = 4;
  const bool partial = gridDim.z > 1;
  const bool ld_c = !partial && a.beta != 0.0f;
  constexpr bool ld_e1 = epi_reads_e1<EPI>();
  constexpr bool use_cv = EPI == EPI_SILU_D4 || EPI == EPI_ZB4, use_rv = EPI == EPI_ZB4;
  if (vec) {
    const int c = 4 * lane, n = n0 + c;
    if (n >= a.N) return;
    float bias[4] = {0.0f, 0.0f, 0.0f, 0.0f}, cv[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (!partial && a.bias) bias[k] = a.bias[n + k];
      if constexpr (use_cv) cv[k] = a.cvec[n + k];
    }
    for (int g = 0; g < BM / WARPS; g += RG) {
      float xc[RG][4], x1[RG][4], x2[RG][4], xo[RG][4], rv[RG];
#pragma unroll
      for (int i = 0; i < RG; ++i) {
        const int m = m0 + warp + (g + i) * WARPS;
        const int64_t idx = (int64_t)m * a.ldc + n;
        const bool in = m < a.M;
#pragma unroll
        for (int k = 0; k < 4; ++k) xc[i][k] = x1[i][k] = x2[i][k] = xo[i][k] = 0.0f;
        rv[i] = 0.0f;
        if constexpr (use_rv) if (in) rv[i] = a.rvec[m];
        if (in && ld_c) ld4(a.C + idx, xc[i]);
        if constexpr (ld_e1) if (in) ld4(a.e1 + idx, x1[i]);
        if constexpr (EPI == EPI_DD) if (in) ld4(a.e2 + idx, x2[i]);
        if constexpr (EPI == EPI_ZBACC) if (in) ld4(a.o1 + idx, xo[i]);
      }
#pragma unroll
      for (int i = 0; i < RG; ++i) {
        const int rr = warp + (g + i) * WARPS, m = m0 + rr;
        if (m >= a.M) continue;
        const float4 t = *reinterpret_cast<const float4*>(out + rr * OUT_STRIDE + c);
        float v[4] = {t.x, t.y, t.z, t.w};
        if (partial) {
          *reinterpret_cast<float4*>(a.part + ((int64_t)blockIdx.z * a.M + m) * a.N + n) = t;
          continue;
        }
        float r1[4], r2[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (ld_c) v[k] = fmaf(a.beta, xc[i][k], v[k]);
          v[k] += bias[k];
          fused_step<EPI>(a, v[k], x1[i][k], x2[i][k], xo[i][k], cv[k], rv[i], r1[k], r2[k]);
        }
        const int64_t idx = (int64_t)m * a.ldc + n;
        if constexpr (epi_stores_c<EPI>()) *reinterpret_cast<float4*>(a.C + idx) = make_float4(v[0], v[1], v[2], v[3]);
        if constexpr (EPI != EPI_NONE)
          *reinterpret_cast<float4*>(a.o1 + idx) = make_float4(r1[0], r1[1], r1[2], r1[3]);
        if constexpr (epi_writes_o2<EPI>())
          *reinterpret_cast<float4*>(a.o2 + idx) = make_float4(r2[0], r2[1], r2[2], r2[3]);
        if (a.img_out) {  // 4 consecutive K of row m: 8 bytes of one 16-byte chunk
          const float* r = a.img_src == 2 ? r2 : r1;
          *reinterpret_cast<uint2*>(a.img_out + (size_t)(m >> 7) * BIMG_BYTES + tc::sw128_offset(128, m & 127, n)) =
              make_uint2(tc::pack_bf16x2(r[0], r[1]), tc::pack_bf16x2(r[2], r[3]));
        }
      }
    }
    return;
  }
  for (int rr = warp; rr < BM; rr += WARPS) {
    const int m = m0 + rr;
    if (m >= a.M) break;
    for (int c = lane; c < BN; c += 32) {
      const int n = n0 + c;
      if (n >= a.N) break;
      float v = out[rr * OUT_STRIDE + c];
      if (partial) {
        a.part[((int64_t)blockIdx.z * a.M + m) * a.N + n] = v;
        continue;
      }
      const int64_t idx = (int64_t)m * a.ldc + n;
      if (ld_c) v = fmaf(a.beta, a.C[idx], v);
      if (a.bias) v += a.bias[n];
      const float x1 = ld_e1 ? a.e1[idx] : 0.0f;
      const float x2 = EPI == EPI_DD ? a.e2[idx] : 0.0f;
      const float xo = EPI == EPI_ZBACC ? a.o1[idx] : 0.0f;
      const float cv = use_cv ? a.cvec[n] : 0.0f, rv = use_rv ? a.rvec[m] : 0.0f;
      float r1 = 0.0f, r2 = 0.0f;
      fused_step<EPI>(a, v, x1, x2, xo, cv, rv, r1, r2);
      if constexpr (epi_stores_c<EPI>()) a.C[idx] = v;
      if constexpr (EPI != EPI_NONE) a.o1[idx] = r1;
      if constexpr (epi_writes_o2<EPI>()) a.o2[idx] = r2;
      if (a.img_out)
        *reinterpret_cast<uint16_t*>(a.img_out + (size_t)(m >> 7) * BIMG_BYTES +
                                     tc::sw128_offset(128, m & 127, n)) = bf16_bits(a.img_src == 2 ? r2 : r1);
    }
  }
}

template <int EPI>
__global__ void __launch_bounds__(NTHREADS, 1) k_tc_gemm(Args a) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  // done[0..1]: stage free again; done[2]: the B image has landed
  uint64_t* done = reinterpret_cast<uint64_t*>(smem + a.bar_off);
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(done + 3);
  const bool bim = a.bimg != nullptr;
  const bool aim = bim && a.aimg != nullptr;  // both operands from images: no staging at all
  uint8_t* const bsm = smem + 2 * a.stage;  // image mode: B, four 16 KB K blocks (A's image below it)
  __shared__ int fail_s;
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  const bool second = a.A2 != nullptr && (int)blockIdx.z >= a.z2;
  const float* const A = second ? a.A2 : a.A;
  const float* const Bm = second ? a.B2 : a.B;
  const int64_t sam = second ? a.sam2 : a.sam, sak = second ? a.sak2 : a.sak;
  const int64_t sbn = second ? a.sbn2 : a.sbn, sbk = second ? a.sbk2 : a.sbk;
  const int split_a = second ? a.split_a2 : a.split_a, split_b = second ? a.split_b2 : a.split_b;
  const int kbeg = (second ? (int)blockIdx.z - a.z2 : (int)blockIdx.z) * a.kchunk;
  const uint32_t b_off = A_BLK * (split_a ? 2u : 1u);  // B hi within a stage
  const int kend = min(a.K, kbeg + a.kchunk);
  const int nk = kend > kbeg ? (kend - kbeg + BK - 1) / BK : 0;
  if (t == 0) {
    fail_s = 0;
    tc::mbar_init(&done[0], 1);
    tc::mbar_init(&done[1], 1);
    tc::mbar_init(&done[2], 1);
    tc::fence_barrier_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(tmem_holder, BN);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  // set-up done; now the previous kernel's results are needed
  tc::pdl_wait();
  if (bim && t == 0 && nk > 0) {
    tc::mbar_expect_tx(&done[2], (uint32_t)nk * (aim ? A_BLK + B_BLK : B_BLK));
    for (int kb = 0; kb < nk; ++kb) {
      tc::bulk_g2s(bsm + kb * B_BLK, a.bimg + (size_t)blockIdx.x * BIMG_BYTES + (size_t)kb * B_BLK, B_BLK, &done[2]);
      if (aim)
        tc::bulk_g2s(smem + kb * A_BLK, a.aimg + (size_t)blockIdx.y * BIMG_BYTES + (size_t)kb * A_BLK, A_BLK,
                     &done[2]);
    }
  }
  constexpr uint32_t idesc = tc::idesc_bf16(BM, BN);
  int committed = 0;  // k blocks whose products were issued (the same count in every thread)
  prefetch_epilogue<EPI>(a, m0, n0);
  Frag<BM> fa;
  Frag<BN> fb;
  if (aim) {
    // both operands arrive by bulk copy: thread 0 waits for them and issues every product
    if (t == 0 && nk > 0) {
      if (!tc::mbar_wait(&done[2], 0, WAIT_LIMIT)) {
        fail_s = 1;
      } else {
        tc::tc_fence_after();
        const uint32_t ab = tc::smem_u32(smem), bb = tc::smem_u32(bsm);
        for (int kb = 0; kb < nk; ++kb)
#pragma unroll
          for (int ks = 0; ks < 4; ++ks)
            tc::mma_bf16(tmem, tc::desc_sw128(ab + kb * A_BLK + ks * 32), tc::desc_sw128(bb + kb * B_BLK + ks * 32),
                         idesc, (kb | ks) != 0);
      }
      tc::mma_commit(&done[0]);
    }
    committed = nk;
  }
  if (!aim && nk > 0) {
    fetch<BM>(fa, A, sam, sak, m0, a.M, kbeg, kend);
    if (!bim) fetch<BN>(fb, Bm, sbn, sbk, n0, a.N, kbeg, kend);
  }
  for (int kb = 0; kb < (aim ? 0 : nk); ++kb) {
    const int s = kb & 1;
    uint8_t* st = smem + s * a.stage;
    if (kb >= 2 && !tc::mbar_wait(&done[s], (uint32_t)((kb / 2 - 1) & 1), WAIT_LIMIT)) fail_s = 1;
    __syncthreads();
    if (fail_s) break;
    put<BM>(fa, st, st + A_BLK, sak == 1, split_a);
    if (!bim) put<BN>(fb, st + b_off, st + b_off + B_BLK, sbk == 1, split_b);
    if (kb + 1 < nk) {  // the next block's loads in flight across the barrier and the product issue
      const int k1 = kbeg + (kb + 1) * BK;
      fetch<BM>(fa, A, sam, sak, m0, a.M, k1, kend);
      if (!bim) fetch<BN>(fb, Bm, sbn, sbk, n0, a.N, k1, kend);
    }
    tc::fence_proxy_async_smem();
    __syncthreads();
    if (t == 0) {
      // image mode: B must have landed before the first product
      const bool b_ok = !bim || kb > 0 || tc::mbar_wait(&done[2], 0, WAIT_LIMIT);
      if (!b_ok) {
        fail_s = 1;  // seen by every thread after the next barrier; the commit below still arrives
      } else {
        tc::tc_fence_after();
        const uint32_t ah = tc::smem_u32(st), al = ah + A_BLK;
        const uint32_t bh = bim ? tc::smem_u32(bsm) + (uint32_t)kb * B_BLK : ah + b_off, bl = bh + B_BLK;
#pragma unroll
        for (int ks = 0; ks < 4; ++ks) {
          tc::mma_bf16(tmem, tc::desc_sw128(ah + ks * 32), tc::desc_sw128(bh + ks * 32), idesc, (kb | ks) != 0);
          if (split_b) tc::mma_bf16(tmem, tc::desc_sw128(ah + ks * 32), tc::desc_sw128(bl + ks * 32), idesc, 1);
          if (split_a) tc::mma_bf16(tmem, tc::desc_sw128(al + ks * 32), tc::desc_sw128(bh + ks * 32), idesc, 1);
        }
      }
      tc::mma_commit(&done[s]);
    }
    committed = kb + 1;
  }
  // the next kernel may be scheduled once every CTA is draining its tile
  tc::pdl_trigger();
  // the last commit arrives once every product issued by this CTA has completed
  if (committed > 0) {
    const int last = committed - 1;
    uint64_t* bar = aim ? &done[0] : &done[last & 1];
    if (!tc::mbar_wait(bar, aim ? 0u : (uint32_t)((last / 2) & 1), WAIT_LIMIT)) fail_s = 1;
  }
  tc::tc_fence_after();
  __syncthreads();
  const bool ok = !fail_s;  // the same in every thread after the barrier
  if (!ok) {
    if (t == 0 && a.err) atomicExch(a.err, 1);
  } else {
    // TMEM -> shared memory (row m = TMEM lane m; warp w reads lane quadrant
    // w % 4, column half w / 4), then rows into C
    float* out = reinterpret_cast<float*>(smem);
    const int quad = warp & 3;
    const int row = quad * 32 + lane;
    const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
    const int c0 = (warp >> 2) * (BN / 2);
    for (int c = c0; c < c0 + BN / 2; c += 32) {
      uint32_t r[32];
      if (committed > 0) {
        tc::tmem_ld32(tmem + lane_base + (uint32_t)c, r);
        tc::tmem_wait_ld();
        tc::tmem_regs_after_wait(r);
      } else {
#pragma unroll
        for (int j = 0; j < 32; ++j) r[j] = 0u;
      }
#pragma unroll
      for (int j = 0; j < 32; j += 4)
        *reinterpret_cast<float4*>(out + row * OUT_STRIDE + c + j) =
            make_float4(__uint_as_float(r[j]), __uint_as_float(r[j + 1]), __uint_as_float(r[j + 2]),
                        __uint_as_float(r[j + 3]));
    }
    __syncthreads();
    auto al16 = [](const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; };
    const bool vec = (a.N & 3) == 0 && (a.ldc & 3) == 0 && al16(a.C) && al16(a.part) && al16(a.e1) &&
                     al16(a.e2) && al16(a.o1) && al16(a.o2);
    store_tile<EPI>(a, out, m0, n0, vec);
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) tc::tmem_dealloc(tmem, BN);
}

// C[m][n] = beta C[m][n] + sum_z part[z][m][n], the slices added in z order.
__global__ void k_splitk_sum(const float* part, int splits, int M, int N, float* C, int64_t ldc, float beta) {
  tc::pdl_wait();
  tc::pdl_trigger();
  const int64_t mn = (int64_t)M * N;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < mn; i += (int64_t)gridDim.x * blockDim.x) {
    float s = 0.0f;
    for (int z = 0; z < splits; ++z) s += part[z * mn + i];
    float* dst = C + (i / N) * ldc + (i % N);
    *dst = beta != 0.0f ? fmaf(beta, *dst, s) : s;
  }
}

}  // namespace tcg
}  // namespace gal
