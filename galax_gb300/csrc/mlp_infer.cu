// Tensor-core inference of the potential-surrogate MLP: potential and its
// gradient (the acceleration) at n positions, one fused kernel.
//
// One CTA per SM, persistent over tiles of 128 points, warp-specialised (a
// weight-copy warp, a tensor-core warp, eight epilogue warps). Per tile:
//   layer 1 (3 -> 256) on CUDA cores -> h1 (bf16) into a shared-memory
//   operand tile; then six 128x256x256 products on the tensor cores
//   (tcgen05.mma kind::f16, bf16 x bf16 -> f32 accumulator in TMEM):
//     z2 = h1 W2^T, z3 = h2 W3^T, z4 = h3 W4^T           (forward)
//     u3 = d4 W4,   u2 = d3 W3,   u1 = d2 W2              (input gradient)
//   with d4 = silu'(z4) w5, d3 = silu'(z3) u3, d2 = silu'(z2) u2 (bf16), and
//   grad_u out = (silu'(z1) u1) W1 on CUDA cores. silu'(z2), silu'(z3) wait in
//   TMEM as packed bf16 pairs.
// Every product runs as two N halves of 128 columns, committed separately, so
// the epilogue of one half overlaps the tensor cores' work on the other, and
// two operand tiles alternate so that an epilogue writes the next product's
// operand while the current one is still read. The next product's first N half
// proceeds in K slices as the epilogues write the operand, 32 columns at a time,
// so after an epilogue only the last slices remain. A tile's layer 1 is computed
// while the tensor cores run the previous tile's last product, so its first
// product starts as soon as that product's accumulator is drained. Weights stream
// through a ring of 16 KB N-halves of K-blocks (bulk copies from pre-swizzled
// global images) run by their own warp ahead of the products. The numerics
// are those of the training kernels' quantised forward/backward (mlp_train.cu).
//
// Every mbarrier wait is bounded: on timeout the kernel records an error code,
// releases its TMEM and returns.
#include <cuda_runtime.h>

#include <atomic>
#include <cstring>
#include <vector>

#include "handle.h"
#include "mlp.cuh"
#include "tc.cuh"

namespace gal {
namespace mlp {

constexpr int TILE = 128;
constexpr int EPI_WARPS = 8;                            // two per TMEM lane quadrant
constexpr int NTHREADS = 64 + 32 * EPI_WARPS;           // warp 0 copies weights, warp 1 issues products
constexpr int STAGES = 5;
constexpr uint32_t HALF_BYTES = 128 * 128;              // one N half of a weight K-block: 128 rows x 64 bf16
constexpr uint32_t KBLOCK_BYTES = 2 * HALF_BYTES;       // a K-block of the global image: 256 rows x 64 bf16
constexpr int KBLOCKS_PER_GEMM = 4;
constexpr int GEMMS = 6;
constexpr int KBLOCKS_PER_TILE = GEMMS * KBLOCKS_PER_GEMM;  // 24 in the global image
constexpr int HALVES_PER_TILE = 2 * KBLOCKS_PER_TILE;       // 48 ring entries per tile
constexpr uint32_t A_BYTES = TILE * 256 * 2;            // 64 KB: one operand tile
constexpr uint32_t SMEM_A = 0;                          // two operand tiles, ping-pong
constexpr uint32_t SMEM_RING = 2 * A_BYTES;
constexpr uint32_t SMEM_SMALL = SMEM_RING + STAGES * HALF_BYTES;
constexpr int SMALL_FLOATS = H * 4 + 4 * H + 1;         // (W1 row, b1) per unit, b2, b3, b4 (halved), w5, b5
constexpr uint32_t SMEM_PART = SMEM_SMALL + ((SMALL_FLOATS * 4 + 255) / 256) * 256;
constexpr uint32_t SMEM_READY = SMEM_PART + TILE * 4 * 4;
constexpr uint32_t SMEM_BAR = SMEM_READY + TILE * 4;
constexpr uint32_t SMEM_TOTAL = SMEM_BAR + 256;
constexpr uint32_t SMEM_ALLOC = SMEM_TOTAL + 1024;      // room to align the base to 1024
constexpr uint32_t WAIT_LIMIT = 1u << 24;
constexpr uint32_t TMEM_COLS = 512;
constexpr uint32_t COL_S2 = 256, COL_S3 = 384;          // packed silu'(z2), silu'(z3)
static_assert(SMEM_ALLOC <= 227 * 1024, "shared memory budget");
static_assert(2 * STAGES + 7 <= 32, "barriers fit their 256 bytes");

struct InferArgs {
  const double* x;       // [3][n]
  int64_t n;
  double inv_length;     // network input u = x * inv_length
  double gscale;         // physical gradient = gscale * grad_u out
  double pscale;         // physical potential = pscale * out
  double* grad;          // [3][n] or NULL
  int32_t accumulate;    // grad += (1) or = (0)
  double* phi;           // [n] or NULL
  const float* small;    // {W1[c][0..2], b1[c]} / 2 for each unit c, then b2 / 2, b3 / 2, b4 / 2, w5, b5
  const uint8_t* wimg;   // 24 pre-swizzled 32 KB K-blocks
  int* err;
};

// Bounded wait that also gives up as soon as another role has aborted.
__device__ __forceinline__ bool wait_bar(uint64_t* bar, uint32_t parity, volatile int* abort_flag) {
  for (uint32_t i = 0; i < WAIT_LIMIT; ++i) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if ((i & 255) == 255 && *abort_flag) return false;
  }
  return false;
}

__device__ __forceinline__ void set_abort(volatile int* abort_flag, int* err, int code) {
  *abort_flag = 1;
  if (err) atomicExch(err, code);
}

// SiLU from one SFU operation. With hz = z / 2 and t = tanh(hz): the sigmoid
// is s = (1 + t) / 2, silu(z) = z s = hz + hz t, and silu'(z) = s + silu (1 - s)
// with 1 - s = (1 - t) / 2. The biases and the first layer's weights are kept
// halved in shared memory (exact), so hz comes straight out of the sums.
//
// The epilogues work on two columns at a time: Blackwell's packed FP32
// instructions (fma.rn.f32x2, mul.rn.f32x2) do two IEEE single-precision
// operations per instruction, rounded as the scalar ones, so they issue half
// the arithmetic instructions for the same results.
__device__ __forceinline__ float2 f2(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ float2 f2u(uint32_t x, uint32_t y) {
  return make_float2(__uint_as_float(x), __uint_as_float(y));
}
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
struct Silu2 {
  float2 h, d;  // silu(z), silu'(z) of two columns
};
__device__ __forceinline__ float2 tanh2(float2 hz) { return f2(tc::tanh_approx(hz.x), tc::tanh_approx(hz.y)); }
__device__ __forceinline__ float2 silu_h2(float2 hz, float2 t) { return fma2(hz, t, hz); }
__device__ __forceinline__ Silu2 silu_hd2(float2 hz) {
  const float2 t = tanh2(hz);
  const float2 h = silu_h2(hz, t);
  const float2 half = f2(0.5f, 0.5f);
  return {h, fma2(h, fma2(f2(-0.5f, -0.5f), t, half), fma2(half, t, half))};
}
// layer 1 for two units from their interleaved parameters {x0, x1, y0, y1},
// {z0, z1, w0, w1} (W1 row {x, y, z}, bias w, all halved): half the argument
__device__ __forceinline__ float2 layer1_hz2(const float4& pxy, const float4& pzw, float2 u0, float2 u1,
                                             float2 u2) {
  return fma2(f2(pxy.x, pxy.y), u0, fma2(f2(pxy.z, pxy.w), u1, fma2(f2(pzw.x, pzw.y), u2, f2(pzw.z, pzw.w))));
}

// write 32 consecutive hidden units [c, c+32) of row `row` into an operand tile
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

// Warp-specialised, persistent over 128-point tiles:
//   warp 0   : streams the weights of every tile through a ring of 16 KB N-halves of K-blocks
//              (bulk copies), in the order the products consume them
//   warp 1   : allocates TMEM and issues the six 128x256x256 products per tile (tcgen05.mma),
//              each as two N halves of 128 columns
//   warps 2-9: epilogues, one thread per (point, quarter of each half's columns); a warp may
//              only touch its TMEM lane quadrant (warp id % 4), so each quadrant has two warps
// Each product splits into its two N halves, committed separately (acc_full[h]), so the
// epilogue of half 0 runs while half 1 is on the tensor cores; the epilogue writes the next
// product's operand into the other of two operand tiles, 32 columns per thread at a time
// (op_ready[2 h + c]: sub-chunk c of operand half h from all eight warps), and the product
// warp issues the next product's first N half two K slices at a time as those arrive.
// Every wait is bounded.
__global__ void __launch_bounds__(NTHREADS, 1) k_mlp_infer(InferArgs a) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = smem_raw + ((1024 - (tc::smem_u32(smem_raw) & 1023)) & 1023);
  uint8_t* tiles = smem + SMEM_A;  // [2][A_BYTES]
  uint8_t* ring = smem + SMEM_RING;
  float* sm = reinterpret_cast<float*>(smem + SMEM_SMALL);
  // {W1 row, b1} of units 2p, 2p+1 interleaved: {x0, x1, y0, y1} at 2p, {z0, z1, w0, w1} at 2p + 1
  const float4* sL1 = reinterpret_cast<const float4*>(sm);
  const float* sb2 = sm + 4 * H;
  const float* sb3 = sb2 + H;
  const float* sb4 = sb3 + H;
  const float* sw5 = sb4 + H;
  float* part = reinterpret_cast<float*>(smem + SMEM_PART);  // [TILE][4]
  volatile int* ready = reinterpret_cast<volatile int*>(smem + SMEM_READY);  // [TILE]
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + SMEM_BAR);
  uint64_t* full = bars;
  uint64_t* empty = bars + STAGES;
  uint64_t* acc_full = bars + 2 * STAGES;  // [2]
  uint64_t* op_ready = acc_full + 2;       // [2 halves][2 sub-chunks]
  uint64_t* drain = op_ready + 4;
  uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(drain + 1);
  __shared__ int abort_s;
  volatile int* abort_flag = &abort_s;

  const int t = threadIdx.x;
  const int warp = t >> 5, lane = t & 31;
  for (int i = t; i < SMALL_FLOATS; i += NTHREADS) {
    int src = i;  // the first 4H floats ({W1 row, b1} per unit) are interleaved by unit pairs
    if (i < 4 * H) src = 8 * (i >> 3) + ((i & 7) >> 1) + 4 * (i & 1);
    sm[i] = a.small[src];
  }
  for (int i = t; i < TILE; i += NTHREADS) ready[i] = 0;
  if (t == 0) {
    abort_s = 0;
    for (int s = 0; s < STAGES; ++s) {
      tc::mbar_init(&full[s], 1);
      tc::mbar_init(&empty[s], 1);
    }
    for (int h = 0; h < 2; ++h) tc::mbar_init(&acc_full[h], 1);
    for (int c = 0; c < 4; ++c) tc::mbar_init(&op_ready[c], EPI_WARPS);
    tc::mbar_init(drain, 1);
    tc::fence_barrier_init();
  }
  if (warp == 1) {
    tc::tmem_alloc(tmem_holder, TMEM_COLS);
    tc::tmem_relinquish();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_holder;
  const int64_t ntiles = (a.n + TILE - 1) / TILE;
  const int64_t my_tiles = ntiles > blockIdx.x ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

  if (warp == 0) {
    // ------------------------------------------------------------ weight producer
    if (lane == 0) {
      const int64_t total = my_tiles * HALVES_PER_TILE;
      int64_t j = 0;
      for (; j < total; ++j) {
        const int s = (int)(j % STAGES);
        const int64_t use = j / STAGES;
        if (use > 0 && !wait_bar(&empty[s], (uint32_t)((use - 1) & 1), abort_flag)) {
          if (!*abort_flag) set_abort(abort_flag, a.err, 3);
          break;
        }
        // entry e of a tile: product g = e / 8, half h = (e / 4) % 2, K-block kb = e % 4
        const int e = (int)(j % HALVES_PER_TILE);
        const int g = e >> 3, h = (e >> 2) & 1, kb = e & 3;
        tc::mbar_expect_tx(&full[s], HALF_BYTES);
        tc::bulk_g2s(ring + (size_t)s * HALF_BYTES,
                     a.wimg + (size_t)(g * KBLOCKS_PER_GEMM + kb) * KBLOCK_BYTES + (size_t)h * HALF_BYTES, HALF_BYTES,
                     &full[s]);
      }
      // every copy issued must have landed before the CTA can exit (bounded)
      for (int64_t q = (j > STAGES ? j - STAGES : 0); q < j; ++q)
        tc::mbar_wait(&full[q % STAGES], (uint32_t)((q / STAGES) & 1), WAIT_LIMIT);
    }
  } else if (warp == 1) {
    // ------------------------------------------------------------ tensor-core products
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_bf16(TILE, 128);
      int64_t j = 0, q = 0;  // ring entries consumed; products started (op_ready phases)
      bool ok = true;
      auto run_blocks = [&](uint32_t a_base, int h, int kb0, int kb1) -> bool {
        for (int kb = kb0; kb < kb1; ++kb, ++j) {
          const int s = (int)(j % STAGES);
          if (!wait_bar(&full[s], (uint32_t)((j / STAGES) & 1), abort_flag)) return false;
          tc::tc_fence_after();
          const uint32_t b_base = tc::smem_u32(ring + (size_t)s * HALF_BYTES);
#pragma unroll
          for (int ks = 0; ks < 4; ++ks) {
            const uint64_t ad = tc::desc_sw128(a_base + kb * (TILE * 128) + ks * 32);
            const uint64_t bd = tc::desc_sw128(b_base + ks * 32);
            tc::mma_bf16(tmem + (uint32_t)(h * 128), ad, bd, idesc, (kb | ks) != 0);
          }
          tc::mma_commit(&empty[s]);  // stage free once these products complete
        }
        return true;
      };
      // N half 0 over one half oh of K (K-blocks 2 oh, 2 oh + 1: ring entries j, j + 1), in two
      // steps of two K slices each as the epilogue writes the operand's sub-chunks
      // (op_ready[2 oh + c]: columns 128 oh + 64 qq + 32 c .. + 31 of both column quarters qq)
      auto half0 = [&](uint32_t a_base, int oh) -> bool {
        for (int d = 0; d < 2; ++d) {
          const int64_t jj = j + d;
          if (!wait_bar(&full[jj % STAGES], (uint32_t)((jj / STAGES) & 1), abort_flag)) return false;
        }
        for (int c = 0; c < 2; ++c) {
          if (!wait_bar(&op_ready[2 * oh + c], (uint32_t)(q & 1), abort_flag)) return false;
          tc::tc_fence_after();
#pragma unroll
          for (int d = 0; d < 2; ++d) {
            const int kb = 2 * oh + d;
            const uint32_t b_base = tc::smem_u32(ring + (size_t)((j + d) % STAGES) * HALF_BYTES);
#pragma unroll
            for (int ks = 2 * c; ks < 2 * c + 2; ++ks) {
              const uint64_t ad = tc::desc_sw128(a_base + kb * (TILE * 128) + ks * 32);
              const uint64_t bd = tc::desc_sw128(b_base + ks * 32);
              tc::mma_bf16(tmem, ad, bd, idesc, (kb | ks) != 0);
            }
          }
        }
        tc::mma_commit(&empty[j % STAGES]);  // both stages free once these products complete
        tc::mma_commit(&empty[(j + 1) % STAGES]);
        j += 2;
        return true;
      };
      for (int64_t it = 0; it < my_tiles && ok; ++it) {
        for (int g = 0; g < GEMMS && ok; ++g, ++q) {
          const uint32_t a_base = tc::smem_u32(tiles + (size_t)(g & 1) * A_BYTES);
          // N half 0 slice by slice as the operand is written, then N half 1 over all of K
          if (!half0(a_base, 0) || !half0(a_base, 1)) { ok = false; break; }
          tc::mma_commit(&acc_full[0]);
          if (!run_blocks(a_base, 1, 0, 4)) { ok = false; break; }
          tc::mma_commit(&acc_full[1]);
        }
      }
      if (!ok && !*abort_flag) set_abort(abort_flag, a.err, 4);
      // no product may still be writing TMEM when it is released
      tc::mma_commit(drain);
      tc::mbar_wait(drain, 0, WAIT_LIMIT);
    }
  } else {
    // ------------------------------------------------------------ epilogues
    const int e = warp - 2;
    const int quad = warp & 3;
    const int row = quad * 32 + lane;
    const int qq = e >= 4 ? 1 : 0;  // which 64-column quarter of each half
    const uint32_t lane_base = (uint32_t)(quad * 32) << 16;
    int64_t q = 0;  // acc_full phases
    // network input of this thread's point of tile `it` (zero past the end)
    auto load_u = [&](int64_t it, float (&u)[3]) {
      const int64_t gi = (blockIdx.x + it * gridDim.x) * TILE + row;
#pragma unroll
      for (int j = 0; j < 3; ++j) u[j] = gi < a.n ? (float)(a.x[j * a.n + gi] * a.inv_length) : 0.f;
    };
    // sub-chunk c (this thread's columns 32 c .. 32 c + 31) of operand half h written and
    // accumulator half h drained: one arrival per warp
    auto signal = [&](int h, int c) {
      tc::fence_proxy_async_smem();
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&op_ready[2 * h + c]);
    };
    // layer 1 on CUDA cores: h1 = silu(W1 u + b1) -> operand tile 0, this thread's columns of
    // both halves; with `each`, every half is signalled as soon as it is written
    auto layer1 = [&](const float (&u)[3], bool each) {
      const float2 u0 = f2(u[0], u[0]), u1 = f2(u[1], u[1]), u2 = f2(u[2], u[2]);
      for (int h = 0; h < 2; ++h) {
        const int cbase = h * 128 + qq * 64;
        for (int c = cbase; c < cbase + 64; c += 32) {
          float v[32];
#pragma unroll
          for (int k = 0; k < 32; k += 2) {
            const float2 hz = layer1_hz2(sL1[c + k], sL1[c + k + 1], u0, u1, u2);  // units c+k, c+k+1
            const float2 hv = silu_h2(hz, tanh2(hz));
            v[k] = hv.x;
            v[k + 1] = hv.y;
          }
          store_row32(tiles, row, c, v);
          if (each) signal(h, (c - cbase) >> 5);
        }
      }
    };
    // The first tile's layer 1 runs here; every later tile's runs while the tensor cores
    // work on the previous tile's last product (operand tile 0 is free once product 4 has
    // completed), so the next tile's first product starts as soon as that product's
    // epilogue has drained the accumulator.
    float u[3] = {0.f, 0.f, 0.f}, un[3] = {0.f, 0.f, 0.f};
    if (my_tiles > 0) {
      load_u(0, u);
      layer1(u, true);
    }
    for (int64_t it = 0; it < my_tiles; ++it) {
      if (*abort_flag) break;
      const int64_t tile = blockIdx.x + it * gridDim.x;
      const int64_t gi = tile * TILE + row;
      const bool valid = gi < a.n;
      const bool has_next = it + 1 < my_tiles;
      if (has_next) load_u(it + 1, un);
      const float2 u0 = f2(u[0], u[0]), u1 = f2(u[1], u[1]), u2 = f2(u[2], u[2]);
      float2 gpart2[3] = {f2(0.f, 0.f), f2(0.f, 0.f), f2(0.f, 0.f)};  // even and odd columns apart
      float2 ppart2 = f2(0.f, 0.f);
      bool ok = true;
#pragma unroll
      for (int g = 0; g < GEMMS; ++g) {
        if (!ok) break;
        uint8_t* tile_out = tiles + (size_t)((g + 1) & 1) * A_BYTES;
#pragma unroll
        for (int h = 0; h < 2; ++h, ++q) {
          if (g == GEMMS - 1 && h == 0 && has_next) layer1(un, false);  // the next tile's, unsignalled
          if (!wait_bar(&acc_full[h], (uint32_t)((q >> 1) & 1), abort_flag)) {
            if (!*abort_flag) set_abort(abort_flag, a.err, 2);
            ok = false;
            break;
          }
          tc::tc_fence_after();
          const int c = h * 128 + qq * 64;  // this thread's 64 columns of half h
          uint32_t acc0[32], acc1[32], sp0[16], sp1[16];
          tc::tmem_ld32(tmem + lane_base + (uint32_t)c, acc0);
          tc::tmem_ld32(tmem + lane_base + (uint32_t)(c + 32), acc1);
          if (g == 3 || g == 4) {
            const uint32_t cs = (g == 3 ? COL_S3 : COL_S2) + c / 2;
            tc::tmem_ld16(tmem + lane_base + cs, sp0);
            tc::tmem_ld16(tmem + lane_base + cs + 16, sp1);
          }
          tc::tmem_wait_ld();
          tc::tmem_regs_after_wait(acc0);
          tc::tmem_regs_after_wait(acc1);
          if (g == 3 || g == 4) {
            tc::tmem_regs_after_wait(sp0);
            tc::tmem_regs_after_wait(sp1);
          }
          // the last product: the next tile's operand (its layer 1) is written already, so its
          // first product may start as soon as this half of the accumulator is drained
          if (g == GEMMS - 1 && has_next) {
            signal(h, 0);
            signal(h, 1);
          }
#pragma unroll
          for (int half = 0; half < 2; ++half) {
            const uint32_t(&acc)[32] = half ? acc1 : acc0;
            const uint32_t(&sp)[16] = half ? sp1 : sp0;
            const int cc0 = c + 32 * half;
            float v[32];
            if (g <= 1) {  // z2 / z3: h = silu(z) -> operand tile, silu'(z) -> TMEM
              const float4* hb = reinterpret_cast<const float4*>((g == 0 ? sb2 : sb3) + cc0);  // halved biases
              uint32_t spk[16];
#pragma unroll
              for (int k = 0; k < 32; k += 4) {
                const float4 b4 = hb[k / 4];
                const Silu2 r0 = silu_hd2(fma2(f2(0.5f, 0.5f), f2u(acc[k], acc[k + 1]), f2(b4.x, b4.y)));
                const Silu2 r1 = silu_hd2(fma2(f2(0.5f, 0.5f), f2u(acc[k + 2], acc[k + 3]), f2(b4.z, b4.w)));
                v[k] = r0.h.x;
                v[k + 1] = r0.h.y;
                v[k + 2] = r1.h.x;
                v[k + 3] = r1.h.y;
                spk[k / 2] = tc::pack_bf16x2(r0.d.x, r0.d.y);
                spk[k / 2 + 1] = tc::pack_bf16x2(r1.d.x, r1.d.y);
              }
              tc::tmem_st16(tmem + lane_base + (uint32_t)((g == 0 ? COL_S2 : COL_S3) + cc0 / 2), spk);
              store_row32(tile_out, row, cc0, v);
            } else if (g == 2) {  // z4: d4 = silu'(z4) w5 -> operand tile; out = w5 . silu(z4)
              const float4* hb = reinterpret_cast<const float4*>(sb4 + cc0);  // halved
              const float4* w5 = reinterpret_cast<const float4*>(sw5 + cc0);
#pragma unroll
              for (int k = 0; k < 32; k += 4) {
                const float4 b4 = hb[k / 4], w4 = w5[k / 4];
                const float2 wa = f2(w4.x, w4.y), wb = f2(w4.z, w4.w);
                const Silu2 r0 = silu_hd2(fma2(f2(0.5f, 0.5f), f2u(acc[k], acc[k + 1]), f2(b4.x, b4.y)));
                const Silu2 r1 = silu_hd2(fma2(f2(0.5f, 0.5f), f2u(acc[k + 2], acc[k + 3]), f2(b4.z, b4.w)));
                ppart2 = fma2(r0.h, wa, ppart2);
                ppart2 = fma2(r1.h, wb, ppart2);
                const float2 d0 = mul2(r0.d, wa), d1 = mul2(r1.d, wb);
                v[k] = d0.x;
                v[k + 1] = d0.y;
                v[k + 2] = d1.x;
                v[k + 3] = d1.y;
              }
              store_row32(tile_out, row, cc0, v);
            } else if (g <= 4) {  // u3 / u2: d = silu'(z) u -> operand tile
#pragma unroll
              for (int k = 0; k < 32; k += 2) {
                const float2 d = mul2(f2(tc::bf16_lo(sp[k / 2]), tc::bf16_hi(sp[k / 2])), f2u(acc[k], acc[k + 1]));
                v[k] = d.x;
                v[k + 1] = d.y;
              }
              store_row32(tile_out, row, cc0, v);
            } else {  // u1: grad_u out = sum_c silu'(z1_c) u1_c W1[c]
#pragma unroll
              for (int k = 0; k < 32; k += 2) {
                // units cc0+k, cc0+k+1; W1 halved: gpart is half the sum, doubled at the end
                const float4 pxy = sL1[cc0 + k], pzw = sL1[cc0 + k + 1];
                const float2 hz = layer1_hz2(pxy, pzw, u0, u1, u2);
                const float2 d1 = mul2(silu_hd2(hz).d, f2u(acc[k], acc[k + 1]));
                gpart2[0] = fma2(d1, f2(pxy.x, pxy.y), gpart2[0]);
                gpart2[1] = fma2(d1, f2(pxy.z, pxy.w), gpart2[1]);
                gpart2[2] = fma2(d1, f2(pzw.x, pzw.y), gpart2[2]);
              }
            }
            // this sub-chunk of the next product's operand written (the accumulator half was
            // drained by the loads above): the product warp may issue its K slices
            if (g < GEMMS - 1) signal(h, half);
          }
          if (g <= 1) tc::tmem_wait_st();
        }
      }
      if (!ok) break;
      const float gpart[3] = {gpart2[0].x + gpart2[0].y, gpart2[1].x + gpart2[1].y, gpart2[2].x + gpart2[2].y};
      const float ppart = ppart2.x + ppart2.y;
      // combine the two column quarters of each row (bounded hand-off through shared memory)
      if (qq == 1) {
        part[row * 4 + 0] = gpart[0];
        part[row * 4 + 1] = gpart[1];
        part[row * 4 + 2] = gpart[2];
        part[row * 4 + 3] = ppart;
        __threadfence_block();
        ready[row] = (int)(it + 1);
      } else {
        uint32_t spins = 0;
        while (ready[row] != (int)(it + 1) && spins < WAIT_LIMIT && !*abort_flag) ++spins;
        if (ready[row] != (int)(it + 1)) {
          if (!*abort_flag) set_abort(abort_flag, a.err, 5);
          break;
        }
        __threadfence_block();
        if (valid) {
#pragma unroll
          for (int j = 0; j < 3; ++j) {
            const double gj = 2.0 * a.gscale * (double)(gpart[j] + part[row * 4 + j]);  // halved W1
            if (a.grad) a.grad[j * a.n + gi] = a.accumulate ? a.grad[j * a.n + gi] + gj : gj;
          }
          if (a.phi) a.phi[gi] = a.pscale * (double)(ppart + part[row * 4 + 3] + sw5[H]);
        }
      }
#pragma unroll
      for (int j = 0; j < 3; ++j) u[j] = un[j];
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, TMEM_COLS);
  }
}

}  // namespace mlp
}  // namespace gal

using namespace gal;
using namespace gal::mlp;

struct gal_mlp {
  float* d_small;      // {W1 row, b1} per unit, b2, b3, b4 (halved), w5, b5
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
  return no_throw([&]() -> gal_status {
    if (!params_host || !out || !(length_scale > 0) || !(phi_scale != 0))
      return fail(GAL_ERR_INVALID_ARGUMENT, "bad gal_mlp_create arguments");
    *out = nullptr;
    const float* P = params_host;
    std::vector<float> small(SMALL_FLOATS);
    // the first layer's weights and biases and the hidden biases halved (exact):
    // the kernel's sums then give z / 2, the argument of its tanh
    for (int c = 0; c < H; ++c) {
      for (int j = 0; j < 3; ++j) small[4 * c + j] = 0.5f * P[OFF_W1 + 3 * c + j];
      small[4 * c + 3] = 0.5f * P[OFF_B1 + c];
    }
    for (int c = 0; c < H; ++c) {
      small[4 * H + c] = 0.5f * P[OFF_B2 + c];
      small[5 * H + c] = 0.5f * P[OFF_B3 + c];
      small[6 * H + c] = 0.5f * P[OFF_B4 + c];
    }
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
    if (e == cudaSuccess)
      e = cudaMemcpy(m->d_small, small.data(), sizeof(float) * small.size(), cudaMemcpyHostToDevice);
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
  });
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
  // the shared-memory opt-in is per device: set once on each (not again while a stream is captured)
  static std::atomic<bool> attr[64] = {};
  int dev = 0;
  cudaError_t e0 = cudaGetDevice(&dev);
  if (e0 != cudaSuccess) return cuda_fail(e0, "cudaGetDevice");
  if (dev < 0 || dev >= 64) return fail(GAL_ERR_UNSUPPORTED, "device index above 63");
  if (!attr[dev].load(std::memory_order_acquire)) {
    cudaError_t e = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_ALLOC);
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute(k_mlp_infer)");
    attr[dev].store(true, std::memory_order_release);
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
