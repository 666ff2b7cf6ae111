// Learned channel estimator: a residual CNN that refines per-stream LS estimates
// of a MIMO grid into the full channel (no counterpart in the reference).
//
//   s  = RMS of the drop's LS estimate (per drop, over pairs, words and columns)
//   x0 = LS / s as 32 channels (16 antenna pairs x re/im) over (word, column)
//   h_l = relu(conv3x3_l(h_{l-1}) + b_l), l = 1..5;  out = LS + s (conv3x3_6(h_5) + b_6)
// so the network works at unit scale whatever the channel energy and SNR.
//
// Every layer is an implicit GEMM (M = grid elements, N = 32 output channels,
// K = 9 taps x 32 input channels) on the BF16 tensor cores with FP32 accumulation.
// Inference (hpx_cnn_refine) runs on TMA + tcgen05 (k_conv3x3_tc: 128 output
// elements of one word per MMA tile, accumulators in tensor memory) with planar
// activations [drop][4 chunks of 8 channels][word][column][8]. Training keeps NHWC
// activations ([drop][word][column][32 channels]) for its mma.sync m16n8k16 kernels:
// forward, the input-gradient pass (the forward kernel's transpose, weights flipped
// and transposed) and the weight gradients; Adam updates FP32 master weights.
#include <cuda.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "hpx_internal.cuh"
#include "tcgen05.cuh"

namespace {

constexpr int CH = 32;          // channels of every layer
constexpr int KK = 9 * CH;      // GEMM depth: 3x3 taps x input channels
constexpr int LAYERS = 6;
constexpr int TH = 2, TW = 64;  // output tile (rows = words, columns)
constexpr int IN_H = TH + 2, IN_W = TW + 2, IN_PX = IN_H * IN_W;
constexpr int WPITCH = KK + 8;  // shared-memory weight row (bf16): 592 bytes, conflict-free ldmatrix
constexpr int NPAIR = CH / 2;   // antenna pairs carried by the 32 channels

// Byte offset of 16-byte chunk q (channels 8q..8q+7) of tile pixel pi: the chunk
// index is XOR-ed with bits 1-2 of the pixel, so 8 consecutive pixels of one chunk
// fall on 8 distinct 16-byte bank groups (ldmatrix without conflicts).
__device__ __forceinline__ int swz(int pi, int q) { return pi * 64 + ((q ^ ((pi >> 1) & 3)) << 4); }

__device__ __forceinline__ uint32_t bf2_bits(float lo, float hi) {
  const __nv_bfloat162 t = __floats2bfloat162_rn(lo, hi);
  uint32_t u;
  memcpy(&u, &t, sizeof(u));
  return u;
}

// Store 16 packed bf16 pairs (64 bytes, one grid element) as four 16-byte stores.
__device__ __forceinline__ void store_px(__nv_bfloat16* dst, const uint32_t (&u)[NPAIR]) {
  uint4* d = reinterpret_cast<uint4*>(dst);
#pragma unroll
  for (int i = 0; i < 4; ++i) d[i] = make_uint4(u[4 * i], u[4 * i + 1], u[4 * i + 2], u[4 * i + 3]);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

__device__ __forceinline__ void mma_bf16(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Load the (TH+2) x (TW+2) input tile with halo around output tile (h0, w0) of
// drop b into swizzled shared memory; elements outside the grid read as zero.
__device__ __forceinline__ void load_tile(unsigned char* sm, const __nv_bfloat16* __restrict__ act, int b, int H, int W,
                                          int h0, int w0) {
  for (int q = threadIdx.x; q < IN_PX * 4; q += blockDim.x) {
    const int pi = q >> 2, ch = q & 3;
    const int ty = pi / IN_W, tx = pi - ty * IN_W;
    const int h = h0 - 1 + ty, w = w0 - 1 + tx;
    uint4 v = make_uint4(0u, 0u, 0u, 0u);
    if (h >= 0 && h < H && w >= 0 && w < W)
      v = __ldg(reinterpret_cast<const uint4*>(act + (((int64_t)b * H + h) * W + w) * CH) + ch);
    *reinterpret_cast<uint4*>(sm + swz(pi, ch)) = v;
  }
}

// EPI 0: + bias, ReLU -> bf16 NHWC.  EPI 1: + bias + residual (complex planes)
// -> complex planes [drop][pair][word][ccols].  EPI 2: times (mask > 0) -> bf16
// NHWC (input gradient through the previous layer's ReLU).
template <int EPI>
__global__ void __launch_bounds__(128) k_conv3x3(int H, int W, const __nv_bfloat16* __restrict__ in,
                                                 const __nv_bfloat16* __restrict__ wt, const float* __restrict__ bias,
                                                 __nv_bfloat16* __restrict__ out, const __nv_bfloat16* __restrict__ mask,
                                                 const float2* __restrict__ resid, float2* __restrict__ out_c,
                                                 int ccols, const float* __restrict__ pw, float inv_count) {
  __shared__ __align__(128) unsigned char s_in[IN_PX * 64];
  __shared__ __align__(128) __nv_bfloat16 s_w[CH * WPITCH];
  const int tiles_w = (W + TW - 1) / TW;
  const int tile = blockIdx.x, b = blockIdx.y;
  const int h0 = (tile / tiles_w) * TH, w0 = (tile - (tile / tiles_w) * tiles_w) * TW;
  for (int q = threadIdx.x; q < CH * (KK / 8); q += blockDim.x) {
    const int n = q / (KK / 8), c16 = q - n * (KK / 8);
    *reinterpret_cast<uint4*>(s_w + n * WPITCH + c16 * 8) = __ldg(reinterpret_cast<const uint4*>(wt + n * KK) + c16);
  }
  load_tile(s_in, in, b, H, W, h0, w0);
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ty = warp >> 1, tx0 = (warp & 1) * 32;
  const int j = lane >> 3, r = lane & 7;
  float acc[2][4][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[mt][nt][i] = 0.f;
  const uint32_t in_base = smem_u32(s_in), w_base = smem_u32(s_w);
#pragma unroll 1
  for (int tap = 0; tap < 9; ++tap) {
    const int dy = tap / 3, dx = tap - dy * 3;
#pragma unroll
    for (int kc = 0; kc < 2; ++kc) {
      uint32_t bf[4][2];
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int n = half * 16 + (j >> 1) * 8 + r;
        const int k = tap * CH + kc * 16 + (j & 1) * 8;
        uint32_t r0, r1, r2, r3;
        ldsm_x4(w_base + (n * WPITCH + k) * 2, r0, r1, r2, r3);
        bf[half * 2][0] = r0;
        bf[half * 2][1] = r1;
        bf[half * 2 + 1][0] = r2;
        bf[half * 2 + 1][1] = r3;
      }
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const int pi = (ty + dy) * IN_W + tx0 + mt * 16 + (j & 1) * 8 + r + dx;
        uint32_t a[4];
        ldsm_x4(in_base + swz(pi, kc * 2 + (j >> 1)), a[0], a[1], a[2], a[3]);
#pragma unroll
        for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], a, bf[nt][0], bf[nt][1]);
      }
    }
  }

  const int h = h0 + ty;
  if (h >= H) return;
  const int g = lane >> 2, cq = (lane & 3) * 2;
  const float scale = EPI == 1 ? sqrtf(pw[b] * inv_count) : 1.f;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int hr = 0; hr < 2; ++hr) {
      const int w = w0 + tx0 + mt * 16 + g + hr * 8;
      if (w >= W) continue;
      const int64_t px = ((int64_t)b * H + h) * W + w;
#pragma unroll
      for (int nt = 0; nt < 4; ++nt) {
        const int n = nt * 8 + cq;
        float v0 = acc[mt][nt][hr * 2], v1 = acc[mt][nt][hr * 2 + 1];
        if (EPI == 0) {
          v0 = fmaxf(v0 + bias[n], 0.f);
          v1 = fmaxf(v1 + bias[n + 1], 0.f);
          *reinterpret_cast<__nv_bfloat162*>(out + px * CH + n) = __floats2bfloat162_rn(v0, v1);
        } else if (EPI == 1) {
          const int64_t e = (((int64_t)b * NPAIR + (n >> 1)) * H + h) * ccols + w;
          const float2 x = resid[e];
          out_c[e] = make_float2(fmaf(scale, v0 + bias[n], x.x), fmaf(scale, v1 + bias[n + 1], x.y));
        } else {
          const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162*>(mask + px * CH + n);
          v0 = __low2float(mk) > 0.f ? v0 : 0.f;
          v1 = __high2float(mk) > 0.f ? v1 : 0.f;
          *reinterpret_cast<__nv_bfloat162*>(out + px * CH + n) = __floats2bfloat162_rn(v0, v1);
        }
      }
    }
}

// ------------------------------------------------------------ tcgen05 forward
// One tile = 128 consecutive output columns of two words of one drop (thread i <->
// TMEM lane i <-> column w0 + i). The input rows h0 - 1 .. h0 + 2 over columns
// w0 - 1 .. w0 + 128 arrive by TMA as four planes of 8 channels: a 4-D tensor map
// over the planar activation (channel in chunk, column, word, 4 drop + chunk) with
// box (8, 130, 4, 1) delivers plane j as four contiguous 2 080-byte rows (row r,
// column p at (r 130 + p) 16 bytes), zero outside the grid. For output row r and
// tap (dy, dx) the A operand (128 elements x 16 channels) is then the K-major,
// unswizzled operand that starts at element (r + dy, dx) of planes 2 kc and 2 kc + 1:
// rows 16 bytes apart (core matrices 128 bytes apart along M), the two 8-channel
// halves a plane apart along K. The weights of tap t and channel half kc form a
// 32 x 16 K-major block. Eighteen MMAs per output row (M = 128, N = 32, K = 16, BF16
// in, FP32 out) give the tile. The CTA walks tiles persistently as a
// warp-specialized pipeline: warp 0 (one thread) issues the TMA copies into two input
// stages and the MMAs into two accumulator slots (32 TMEM columns per output row);
// warps 1-4 each read a quarter of a slot's lanes, release the slot through an
// mbarrier and run the epilogue, so the MMAs of tile k + 1 queue while tile k is
// stored. No CTA-wide barrier inside the loop. A tensor-core or TMA wait that times
// out writes NaN outputs and sets *fail.
constexpr int TCW = 128;                           // output columns per tile
constexpr int TC_INW = TCW + 2;                    // input columns with halo
constexpr int TC_ROWS = 2;                         // output rows (words) per tile
constexpr int TC_INH = TC_ROWS + 2;                // input rows with halo
constexpr int TC_BOX = TC_INH * TC_INW * 16;       // bytes of one TMA box (one plane)
constexpr int TC_PLANE = (TC_BOX + 127) / 128 * 128;  // plane stride (TMA destinations 128-byte aligned)
constexpr int TC_BUF = 4 * TC_PLANE;               // one input stage
constexpr int TC_STAGES = 2;                       // input stages in flight per CTA
constexpr int TC_WBLK = CH * 16 * 2;               // one 32 x 16 bf16 weight block
constexpr int TC_SMEM = TC_STAGES * TC_BUF + 18 * TC_WBLK + 128;  // + alignment slack
constexpr uint32_t TC_IDESC = tc::idesc_f16_f32(128, CH) | (1u << 7) | (1u << 10);  // A, B: BF16
constexpr long long TC_CONV_WAIT = 40ll * 1000 * 1000;  // cycles (~20 ms)
constexpr int TC_CTAS_PER_SM = 2;                  // shared memory: 2 x 83 KB
constexpr int TC_SLOT = TC_ROWS * 32;              // TMEM columns of one accumulator slot
constexpr int TC_THREADS = 160;                    // warp 0: TMA + MMA issue; warps 1-4: epilogue

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(tc::smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(tc::smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(tc::smem_u32(bar))
      : "memory");
}

template <int EPI>
__global__ void __launch_bounds__(TC_THREADS, TC_CTAS_PER_SM) k_conv3x3_tc(
    const __grid_constant__ CUtensorMap tmap, int B, int H, int W, const __nv_bfloat16* __restrict__ wt,
    const float* __restrict__ bias, __nv_bfloat16* __restrict__ out, const float2* resid, float2* out_c, int ccols,
    const float* __restrict__ pw, float inv_count, int* fail) {
  extern __shared__ unsigned char sm_raw[];
  unsigned char* sm = sm_raw + ((128u - (tc::smem_u32(sm_raw) & 127u)) & 127u);
  unsigned char* s_in = sm;                      // [TC_STAGES][4 planes]
  unsigned char* s_w = sm + TC_STAGES * TC_BUF;  // [9 taps x 2 halves] weight blocks
  __shared__ uint64_t bar_in[TC_STAGES], bar_mma[2], bar_free[2];
  __shared__ uint32_t tmem_slot;
  __shared__ float s_bias[CH];
  __shared__ int skip;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // weights: element (n, tap 32 + c) -> block (tap, c / 16), K-major inside
  for (int q = tid; q < CH * 36; q += TC_THREADS) {
    const int n = q / 36, r = q - n * 36, tap = r >> 2, c8 = r & 3;
    const uint4 v = __ldg(reinterpret_cast<const uint4*>(wt + n * KK + tap * CH + c8 * 8));
    *reinterpret_cast<uint4*>(s_w + (tap * 2 + (c8 >> 1)) * TC_WBLK + tc::kmajor_offset(n, (c8 & 1) * 8, 16)) = v;
  }
  if (tid < CH) s_bias[tid] = bias[tid];
  if (tid == 0) {
    skip = *(volatile int*)fail;
    for (int i = 0; i < TC_STAGES; ++i) tc::mbar_init(&bar_in[i], 1);
    for (int i = 0; i < 2; ++i) {
      tc::mbar_init(&bar_mma[i], 1);
      tc::mbar_init(&bar_free[i], 128);  // every epilogue thread releases the slot
    }
  }
  if (warp == 0) {
    tc::tmem_alloc(&tmem_slot, 2 * TC_SLOT);  // two accumulator slots, 32 columns per output row
    tc::tmem_relinquish();
  }
  tc::fence_proxy_async_smem();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  bool ok = skip == 0;
  const int tiles_w = (W + TCW - 1) / TCW, tiles_h = (H + TC_ROWS - 1) / TC_ROWS;
  const int64_t ntiles = (int64_t)B * tiles_h * tiles_w;
  // tiles of this CTA: blockIdx.x + k gridDim.x, k < K
  const int K = blockIdx.x < ntiles ? (int)((ntiles - 1 - blockIdx.x) / gridDim.x) + 1 : 0;
  auto decode = [&](int k, int& b, int& h, int& w0) {
    const int64_t tile = blockIdx.x + (int64_t)k * gridDim.x;
    const int64_t bh = tile / tiles_w;
    w0 = (int)(tile - bh * tiles_w) * TCW;
    b = (int)(bh / tiles_h);
    h = (int)(bh - (int64_t)b * tiles_h) * TC_ROWS;  // first output row of the tile
  };
  if (warp == 0) {
    // ---- producer: lane 0 issues the TMA into the stages and the MMAs into the two
    // slots; the warp walks the loop together (status broadcast from lane 0)
    int issued[TC_STAGES] = {}, landed[TC_STAGES] = {};
    auto issue = [&](int k) {  // the four planes of tile k into stage k % TC_STAGES
      const int st = k % TC_STAGES;
      int b, h, w0;
      decode(k, b, h, w0);
      ++issued[st];
      mbar_expect_tx(&bar_in[st], 4 * TC_BOX);
#pragma unroll
      for (int j = 0; j < 4; ++j)
        tma_load_4d(s_in + st * TC_BUF + j * TC_PLANE, &tmap, 0, w0 - 1, h - 1, 4 * b + j, &bar_in[st]);
    };
    const uint64_t b_desc = tc::smem_desc(s_w, 128, 256);
    if (lane == 0 && ok)
      for (int k = 0; k < TC_STAGES && k < K; ++k) issue(k);
    for (int k = 0; k < K && ok; ++k) {
      bool go = true;
      if (lane == 0) {
        const int st = k % TC_STAGES, slot = k & 1;
        go = tc::mbar_wait(&bar_in[st], (uint32_t)((k / TC_STAGES) & 1), TC_CONV_WAIT);
        if (go) ++landed[st];
        // the epilogue of tile k - 2 has read this slot
        if (go && k >= 2) go = tc::mbar_wait(&bar_free[slot], (uint32_t)(((k - 2) >> 1) & 1), TC_CONV_WAIT);
        tc::fence_after_sync();
        if (go) {
          // every operand is a fixed offset from the two buffers: the descriptors
          // differ from the buffers' only in the start-address field (address / 16)
          const uint64_t a_desc = tc::smem_desc(s_in + st * TC_BUF, TC_PLANE, 128);
#pragma unroll
          for (int r = 0; r < TC_ROWS; ++r) {  // output row r reads input rows r .. r + 2
            const uint32_t d = tmem + (uint32_t)(slot * TC_SLOT + r * 32);
#pragma unroll
            for (int tap = 0; tap < 9; ++tap) {
              const int dy = tap / 3, dx = tap - dy * 3;
#pragma unroll
              for (int kc = 0; kc < 2; ++kc) {
                const uint64_t ad =
                    a_desc + (uint64_t)((2 * kc * TC_PLANE + ((r + dy) * TC_INW + dx) * 16) >> 4);
                const uint64_t bd = b_desc + (uint64_t)(((tap * 2 + kc) * TC_WBLK) >> 4);
                tc::mma_f16(d, ad, bd, TC_IDESC, (tap | kc) != 0);
              }
            }
          }
          tc::mma_commit(&bar_mma[slot]);
          // tile k - 1's MMAs (queued ahead of these) have read their stage: refill it
          if (k >= 1 && k - 1 + TC_STAGES < K) {
            go = tc::mbar_wait(&bar_mma[(k - 1) & 1], (uint32_t)(((k - 1) >> 1) & 1), TC_CONV_WAIT);
            if (go) issue(k - 1 + TC_STAGES);
          }
        }
      }
      ok = __shfl_sync(0xffffffffu, go ? 1 : 0, 0) != 0;
    }
    if (lane == 0) {
      // after a timeout: let copies still in flight land (bounded) before leaving
      for (int st = 0; st < TC_STAGES; ++st)
        for (; landed[st] < issued[st]; ++landed[st])
          tc::mbar_wait(&bar_in[st], (uint32_t)(landed[st] & 1), TC_CONV_WAIT);
      if (!ok && skip == 0) atomicExch(fail, 1);
    }
    __syncwarp();
  } else {
    // ---- epilogue warps: warp w reads TMEM lanes 32 (w % 4) .. + 31
    const int qtr = warp & 3;
    for (int k = 0; k < K; ++k) {
      const int slot = k & 1;
      if (ok) ok = tc::mbar_wait(&bar_mma[slot], (uint32_t)((k >> 1) & 1), TC_CONV_WAIT);
      tc::fence_after_sync();
      float accs[TC_ROWS][32];
#pragma unroll
      for (int r = 0; r < TC_ROWS; ++r)
        tc::tmem_ld32(tmem + ((uint32_t)(qtr * 32) << 16) + (uint32_t)(slot * TC_SLOT + r * 32), accs[r]);
      tc::fence_before_sync();
      tc::mbar_arrive(&bar_free[slot]);  // the slot may take tile k + 2
      int b, h0, w0;
      decode(k, b, h0, w0);
      const int w = w0 + qtr * 32 + lane;
#pragma unroll
      for (int r = 0; r < TC_ROWS; ++r) {
      const int h = h0 + r;
      const float* acc = accs[r];
      if (w < W && h < H) {
        const float nan = __int_as_float(0x7fc00000);
        if (EPI == 0) {
          uint32_t u[NPAIR];
#pragma unroll
          for (int i = 0; i < NPAIR; ++i)
            u[i] = ok ? bf2_bits(fmaxf(acc[2 * i] + s_bias[2 * i], 0.f), fmaxf(acc[2 * i + 1] + s_bias[2 * i + 1], 0.f))
                      : bf2_bits(nan, nan);
#pragma unroll
          for (int j = 0; j < 4; ++j)
            *reinterpret_cast<uint4*>(out + ((((int64_t)b * 4 + j) * H + h) * W + w) * 8) =
                make_uint4(u[4 * j], u[4 * j + 1], u[4 * j + 2], u[4 * j + 3]);
        } else {
          // resid may be out_c itself: every residual of this element is read before
          // the first store, so the 16 loads are in flight together
          const float scale = sqrtf(pw[b] * inv_count);
          const int64_t e0 = ((int64_t)b * NPAIR * H + h) * ccols + w, es = (int64_t)H * ccols;
          float2 x[NPAIR];
#pragma unroll
          for (int i = 0; i < NPAIR; ++i) x[i] = resid[e0 + i * es];
#pragma unroll
          for (int i = 0; i < NPAIR; ++i)
            out_c[e0 + i * es] = ok ? make_float2(fmaf(scale, acc[2 * i] + s_bias[2 * i], x[i].x),
                                                  fmaf(scale, acc[2 * i + 1] + s_bias[2 * i + 1], x[i].y))
                                    : make_float2(nan, nan);
        }
      }
      }
    }
    if (!ok && skip == 0) atomicExch(fail, 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, 2 * TC_SLOT);
}

// Tensor map of a planar BF16 activation [B][4 chunks][H][W][8] with the conv tile's box:
// dimensions (channel in chunk, column, word, 4 drop + chunk).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

hpx_status activation_map(const __nv_bfloat16* act, int B, int H, int W, CUtensorMap* map) {
  static EncodeTiledFn encode = nullptr;
  if (!encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    HPX_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !fn)
      return hpx_fail(HPX_ERR_CUDA, "cnn: cuTensorMapEncodeTiled unavailable");
    encode = reinterpret_cast<EncodeTiledFn>(fn);
  }
  const cuuint64_t dims[4] = {8, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)B * 4};
  const cuuint64_t strides[3] = {16, (cuuint64_t)W * 16, (cuuint64_t)H * W * 16};
  const cuuint32_t box[4] = {8, (cuuint32_t)TC_INW, (cuuint32_t)TC_INH, 1};
  const cuuint32_t estride[4] = {1, 1, 1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<__nv_bfloat16*>(act), dims, strides,
                            box, estride, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return hpx_fail(HPX_ERR_CUDA, "cnn: tensor map encoding failed (%d)", (int)r);
  return HPX_OK;
}

// Weight and bias gradients of one layer: dW[n][tap*32 + c] += sum_p dY[p][n] X[p + tap][c],
// db[n] += sum_p dY[p][n] over all grid elements of the batch. Nine warps, warp = tap;
// each block walks a contiguous range of tiles and adds its partial sums once.
__global__ void __launch_bounds__(288) k_conv3x3_wgrad(int H, int W, int B, const __nv_bfloat16* __restrict__ x,
                                                       const __nv_bfloat16* __restrict__ dy, float* __restrict__ dw,
                                                       float* __restrict__ db) {
  __shared__ __align__(128) unsigned char s_x[IN_PX * 64];
  __shared__ __align__(128) unsigned char s_d[TH * TW * 64];
  const int tiles_w = (W + TW - 1) / TW, tiles_h = (H + TH - 1) / TH;
  const int64_t tiles = (int64_t)B * tiles_h * tiles_w;
  const int64_t per = (tiles + gridDim.x - 1) / gridDim.x;
  const int64_t t0 = (int64_t)blockIdx.x * per, t1 = min(tiles, t0 + per);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tap = warp, ddy = tap / 3, ddx = tap - ddy * 3;
  const int j = lane >> 3, r = lane & 7;
  float acc[2][4][4];
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int i = 0; i < 4; ++i) acc[mt][nt][i] = 0.f;
  float bsum = 0.f;
  const uint32_t xb = smem_u32(s_x), dbase = smem_u32(s_d);
  for (int64_t t = t0; t < t1; ++t) {
    const int b = (int)(t / (tiles_h * tiles_w));
    const int rem = (int)(t - (int64_t)b * tiles_h * tiles_w);
    const int h0 = (rem / tiles_w) * TH, w0 = (rem - (rem / tiles_w) * tiles_w) * TW;
    __syncthreads();  // previous tile consumed
    load_tile(s_x, x, b, H, W, h0, w0);
    for (int q = threadIdx.x; q < TH * TW * 4; q += blockDim.x) {
      const int pd = q >> 2, ch = q & 3;
      const int ty = pd / TW, tx = pd - ty * TW;
      const int h = h0 + ty, w = w0 + tx;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (h < H && w < W) v = __ldg(reinterpret_cast<const uint4*>(dy + (((int64_t)b * H + h) * W + w) * CH) + ch);
      *reinterpret_cast<uint4*>(s_d + swz(pd, ch)) = v;
    }
    __syncthreads();
    if (threadIdx.x < CH) {
      const __nv_bfloat16* sd = reinterpret_cast<const __nv_bfloat16*>(s_d);
      const int n = threadIdx.x, q = n >> 3, e = n & 7;
      for (int pd = 0; pd < TH * TW; ++pd) bsum += __bfloat162float(sd[swz(pd, q) / 2 + e]);
    }
#pragma unroll
    for (int ty = 0; ty < TH; ++ty)
#pragma unroll 1
      for (int ks = 0; ks < TW / 16; ++ks) {
        uint32_t a[2][4];
#pragma unroll
        for (int mt = 0; mt < 2; ++mt) {
          const int pd = ty * TW + ks * 16 + (j >> 1) * 8 + r;
          ldsm_x4_t(dbase + swz(pd, mt * 2 + (j & 1)), a[mt][0], a[mt][1], a[mt][2], a[mt][3]);
        }
        uint32_t bf[4][2];
#pragma unroll
        for (int half = 0; half < 2; ++half) {
          const int pi = (ty + ddy) * IN_W + ks * 16 + (j & 1) * 8 + r + ddx;
          uint32_t r0, r1, r2, r3;
          ldsm_x4_t(xb + swz(pi, half * 2 + (j >> 1)), r0, r1, r2, r3);
          bf[half * 2][0] = r0;
          bf[half * 2][1] = r1;
          bf[half * 2 + 1][0] = r2;
          bf[half * 2 + 1][1] = r3;
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
          for (int nt = 0; nt < 4; ++nt) mma_bf16(acc[mt][nt], a[mt], bf[nt][0], bf[nt][1]);
      }
  }
  const int g = lane >> 2, cq = (lane & 3) * 2;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 4; ++nt)
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int n = mt * 16 + g + (i >> 1) * 8;
        const int c = nt * 8 + cq + (i & 1);
        atomicAdd(dw + n * KK + tap * CH + c, acc[mt][nt][i]);
      }
  if (threadIdx.x < CH) atomicAdd(db + threadIdx.x, bsum);
}

// Per drop: pw[b] = sum of |LS|^2 over pairs, words and columns, one block per drop
// (blockIdx.x): every warp takes (pair, word) rows in a fixed order and the block
// adds the warp sums in warp order, so the sum (and every refined estimate that the
// input scale enters) is the same from run to run.
constexpr int POWER_THREADS = 512;
__global__ void __launch_bounds__(POWER_THREADS) k_cnn_power(int H, int W, int ccols, const float2* __restrict__ csi,
                                                             float* __restrict__ pw) {
  __shared__ float wsum[POWER_THREADS / 32];
  const int b = blockIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  float e = 0.f;
  for (int row = warp; row < NPAIR * H; row += POWER_THREADS / 32) {
    const float2* r = csi + ((int64_t)b * NPAIR * H + row) * ccols;
    for (int w = lane; w < W; w += 32) {
      const float2 z = r[w];
      e = fmaf(z.x, z.x, fmaf(z.y, z.y, e));
    }
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  if (lane == 0) wsum[warp] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    float t = 0.f;
    for (int i = 0; i < POWER_THREADS / 32; ++i) t += wsum[i];
    pw[b] = t;
  }
}

// complex planes [drop][pair][word][ccols] / s -> bf16 NHWC [drop][word][column][32]
// PLANAR: the tensor-core forward's layout [drop][4 chunks][word][column][8 channels];
// else NHWC.
template <bool PLANAR>
__global__ void k_cnn_pack(int H, int W, int ccols, int B, const float2* __restrict__ csi, const float* __restrict__ pw,
                           float inv_count, __nv_bfloat16* __restrict__ out) {
  const int64_t total = (int64_t)B * H * W;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = q / ((int64_t)H * W);
    const int rem = (int)(q - b * H * W);
    const int h = rem / W, w = rem - h * W;
    const float is = rsqrtf(fmaxf(pw[b] * inv_count, 1e-30f));
    uint32_t v[NPAIR];
#pragma unroll
    for (int p = 0; p < NPAIR; ++p) {
      const float2 z = csi[((b * NPAIR + p) * H + h) * ccols + w];
      v[p] = bf2_bits(z.x * is, z.y * is);
    }
    if (PLANAR) {
#pragma unroll
      for (int j = 0; j < 4; ++j)
        *reinterpret_cast<uint4*>(out + (((b * 4 + j) * H + h) * W + w) * 8) =
            make_uint4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
    } else {
      store_px(out + q * CH, v);
    }
  }
}

// dY = (out - truth) / s as bf16 NHWC and the batch's sum of |out - truth|^2 / s^2
// (the loss at the network's unit scale).
__global__ void k_cnn_loss_grad(int H, int W, int ccols, int B, const float2* __restrict__ outc,
                                const float2* __restrict__ truth, const float* __restrict__ pw, float inv_count,
                                __nv_bfloat16* __restrict__ dy, double* __restrict__ loss) {
  const int64_t total = (int64_t)B * H * W;
  float e = 0.f;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = q / ((int64_t)H * W);
    const int rem = (int)(q - b * H * W);
    const int h = rem / W, w = rem - h * W;
    const float is = rsqrtf(fmaxf(pw[b] * inv_count, 1e-30f));
    uint32_t v[NPAIR];
#pragma unroll
    for (int p = 0; p < NPAIR; ++p) {
      const int64_t i = ((b * NPAIR + p) * H + h) * ccols + w;
      const float2 o = outc[i], t = truth[i];
      const float dx = (o.x - t.x) * is, dyv = (o.y - t.y) * is;
      e = fmaf(dx, dx, fmaf(dyv, dyv, e));
      v[p] = bf2_bits(dx, dyv);
    }
    store_px(dy + q * CH, v);
  }
  for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, (double)e);
}

// Adam on the FP32 master parameters; refreshes the BF16 forward weights and the
// flipped, transposed copies used for input gradients:
//   wd[l][c][(8 - tap) * 32 + n] = w[l][n][tap * 32 + c].
__global__ void k_cnn_adam(int nparam, float* __restrict__ p, float* __restrict__ m, float* __restrict__ v,
                           const float* __restrict__ grad, float lr, float b1, float b2, float eps, float c1, float c2,
                           float gscale, __nv_bfloat16* __restrict__ wbf, __nv_bfloat16* __restrict__ wdf) {
  const int nw = LAYERS * CH * KK;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nparam; i += gridDim.x * blockDim.x) {
    const float g = grad[i] * gscale;
    const float mi = b1 * m[i] + (1.f - b1) * g;
    const float vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    p[i] = pi;
    if (i < nw) {
      const int l = i / (CH * KK), rem = i - l * CH * KK;
      const int n = rem / KK, k = rem - n * KK, tap = k / CH, c = k - tap * CH;
      wbf[i] = __float2bfloat16_rn(pi);
      wdf[(size_t)l * CH * KK + c * KK + (8 - tap) * CH + n] = __float2bfloat16_rn(pi);
    }
  }
}

}  // namespace

struct hpx_cnn {
  int H = 0, W = 0, max_batch = 0;
  int64_t step = 0;
  // parameters: weights [6][32][288] then biases [6][32] (FP32 master, Adam state, gradients)
  float* d_param = nullptr;
  float* d_m = nullptr;
  float* d_v = nullptr;
  float* d_grad = nullptr;
  __nv_bfloat16* d_w = nullptr;   // [6][32][288]
  __nv_bfloat16* d_wd = nullptr;  // [6][32][288] flipped / transposed
  __nv_bfloat16* d_act = nullptr; // [6][max_batch][H][W][32]: x0, h1..h5
  __nv_bfloat16* d_g = nullptr;   // [2][max_batch][H][W][32] gradient ping-pong
  float2* d_out = nullptr;        // [max_batch][16][H][W] training output
  float* d_pw = nullptr;          // [max_batch] per-drop LS power sums
  double* d_loss = nullptr;
  int* d_fail = nullptr;          // set when a tensor-core wait of the forward pass timed out
  int num_sms = 0;
};

namespace {

constexpr int NW = LAYERS * CH * KK, NB = LAYERS * CH, NPARAM = NW + NB;

void cnn_release(hpx_cnn* c) {
  if (!c) return;
  void* p[] = {c->d_param, c->d_m, c->d_v, c->d_grad, c->d_w,  c->d_wd,
               c->d_act,   c->d_g, c->d_out, c->d_pw,  c->d_loss, c->d_fail};
  for (void* q : p)
    if (q) cudaFree(q);
  delete c;
}

hpx_status refresh_bf16(hpx_cnn* c) {
  // an Adam step with zero learning rate and zero gradient rewrites both bf16 copies
  HPX_CUDA(cudaMemset(c->d_grad, 0, sizeof(float) * NPARAM));
  std::vector<float> zero(NPARAM, 0.f);
  float* tmp_m = nullptr;
  float* tmp_v = nullptr;
  HPX_CUDA(cudaMalloc(&tmp_m, sizeof(float) * NPARAM));
  HPX_CUDA(cudaMalloc(&tmp_v, sizeof(float) * NPARAM));
  cudaMemset(tmp_m, 0, sizeof(float) * NPARAM);
  cudaMemset(tmp_v, 0, sizeof(float) * NPARAM);
  k_cnn_adam<<<(NPARAM + 255) / 256, 256>>>(NPARAM, c->d_param, tmp_m, tmp_v, c->d_grad, 0.f, 0.9f, 0.999f, 1e-8f,
                                             1.f, 1.f, 1.f, c->d_w, c->d_wd);
  const cudaError_t e = cudaDeviceSynchronize();
  cudaFree(tmp_m);
  cudaFree(tmp_v);
  if (e != cudaSuccess) return hpx_cuda_status(e, "cnn weights");
  return HPX_OK;
}

int conv_tiles(int H, int W) { return ((H + TH - 1) / TH) * ((W + TW - 1) / TW); }

// Power sums and the packed, scaled input of B drops of complex planes.
hpx_status prepare(const hpx_cnn* c, int B, const float2* csi, int ccols, __nv_bfloat16* x0, bool planar,
                   cudaStream_t s) {
  const float inv = 1.f / (float)(NPAIR * c->H * c->W);
  k_cnn_power<<<B, POWER_THREADS, 0, s>>>(c->H, c->W, ccols, csi, c->d_pw);
  HPX_LAUNCHED("cnn power");
  const int64_t px = (int64_t)B * c->H * c->W;
  if (planar)
    k_cnn_pack<true><<<(int)((px + 255) / 256), 256, 0, s>>>(c->H, c->W, ccols, B, csi, c->d_pw, inv, x0);
  else
    k_cnn_pack<false><<<(int)((px + 255) / 256), 256, 0, s>>>(c->H, c->W, ccols, B, csi, c->d_pw, inv, x0);
  HPX_LAUNCHED("cnn pack");
  return HPX_OK;
}

// Training forward (NHWC activations kept for the backward pass): mma.sync layers.
hpx_status forward(const hpx_cnn* c, int B, const __nv_bfloat16* x0, __nv_bfloat16* const* act_out,
                   const float2* resid, float2* out_c, int ccols, cudaStream_t s) {
  const float inv = 1.f / (float)(NPAIR * c->H * c->W);
  dim3 g(conv_tiles(c->H, c->W), B);
  const __nv_bfloat16* in = x0;
  for (int l = 0; l < LAYERS - 1; ++l) {
    k_conv3x3<0><<<g, 128, 0, s>>>(c->H, c->W, in, c->d_w + (size_t)l * CH * KK, c->d_param + NW + l * CH,
                                   act_out[l], nullptr, nullptr, nullptr, 0, nullptr, 0.f);
    in = act_out[l];
  }
  k_conv3x3<1><<<g, 128, 0, s>>>(c->H, c->W, in, c->d_w + (size_t)(LAYERS - 1) * CH * KK,
                                 c->d_param + NW + (LAYERS - 1) * CH, nullptr, nullptr, resid, out_c, ccols, c->d_pw,
                                 inv);
  HPX_LAUNCHED("cnn forward");
  return HPX_OK;
}

// Inference forward on the tensor cores (TMA + tcgen05), planar activations.
hpx_status forward_tc(const hpx_cnn* c, int B, const __nv_bfloat16* x0, __nv_bfloat16* const* act_out,
                      const float2* resid, float2* out_c, int ccols, cudaStream_t s) {
  const float inv = 1.f / (float)(NPAIR * c->H * c->W);
  const int64_t tiles = (int64_t)B * ((c->H + TC_ROWS - 1) / TC_ROWS) * ((c->W + TCW - 1) / TCW);
  const int grid = (int)std::min<int64_t>(tiles, (int64_t)c->num_sms * TC_CTAS_PER_SM);
  // per call: the attribute belongs to the current device's context
  HPX_CUDA(cudaFuncSetAttribute(k_conv3x3_tc<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
  HPX_CUDA(cudaFuncSetAttribute(k_conv3x3_tc<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM));
  const __nv_bfloat16* in = x0;
  CUtensorMap map;
  for (int l = 0; l < LAYERS - 1; ++l) {
    HPX_TRY(activation_map(in, B, c->H, c->W, &map));
    k_conv3x3_tc<0><<<grid, TC_THREADS, TC_SMEM, s>>>(map, B, c->H, c->W, c->d_w + (size_t)l * CH * KK,
                                               c->d_param + NW + l * CH, act_out[l], nullptr, nullptr, 0, nullptr,
                                               0.f, c->d_fail);
    HPX_LAUNCHED("cnn forward");
    in = act_out[l];
  }
  HPX_TRY(activation_map(in, B, c->H, c->W, &map));
  k_conv3x3_tc<1><<<grid, TC_THREADS, TC_SMEM, s>>>(map, B, c->H, c->W, c->d_w + (size_t)(LAYERS - 1) * CH * KK,
                                             c->d_param + NW + (LAYERS - 1) * CH, nullptr, resid, out_c, ccols,
                                             c->d_pw, inv, c->d_fail);
  HPX_LAUNCHED("cnn forward");
  return HPX_OK;
}

}  // namespace

extern "C" {

hpx_status hpx_cnn_create(int32_t num_words, int32_t num_columns, int32_t max_batch, const float* params,
                          uint64_t seed, hpx_cnn** out) {
  if (!out) return hpx_fail(HPX_ERR_ARG, "cnn: null argument");
  *out = nullptr;
  if (num_words < 1 || num_columns < 1 || max_batch < 1 || max_batch > 65535)
    return hpx_fail(HPX_ERR_ARG, "cnn: bad grid or batch size");
  hpx_cnn* c = new hpx_cnn();
  c->H = num_words;
  c->W = num_columns;
  c->max_batch = max_batch;
  std::vector<float> host(NPARAM, 0.f);
  if (params) {
    host.assign(params, params + NPARAM);
  } else {
    // He-normal convolutions; the last layer starts near zero so the network
    // starts as the identity on its LS input.
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, std::sqrt(2.0f / KK));
    for (int l = 0; l < LAYERS; ++l)
      for (int i = 0; i < CH * KK; ++i) host[(size_t)l * CH * KK + i] = nd(rng) * (l == LAYERS - 1 ? 0.01f : 1.f);
  }
  const size_t act = (size_t)max_batch * num_words * num_columns * CH;
  cudaError_t e;
  if ((e = cudaMalloc(&c->d_param, sizeof(float) * NPARAM)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_m, sizeof(float) * NPARAM)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_v, sizeof(float) * NPARAM)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_grad, sizeof(float) * NPARAM)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_w, sizeof(__nv_bfloat16) * NW)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_wd, sizeof(__nv_bfloat16) * NW)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_act, sizeof(__nv_bfloat16) * act * LAYERS)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_g, sizeof(__nv_bfloat16) * act * 2)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_out, sizeof(float2) * (size_t)max_batch * NPAIR * num_words * num_columns)) !=
          cudaSuccess ||
      (e = cudaMalloc(&c->d_loss, sizeof(double))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_pw, sizeof(float) * max_batch)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_fail, sizeof(int))) != cudaSuccess ||
      (e = cudaMemset(c->d_fail, 0, sizeof(int))) != cudaSuccess ||
      (e = cudaMemcpy(c->d_param, host.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemset(c->d_m, 0, sizeof(float) * NPARAM)) != cudaSuccess ||
      (e = cudaMemset(c->d_v, 0, sizeof(float) * NPARAM)) != cudaSuccess) {
    cnn_release(c);
    return hpx_cuda_status(e, "cnn buffers");
  }
  int dev = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) {
    cnn_release(c);
    return hpx_cuda_status(e, "cnn device");
  }
  const hpx_status st = refresh_bf16(c);
  if (st != HPX_OK) {
    cnn_release(c);
    return st;
  }
  *out = c;
  return HPX_OK;
}

hpx_status hpx_cnn_destroy(hpx_cnn* c) {
  cnn_release(c);
  return HPX_OK;
}

int32_t hpx_cnn_num_params(void) { return NPARAM; }

hpx_status hpx_cnn_get_params(const hpx_cnn* c, float* params) {
  if (!c || !params) return hpx_fail(HPX_ERR_ARG, "cnn_get_params: null argument");
  HPX_CUDA(cudaMemcpy(params, c->d_param, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  return HPX_OK;
}

hpx_status hpx_cnn_get_grads(const hpx_cnn* c, float* grads) {
  if (!c || !grads) return hpx_fail(HPX_ERR_ARG, "cnn_get_grads: null argument");
  HPX_CUDA(cudaMemcpy(grads, c->d_grad, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost));
  return HPX_OK;
}

hpx_status hpx_cnn_refine(const hpx_cnn* c, hpx_cf32* csi, int32_t ccols, int32_t B, void* stream) {
  if (!c || !csi) return hpx_fail(HPX_ERR_ARG, "cnn_refine: null argument");
  if (B < 0) return hpx_fail(HPX_ERR_ARG, "cnn_refine: negative batch");
  if (ccols < c->W) return hpx_fail(HPX_ERR_SHAPE, "cnn_refine: CSI narrower than the network's grid");
  cudaStream_t s = as_stream(stream);
  const size_t act = (size_t)c->max_batch * c->H * c->W * CH;
  for (int b0 = 0; b0 < B; b0 += c->max_batch) {
    const int n = B - b0 < c->max_batch ? B - b0 : c->max_batch;
    float2* cs = reinterpret_cast<float2*>(csi) + (size_t)b0 * NPAIR * c->H * ccols;
    __nv_bfloat16* x0 = c->d_act;
    __nv_bfloat16* pp[2] = {c->d_g, c->d_g + act};
    __nv_bfloat16* outs[LAYERS - 1] = {pp[0], pp[1], pp[0], pp[1], pp[0]};
    HPX_TRY(prepare(c, n, cs, ccols, x0, true, s));
    HPX_TRY(forward_tc(c, n, x0, outs, cs, cs, ccols, s));
  }
  return HPX_OK;
}

hpx_status hpx_cnn_status(hpx_cnn* c, int32_t clear, void* stream) {
  if (!c) return hpx_fail(HPX_ERR_ARG, "cnn_status: null argument");
  cudaStream_t s = as_stream(stream);
  int flag = 0;
  HPX_CUDA(cudaMemcpyAsync(&flag, c->d_fail, sizeof(int), cudaMemcpyDeviceToHost, s));
  if (clear) HPX_CUDA(cudaMemsetAsync(c->d_fail, 0, sizeof(int), s));
  HPX_CUDA(cudaStreamSynchronize(s));
  if (flag) return hpx_fail(HPX_ERR_TIMEOUT, "cnn_refine: a bounded TMA / tensor-core wait ran out (estimates are NaN)");
  return HPX_OK;
}

hpx_status hpx_cnn_inject_timeout(hpx_cnn* c, void* stream) {
  if (!c) return hpx_fail(HPX_ERR_ARG, "cnn_inject_timeout: null argument");
  HPX_CUDA(cudaMemsetAsync(c->d_fail, 0x01, 1, as_stream(stream)));  // the int word becomes 1
  return HPX_OK;
}

hpx_status hpx_cnn_train_step(hpx_cnn* c, const hpx_cf32* ls, const hpx_cf32* truth, int32_t ccols, int32_t B,
                              float lr, double* loss, void* stream) {
  if (!c || !ls || !truth) return hpx_fail(HPX_ERR_ARG, "cnn_train_step: null argument");
  if (B < 1 || B > c->max_batch) return hpx_fail(HPX_ERR_ARG, "cnn_train_step: batch must be in [1, %d]", c->max_batch);
  if (ccols != c->W) return hpx_fail(HPX_ERR_SHAPE, "cnn_train_step: CSI columns must equal the network's grid width");
  cudaStream_t s = as_stream(stream);
  const size_t act = (size_t)c->max_batch * c->H * c->W * CH;
  __nv_bfloat16* a[LAYERS];
  for (int l = 0; l < LAYERS; ++l) a[l] = c->d_act + act * l;
  const int64_t px = (int64_t)B * c->H * c->W;
  const int blocks = (int)((px + 255) / 256);
  const float inv = 1.f / (float)(NPAIR * c->H * c->W);
  HPX_TRY(prepare(c, B, reinterpret_cast<const float2*>(ls), ccols, a[0], false, s));
  HPX_TRY(forward(c, B, a[0], a + 1, reinterpret_cast<const float2*>(ls), c->d_out, ccols, s));
  HPX_CUDA(cudaMemsetAsync(c->d_loss, 0, sizeof(double), s));
  __nv_bfloat16* g[2] = {c->d_g, c->d_g + act};
  k_cnn_loss_grad<<<blocks, 256, 0, s>>>(c->H, c->W, ccols, B, c->d_out, reinterpret_cast<const float2*>(truth),
                                         c->d_pw, inv, g[0], c->d_loss);
  HPX_LAUNCHED("cnn loss");
  HPX_CUDA(cudaMemsetAsync(c->d_grad, 0, sizeof(float) * NPARAM, s));
  const int tiles = B * conv_tiles(c->H, c->W);
  const int wblocks = tiles < 4 * 152 ? tiles : 4 * 152;
  dim3 gd(conv_tiles(c->H, c->W), B);
  int cur = 0;
  for (int l = LAYERS - 1; l >= 0; --l) {
    k_conv3x3_wgrad<<<wblocks, 288, 0, s>>>(c->H, c->W, B, a[l], g[cur], c->d_grad + (size_t)l * CH * KK,
                                            c->d_grad + NW + l * CH);
    HPX_LAUNCHED("cnn wgrad");
    if (l > 0) {
      k_conv3x3<2><<<gd, 128, 0, s>>>(c->H, c->W, g[cur], c->d_wd + (size_t)l * CH * KK, nullptr, g[cur ^ 1], a[l],
                                      nullptr, nullptr, 0, nullptr, 0.f);
      HPX_LAUNCHED("cnn dgrad");
      cur ^= 1;
    }
  }
  c->step += 1;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f / (1.f - std::pow(b1, (float)c->step)), c2 = 1.f / (1.f - std::pow(b2, (float)c->step));
  // gradients are sums over the batch's grid elements and channels: average them
  const float gscale = 1.f / (float)(px * CH);
  k_cnn_adam<<<(NPARAM + 255) / 256, 256, 0, s>>>(NPARAM, c->d_param, c->d_m, c->d_v, c->d_grad, lr, b1, b2, 1e-8f, c1,
                                                   c2, gscale, c->d_w, c->d_wd);
  HPX_LAUNCHED("cnn adam");
  if (loss) HPX_CUDA(cudaMemcpyAsync(loss, c->d_loss, sizeof(double), cudaMemcpyDeviceToDevice, s));
  return HPX_OK;
}

}  // extern "C"
