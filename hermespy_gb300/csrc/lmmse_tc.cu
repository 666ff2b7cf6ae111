// Fused tap-domain LMMSE receiver of the 4 x 4 pilot-comb link on the tcgen05
// tensor cores.
//
// The per-element channel of every antenna pair is a tap DFT,
//   H[w][c][pair] = sum_u g[w][u][pair] exp(-2 pi i bin(c) d_u / N),
// i.e. for one drop a GEMM of (subcarriers x 2U) twiddles by (2U x words*pairs*{re,im})
// gains: [Re H | Im H] = [F_re | F_im] [[G_re, G_im], [-G_im, G_re]]. It runs in three
// kernels per chunk of drops:
//   k_lmmse_ls     (one CTA per pilot word of a stream and 32 drops): the pilot LS of
//                  the tap gains, as a complex GEMM over drops with the weighted-LS
//                  operator held in shared memory;
//   k_lmmse_gains  (one CTA per drop): per-tap LMMSE weights over the pilot words
//                  and the gains of every data word and pair, written to a
//                  workspace as the GEMM's FP16 (hi, lo) operand in its shared-memory
//                  layout, scaled by a power of two bounding them by 1;
//   k_lmmse_tc     (one CTA per drop and 128 subcarriers): the GEMM as FP16 MMAs
//                  with FP32 accumulation in tensor memory, operands split
//                  x = hi + lo and multiplied hi*hi + hi*lo + lo*hi (~2^-22 of the
//                  largest term), four words (128 accumulator columns) per pass;
//                  then every thread owns one subcarrier (its TMEM lane), reads a
//                  word's 16 complex gains with one tcgen05.ld, equalizes (LMMSE /
//                  ZF, Cholesky), demaps and counts bit errors against the
//                  regenerated Philox bits.
// The twiddle operand (hi, lo) of each 128-subcarrier tile is built once at
// handle creation. Other antenna configurations use the FP32 kernel in detect.cu.
#include <cuda_fp16.h>

#include <algorithm>
#include <cmath>

#include "equalize_dev.cuh"
#include "lmmse_dev.cuh"
#include "tcgen05.cuh"

namespace {

constexpr int TC_THREADS = 256;   // 8 warps: 4 lane quarters x 2 word slots
constexpr int TC_M = 128;         // subcarriers per CTA (TMEM lanes)
constexpr int TC_WORDS = 4;       // words per pass: 4 x 16 pairs x {re, im} = 128 columns
constexpr int TC_N = TC_WORDS * 32;
constexpr int TC_BITBLK = 10;     // Philox blocks staged per (word slot, stream)
constexpr int TC_NP = 16;         // antenna pairs (4 x 4)
constexpr long long TC_WAIT = 40ll * 1000 * 1000;  // cycles (~20 ms) before a wait gives up
constexpr int TC_CTAS = 3;        // CTAs per SM: 3 x 128 TMEM columns, ~68 KB shared memory, 85 registers

struct TcView {
  int W, FC, U, KP, mtiles, nwl, m;
  const int32_t* wlist;   // [nwl] data words, -1 padding
  const int32_t* kfirst;  // [W][mtiles] first data element of row w in tile, -1: none
  const int32_t* etab;    // [W][FC] data element index, -1 for reference / null elements
  const uint16_t* ftab;   // [mtiles][2][TC_M x KP] K-major FP16 (hi, lo)
  const uint16_t* bop;    // [drops][passes][2][TC_M x KP] FP16 gains operand (hi, lo)
  const float* scale;     // [drops]
};

// ------------------------------------------------------- kernel 0: pilot LS
// The weighted LS of every tap gain on every pilot word (step 1 of lmmse_drop_taps),
// batched over drops as a complex GEMM: CTA (pilot word p, DROPS drops) computes
// gls[b][r ntx + t][p][u] = sum_k G_tp[u][k] y(b, r, word_p, pcol_tp[k]) for all four
// streams t, its drops and the 4 receive antennas. The received rows of the word pass
// through shared memory in chunks of LS_CC columns (whole 32-byte sectors: every
// pilot of every stream in them is used), with the weighted-LS rows of the pilots
// that fall in the chunk, by cp.async S stages deep. Rows are stored as (gr, gr, gi,
// gi) and pilots as received, so that P += (yr, yi) (gr, gr) and Q += (yr, yi) (gi, gi)
// are packed FP32x2 FMAs and the gain is (P.x - Q.y, Q.x + P.y). Thread (t, g, d)
// accumulates taps g, g + 8, ... of stream t for drop d's four antennas.
// A chunk column holds (drop d, antenna r) at 8-byte slot 4 d + r, columns ROWS + 2
// slots apart: a staging copy instruction writes 32 columns of one row (one 256-byte
// run in global memory, 4-way bank aliasing in shared memory), and the FMA loop reads
// a drop's antennas (0, 1) and (2, 3) as 16-byte pairs, the warp's 4 drops without
// conflicts.
constexpr int LS_CC = 32;  // columns per chunk

template <int TU>
struct LsShape {
  static constexpr int DROPS = TU <= 4 ? 16 : 8;  // accumulator registers: 16 TU per thread
  static constexpr int THREADS = 4 * 8 * DROPS;   // 4 streams x 8 tap groups x DROPS
  static constexpr int ROWS = 4 * DROPS;          // received rows (drop, antenna) of a chunk
  static constexpr int CS = ROWS + 2;             // slots per staged column
};

struct LsView {
  const int32_t* cspan;  // [np][2] first pilot column of the word, columns spanned
  const int2* krange;    // [np][nch_max][4]: stream t's pilots in chunk c, [kb, ke)
  int nch_max, kcm, cnt_max;
};

size_t lmmse_ls_smem(int tu, int stages, int kcm, int cnt_max, int nch_max) {
  const int cs = (tu <= 4 ? 64 : 32) + 2;
  return (size_t)stages * LS_CC * cs * sizeof(float2) + (size_t)stages * 4 * kcm * 8 * tu * sizeof(float4) +
         (size_t)4 * cnt_max * 4 + (size_t)nch_max * 4 * sizeof(int2);
}

__device__ __forceinline__ void cp_async8(void* dst, const void* src, bool fill) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(src), "r"(fill ? 8 : 0) : "memory");
}
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool fill) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(s), "l"(src), "r"(fill ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <int TU, int S>  // taps per thread (U <= 8 TU), pipeline stages
__global__ void __launch_bounds__(LsShape<TU>::THREADS, 1)
    k_lmmse_ls(LmmseView e, LsView lv, const float4* __restrict__ gtab, const float2* __restrict__ grid, int gcols,
               int nb, float2* __restrict__ gls_out) {
  using SH = LsShape<TU>;
  constexpr int UP = 8 * TU;
  extern __shared__ float4 smem4[];
  const int kcm = lv.kcm, cmax = lv.cnt_max;
  float2* ys = reinterpret_cast<float2*>(smem4);               // [S][LS_CC][CS]
  float4* gs = reinterpret_cast<float4*>(ys + S * LS_CC * SH::CS);  // [S][4][kcm][UP]
  int* pcs = reinterpret_cast<int*>(gs + S * 4 * kcm * UP);    // [4][cnt_max] column - first column
  int2* kr = reinterpret_cast<int2*>(pcs + 4 * cmax);          // [nch][4]
  const int W = e.W, U = e.U, np = e.np, P = e.P;
  const int p = blockIdx.x, b0 = blockIdx.y * SH::DROPS;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int word = e.pw_word[p];  // every stream carries pilots in the same words
  const int c_first = lv.cspan[2 * p], span = lv.cspan[2 * p + 1];
  const int nch = (span + LS_CC - 1) / LS_CC;
  __shared__ int offt[4];  // first pilot of each stream's word p in the pilot tables
  if (tid < 4) offt[tid] = e.pw_off[tid * P + p];
  for (int i = tid; i < 4 * cmax; i += SH::THREADS) {
    const int t = i / cmax, k = i - t * cmax;
    if (k < e.pw_count[t * P + p]) pcs[i] = e.pcol[e.pw_off[t * P + p] + k] - c_first;
  }
  for (int i = tid; i < nch * 4; i += SH::THREADS) kr[i] = lv.krange[(size_t)p * lv.nch_max * 4 + i];
  __syncthreads();
  // staging: copy m of this thread is row warp + (THREADS / 32) m, column lane of the chunk
  constexpr int NM = SH::ROWS * LS_CC / SH::THREADS;
  static_assert(NM * SH::THREADS == SH::ROWS * LS_CC && SH::THREADS / 32 * NM == SH::ROWS, "staging rounds");
  const float2* rp[NM];
  int ys_off[NM];
#pragma unroll
  for (int m = 0; m < NM; ++m) {
    const int row = warp + (SH::THREADS / 32) * m, dd = row >> 2, r = row & 3;
    rp[m] = grid + (((int64_t)min(b0 + dd, nb - 1) * 4 + r) * W + word) * gcols + c_first;
    ys_off[m] = lane * SH::CS + 4 * dd + r;
  }
  const int g = tid & 7, d = (tid >> 3) % SH::DROPS;
  const int ts = tid / (8 * SH::DROPS);  // this thread's stream
  auto stage = [&](int c, int st) {
    const int col = c * LS_CC + lane;
    const bool ok = col < span;
    float2* yd = ys + st * LS_CC * SH::CS;
#pragma unroll
    for (int m = 0; m < NM; ++m) cp_async8(yd + ys_off[m], rp[m] + (ok ? col : 0), ok);
    // the operator rows of this thread's stream: its 8 DROPS threads copy kcm x UP rows
    float4* gd = gs + (st * 4 + ts) * kcm * UP;
    const int2 k = kr[c * 4 + ts];
    const float4* gsrc = gtab + (int64_t)(offt[ts] + k.x) * UP;
    for (int j = tid - ts * 8 * SH::DROPS; j < kcm * UP; j += 8 * SH::DROPS) {
      const bool v = j < (k.y - k.x) * UP;
      cp_async16(gd + j, v ? gsrc + j : gtab, v);
    }
  };
  float2 Pa[TU][4], Qa[TU][4];
#pragma unroll
  for (int i = 0; i < TU; ++i)
#pragma unroll
    for (int r = 0; r < 4; ++r) Pa[i][r] = Qa[i][r] = make_float2(0.f, 0.f);
#pragma unroll
  for (int s = 0; s < S - 1; ++s) {
    if (s < nch) stage(s, s);
    cp_async_commit();
  }
  const int* pct = pcs + ts * cmax;
  for (int c = 0; c < nch; ++c) {
    cp_async_wait<S - 2>();
    __syncthreads();  // chunk c landed everywhere; chunk c - 1's stage is free
    if (c + S - 1 < nch) stage(c + S - 1, (c + S - 1) % S);
    cp_async_commit();
    const int st = c % S;
    const float2* yst = ys + st * LS_CC * SH::CS + 4 * d;
    const float4* gst = gs + (st * 4 + ts) * kcm * UP + g;
    const int2 k = kr[c * 4 + ts];
#pragma unroll 2
    for (int kk = k.x; kk < k.y; ++kk) {
      const float2* yc = yst + (pct[kk] - c * LS_CC) * SH::CS;
      const float4 y01 = *reinterpret_cast<const float4*>(yc);
      const float4 y23 = *reinterpret_cast<const float4*>(yc + 2);
      const float2 y[4] = {make_float2(y01.x, y01.y), make_float2(y01.z, y01.w), make_float2(y23.x, y23.y),
                           make_float2(y23.z, y23.w)};
      const float4* gk = gst + (kk - k.x) * UP;
#pragma unroll
      for (int i = 0; i < TU; ++i) {
        const float4 gv = gk[8 * i];
#pragma unroll
        for (int r = 0; r < 4; ++r) {
          Pa[i][r] = __ffma2_rn(y[r], make_float2(gv.x, gv.y), Pa[i][r]);
          Qa[i][r] = __ffma2_rn(y[r], make_float2(gv.z, gv.w), Qa[i][r]);
        }
      }
    }
  }
  const int b = b0 + d;
  if (b >= nb) return;
  float2* dst = gls_out + (int64_t)b * 16 * np * U;
#pragma unroll
  for (int i = 0; i < TU; ++i) {
    const int u = 8 * i + g;
    if (u < U)
#pragma unroll
      for (int r = 0; r < 4; ++r)
        dst[((r * 4 + ts) * np + p) * U + u] = make_float2(Pa[i][r].x - Qa[i][r].y, Qa[i][r].x + Pa[i][r].y);
  }
}

// ------------------------------------------------------------ kernel 1: gains
// Per drop: the per-tap LMMSE weights over the pilot words (lmmse_word_weights), the
// gains g[w][u][pair] = sum_p weight * LS gain of every data word, and from them,
// per pass of four data words, the FP16 (hi, lo) gains operand of the GEMM in its
// K-major shared-memory layout: row n = slot * 32 + q (q < 16: Re H of pair q, else
// Im H of pair q - 16), k < U: the coefficient of Re F (G_re or G_im), U <= k < 2U:
// of Im F (-G_im or G_re), scaled by a power of two bounding the drop's gains by 1.
// The gains are kept as gx[i][row][q] (row < U: tap, U <= row < KP - U: zero) for
// data word i of the pass list, q < 16: Re of pair q, else Im of pair q - 16; operand
// column k reads row k (column q) for k < U and row k - U (column q ^ 16, negated for
// q < 16) above, so k >= 2U meets the zero rows. Lane q of a warp writes row n.
__global__ void __launch_bounds__(512, 2) k_lmmse_gains(LmmseView e, const float* __restrict__ nv,
                                                         const int32_t* __restrict__ wlist, int nwl, int KP,
                                                         uint16_t* __restrict__ bop, float* __restrict__ scale_ws,
                                                         const float2* __restrict__ gls_ws) {
  extern __shared__ float4 smem4[];
  __shared__ float red[16];
  __shared__ float sscale;
  const int b = blockIdx.x, tid = threadIdx.x;
  const int W = e.W, U = e.U, np = e.np, ntx = e.ntx, R = KP - U;
  float* gx = reinterpret_cast<float*>(smem4);   // [nwl][R][32]
  float* cw = gx + (size_t)nwl * R * 32;         // [ntx][U][W][np]
  for (int i = tid; i < nwl * (R - U) * 32; i += blockDim.x) {
    const int wi = i / ((R - U) * 32), rest = i - wi * (R - U) * 32;
    gx[((size_t)wi * R + U) * 32 + rest] = 0.0f;
  }
  const float s2 = nv ? nv[b] : 0.0f;
  switch (np) {  // the data words' systems in parallel for the usual pilot-word counts
    case 1: lmmse_listed_word_weights<1>(e, s2, wlist, nwl, cw); break;
    case 2: lmmse_listed_word_weights<2>(e, s2, wlist, nwl, cw); break;
    case 3: lmmse_listed_word_weights<3>(e, s2, wlist, nwl, cw); break;
    case 4: lmmse_listed_word_weights<4>(e, s2, wlist, nwl, cw); break;
    default: lmmse_word_weights<kMaxPilotWords>(e, s2, cw, np); break;
  }
  __syncthreads();
  const float2* gsrc = gls_ws + (int64_t)b * TC_NP * np * U;
  float mx = 0.0f;
  for (int q = tid; q < U * TC_NP; q += blockDim.x) {
    const int u = q >> 4, pair = q & 15, t = pair % ntx;
    float2 gl[kMaxPilotWords];
#pragma unroll
    for (int p = 0; p < kMaxPilotWords; ++p) gl[p] = p < np ? gsrc[(pair * np + p) * U + u] : make_float2(0.f, 0.f);
    const float* cu = cw + ((size_t)t * U + u) * W * np;
    for (int i = 0; i < nwl; ++i) {
      const int w = wlist[i];
      float2 acc = make_float2(0.f, 0.f);
      if (w >= 0) {
#pragma unroll
        for (int p = 0; p < kMaxPilotWords; ++p)
          if (p < np) {
            const float c = cu[w * np + p];
            acc.x = fmaf(c, gl[p].x, acc.x);
            acc.y = fmaf(c, gl[p].y, acc.y);
          }
      }
      float* row = gx + ((size_t)i * R + u) * 32;
      row[pair] = acc.x;
      row[16 + pair] = acc.y;
      mx = fmaxf(mx, fmaxf(fabsf(acc.x), fabsf(acc.y)));
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((tid & 31) == 0) red[tid >> 5] = mx;
  __syncthreads();
  if (tid == 0) {
    float m = 0.0f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, red[w]);
    int ex = 0;
    frexpf(m, &ex);  // m < 2^ex
    sscale = (m > 0.0f && isfinite(m)) ? ldexpf(1.0f, ex) : 1.0f;
    scale_ws[b] = sscale;
  }
  __syncthreads();
  const float inv = 1.0f / sscale;
  const int q = tid & 31;
  const float inv_hi = q < 16 ? -inv : inv;          // k >= U: -G_im for Re rows, G_re for Im rows
  const int step_hi = ((q ^ 16) - q) - U * 32;       // from (row k, column q) to (row k - U, column q ^ 16)
  const int kg = KP / 8;
  const size_t opel = (size_t)TC_M * KP;  // halves per operand
  uint16_t* dst = bop + (size_t)b * (nwl / TC_WORDS) * 2 * opel;
  for (int it = tid >> 5; it < nwl * kg; it += blockDim.x >> 5) {
    const int i = it / kg, gk = it - i * kg;
    const int pass = i / TC_WORDS, n = (i - pass * TC_WORDS) * 32 + q;
    const float* src = gx + (size_t)i * R * 32 + q;
    uint32_t hw[4], lw[4];
#pragma unroll
    for (int j = 0; j < 8; j += 2) {
      const int k0 = gk * 8 + j, k1 = k0 + 1;
      const float v0 = src[k0 * 32 + (k0 >= U ? step_hi : 0)] * (k0 >= U ? inv_hi : inv);
      const float v1 = src[k1 * 32 + (k1 >= U ? step_hi : 0)] * (k1 >= U ? inv_hi : inv);
      const __half2 h = __floats2half2_rn(v0, v1);
      const float2 hf = __half22float2(h);
      const __half2 l = __floats2half2_rn(v0 - hf.x, v1 - hf.y);
      hw[j >> 1] = *reinterpret_cast<const uint32_t*>(&h);
      lw[j >> 1] = *reinterpret_cast<const uint32_t*>(&l);
    }
    uint16_t* base = dst + (size_t)pass * 2 * opel;
    const uint32_t off = tc::kmajor_offset(n, gk * 8, KP) / 2;
    *reinterpret_cast<uint4*>(base + off) = make_uint4(hw[0], hw[1], hw[2], hw[3]);
    *reinterpret_cast<uint4*>(base + opel + off) = make_uint4(lw[0], lw[1], lw[2], lw[3]);
  }
}

// ------------------------------------------------------- kernel 2: GEMM + detect
// Operands and received samples arrive by bulk copies issued by thread 0 at the start
// of each pass (the twiddle tile with the first pass), completing on mbar_ld: the
// pass's gains operand (hi, lo) and, when the grid's rows are 16-byte aligned, the
// pass's received rows (4 words x 4 antennas x this tile's columns) into `ys`. The
// epilogue thus reads its received samples from shared memory; every thread waits
// on mbar_ld itself before reading them. The tile's element table (data element
// index of each column of each data word, -1 for other elements) and the drop's
// gains scale are read before the tensor-memory load of each word.
// The equalizer works on the unscaled GEMM output A = H / scale with the regularizer
// s2 / scale^2 and divides the solution by scale: the scale is a power of two, so
// the result is the one of H itself.
template <int ORDER>  // modulation order: the demapper's branches and the bit widths are fixed
__global__ void __launch_bounds__(TC_THREADS, TC_CTAS) k_lmmse_tc(TcView v, int W, const float2* __restrict__ grid,
                                                                  int gcols, int bulk_y, const float* __restrict__ nv,
                                                                  const __grid_constant__ QamDemapTable qt, int mode,
                                                                  uint64_t seed, int64_t drop0,
                                                                  uint32_t* __restrict__ errors, int* fail) {
  extern __shared__ __align__(128) unsigned char sm[];
  __shared__ uint64_t mbar, mbar_ld;
  __shared__ uint32_t tmem_slot;
  const int mt = blockIdx.x, b = blockIdx.y;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  constexpr int m = ORDER == 2 ? 1 : ORDER == 4 ? 2 : ORDER == 16 ? 4 : ORDER == 64 ? 6 : 8;
  const int KP = v.KP;
  const uint32_t opbytes = (uint32_t)TC_M * KP * 2;  // one 128-row FP16 operand
  unsigned char* a_hi = sm;
  unsigned char* a_lo = sm + opbytes;
  unsigned char* b_hi = sm + 2 * opbytes;
  unsigned char* b_lo = sm + 3 * opbytes;
  float2* ys = reinterpret_cast<float2*>(sm + 4 * opbytes);  // [TC_WORDS][4 antennas][TC_M]
  uint32_t* bits = reinterpret_cast<uint32_t*>(sm + 4 * opbytes + TC_WORDS * 4 * TC_M * sizeof(float2));

  __shared__ int skip;
  if (tid == 0) skip = *(volatile int*)fail;
  __syncthreads();
  if (skip) {  // an earlier CTA timed out on the tensor core: flag and leave
    if (tid == 0) atomicOr(errors + b, HPX_DROP_TIMEOUT);
    return;
  }
  if (warp == 0) {
    tc::tmem_alloc(&tmem_slot, TC_N);
    tc::tmem_relinquish();
  }
  if (tid == 0) {
    tc::mbar_init(&mbar, 1);
    tc::mbar_init(&mbar_ld, 1);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tmem_slot;
  const int c0 = mt * TC_M;
  const int ncol = min(TC_M, v.FC - c0);
  const uint32_t rowbytes = (uint32_t)ncol * sizeof(float2);  // ncol even when bulk_y (checked on the host)
  const unsigned char* bop = reinterpret_cast<const unsigned char*>(v.bop) + (size_t)b * (v.nwl / TC_WORDS) * 2 * opbytes;
  const float scl = v.scale[b];
  const float s2 = nv ? nv[b] : 0.0f;
  const float inv_scl = 1.0f / scl;          // powers of two: exact
  const float s2a = s2 * inv_scl * inv_scl;  // regularizer of the unscaled system
  bool ok = true, fin = finite_f(s2);        // a NaN / inf noise power is an invalid drop too
  unsigned int local = 0;
  const uint32_t idesc = tc::idesc_f16_f32(TC_M, TC_N);
  const int npass = v.nwl / TC_WORDS;
  const int qtr = warp & 3;
  const int cl = qtr * 32 + lane;  // this thread's column in the tile (TMEM lane)
  const int c = c0 + cl;
  int issued = 0;                  // mbar_ld phases armed by thread 0
  for (int p = 0; p < npass; ++p) {
    if (p > 0) __syncthreads();  // every thread is done with the previous pass's bits and samples
    if (tid == 0) {
      uint32_t bytes = 2 * opbytes + (p == 0 ? 2 * opbytes : 0);
      if (bulk_y)
        for (int s = 0; s < TC_WORDS; ++s) bytes += v.wlist[p * TC_WORDS + s] >= 0 ? 4 * rowbytes : 0;
      tc::mbar_arrive_expect_tx(&mbar_ld, bytes);
      if (p == 0) tc::bulk_g2s(a_hi, v.ftab + (size_t)mt * 2 * TC_M * KP, 2 * opbytes, &mbar_ld);
      tc::bulk_g2s(b_hi, bop + (size_t)p * 2 * opbytes, 2 * opbytes, &mbar_ld);
      if (bulk_y) {
        for (int s = 0; s < TC_WORDS; ++s) {
          const int w = v.wlist[p * TC_WORDS + s];
          if (w < 0) continue;
          for (int r = 0; r < 4; ++r)
            tc::bulk_g2s(ys + (s * 4 + r) * TC_M, grid + (((int64_t)b * 4 + r) * W + w) * gcols + c0, rowbytes,
                         &mbar_ld);
        }
      }
      ++issued;
    }
    // this thread's two word slots: word, data element index (-1: none), first
    // element of the word in the tile, loaded ahead of the bits and the waits
    int wsl[2], ksl[2], kfsl[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const int w = v.wlist[p * TC_WORDS + (warp >> 2) + 2 * j];
      ksl[j] = (w >= 0 && c < v.FC) ? v.etab[w * v.FC + c] : -1;
      kfsl[j] = w >= 0 ? v.kfirst[w * v.mtiles + mt] : 0;
      wsl[j] = w;
    }
    // ---- Philox bits of the elements of the pass's rows in this tile
    for (int it = tid; it < TC_WORDS * 4 * TC_BITBLK; it += TC_THREADS) {
      const int s = it / (4 * TC_BITBLK), r = it - s * 4 * TC_BITBLK;
      const int t = r / TC_BITBLK, j = r - t * TC_BITBLK;
      const int w = v.wlist[p * TC_WORDS + s];
      const int kf = w >= 0 ? v.kfirst[w * v.mtiles + mt] : -1;
      uint4 blk = make_uint4(0u, 0u, 0u, 0u);
      if (kf >= 0) {
        const int64_t blk0 = ((int64_t)kf * m) >> 7;
        blk = hpx_random_block(seed, drop0 + b, (uint32_t)t, HPX_DOMAIN_BITS, (uint32_t)(blk0 + j));
      }
      *reinterpret_cast<uint4*>(bits + (size_t)(s * 4 + t) * TC_BITBLK * 4 + j * 4) = blk;
    }
    tc::fence_before_sync();
    __syncthreads();  // bits written; previous pass's TMEM reads done
    tc::fence_after_sync();
    const bool landed = tc::mbar_wait(&mbar_ld, (uint32_t)(p & 1), TC_WAIT);  // operands and samples in place
    ok = ok && landed;
    if (tid == 0) {
      if (landed) {
        for (int ks = 0; ks < KP / 16; ++ks) {
          const uint32_t koff = (uint32_t)ks * 256;  // two core matrices along K
          const uint64_t ah = tc::smem_desc(a_hi + koff, 128, KP * 16), al = tc::smem_desc(a_lo + koff, 128, KP * 16);
          const uint64_t bh = tc::smem_desc(b_hi + koff, 128, KP * 16), bl = tc::smem_desc(b_lo + koff, 128, KP * 16);
          tc::mma_f16(tmem, ah, bh, idesc, ks > 0);
          tc::mma_f16(tmem, ah, bl, idesc, true);
          tc::mma_f16(tmem, al, bh, idesc, true);
        }
      }
      tc::mma_commit(&mbar);  // arrives at once if nothing was issued
    }
    ok = ok && tc::mbar_wait(&mbar, (uint32_t)(p & 1), TC_WAIT);
    tc::fence_after_sync();
    // ---- epilogue: thread = subcarrier (TMEM lane), two word slots per warp
#pragma unroll 1
    for (int s = warp >> 2; s < TC_WORDS; s += 2) {
      const bool second = s >= 2;
      const int w = second ? wsl[1] : wsl[0];
      const int k = ok ? (second ? ksl[1] : ksl[0]) : -1;  // data element index, -1: not a data element
      float2 y[4];
#pragma unroll
      for (int r = 0; r < 4; ++r)
        y[r] = k < 0 ? make_float2(0.f, 0.f)
                     : (bulk_y ? ys[(s * 4 + r) * TC_M + cl] : grid[(((int64_t)b * 4 + r) * W + w) * gcols + c]);
      float acc[32];
      tc::tmem_ld32(tmem + ((uint32_t)(qtr * 32) << 16) + (uint32_t)(s * 32), acc);
      if (k < 0) continue;
      float2 A[4][4], x[4];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int t = 0; t < 4; ++t) A[r][t] = make_float2(acc[r * 4 + t], acc[16 + r * 4 + t]);
      fin &= equalize_one<4, 4>(mode, A, y, s2a, x);
      const int kf = second ? kfsl[1] : kfsl[0];
      const int64_t pos = (int64_t)k * m - ((((int64_t)kf * m) >> 7) << 7);
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        const uint32_t rx_v = qam_decide_t<ORDER>(qt, make_float2(x[t].x * inv_scl, x[t].y * inv_scl));
        const uint32_t tx_v = extract_bits_msb(bits + (size_t)(s * 4 + t) * TC_BITBLK * 4, pos, m);
        local += __popc(rx_v ^ tx_v);
      }
    }
    tc::fence_before_sync();
  }
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, TC_N);
  // copies of a pass whose wait gave up may still be landing: let them land (bounded)
  if (tid == 0 && !ok)
    for (int p = 0; p < issued; ++p) tc::mbar_wait(&mbar_ld, (uint32_t)(p & 1), TC_WAIT);
  // block error count
  for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
  __shared__ unsigned int wsum[TC_THREADS / 32];
  if (lane == 0) wsum[warp] = local;
  const int okall = __syncthreads_and(ok);
  const int any_bad = __syncthreads_or(!fin);
  if (tid == 0) {
    unsigned int tot = 0;
    for (int i = 0; i < TC_THREADS / 32; ++i) tot += wsum[i];
    if (!okall) {  // the tensor core or a bulk copy never signalled completion
      atomicOr(errors + b, HPX_DROP_TIMEOUT);
      atomicExch(fail, 1);
    } else {
      if (tot) atomicAdd(errors + b, tot);
      if (any_bad) atomicOr(errors + b, HPX_DROP_NUMERIC);
    }
  }
}

void upload_raw(void** dst, const void* src, size_t bytes, cudaError_t* err) {
  if (*err != cudaSuccess) return;
  *err = cudaMalloc(dst, bytes);
  if (*err == cudaSuccess && src) *err = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
}

}  // namespace

// Host tables of the tensor-core receiver (called by hpx_lmmse_create for 4 x 4).
hpx_status lmmse_tc_prepare(hpx_lmmse* e, const std::vector<int>& delays, const std::vector<float2>& G,
                            const std::vector<int32_t>& pw_count, const std::vector<int32_t>& pw_off,
                            const std::vector<int32_t>& pcol) {
  const hpx_frame* fr = e->frame;
  const int N = e->N, W = e->W, FC = fr->info.num_columns, U = e->U;
  const int KP = ((2 * U + 15) / 16) * 16;
  const int mtiles = (e->C + TC_M - 1) / TC_M;
  // twiddle operand per tile: row c (subcarrier), k < U: Re F, U <= k < 2U: Im F
  std::vector<float2> tw(N);
  for (int t = 0; t < N; ++t) {
    const double a = -2.0 * M_PI * (double)t / (double)N;
    tw[t] = make_float2((float)std::cos(a), (float)std::sin(a));
  }
  std::vector<uint16_t> ftab((size_t)mtiles * 2 * TC_M * KP, 0);
  for (int mt = 0; mt < mtiles; ++mt)
    for (int r = 0; r < TC_M; ++r) {
      const int c = mt * TC_M + r;
      if (c >= e->C) continue;
      for (int k = 0; k < 2 * U; ++k) {
        const int u = k < U ? k : k - U;
        const float2 f = tw[((int64_t)fr->h_bins[c] * delays[u]) & (N - 1)];
        const float val = k < U ? f.x : f.y;
        const __half hi = __float2half_rn(val);
        const __half lo = __float2half_rn(val - __half2float(hi));
        const size_t base = ((size_t)mt * 2) * TC_M * KP;
        const uint32_t off = tc::kmajor_offset(r, k, KP) / 2;
        ftab[base + off] = static_cast<__half_raw>(hi).x;
        ftab[base + (size_t)TC_M * KP + off] = static_cast<__half_raw>(lo).x;
      }
    }
  // words holding data, padded to whole passes
  std::vector<int32_t> wl;
  for (int w = 0; w < W; ++w) {
    bool any = false;
    for (int c = 0; c < FC && !any; ++c) any = fr->h_kind[(size_t)w * FC + c] == HPX_RE_DATA;
    if (any) wl.push_back(w);
  }
  while (wl.empty() || wl.size() % TC_WORDS) wl.push_back(-1);
  std::vector<int32_t> etab((size_t)W * FC, -1);
  for (size_t i = 0; i < etab.size(); ++i)
    if (fr->h_kind[i] == HPX_RE_DATA) etab[i] = fr->h_index[i];
  std::vector<int32_t> kfirst((size_t)W * mtiles, -1);
  for (int w = 0; w < W; ++w)
    for (int c = 0; c < FC; ++c)
      if (fr->h_kind[(size_t)w * FC + c] == HPX_RE_DATA) {
        int32_t& kf = kfirst[(size_t)w * mtiles + c / TC_M];
        if (kf < 0) kf = fr->h_index[(size_t)w * FC + c];
      }
  // weighted-LS rows transposed to [pilot][tap] for the batched LS, (gr, gr, gi, gi),
  // taps padded with zeros to 8 per thread
  e->tc_ls_tu = U <= 24 ? 3 : 8;
  const int up = 8 * e->tc_ls_tu;
  std::vector<float4> gt(G.size() / U * up, make_float4(0.f, 0.f, 0.f, 0.f));
  for (int q = 0; q < e->ntx * kMaxPilotWords; ++q) {
    const int cnt = pw_count[q];
    const size_t off = (size_t)pw_off[q];  // pilot word q's rows: G[off U ..], [U][cnt]
    e->tc_cnt_max = std::max(e->tc_cnt_max, cnt);
    for (int u = 0; u < U; ++u)
      for (int k = 0; k < cnt; ++k) {
        const float2 g = G[off * U + (size_t)u * cnt + k];
        gt[(off + k) * up + u] = make_float4(g.x, g.x, g.y, g.y);
      }
  }
  // column chunks of each pilot word for the batched LS: span, and per chunk and stream
  // the range of the stream's pilots (columns increase with the pilot index)
  std::vector<int32_t> cspan(2 * e->np);
  for (int p = 0; p < e->np; ++p) {
    int lo = 1 << 30, hi = -1;
    for (int t = 0; t < e->ntx; ++t) {
      const int q = t * kMaxPilotWords + p;
      for (int k = 0; k < pw_count[q]; ++k) {
        lo = std::min(lo, pcol[pw_off[q] + k]);
        hi = std::max(hi, pcol[pw_off[q] + k]);
      }
    }
    cspan[2 * p] = lo;
    cspan[2 * p + 1] = hi - lo + 1;
    e->tc_ls_nch_max = std::max(e->tc_ls_nch_max, (hi - lo + LS_CC) / LS_CC);
  }
  std::vector<int2> krange((size_t)e->np * e->tc_ls_nch_max * 4, make_int2(0, 0));
  for (int p = 0; p < e->np; ++p)
    for (int t = 0; t < e->ntx; ++t) {
      const int q = t * kMaxPilotWords + p;
      for (int k = 0; k < pw_count[q]; ++k) {
        const int c = (pcol[pw_off[q] + k] - cspan[2 * p]) / LS_CC;
        int2& r = krange[((size_t)p * e->tc_ls_nch_max + c) * 4 + t];
        if (r.y == r.x) r.x = r.y = k;  // first pilot of the chunk
        r.y = k + 1;
      }
    }
  for (const int2& r : krange) e->tc_ls_kcm = std::max(e->tc_ls_kcm, r.y - r.x);
  e->tc_ls_stages = 0;
  for (const int st : {6, 3, 2})  // deepest pipeline that fits
    if (!e->tc_ls_stages &&
        lmmse_ls_smem(e->tc_ls_tu, st, e->tc_ls_kcm, e->tc_cnt_max, e->tc_ls_nch_max) <= 220 * 1024)
      e->tc_ls_stages = st;
  e->tc_KP = KP;
  e->tc_mtiles = mtiles;
  e->tc_nwl = (int)wl.size();
  e->tc_ws_drops = kLmmseTcChunk;
  cudaError_t err = cudaSuccess;
  upload_raw(reinterpret_cast<void**>(&e->d_tc_ftab), ftab.data(), ftab.size() * 2, &err);
  upload_raw(reinterpret_cast<void**>(&e->d_tc_wlist), wl.data(), wl.size() * 4, &err);
  upload_raw(reinterpret_cast<void**>(&e->d_tc_kfirst), kfirst.data(), kfirst.size() * 4, &err);
  upload_raw(reinterpret_cast<void**>(&e->d_tc_etab), etab.data(), etab.size() * 4, &err);
  upload_raw(reinterpret_cast<void**>(&e->d_tc_bop), nullptr,
             (size_t)kLmmseTcChunk * (wl.size() / TC_WORDS) * 2 * TC_M * KP * 2, &err);
  upload_raw(reinterpret_cast<void**>(&e->d_tc_scale), nullptr, (size_t)kLmmseTcChunk * 4, &err);
  upload_raw(reinterpret_cast<void**>(&e->d_tc_fail), nullptr, sizeof(int), &err);
  upload_raw(reinterpret_cast<void**>(&e->d_tc_gt), gt.data(), gt.size() * sizeof(float4), &err);
  upload_raw(reinterpret_cast<void**>(&e->d_tc_ls_cspan), cspan.data(), cspan.size() * 4, &err);
  upload_raw(reinterpret_cast<void**>(&e->d_tc_ls_krange), krange.data(), krange.size() * sizeof(int2), &err);
  upload_raw(reinterpret_cast<void**>(&e->d_tc_gls), nullptr,
             (size_t)kLmmseTcChunk * TC_NP * e->np * U * sizeof(float2), &err);
  if (err == cudaSuccess) err = cudaMemset(e->d_tc_fail, 0, sizeof(int));
  if (err != cudaSuccess) return hpx_cuda_status(err, "lmmse tensor-core tables");
  return HPX_OK;
}

void lmmse_tc_release(hpx_lmmse* e) {
  void* p[] = {e->d_tc_ftab, e->d_tc_wlist, e->d_tc_kfirst, e->d_tc_bop,  e->d_tc_scale,
               e->d_tc_fail, e->d_tc_etab,  e->d_tc_gt,     e->d_tc_gls,
               e->d_tc_ls_cspan, e->d_tc_ls_krange};
  for (void* q : p)
    if (q) cudaFree(q);
}

// At least 48 KB, so that at most four CTAs (4 x 128 TMEM columns) share an SM.
size_t lmmse_tc_smem(const hpx_lmmse* e) {
  // operands (twiddles, gains: hi and lo), received samples of a pass, staged bits
  return (size_t)4 * TC_M * e->tc_KP * 2 + (size_t)TC_WORDS * 4 * TC_M * sizeof(float2) +
         (size_t)TC_WORDS * 4 * TC_BITBLK * 16 + 128;
}

// The 4 x 4 receiver over B drops in chunks of the workspace size.
hpx_status lmmse_tc_detect(const hpx_lmmse* e, int mode, const float2* grid, int gcols, const float* nv,
                           uint64_t seed, int64_t drop0, int B, uint32_t* errors, cudaStream_t s) {
  const hpx_frame* fr = e->frame;
  QamDemapTable qt;
  HPX_TRY(qam_demap_table(fr->info.modulation_order, &qt));
  const size_t smem_g = ((size_t)e->tc_nwl * (e->tc_KP - e->U) * 32 + (size_t)e->ntx * e->U * e->W * e->np) * 4;
  const size_t smem_t = lmmse_tc_smem(e);
  if (smem_g > 220 * 1024 || smem_t > 220 * 1024)
    return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_lmmse: frame needs too much shared memory");
  if (!e->tc_ls_stages)  // the caller routes such layouts to the FP32 receiver
    return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_lmmse: pilot layout needs too much shared memory");
  const int ls_st = e->tc_ls_stages, ls_tu = e->tc_ls_tu;
  const size_t smem_ls = lmmse_ls_smem(ls_tu, ls_st, e->tc_ls_kcm, e->tc_cnt_max, e->tc_ls_nch_max);
  auto* kls = ls_tu == 3 ? (ls_st == 6 ? k_lmmse_ls<3, 6> : ls_st == 3 ? k_lmmse_ls<3, 3> : k_lmmse_ls<3, 2>)
                         : (ls_st == 6 ? k_lmmse_ls<8, 6> : ls_st == 3 ? k_lmmse_ls<8, 3> : k_lmmse_ls<8, 2>);
  const int ls_drops = ls_tu == 3 ? LsShape<3>::DROPS : LsShape<8>::DROPS;
  const int ls_threads = ls_tu == 3 ? LsShape<3>::THREADS : LsShape<8>::THREADS;
  const LsView lsv{e->d_tc_ls_cspan, e->d_tc_ls_krange, e->tc_ls_nch_max, e->tc_ls_kcm, e->tc_cnt_max};
  HPX_CUDA(cudaFuncSetAttribute(kls, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_ls));
  HPX_CUDA(cudaFuncSetAttribute(k_lmmse_gains, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_g));
  // gains CTAs of 256 threads where four fit an SM (their phases keep few threads busy,
  // so more CTAs overlap better), else 512 (e.g. 64 design taps: one CTA per SM)
  const int gthreads = smem_g <= 56 * 1024 ? 256 : 512;
  const int order = fr->info.modulation_order;
  auto* ktc = order == 2 ? k_lmmse_tc<2> : order == 4 ? k_lmmse_tc<4> : order == 16 ? k_lmmse_tc<16>
            : order == 64 ? k_lmmse_tc<64> : k_lmmse_tc<256>;  // qam_demap_table accepted the order
  HPX_CUDA(cudaFuncSetAttribute(ktc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_t));
  const LmmseView lv = lmmse_view(e);
  TcView tv{e->W, fr->info.num_columns, e->U, e->tc_KP, e->tc_mtiles, e->tc_nwl, fr->info.bits_per_symbol,
            e->d_tc_wlist, e->d_tc_kfirst, e->d_tc_etab, e->d_tc_ftab, e->d_tc_bop, e->d_tc_scale};
  // received rows by bulk copy: 16-byte aligned rows and an even number of columns per tile
  const int bulk_y = (gcols % 2 == 0) && (fr->info.num_columns % 2 == 0) &&
                     (reinterpret_cast<uintptr_t>(grid) % 16 == 0);
  const int64_t per_drop = (int64_t)4 * e->W * gcols;  // grid samples per drop
  for (int d = 0; d < B; d += e->tc_ws_drops) {
    const int nb = std::min(e->tc_ws_drops, B - d);
    const float2* g = grid + (int64_t)d * per_drop;
    const float* n = nv ? nv + d : nullptr;
    kls<<<dim3(e->np, (nb + ls_drops - 1) / ls_drops), ls_threads, smem_ls, s>>>(lv, lsv, e->d_tc_gt, g, gcols, nb,
                                                                                 e->d_tc_gls);
    HPX_LAUNCHED("lmmse_ls");
    k_lmmse_gains<<<nb, gthreads, smem_g, s>>>(lv, n, e->d_tc_wlist, e->tc_nwl, e->tc_KP, e->d_tc_bop,
                                          e->d_tc_scale, e->d_tc_gls);
    HPX_LAUNCHED("lmmse_gains");
    ktc<<<dim3(e->tc_mtiles, nb), TC_THREADS, smem_t, s>>>(tv, e->W, g, gcols, bulk_y, n, qt, mode, seed,
                                                                  drop0 + d, errors + d, e->d_tc_fail);
    HPX_LAUNCHED("lmmse_tc");
  }
  return HPX_OK;
}
