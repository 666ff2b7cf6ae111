// Internal definitions shared by the engine's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdarg>
#include <cstdio>
#include <vector>

#include "../../include/hpx.h"

// ------------------------------------------------------------------ errors

hpx_status hpx_fail(hpx_status code, const char* fmt, ...);
hpx_status hpx_cuda_status(cudaError_t err, const char* what);
// True if an LS table was built for a grid of this frame's layout (detect.cu).
bool hpx_ls_matches_frame(const hpx_ls* ls, const hpx_frame* frame);

#define HPX_TRY(expr)                      \
  do {                                     \
    hpx_status _s = (expr);                \
    if (_s != HPX_OK) return _s;           \
  } while (0)

#define HPX_CUDA(expr)                                         \
  do {                                                         \
    cudaError_t _e = (expr);                                   \
    if (_e != cudaSuccess) return hpx_cuda_status(_e, #expr);  \
  } while (0)

// Check the launch of the kernel enqueued just before.
#define HPX_LAUNCHED(name) HPX_CUDA(cudaPeekAtLastError())

static inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// -------------------------------------------------------------- complex math

__host__ __device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cmulc(float2 a, float2 b) {  // conj(a) * b
  return make_float2(a.x * b.x + a.y * b.y, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// acc += a * b
__device__ __forceinline__ void cfma(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(-a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(a.y, b.x, acc.y);
}
// acc += conj(a) * b
__device__ __forceinline__ void cfmac(float2& acc, float2 a, float2 b) {
  acc.x = fmaf(a.x, b.x, acc.x);
  acc.x = fmaf(a.y, b.y, acc.x);
  acc.y = fmaf(a.x, b.y, acc.y);
  acc.y = fmaf(-a.y, b.x, acc.y);
}

// ------------------------------------------------------------- Philox4x32-10
// Salmon et al., "Parallel random numbers: as easy as 1, 2, 3" (SC'11).

// Each round's products are formed as one 32 x 32 -> 64-bit multiply (a single wide
// multiply-add on the GPU gives both halves).
__host__ __device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
  for (int i = 0; i < 10; ++i) {
    const uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
    const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

// Random-stream layout: c0 = block, c1 = stream id, c2 = drop (low 32 bits),
// c3 = domain | drop bits 32..55 << 8; key = 64-bit campaign seed.
enum { HPX_DOMAIN_BITS = 1, HPX_DOMAIN_FADING = 2, HPX_DOMAIN_NOISE = 3 };

__host__ __device__ __forceinline__ uint4 hpx_random_block(uint64_t seed, int64_t drop, uint32_t stream_id,
                                                           uint32_t domain, uint32_t block) {
  const uint64_t d = (uint64_t)drop;
  uint4 c = make_uint4(block, stream_id, (uint32_t)(d & 0xFFFFFFFFu),
                       (domain & 0xFFu) | ((uint32_t)((d >> 32) & 0xFFFFFFu) << 8));
  return philox4x32_10(c, make_uint2((uint32_t)(seed & 0xFFFFFFFFu), (uint32_t)(seed >> 32)));
}

// Round keys of one seed (k0 + r W0, k1 + r W1 for the ten rounds), computed on the
// host and passed by value, so that a kernel drawing many blocks with one seed reads
// them as constant operands instead of re-deriving the key schedule in every block.
struct PhiloxKeys {
  uint32_t k[20];
};

static inline PhiloxKeys philox_keys(uint64_t seed) {
  PhiloxKeys r;
  uint32_t k0 = (uint32_t)(seed & 0xFFFFFFFFu), k1 = (uint32_t)(seed >> 32);
  for (int i = 0; i < 10; ++i) {
    r.k[2 * i] = k0;
    r.k[2 * i + 1] = k1;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  return r;
}

// hpx_random_block with the seed's round keys (same values).
__device__ __forceinline__ uint4 hpx_random_block_k(const PhiloxKeys& rk, int64_t drop, uint32_t stream_id,
                                                   uint32_t domain, uint32_t block) {
  const uint64_t d = (uint64_t)drop;
  uint4 c = make_uint4(block, stream_id, (uint32_t)(d & 0xFFFFFFFFu),
                       (domain & 0xFFu) | ((uint32_t)((d >> 32) & 0xFFFFFFu) << 8));
#pragma unroll
  for (int i = 0; i < 10; ++i) {  // (separate high and low products measured faster here than one wide product)
    const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), hi1 = __umulhi(0xCD9E8D57u, c.z);
    const uint32_t lo0 = 0xD2511F53u * c.x, lo1 = 0xCD9E8D57u * c.z;
    c = make_uint4(hi1 ^ c.y ^ rk.k[2 * i], lo1, hi0 ^ c.w ^ rk.k[2 * i + 1], lo0);
  }
  return c;
}

__host__ __device__ __forceinline__ uint32_t uint4_get(const uint4& v, int i) {
  return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// Uniform on (0, 1) from one 32-bit word: (w + 0.5) * 2^-32.
__host__ __device__ __forceinline__ double u01_f64(uint32_t w) { return ((double)w + 0.5) * 2.3283064365386963e-10; }
__device__ __forceinline__ float u01_f32(uint32_t w) { return ((float)(w >> 8) + 0.5f) * 5.9604644775390625e-08f; }

// Box-Muller pair of unit normals from two words: r (cos 2 pi u2, sin 2 pi u2),
// evaluated as -r (cos a, sin a) with a = 2 pi (u2 - 1/2) in (-pi, pi), where the
// fast hardware sine and cosine are accurate to a few 1e-7.
// The radius uses the hardware logarithm and reciprocal square root (a few 1e-7
// relative, about 1e-6 RMS over the normal distribution).
__device__ __forceinline__ float2 box_muller(uint32_t a, uint32_t b) {
  const float u1 = u01_f32(a);
  const float u2 = u01_f32(b);
  const float x = -2.0f * __logf(u1);
  const float r = x * rsqrtf(fmaxf(x, 1e-30f));
  float s, c;
  __sincosf(6.283185307179586f * (u2 - 0.5f), &s, &c);
  return make_float2(-r * c, -r * s);
}

// ------------------------------------------------------ fixed-point phases
// A phase in turns is held as a 64-bit two's-complement fraction of a turn, so
// that phase(t) = P0 + W * t wraps exactly modulo one turn for any sample index.

__host__ __device__ __forceinline__ int64_t turns_to_fixed(double turns) {
  const double frac = turns - floor(turns);  // [0, 1)
  // 2^64 * frac, computed as two 32-bit halves to stay exact in double
  const double hi = floor(frac * 4294967296.0);
  const double lo = floor((frac * 4294967296.0 - hi) * 4294967296.0);
  return (int64_t)(((uint64_t)hi << 32) | (uint64_t)lo);
}

// Fixed-point initial phase u - 1/2 of a sinusoid whose uniform is u = (w + 1/2) 2^-32
// (u01_f64 of the drawn word w): 2^64 (u - 1/2) mod 2^64 = w 2^32 + 2^31 - 2^63,
// exactly turns_to_fixed of the FP64 value, without FP64 arithmetic.
__host__ __device__ __forceinline__ int64_t phase_from_word(uint32_t w) {
  return (int64_t)((((uint64_t)w) << 32) + 0x80000000ull + 0x8000000000000000ull);
}

// Fixed-point rate of a turns-per-sample value held in FP32 (|turns| < 1/2): the
// float's exact multiple of 2^-64. With the FP32 cosine behind it the rate is off by
// about 2^-23 |turns|, so the phase of sample t by 2^-23 |turns| t: the realization uses
// FP32 rates only while the largest rate is at most kFp32RateLimit turns per sample,
// which keeps that error under 1.2e-7 turns (7.5e-7 relative in the taps) for frames of
// up to 65 536 samples; faster channels take the FP64 path.
constexpr double kFp32RateLimit = 1.0 / 65536.0;
__device__ __forceinline__ int64_t rate_to_fixed(float turns) { return __float2ll_rn(turns * 18446744073709551616.0f); }

// Angle in radians in [-pi, pi) of a fixed-point phase.
__device__ __forceinline__ float fixed_to_angle(uint64_t p) {
  return (float)(int32_t)(uint32_t)(p >> 32) * 1.4629180792671596e-09f;  // 2*pi / 2^32
}

// ------------------------------------------------------------- frame tables

struct hpx_frame {
  hpx_frame_info info;
  int dc_suppression;
  int pilot_comb;  // 0/1: all streams send every reference element; P > 1: stream s only on columns c % P == s % P
  // host copies
  std::vector<int32_t> h_prefix, h_zero_prefix, h_word_start, h_window_start;
  std::vector<int32_t> h_data_offset, h_ref_offset;  // first data / ref index of each word
  std::vector<int8_t> h_kind;                        // [W * C]
  std::vector<int32_t> h_index;                      // [W * C] data or ref index within the frame
  std::vector<int32_t> h_bins;                       // [N] FFT bin of grid column c
  int32_t max_data_word = 0;                         // most data elements in one word
  // device copies
  int32_t* d_prefix = nullptr;
  int32_t* d_zero_prefix = nullptr;
  int32_t* d_word_start = nullptr;
  int32_t* d_window_start = nullptr;
  int32_t* d_data_offset = nullptr;
  int32_t* d_num_data_word = nullptr;  // data elements per word
  int8_t* d_kind = nullptr;
  int32_t* d_index = nullptr;
  int32_t* d_bins = nullptr;
  int32_t* d_data_column = nullptr;    // [num_data] column of data element k (word via search)
  int32_t* d_data_word = nullptr;      // [num_data] word of data element k
  float2* d_twiddle = nullptr;         // [N] exp(-2 pi i t / N)
  float2* d_stage_twiddle = nullptr;   // [2N] per-stage tables of the OFDM FFT (fft.cuh)
  float2* d_pilots = nullptr;          // [num_refs]
  int32_t* d_bin_code = nullptr;       // [W * N] per (word, FFT bin): data index, ~pilot index, or INT32_MIN (null)
  float2* d_constellation = nullptr;   // [M] symbols in MSB-first bit-value order
  // transmitter from Philox bits (k_ofdm_tx): per (word, bin) the bit offset of a data
  // element within the word's staged words, -2 - (reference index * 64 + comb phase) for
  // a reference element, -1 for nothing; per word 1 if its columns are data elements in
  // column order (then the offset is column * m + word bit offset) and that bit offset
  int32_t* d_tx_src = nullptr;         // [W * N]
  int32_t* d_tx_regular = nullptr;     // [W]
  int32_t* d_tx_bitoff = nullptr;      // [W] (first data index * m) mod 128
  float2* d_constellation_lsb = nullptr;  // [M] symbols by LSB-first bit value (bit-reversed index)
};

// ------------------------------------------------------------ fading state

struct hpx_fading {
  int L, S, S1;  // taps, sinusoids, sinusoids + LOS component
  int nrx, ntx;
  double fs, doppler, los_doppler, gain;
  int max_delay;  // D
  int G;          // distinct tap delays (taps sharing one sample delay form a group)
  std::vector<int32_t> h_delay;
  std::vector<float> h_amp_nlos, h_amp_los;  // sqrt(gain g_l) * gain_{nlos,los}
  std::vector<double> h_rx_corr, h_tx_corr;  // complex interleaved, empty if none
  // device copies
  int32_t* d_delay = nullptr;
  int32_t* d_group = nullptr;   // [G + 1] first tap of each delay group, then [G] group delays
  float* d_amp = nullptr;       // [L][2] (nlos, los)
  double* d_rx_corr = nullptr;  // [nrx*nrx*2] or null
  double* d_tx_corr = nullptr;
  // per-drop state layout (bytes)
  size_t off_w, off_p0, off_spatial, stride;
};

// Tap-domain LMMSE channel estimator tables (estimate.cu builds them, the fused
// receiver in detect.cu reads them).
constexpr int kMaxPilotWords = 8;
struct hpx_lmmse {
  const hpx_frame* frame = nullptr;
  int C = 0, ntx = 0, U = 0, P = 0, N = 0, W = 0;
  int np = 0;  // pilot words per stream (the same for every stream)
  int32_t* d_delay = nullptr;     // [U] distinct tap delays (samples)
  int32_t* d_pw_word = nullptr;   // [ntx][P] word of pilot word p (-1: none)
  int32_t* d_pw_count = nullptr;  // [ntx][P] pilots in that word
  int32_t* d_pw_off = nullptr;    // [ntx][P] offset into d_pcol / d_G (in pilots)
  int32_t* d_pcol = nullptr;      // [total pilots] grid column
  float2* d_G = nullptr;          // per pilot word [U][count] weighted-LS rows
  float* d_E = nullptr;           // [ntx][P][U] diag((A^H A)^-1)
  float* d_R = nullptr;           // [U][P][P]
  float* d_r = nullptr;           // [U][W][P]
  int32_t* d_np = nullptr;        // [ntx] pilot words per stream
  // tensor-core receiver of the 4 x 4 link (lmmse_tc.cu)
  int tc_KP = 0, tc_mtiles = 0, tc_nwl = 0, tc_ws_drops = 0;
  uint16_t* d_tc_ftab = nullptr;   // [mtiles][2][128 x KP] FP16 twiddle operand (hi, lo)
  int32_t* d_tc_wlist = nullptr;   // [nwl] data words, -1 padding
  int32_t* d_tc_kfirst = nullptr;  // [W][mtiles] first data element of row w in the tile
  uint16_t* d_tc_bop = nullptr;    // [tc_ws_drops][passes][2][128 x KP] FP16 gains operand
  float* d_tc_scale = nullptr;     // [tc_ws_drops]
  int* d_tc_fail = nullptr;        // set if a tensor-core wait timed out (later CTAs skip)
  int32_t* d_tc_etab = nullptr;    // [W][FC] data element index, -1 for other elements
  int tc_cnt_max = 0;              // most pilots of one stream in one word
  int tc_ls_tu = 0;                // taps per thread of the batched pilot LS (rows padded to 8 of them)
  int tc_ls_stages = 0;            // its cp.async pipeline depth (0: the frame does not fit)
  int tc_ls_nch_max = 0, tc_ls_kcm = 0;  // column chunks per pilot word, most pilots of a stream in one
  int32_t* d_tc_ls_cspan = nullptr;      // [np][2] first pilot column of the word, columns spanned
  int2* d_tc_ls_krange = nullptr;        // [np][nch_max][4] pilots of stream t in chunk c: [kb, ke)
  float4* d_tc_gt = nullptr;       // [total pilots][8 tc_ls_tu] weighted-LS rows transposed, (gr, gr, gi, gi)
  float2* d_tc_gls = nullptr;      // [tc_ws_drops][16 pairs][np][U] pilot LS gains
};
constexpr int kLmmseTcChunk = 8192;  // drops per gains/GEMM launch pair (workspace 72 KB per drop)
hpx_status lmmse_tc_prepare(hpx_lmmse* e, const std::vector<int>& delays, const std::vector<float2>& G,
                            const std::vector<int32_t>& pw_count, const std::vector<int32_t>& pw_off,
                            const std::vector<int32_t>& pcol);
void lmmse_tc_release(hpx_lmmse* e);
hpx_status lmmse_tc_detect(const hpx_lmmse* e, int mode, const float2* grid, int gcols, const float* nv,
                           uint64_t seed, int64_t drop0, int B, uint32_t* errors, cudaStream_t s);

// Per-drop realization state, read by the kernels.
struct FadingView {
  const unsigned char* base;
  size_t stride, off_w, off_p0, off_spatial;
  int L, S1, nrx, ntx;
  __device__ __forceinline__ const int64_t* W(int b) const {
    return reinterpret_cast<const int64_t*>(base + b * stride + off_w);
  }
  __device__ __forceinline__ const int64_t* P0(int b) const {
    return reinterpret_cast<const int64_t*>(base + b * stride + off_p0);
  }
  __device__ __forceinline__ const float2* spatial(int b) const {
    return reinterpret_cast<const float2*>(base + b * stride + off_spatial);
  }
};

static inline FadingView fading_view(const hpx_fading* f, const void* state) {
  FadingView v;
  v.base = static_cast<const unsigned char*>(state);
  v.stride = f->stride;
  v.off_w = f->off_w;
  v.off_p0 = f->off_p0;
  v.off_spatial = f->off_spatial;
  v.L = f->L;
  v.S1 = f->S1;
  v.nrx = f->nrx;
  v.ntx = f->ntx;
  return v;
}

// QAM tables (mapping.cu)
hpx_status qam_bits_per_symbol(int32_t order, int* bits);
// Exact hard decisions of PskQamMapping.detect_bits on float32 amplitudes. The
// reference's scaled amplitude r(x) = (x sqrt 2) sqrt c is odd and monotone, so per
// real dimension the first bit is the sign and every further bit is 1 exactly when
// |x| lies in one of up to three open intervals (lo, hi) of float32 cut points
// (lo = -1 encodes an interval closed at 0).
struct QamDemapTable {
  int order, bits, pam_bits;  // pam_bits: bits per real dimension
  float lo[4][3], hi[4][3];   // PAM bits 1..pam_bits-1 over |x|
  int count[4];
};
hpx_status qam_demap_table(int32_t order, QamDemapTable* table);

// PAM level (3GPP Gray) of `nb` bits MSB-first packed in `v` (bit nb-1 is the first bit).
__host__ __device__ __forceinline__ float pam_level(int nb, uint32_t v) {
  // Unnormalized amplitudes of generate_pam_symbol_3gpp (psk_qam_mapping.py:261-298)
  float b0 = (float)((v >> (nb - 1)) & 1u);
  if (nb == 1) return 1.0f - 2.0f * b0;
  float b1 = (float)((v >> (nb - 2)) & 1u);
  if (nb == 2) return (1.0f - 2.0f * b0) * (1.0f + 2.0f * b1);
  float b2 = (float)((v >> (nb - 3)) & 1u);
  if (nb == 3) return (2.0f * b0 - 1.0f) * ((1.0f - 2.0f * b1) * (1.0f + 2.0f * b2) - 4.0f);
  float b3 = (float)((v >> (nb - 4)) & 1u);
  return ((((1.0f - 2.0f * b2) * (1.0f + 2.0f * b3) - 4.0f) * (-1.0f + 2.0f * b1)) - 8.0f) * (-1.0f + 2.0f * b0);
}

// Symbol of an M-ary constellation from its MSB-first bit value (0..M-1).
__host__ __device__ __forceinline__ float2 qam_symbol(int order, uint32_t v) {
  switch (order) {
    case 2: return make_float2(pam_level(1, v), 0.0f);
    case 4: {
      const float s = 0.70710678118654752f;
      return make_float2(pam_level(1, v >> 1) * s, pam_level(1, v & 1u) * s);
    }
    default: {
      // bits b0 b1 b2 ... : real gets b0 b2 b4.., imag gets b1 b3 b5..
      const int m = order == 16 ? 4 : (order == 64 ? 6 : 8);
      const int h = m / 2;
      uint32_t re = 0, im = 0;
      for (int i = 0; i < h; ++i) {
        re = (re << 1) | ((v >> (m - 1 - 2 * i)) & 1u);
        im = (im << 1) | ((v >> (m - 2 - 2 * i)) & 1u);
      }
      const float s = order == 16 ? 0.31622776601683794f : (order == 64 ? 0.15430334996209191f : 0.07669649888473704f);
      return make_float2(pam_level(h, re) * s, pam_level(h, im) * s);
    }
  }
}

// Hard decisions of one symbol with a demap table; returns MSB-first bit value.
// BPSK and QPSK LLRs are plain linear functions of the amplitude (no masked
// pieces), so -inf decides 1 there, while the masked piecewise LLRs of the larger
// constellations turn any infinity into NaN and decide 0 for every bit.
// Bit i (1 <= i < PB) of a PAM axis is 1 on i open intervals of |x|. Kernels pass
// the table as a __grid_constant__ parameter, so every bound is a constant-bank
// operand of its compare.
// The tables' intervals have a fixed shape (checked where qam_demap_table builds them):
// bit i has i intervals, the first of them open below (lower bound -1, below every |x|)
// for i >= 2 and the last open above (upper bound +inf). So the lower test of such a
// first interval only rejects NaN, which its upper test rejects too, and the upper test
// of a last interval is the sign bit's finiteness test: both are shared, not repeated.
__host__ __device__ constexpr bool pam_interval_open_below(int i, int k) { return k == 0 && i >= 2; }
__host__ __device__ constexpr bool pam_interval_open_above(int i, int k) { return k == i - 1; }

// SHARED: use that shape (fewer compares); otherwise every bound is tested, which the
// register-tight CSI receiver compiles without spills. Both decide the same bits.
template <int PB, bool SHARED = true>
__device__ __forceinline__ uint32_t pam_decide(const QamDemapTable& t, float x) {
  const float ax = fabsf(x);
  const bool fin = ax < INFINITY;
  uint32_t v = ((x < 0.0f) & fin) ? 1u : 0u;  // plain compares, no short circuits
#pragma unroll
  for (int i = 1; i < PB; ++i) {
    bool in = false;
#pragma unroll
    for (int k = 0; k < i; ++k) {
      const bool above = (SHARED && pam_interval_open_below(i, k)) ? true : (ax > t.lo[i][k]);
      const bool below = (SHARED && pam_interval_open_above(i, k)) ? fin : (ax < t.hi[i][k]);
      in |= above & below;
    }
    v = (v << 1) | (in ? 1u : 0u);
  }
  return v;
}

template <int PB, bool SHARED = true>
__device__ __forceinline__ uint32_t qam_decide_pb(const QamDemapTable& t, float2 y) {
  const uint32_t re = pam_decide<PB, SHARED>(t, y.x), im = pam_decide<PB, SHARED>(t, y.y);
  // interleave: b0 = re0, b1 = im0, b2 = re1, ... (MSB first)
  uint32_t v = 0;
#pragma unroll
  for (int i = PB - 1; i >= 0; --i) v = (v << 2) | (((re >> i) & 1u) << 1) | ((im >> i) & 1u);
  return v;
}

// qam_decide for a modulation order known at compile time.
template <int ORDER>
__device__ __forceinline__ uint32_t qam_decide_t(const QamDemapTable& t, float2 y) {
  if constexpr (ORDER == 2) return (y.x < 0.0f) ? 1u : 0u;
  else if constexpr (ORDER == 4) return ((y.x < 0.0f) ? 2u : 0u) | ((y.y < 0.0f) ? 1u : 0u);
  else if constexpr (ORDER == 16) return qam_decide_pb<2>(t, y);
  else if constexpr (ORDER == 64) return qam_decide_pb<3>(t, y);
  else return qam_decide_pb<4>(t, y);
}

template <int ORDER, int NTX>
__device__ __forceinline__ void qam_decide_all(const QamDemapTable& t, const float2 (&x)[NTX], int n,
                                               uint32_t (&v)[NTX]) {
#pragma unroll
  for (int i = 0; i < NTX; ++i) v[i] = i < n ? qam_decide_t<ORDER>(t, x[i]) : 0u;
}

// Hard decisions of the NTX equalized streams of one element, zero for streams at or
// past n: one branch on the order for all of them.
template <int NTX>
__device__ __forceinline__ void qam_decide_n(const QamDemapTable& t, const float2 (&x)[NTX], int n,
                                             uint32_t (&v)[NTX]) {
  switch (t.order) {
    case 2: qam_decide_all<2>(t, x, n, v); break;
    case 4: qam_decide_all<4>(t, x, n, v); break;
    case 16: qam_decide_all<16>(t, x, n, v); break;
    case 64: qam_decide_all<64>(t, x, n, v); break;
    default: qam_decide_all<256>(t, x, n, v); break;
  }
}

__device__ __forceinline__ uint32_t qam_decide(const QamDemapTable& t, float2 y) {
  switch (t.order) {
    case 2: return (y.x < 0.0f) ? 1u : 0u;
    case 4: return ((y.x < 0.0f) ? 2u : 0u) | ((y.y < 0.0f) ? 1u : 0u);
    case 16: return qam_decide_pb<2, false>(t, y);
    case 64: return qam_decide_pb<3, false>(t, y);
    default: return qam_decide_pb<4, false>(t, y);
  }
}

// Words of packed Philox bits staged for the data elements of one OFDM word with
// C columns and m bits per symbol: the covered words, rounding to whole Philox
// blocks of 4 words at both ends, and one spare word for 64-bit windows.
__host__ __device__ inline int staged_bit_words(int C, int m) { return ((C * m) >> 5) + 9; }

// Extract `nb` (<= 8) bits MSB-first starting at stream bit position `pos` from
// packed bit storage (stream bit b = bit b%32 of word b/32): one 64-bit window,
// then a bit reversal puts the first stream bit in the most significant place.
// `words` must hold one readable word past the last one touched.
__device__ __forceinline__ uint32_t extract_bits_msb(const uint32_t* words, int64_t pos, int nb) {
  const int64_t w = pos >> 5;
  const uint64_t win = (uint64_t)words[w] | ((uint64_t)words[w + 1] << 32);
  const uint32_t raw = (uint32_t)(win >> (pos & 31)) & ((1u << nb) - 1u);
  return __brev(raw) >> (32 - nb);
}
