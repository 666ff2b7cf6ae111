// OFDM transmit (bits -> QAM -> place -> IFFT -> prefix) and receive
// (prefix strip -> FFT -> bin gather) kernels with a block-cooperative
// Stockham FFT in shared memory.
#include <climits>

#include "fft.cuh"
#include "hpx_internal.cuh"

namespace {


struct FrameDev {
  int N, W, C, m, order, T, num_data, dc;
  int comb;  // pilot comb (0/1: every stream sends every reference element)
  const int32_t* prefix;
  const int32_t* zero_prefix;
  const int32_t* word_start;
  const int32_t* window_start;
  const int32_t* data_offset;
  const int32_t* num_data_word;
  const int8_t* kind;
  const int32_t* index;
  const int32_t* bins;
  const int32_t* data_column;
  const int32_t* data_word;
  const float2* twiddle;
  const float2* stage_twiddle;
  const float2* pilots;
  const int32_t* bin_code;
  const float2* constellation;
  const int32_t* tx_src;
  const int32_t* tx_regular;
  const int32_t* tx_bitoff;
  const float2* constellation_lsb;
};

FrameDev frame_dev(const hpx_frame* f) {
  FrameDev d;
  d.N = f->info.num_subcarriers;
  d.W = f->info.num_words;
  d.C = f->info.num_columns;
  d.m = f->info.bits_per_symbol;
  d.order = f->info.modulation_order;
  d.T = f->info.samples_per_frame;
  d.num_data = f->info.num_data;
  d.dc = f->dc_suppression;
  d.comb = f->pilot_comb;
  d.prefix = f->d_prefix;
  d.zero_prefix = f->d_zero_prefix;
  d.word_start = f->d_word_start;
  d.window_start = f->d_window_start;
  d.data_offset = f->d_data_offset;
  d.num_data_word = f->d_num_data_word;
  d.kind = f->d_kind;
  d.index = f->d_index;
  d.bins = f->d_bins;
  d.data_column = f->d_data_column;
  d.data_word = f->d_data_word;
  d.twiddle = f->d_twiddle;
  d.stage_twiddle = f->d_stage_twiddle;
  d.pilots = f->d_pilots;
  d.bin_code = f->d_bin_code;
  d.constellation = f->d_constellation;
  d.tx_src = f->d_tx_src;
  d.tx_regular = f->d_tx_regular;
  d.tx_bitoff = f->d_tx_bitoff;
  d.constellation_lsb = f->d_constellation_lsb;
  return d;
}

// Grid column of an FFT bin (inverse of hpx_frame::h_bins; ofdm.py:116-128, 146-151).
__device__ __forceinline__ int column_of_bin(int b, int N, bool dc) {
  if (!dc) return (b + N / 2) & (N - 1);
  if (b >= N / 2) return b - N / 2;
  return b == 0 ? N - 1 : b + N / 2 - 1;
}


template <int N>
constexpr int groups_per_block() {
  return fft::Plan<N>::TP >= 128 ? 1 : 128 / fft::Plan<N>::TP;
}

// MODE 0: data symbols `data` [items][num_data]; MODE 1: Philox bits of drop
// item / num_streams, stream item % num_streams; MODE 2: a placed grid `data`
// [items][W][G] with G = num_streams columns.
// Resident CTAs per SM the FFT kernels are compiled for: the transforms are latency
// bound, so the 128-thread CTAs of N <= 2048 take a 64-register cap (8 CTAs per SM),
// without spills: for 8 192 drops of the 1024-point 4x4 link that measured 2 % (transmit)
// and 5 % (receive) faster than 7 and 6 CTAs; the 256-thread CTAs of N = 4096 keep 85.
template <int N>
constexpr int tx_min_blocks() { return fft::Plan<N>::TP * groups_per_block<N>() >= 256 ? 3 : 8; }
template <int N>
constexpr int rx_min_blocks() { return fft::Plan<N>::TP * groups_per_block<N>() >= 256 ? 3 : 8; }

template <int N, int MODE>
__global__ void __launch_bounds__(fft::Plan<N>::TP * groups_per_block<N>(), tx_min_blocks<N>())
    k_ofdm_tx(FrameDev fr, int num_pairs, const float2* __restrict__ data, uint64_t seed, int64_t drop0,
              int num_streams, float2* __restrict__ out) {
  constexpr int TP = fft::Plan<N>::TP;
  constexpr int F = groups_per_block<N>();
  constexpr int PN = fft::padded<N>();
  extern __shared__ float4 smem4[];
  const int g = threadIdx.x / TP, t = threadIdx.x - g * TP;
  float2* buf = reinterpret_cast<float2*>(smem4) + g * PN;
  const int BW = staged_bit_words(fr.C, fr.m);
  float2* cons = reinterpret_cast<float2*>(smem4) + F * PN;  // [M] constellation (MODE 1)
  uint32_t* bits = reinterpret_cast<uint32_t*>(cons + (MODE == 1 ? fr.order : 0)) + g * BW;
  const int p = blockIdx.x * F + g;
  const bool valid = p < num_pairs;
  const int item = valid ? p / fr.W : 0, w = valid ? p - item * fr.W : 0;
  const bool dc = fr.dc != 0;
  const float scale = rsqrtf((float)N);
  if (MODE == 1 && valid) {
    const int drop = item / num_streams, s = item - drop * num_streams;
    const int64_t k0 = fr.data_offset[w];
    const int nd = fr.num_data_word[w];
    if (nd > 0) {
      const int64_t blk0 = ((k0 * fr.m) >> 5) >> 2, blk1 = (((k0 + nd) * fr.m - 1) >> 5) >> 2;
      for (int64_t blk = blk0 + t; blk <= blk1; blk += TP) {
        const uint4 r = hpx_random_block(seed, drop0 + drop, (uint32_t)s, HPX_DOMAIN_BITS, (uint32_t)blk);
        uint32_t* dst = bits + (blk - blk0) * 4;
        dst[0] = r.x;
        dst[1] = r.y;
        dst[2] = r.z;
        dst[3] = r.w;
      }
    }
  }
  // MODE 1: the constellation by LSB-first bit value, scaled, in shared memory
  if (MODE == 1) {
    for (int i = threadIdx.x; i < fr.order; i += blockDim.x) cons[i] = cscale(fr.constellation_lsb[i], scale);
    __syncthreads();
  }
  const int32_t* codes = fr.bin_code + (int64_t)w * N;
  const int32_t* srcs = fr.tx_src + (int64_t)w * N;
  // stream of this item (MODE 1: items are (drop, stream); MODE 0: stream 0)
  const int stream = MODE == 1 ? item % num_streams : 0;
  const int phase = fr.comb > 1 ? stream % fr.comb : 0;
  const bool regular = MODE == 1 && valid && fr.tx_regular[w] != 0;
  const int bitoff = MODE == 1 && valid ? fr.tx_bitoff[w] : 0;
  const uint32_t mask = (1u << fr.m) - 1u;
  // symbol of the m staged bits at bit offset d (LSB-first window, so no bit reversal)
  auto symbol = [&](int d) -> float2 {
    const int wi = d >> 5;
    return cons[__funnelshift_r(bits[wi], bits[wi + 1], d & 31) & mask];
  };
  auto load = [&](int b) -> float2 {
    if (!valid) return make_float2(0.f, 0.f);
    float2 v = make_float2(0.f, 0.f);
    if (MODE == 2) {
      const int c = column_of_bin(b, N, dc);
      if (c < num_streams) v = data[(int64_t)p * num_streams + c];
      return cscale(v, scale);
    }
    if (MODE == 1) {
      if (regular) {  // every column a data element in column order: no table lookup
        const int c = column_of_bin(b, N, dc);
        return c < fr.C ? symbol(c * fr.m + bitoff) : v;
      }
      const int32_t d = __ldg(srcs + b);
      if (d >= 0) return symbol(d);
      if (d != -1) {
        const int q = -2 - d;  // reference index * 64 + comb phase of its column
        if (fr.comb <= 1 || (q & 63) == phase) v = cscale(fr.pilots[q >> 6], scale);
      }
      return v;
    }
    const int32_t code = __ldg(codes + b);
    if (code >= 0) v = data[(int64_t)item * fr.num_data + code];
    else if (code != INT32_MIN) {
      if (fr.comb <= 1 || column_of_bin(b, N, dc) % fr.comb == stream % fr.comb) v = fr.pilots[~code];
    }
    return cscale(v, scale);
  };
  float2* dst = out + (int64_t)item * fr.T + fr.word_start[w];
  const int P = valid ? fr.prefix[w] : 0;
  const bool zp = valid && fr.zero_prefix[w] != 0;
  auto store = [&](int n, float2 v) {
    if (!valid) return;
    dst[P + n] = v;
    if (n >= N - P) dst[n - (N - P)] = zp ? make_float2(0.f, 0.f) : v;
  };
  fft::transform<N, true>(buf, t, fr.stage_twiddle, load, store);
}

template <int N>
__global__ void __launch_bounds__(fft::Plan<N>::TP * groups_per_block<N>(), rx_min_blocks<N>())
    k_ofdm_rx(FrameDev fr, int num_pairs, const float2* __restrict__ in, int64_t stride, int ncols,
              float2* __restrict__ grid) {
  constexpr int TP = fft::Plan<N>::TP;
  constexpr int F = groups_per_block<N>();
  constexpr int PN = fft::padded<N>();
  extern __shared__ float4 smem4[];
  const int g = threadIdx.x / TP, t = threadIdx.x - g * TP;
  float2* buf = reinterpret_cast<float2*>(smem4) + g * PN;
  const int p = blockIdx.x * F + g;
  const bool valid = p < num_pairs;
  const int item = valid ? p / fr.W : 0, w = valid ? p - item * fr.W : 0;
  const bool dc = fr.dc != 0;
  const float scale = rsqrtf((float)N);
  const float2* src = in + (int64_t)item * stride + fr.window_start[w];
  float2* dst = grid + (int64_t)p * ncols;
  auto load = [&](int n) -> float2 { return valid ? __ldg(src + n) : make_float2(0.f, 0.f); };
  auto store = [&](int b, float2 v) {
    const int c = column_of_bin(b, N, dc);
    if (valid && c < ncols) dst[c] = cscale(v, scale);
  };
  fft::transform<N, false>(buf, t, fr.stage_twiddle, load, store);
}

__global__ void k_ofdm_pick(FrameDev fr, const float2* __restrict__ grid, int gcols, int batch, float2* __restrict__ out) {
  const int64_t total = (int64_t)batch * fr.num_data;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t item = q / fr.num_data;
    const int k = (int)(q - item * fr.num_data);
    out[q] = grid[(item * fr.W + fr.data_word[k]) * gcols + fr.data_column[k]];
  }
}

template <int N, int MODE>
hpx_status launch_tx_n(const FrameDev& d, int pairs, const float2* data, uint64_t seed, int64_t drop0, int ns,
                       float2* out, cudaStream_t s) {
  constexpr int F = groups_per_block<N>();
  constexpr int threads = fft::Plan<N>::TP * F;
  const size_t smem = (size_t)F * (N + N / 16) * sizeof(float2) +
                      (MODE == 1 ? (size_t)d.order * sizeof(float2) + (size_t)F * staged_bit_words(d.C, d.m) * 4 : 0);
  auto kern = k_ofdm_tx<N, MODE>;
  if (smem > 48 * 1024) HPX_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int blocks = (pairs + F - 1) / F;
  kern<<<blocks, threads, smem, s>>>(d, pairs, data, seed, drop0, ns, out);
  HPX_LAUNCHED("ofdm_tx");
  return HPX_OK;
}

template <int MODE>
hpx_status launch_tx(const FrameDev& d, int pairs, const float2* data, uint64_t seed, int64_t drop0, int ns,
                     float2* out, cudaStream_t s) {
  switch (d.N) {
    case 64: return launch_tx_n<64, MODE>(d, pairs, data, seed, drop0, ns, out, s);
    case 128: return launch_tx_n<128, MODE>(d, pairs, data, seed, drop0, ns, out, s);
    case 256: return launch_tx_n<256, MODE>(d, pairs, data, seed, drop0, ns, out, s);
    case 512: return launch_tx_n<512, MODE>(d, pairs, data, seed, drop0, ns, out, s);
    case 1024: return launch_tx_n<1024, MODE>(d, pairs, data, seed, drop0, ns, out, s);
    case 2048: return launch_tx_n<2048, MODE>(d, pairs, data, seed, drop0, ns, out, s);
    case 4096: return launch_tx_n<4096, MODE>(d, pairs, data, seed, drop0, ns, out, s);
    default: return hpx_fail(HPX_ERR_UNSUPPORTED, "FFT size %d not supported", d.N);
  }
}

template <int N>
hpx_status launch_rx_n(const FrameDev& d, int pairs, const float2* in, int64_t stride, int ncols, float2* grid,
                       cudaStream_t s) {
  constexpr int F = groups_per_block<N>();
  constexpr int threads = fft::Plan<N>::TP * F;
  const size_t smem = (size_t)F * (N + N / 16) * sizeof(float2);
  auto kern = k_ofdm_rx<N>;
  if (smem > 48 * 1024) HPX_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int blocks = (pairs + F - 1) / F;
  kern<<<blocks, threads, smem, s>>>(d, pairs, in, stride, ncols, grid);
  HPX_LAUNCHED("ofdm_rx");
  return HPX_OK;
}

hpx_status launch_rx(const FrameDev& d, int pairs, const float2* in, int64_t stride, int ncols, float2* grid,
                     cudaStream_t s) {
  switch (d.N) {
    case 64: return launch_rx_n<64>(d, pairs, in, stride, ncols, grid, s);
    case 128: return launch_rx_n<128>(d, pairs, in, stride, ncols, grid, s);
    case 256: return launch_rx_n<256>(d, pairs, in, stride, ncols, grid, s);
    case 512: return launch_rx_n<512>(d, pairs, in, stride, ncols, grid, s);
    case 1024: return launch_rx_n<1024>(d, pairs, in, stride, ncols, grid, s);
    case 2048: return launch_rx_n<2048>(d, pairs, in, stride, ncols, grid, s);
    case 4096: return launch_rx_n<4096>(d, pairs, in, stride, ncols, grid, s);
    default: return hpx_fail(HPX_ERR_UNSUPPORTED, "FFT size %d not supported", d.N);
  }
}

}  // namespace

extern "C" {

hpx_status hpx_ofdm_modulate(const hpx_frame* frame, const hpx_cf32* data, int32_t batch, hpx_cf32* samples,
                             void* stream) {
  if (!frame) return hpx_fail(HPX_ERR_ARG, "modulate: null frame");
  if (batch < 0) return hpx_fail(HPX_ERR_ARG, "modulate: negative batch");
  if (batch == 0) return HPX_OK;
  if (!samples || (!data && frame->info.num_data > 0)) return hpx_fail(HPX_ERR_ARG, "modulate: null pointer");
  const FrameDev d = frame_dev(frame);
  const int64_t pairs = (int64_t)batch * d.W;
  if (pairs > (1ll << 31) - 1) return hpx_fail(HPX_ERR_ARG, "modulate: batch too large");
  return launch_tx<0>(d, (int)pairs, reinterpret_cast<const float2*>(data), 0, 0, 1, reinterpret_cast<float2*>(samples),
                      as_stream(stream));
}

hpx_status hpx_ofdm_modulate_grid(const hpx_frame* frame, const hpx_cf32* grid, int32_t grid_columns, int32_t batch,
                                  hpx_cf32* samples, void* stream) {
  if (!frame) return hpx_fail(HPX_ERR_ARG, "modulate_grid: null frame");
  if (batch < 0) return hpx_fail(HPX_ERR_ARG, "modulate_grid: negative batch");
  const FrameDev d = frame_dev(frame);
  if (grid_columns < 1 || grid_columns > d.N) return hpx_fail(HPX_ERR_SHAPE, "modulate_grid: grid width out of range");
  if (batch == 0) return HPX_OK;
  if (!samples || !grid) return hpx_fail(HPX_ERR_ARG, "modulate_grid: null pointer");
  const int64_t pairs = (int64_t)batch * d.W;
  if (pairs > (1ll << 31) - 1) return hpx_fail(HPX_ERR_ARG, "modulate_grid: batch too large");
  return launch_tx<2>(d, (int)pairs, reinterpret_cast<const float2*>(grid), 0, 0, grid_columns,
                      reinterpret_cast<float2*>(samples), as_stream(stream));
}

hpx_status hpx_ofdm_modulate_bits(const hpx_frame* frame, uint64_t seed, int64_t drop0, int32_t num_drops,
                                  int32_t num_streams, hpx_cf32* samples, void* stream) {
  if (!frame) return hpx_fail(HPX_ERR_ARG, "modulate_bits: null frame");
  if (num_drops < 0 || num_streams < 1 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "modulate_bits: bad sizes");
  if (num_drops == 0) return HPX_OK;
  if (!samples) return hpx_fail(HPX_ERR_ARG, "modulate_bits: null output");
  const FrameDev d = frame_dev(frame);
  const int64_t pairs = (int64_t)num_drops * num_streams * d.W;
  if (pairs > (1ll << 31) - 1) return hpx_fail(HPX_ERR_ARG, "modulate_bits: batch too large");
  return launch_tx<1>(d, (int)pairs, nullptr, seed, drop0, num_streams, reinterpret_cast<float2*>(samples),
                      as_stream(stream));
}

hpx_status hpx_ofdm_demodulate(const hpx_frame* frame, const hpx_cf32* samples, int64_t sample_stride, int32_t batch,
                               int32_t num_columns, hpx_cf32* grid, void* stream) {
  if (!frame) return hpx_fail(HPX_ERR_ARG, "demodulate: null frame");
  if (batch < 0) return hpx_fail(HPX_ERR_ARG, "demodulate: negative batch");
  if (batch == 0) return HPX_OK;
  const FrameDev d = frame_dev(frame);
  if (num_columns < 1 || num_columns > d.N) return hpx_fail(HPX_ERR_ARG, "demodulate: num_columns out of range");
  if (sample_stride < d.T) return hpx_fail(HPX_ERR_SHAPE, "demodulate: fewer samples than one frame");
  if (!samples || !grid) return hpx_fail(HPX_ERR_ARG, "demodulate: null pointer");
  const int64_t pairs = (int64_t)batch * d.W;
  if (pairs > (1ll << 31) - 1) return hpx_fail(HPX_ERR_ARG, "demodulate: batch too large");
  return launch_rx(d, (int)pairs, reinterpret_cast<const float2*>(samples), sample_stride, num_columns,
                   reinterpret_cast<float2*>(grid), as_stream(stream));
}

hpx_status hpx_ofdm_pick(const hpx_frame* frame, const hpx_cf32* grid, int32_t grid_columns, int32_t batch,
                         hpx_cf32* out, void* stream) {
  if (!frame) return hpx_fail(HPX_ERR_ARG, "pick: null frame");
  if (batch < 0) return hpx_fail(HPX_ERR_ARG, "pick: negative batch");
  const FrameDev d = frame_dev(frame);
  if (grid_columns < d.C) return hpx_fail(HPX_ERR_SHAPE, "pick: grid narrower than the frame's columns");
  if (batch == 0 || d.num_data == 0) return HPX_OK;
  if (!grid || !out) return hpx_fail(HPX_ERR_ARG, "pick: null pointer");
  const int64_t total = (int64_t)batch * d.num_data;
  int blocks = (int)((total + 255) / 256);
  if (blocks > 152 * 16) blocks = 152 * 16;
  k_ofdm_pick<<<blocks, 256, 0, as_stream(stream)>>>(d, reinterpret_cast<const float2*>(grid), grid_columns, batch,
                                                     reinterpret_cast<float2*>(out));
  HPX_LAUNCHED("pick");
  return HPX_OK;
}

}  // extern "C"
