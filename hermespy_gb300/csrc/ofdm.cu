// OFDM transmit (bits -> QAM -> place -> IFFT -> prefix) and receive
// (prefix strip -> FFT -> bin gather) kernels with a block-cooperative
// Stockham FFT in shared memory.
#include "hpx_internal.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxButterflies = 4;  // per thread and stage for N <= 4096 with 256 threads

struct FrameDev {
  int N, logN, W, C, m, order, T, num_data;
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
  const float2* pilots;
};

FrameDev frame_dev(const hpx_frame* f) {
  FrameDev d;
  d.N = f->info.num_subcarriers;
  d.logN = 0;
  while ((1 << d.logN) < d.N) ++d.logN;
  d.W = f->info.num_words;
  d.C = f->info.num_columns;
  d.m = f->info.bits_per_symbol;
  d.order = f->info.modulation_order;
  d.T = f->info.samples_per_frame;
  d.num_data = f->info.num_data;
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
  d.pilots = f->d_pilots;
  return d;
}

// Transforms per block: 1024 samples of shared memory work per block for N <= 1024.
int transforms_per_block(int N) { return N >= 1024 ? 1 : 1024 / N; }

// In-place Stockham autosort FFT of F transforms of length N = 2^logN stored
// back to back in `buf`, executed by all threads of the block. Stage with radix R
// and span Ns: butterfly j reads buf[j + r N/R], applies exp(-+2 pi i r k/(Ns R))
// with k = j mod Ns, and writes buf[(j - k) R + k + r Ns]. Forward: exp(-2 pi i ...);
// INVERSE: exp(+2 pi i ...), unscaled.
template <bool INVERSE>
__device__ void block_fft(float2* buf, int N, int logN, int F, const float2* __restrict__ tw) {
  const int tid = threadIdx.x;
  int Ns = 1;
  if (logN & 1) {
    const int half = N >> 1;
    const int nb = F * half;
    float2 y[kMaxButterflies][2];
    int jj[kMaxButterflies], ff[kMaxButterflies];
#pragma unroll
    for (int i = 0; i < kMaxButterflies; ++i) {
      const int q = tid + i * kThreads;
      if (q < nb) {
        const int f = q / half, j = q - f * half;
        const float2 a0 = buf[f * N + j], a1 = buf[f * N + j + half];
        y[i][0] = cadd(a0, a1);
        y[i][1] = csub(a0, a1);
        jj[i] = j;
        ff[i] = f;
      }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kMaxButterflies; ++i) {
      const int q = tid + i * kThreads;
      if (q < nb) {
        float2* b = buf + ff[i] * N;
        b[2 * jj[i]] = y[i][0];
        b[2 * jj[i] + 1] = y[i][1];
      }
    }
    __syncthreads();
    Ns = 2;
  }
  const int quarter = N >> 2;
  const int nb = F * quarter;
  for (; Ns < N; Ns <<= 2) {
    const int stride = N / (Ns * 4);
    float2 y[kMaxButterflies][4];
    int jj[kMaxButterflies], ff[kMaxButterflies];
#pragma unroll
    for (int i = 0; i < kMaxButterflies; ++i) {
      const int q = tid + i * kThreads;
      if (q < nb) {
        const int f = q / quarter, j = q - f * quarter;
        const int k = j & (Ns - 1);
        const float2* b = buf + f * N;
        float2 a0 = b[j], a1 = b[j + quarter], a2 = b[j + 2 * quarter], a3 = b[j + 3 * quarter];
        if (Ns > 1) {
          const int t1 = (k * stride) & (N - 1);
          const int t2 = (2 * k * stride) & (N - 1);
          const int t3 = (3 * k * stride) & (N - 1);
          float2 w1 = __ldg(tw + t1), w2 = __ldg(tw + t2), w3 = __ldg(tw + t3);
          if (INVERSE) {
            w1.y = -w1.y;
            w2.y = -w2.y;
            w3.y = -w3.y;
          }
          a1 = cmul(a1, w1);
          a2 = cmul(a2, w2);
          a3 = cmul(a3, w3);
        }
        const float2 t0 = cadd(a0, a2), t1 = csub(a0, a2), t2 = cadd(a1, a3);
        const float2 d = csub(a1, a3);
        // forward: (a1 - a3) * (-i); inverse: (a1 - a3) * (+i)
        const float2 t3 = INVERSE ? make_float2(-d.y, d.x) : make_float2(d.y, -d.x);
        y[i][0] = cadd(t0, t2);
        y[i][1] = cadd(t1, t3);
        y[i][2] = csub(t0, t2);
        y[i][3] = csub(t1, t3);
        jj[i] = (j - k) * 4 + k;
        ff[i] = f;
      }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < kMaxButterflies; ++i) {
      const int q = tid + i * kThreads;
      if (q < nb) {
        float2* b = buf + ff[i] * N + jj[i];
        b[0] = y[i][0];
        b[Ns] = y[i][1];
        b[2 * Ns] = y[i][2];
        b[3 * Ns] = y[i][3];
      }
    }
    __syncthreads();
  }
}

// Words of packed Philox bits a block stages per transform.
__host__ __device__ inline int bit_words(int C, int m) { return ((C * m) >> 5) + 8; }

// MODE 0: data symbols from `data` [items][num_data]; MODE 1: Philox bits of
// drop item / num_streams, stream item % num_streams; MODE 2: a placed grid
// `data` [items][W][num_streams] (num_streams carries the grid width).
template <int MODE>
__global__ void __launch_bounds__(kThreads) k_ofdm_tx(FrameDev fr, int F, int num_pairs, const float2* __restrict__ data,
                                                      uint64_t seed, int64_t drop0, int num_streams,
                                                      float2* __restrict__ out) {
  extern __shared__ float4 smem4[];
  float2* sm = reinterpret_cast<float2*>(smem4);
  const int N = fr.N, W = fr.W, C = fr.C;
  const int BW = bit_words(C, fr.m);
  uint32_t* bitsm = reinterpret_cast<uint32_t*>(sm + F * N);
  const int p0 = blockIdx.x * F;
  const int tid = threadIdx.x;

  for (int i = tid; i < F * N; i += kThreads) sm[i] = make_float2(0.f, 0.f);
  if (MODE == 1) {
    for (int f = 0; f < F; ++f) {
      const int p = p0 + f;
      if (p >= num_pairs) break;
      const int item = p / W, w = p - item * W;
      const int drop = item / num_streams, s = item - drop * num_streams;
      const int64_t k0 = fr.data_offset[w];
      const int nd = fr.num_data_word[w];
      if (nd == 0) continue;
      const int64_t wa = (k0 * fr.m) >> 5, wb = ((k0 + nd) * fr.m - 1) >> 5;
      const int64_t blk0 = wa >> 2, blk1 = wb >> 2;
      for (int64_t blk = blk0 + tid; blk <= blk1; blk += kThreads) {
        const uint4 r = hpx_random_block(seed, drop0 + drop, (uint32_t)s, HPX_DOMAIN_BITS, (uint32_t)blk);
        uint32_t* dst = bitsm + f * BW + (blk - blk0) * 4;
        dst[0] = r.x;
        dst[1] = r.y;
        dst[2] = r.z;
        dst[3] = r.w;
      }
    }
  }
  __syncthreads();
  const float inv_sqrt_n = rsqrtf((float)N);
  if (MODE == 2) {
    const int G = num_streams;
    for (int q = tid; q < F * G; q += kThreads) {
      const int f = q / G, c = q - f * G;
      const int p = p0 + f;
      if (p >= num_pairs) continue;
      sm[f * N + fr.bins[c]] = cscale(data[(int64_t)p * G + c], inv_sqrt_n);
    }
  }
  for (int q = tid; MODE != 2 && q < F * C; q += kThreads) {
    const int f = q / C, c = q - f * C;
    const int p = p0 + f;
    if (p >= num_pairs) continue;
    const int item = p / W, w = p - item * W;
    const int kind = fr.kind[w * C + c];
    float2 v = make_float2(0.f, 0.f);
    if (kind == HPX_RE_DATA) {
      const int k = fr.index[w * C + c];
      if (MODE == 0) {
        v = data[(int64_t)item * fr.num_data + k];
      } else {
        const int64_t k0 = fr.data_offset[w];
        const int64_t blk0 = ((k0 * fr.m) >> 5) >> 2;
        const uint32_t* words = bitsm + f * BW - blk0 * 4;
        v = qam_symbol(fr.order, extract_bits_msb(words, (int64_t)k * fr.m, fr.m));
      }
    } else if (kind == HPX_RE_REFERENCE) {
      v = fr.pilots[fr.index[w * C + c]];
    }
    sm[f * N + fr.bins[c]] = cscale(v, inv_sqrt_n);
  }
  __syncthreads();
  block_fft<true>(sm, N, fr.logN, F, fr.twiddle);
  for (int f = 0; f < F; ++f) {
    const int p = p0 + f;
    if (p >= num_pairs) break;
    const int item = p / W, w = p - item * W;
    const int P = fr.prefix[w];
    const bool zp = fr.zero_prefix[w] != 0;
    float2* dst = out + (int64_t)item * fr.T + fr.word_start[w];
    const float2* src = sm + f * N;
    for (int i = tid; i < P + N; i += kThreads) {
      float2 v;
      if (i < P) v = zp ? make_float2(0.f, 0.f) : src[N - P + i];
      else v = src[i - P];
      dst[i] = v;
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_ofdm_rx(FrameDev fr, int F, int num_pairs, const float2* __restrict__ in,
                                                      int64_t stride, int ncols, float2* __restrict__ grid) {
  extern __shared__ float4 smem4[];
  float2* sm = reinterpret_cast<float2*>(smem4);
  const int N = fr.N, W = fr.W;
  const int p0 = blockIdx.x * F;
  const int tid = threadIdx.x;
  for (int f = 0; f < F; ++f) {
    const int p = p0 + f;
    if (p >= num_pairs) {
      for (int i = tid; i < N; i += kThreads) sm[f * N + i] = make_float2(0.f, 0.f);
      continue;
    }
    const int item = p / W, w = p - item * W;
    const float2* src = in + (int64_t)item * stride + fr.window_start[w];
    for (int i = tid; i < N; i += kThreads) sm[f * N + i] = __ldg(src + i);
  }
  __syncthreads();
  block_fft<false>(sm, N, fr.logN, F, fr.twiddle);
  const float inv_sqrt_n = rsqrtf((float)N);
  for (int q = tid; q < F * ncols; q += kThreads) {
    const int f = q / ncols, c = q - f * ncols;
    const int p = p0 + f;
    if (p >= num_pairs) continue;
    grid[(int64_t)p * ncols + c] = cscale(sm[f * N + fr.bins[c]], inv_sqrt_n);
  }
}

__global__ void k_ofdm_pick(FrameDev fr, const float2* __restrict__ grid, int gcols, int batch, float2* __restrict__ out) {
  const int64_t total = (int64_t)batch * fr.num_data;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < total; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t item = q / fr.num_data;
    const int k = (int)(q - item * fr.num_data);
    out[q] = grid[(item * fr.W + fr.data_word[k]) * gcols + fr.data_column[k]];
  }
}

size_t tx_smem(const FrameDev& d, int F, int mode) {
  return (size_t)F * d.N * sizeof(float2) + (mode == 1 ? (size_t)F * bit_words(d.C, d.m) * 4 : 0);
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
  const int F = transforms_per_block(d.N);
  const int64_t pairs = (int64_t)batch * d.W;
  if (pairs > (1ll << 31) - 1) return hpx_fail(HPX_ERR_ARG, "modulate: batch too large");
  const size_t smem = tx_smem(d, F, 0);
  const int blocks = (int)((pairs + F - 1) / F);
  k_ofdm_tx<0><<<blocks, kThreads, smem, as_stream(stream)>>>(d, F, (int)pairs, reinterpret_cast<const float2*>(data),
                                                                0, 0, 1, reinterpret_cast<float2*>(samples));
  HPX_LAUNCHED("modulate");
  return HPX_OK;
}

hpx_status hpx_ofdm_modulate_grid(const hpx_frame* frame, const hpx_cf32* grid, int32_t grid_columns, int32_t batch,
                                  hpx_cf32* samples, void* stream) {
  if (!frame) return hpx_fail(HPX_ERR_ARG, "modulate_grid: null frame");
  if (batch < 0) return hpx_fail(HPX_ERR_ARG, "modulate_grid: negative batch");
  const FrameDev d = frame_dev(frame);
  if (grid_columns < 1 || grid_columns > d.N) return hpx_fail(HPX_ERR_SHAPE, "modulate_grid: grid width out of range");
  if (batch == 0) return HPX_OK;
  if (!samples || !grid) return hpx_fail(HPX_ERR_ARG, "modulate_grid: null pointer");
  const int F = transforms_per_block(d.N);
  const int64_t pairs = (int64_t)batch * d.W;
  if (pairs > (1ll << 31) - 1) return hpx_fail(HPX_ERR_ARG, "modulate_grid: batch too large");
  const size_t smem = tx_smem(d, F, 0);
  const int blocks = (int)((pairs + F - 1) / F);
  k_ofdm_tx<2><<<blocks, kThreads, smem, as_stream(stream)>>>(d, F, (int)pairs, reinterpret_cast<const float2*>(grid),
                                                                0, 0, grid_columns, reinterpret_cast<float2*>(samples));
  HPX_LAUNCHED("modulate_grid");
  return HPX_OK;
}

hpx_status hpx_ofdm_modulate_bits(const hpx_frame* frame, uint64_t seed, int64_t drop0, int32_t num_drops,
                                  int32_t num_streams, hpx_cf32* samples, void* stream) {
  if (!frame) return hpx_fail(HPX_ERR_ARG, "modulate_bits: null frame");
  if (num_drops < 0 || num_streams < 1 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "modulate_bits: bad sizes");
  if (num_drops == 0) return HPX_OK;
  if (!samples) return hpx_fail(HPX_ERR_ARG, "modulate_bits: null output");
  const FrameDev d = frame_dev(frame);
  const int F = transforms_per_block(d.N);
  const int64_t pairs = (int64_t)num_drops * num_streams * d.W;
  if (pairs > (1ll << 31) - 1) return hpx_fail(HPX_ERR_ARG, "modulate_bits: batch too large");
  const size_t smem = tx_smem(d, F, 1);
  if (smem > 48 * 1024)
    HPX_CUDA(cudaFuncSetAttribute(k_ofdm_tx<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int blocks = (int)((pairs + F - 1) / F);
  k_ofdm_tx<1><<<blocks, kThreads, smem, as_stream(stream)>>>(d, F, (int)pairs, nullptr, seed, drop0, num_streams,
                                                                reinterpret_cast<float2*>(samples));
  HPX_LAUNCHED("modulate_bits");
  return HPX_OK;
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
  const int F = transforms_per_block(d.N);
  const int64_t pairs = (int64_t)batch * d.W;
  if (pairs > (1ll << 31) - 1) return hpx_fail(HPX_ERR_ARG, "demodulate: batch too large");
  const size_t smem = (size_t)F * d.N * sizeof(float2);
  const int blocks = (int)((pairs + F - 1) / F);
  k_ofdm_rx<<<blocks, kThreads, smem, as_stream(stream)>>>(d, F, (int)pairs, reinterpret_cast<const float2*>(samples),
                                                           sample_stride, num_columns, reinterpret_cast<float2*>(grid));
  HPX_LAUNCHED("demodulate");
  return HPX_OK;
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
