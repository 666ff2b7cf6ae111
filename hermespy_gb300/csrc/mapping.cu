// Bits, Gray PSK/QAM mapping, hard demapping and bit-error counting.
#include <cmath>
#include <cstring>
#include <mutex>

#include "hpx_internal.cuh"

// ---------------------------------------------------------------- QAM tables

hpx_status qam_bits_per_symbol(int32_t order, int* bits) {
  switch (order) {
    case 2: *bits = 1; return HPX_OK;
    case 4: *bits = 2; return HPX_OK;
    case 16: *bits = 4; return HPX_OK;
    case 64: *bits = 6; return HPX_OK;
    case 256: *bits = 8; return HPX_OK;
    default: return hpx_fail(HPX_ERR_ARG, "Unsupported modulation order (%d)", order);
  }
}

namespace {

// Scaled amplitude of PskQamMapping.get_llr_3gpp for a float32 input, evaluated
// exactly as the reference does in float64: r = (x * sqrt(2)) * sqrt(c)
// (psk_qam_mapping.py:331-344, 363, 411, 450).
double scaled_amplitude(float x, double c) {
  volatile double r = (double)x * std::sqrt(2.0);
  if (c > 1.0) r = r * std::sqrt(c);
  return r;
}

// Order-preserving integer of a float32.
int64_t f2ord(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  return (u & 0x80000000u) ? -(int64_t)(u & 0x7FFFFFFFu) : (int64_t)u;
}
float ord2f(int64_t o) {
  uint32_t u = o < 0 ? (uint32_t)(-o) | 0x80000000u : (uint32_t)o;
  float x;
  std::memcpy(&x, &u, 4);
  return x;
}

// Largest float32 x with r(x) <= e (so r > e <=> x > result).
float x_upper(double e, double c) {
  int64_t lo = f2ord(-3.0e38f), hi = f2ord(3.0e38f);
  while (hi - lo > 1) {
    const int64_t mid = lo + (hi - lo) / 2;
    if (scaled_amplitude(ord2f(mid), c) <= e) lo = mid; else hi = mid;
  }
  return ord2f(lo);
}
// Smallest float32 x with r(x) >= e (so r < e <=> x < result).
float x_lower(double e, double c) {
  int64_t lo = f2ord(-3.0e38f), hi = f2ord(3.0e38f);
  while (hi - lo > 1) {
    const int64_t mid = lo + (hi - lo) / 2;
    if (scaled_amplitude(ord2f(mid), c) >= e) hi = mid; else lo = mid;
  }
  return ord2f(hi);
}

// Open intervals of |r| (r the scaled amplitude) where PAM bit i >= 1 has a positive
// LLR (psk_qam_mapping.py:331-497). Every sign change of those piecewise-linear LLRs
// sits on an exact zero, so ties give bit 0; a = -1 marks an interval closed at 0
// and b = INF an unbounded one. Bit 0 is the sign of r.
const double INF = 1e300;
struct Iv { double a, b; };
const Iv PAM4[2][3] = {{}, {{2, INF}}};
const Iv PAM8[3][3] = {{}, {{4, INF}}, {{-1, 2}, {6, INF}}};
const Iv PAM16[4][3] = {{}, {{8, INF}}, {{-1, 4}, {12, INF}}, {{-1, 2}, {6, 10}, {14, INF}}};
const int PAM4_N[2] = {0, 1};
const int PAM8_N[3] = {0, 1, 2};
const int PAM16_N[4] = {0, 1, 2, 3};

std::mutex g_table_mutex;
QamDemapTable g_tables[9];
bool g_table_ready[9] = {false};

}  // namespace

hpx_status qam_demap_table(int32_t order, QamDemapTable* out) {
  int m;
  HPX_TRY(qam_bits_per_symbol(order, &m));
  const int slot = m;
  std::lock_guard<std::mutex> lock(g_table_mutex);
  if (!g_table_ready[slot]) {
    QamDemapTable t;
    std::memset(&t, 0, sizeof(t));
    t.order = order;
    t.bits = m;
    t.pam_bits = order == 2 ? 1 : m / 2;
    const double c = order == 16 ? 5.0 : (order == 64 ? 21.0 : (order == 256 ? 85.0 : 1.0));
    for (int i = 1; i < t.pam_bits; ++i) {
      const Iv* ivs;
      int n;
      if (order == 16) { ivs = PAM4[i]; n = PAM4_N[i]; }
      else if (order == 64) { ivs = PAM8[i]; n = PAM8_N[i]; }
      else { ivs = PAM16[i]; n = PAM16_N[i]; }
      t.count[i] = n;
      if (n != i) return hpx_fail(HPX_ERR_UNSUPPORTED, "demap table: bit %d has %d intervals", i, n);
      for (int k = 0; k < n; ++k) {
        t.lo[i][k] = ivs[k].a < 0 ? -1.0f : x_upper(ivs[k].a, c);
        t.hi[i][k] = ivs[k].b >= INF ? INFINITY : x_lower(ivs[k].b, c);
        // the shape pam_decide relies on
        if ((ivs[k].a < 0) != pam_interval_open_below(i, k) || (ivs[k].b >= INF) != pam_interval_open_above(i, k))
          return hpx_fail(HPX_ERR_UNSUPPORTED, "demap table: interval %d of bit %d has an unexpected shape", k, i);
      }
    }
    g_tables[slot] = t;
    g_table_ready[slot] = true;
  }
  *out = g_tables[slot];
  return HPX_OK;
}

// ------------------------------------------------------------------ kernels

__global__ void k_bits_generate(uint64_t seed, int64_t drop0, int num_streams, int64_t nbits, uint8_t* bits) {
  // grid: (blocks over 128-bit Philox blocks, num_streams, num_drops)
  const int s = blockIdx.y;
  const int d = blockIdx.z;
  const int64_t nblk = (nbits + 127) / 128;
  uint8_t* out = bits + ((int64_t)d * num_streams + s) * nbits;
  for (int64_t blk = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; blk < nblk;
       blk += (int64_t)gridDim.x * blockDim.x) {
    const uint4 r = hpx_random_block(seed, drop0 + d, (uint32_t)s, HPX_DOMAIN_BITS, (uint32_t)blk);
    const uint32_t w[4] = {r.x, r.y, r.z, r.w};
    const int64_t b0 = blk * 128;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      for (int i = 0; i < 32; ++i) {
        const int64_t b = b0 + j * 32 + i;
        if (b < nbits) out[b] = (uint8_t)((w[j] >> i) & 1u);
      }
    }
  }
}

__global__ void k_qam_map(int order, int m, const uint8_t* __restrict__ bits, int64_t n, float2* __restrict__ sym) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    uint32_t v = 0;
    for (int i = 0; i < m; ++i) v = (v << 1) | (bits[k * m + i] & 1u);
    sym[k] = qam_symbol(order, v);
  }
}

__global__ void k_qam_demap(const __grid_constant__ QamDemapTable t, const float2* __restrict__ sym, int64_t n, uint8_t* __restrict__ bits) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t v = qam_decide(t, sym[k]);
    for (int i = 0; i < t.bits; ++i) bits[k * t.bits + i] = (uint8_t)((v >> (t.bits - 1 - i)) & 1u);
  }
}

__global__ void k_count_errors(const uint8_t* __restrict__ a, int64_t na, const uint8_t* __restrict__ b, int64_t nb,
                               unsigned long long* errors) {
  const int item = blockIdx.y;
  const int64_t n = na > nb ? na : nb;
  const uint8_t* pa = a + item * na;
  const uint8_t* pb = b + item * nb;
  unsigned int local = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int va = i < na ? (pa[i] & 1) : 0;
    const int vb = i < nb ? (pb[i] & 1) : 0;
    local += (unsigned)(va != vb);
  }
  for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
  __shared__ unsigned int warp_sums[32];
  if ((threadIdx.x & 31) == 0) warp_sums[threadIdx.x >> 5] = local;
  __syncthreads();
  if (threadIdx.x < 32) {
    unsigned int v = threadIdx.x < (blockDim.x >> 5) ? warp_sums[threadIdx.x] : 0u;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (threadIdx.x == 0 && v) atomicAdd(errors + item, (unsigned long long)v);
  }
}

static int grid_for(int64_t n, int threads) {
  int64_t g = (n + threads - 1) / threads;
  if (g < 1) g = 1;
  if (g > 152 * 32) g = 152 * 32;
  return (int)g;
}

extern "C" {

hpx_status hpx_bits_generate(uint64_t seed, int64_t drop0, int32_t num_drops, int32_t num_streams,
                             int64_t bits_per_stream, uint8_t* bits, void* stream) {
  if (num_drops < 0 || num_streams < 0 || bits_per_stream < 0 || drop0 < 0)
    return hpx_fail(HPX_ERR_ARG, "bits: negative size");
  if (num_drops == 0 || num_streams == 0 || bits_per_stream == 0) return HPX_OK;
  if (!bits) return hpx_fail(HPX_ERR_ARG, "bits: null output");
  if (num_streams > 65535 || num_drops > 65535) return hpx_fail(HPX_ERR_ARG, "bits: batch too large");
  const int64_t nblk = (bits_per_stream + 127) / 128;
  dim3 grid((unsigned)((nblk + 127) / 128 > 1024 ? 1024 : (nblk + 127) / 128), num_streams, num_drops);
  k_bits_generate<<<grid, 128, 0, as_stream(stream)>>>(seed, drop0, num_streams, bits_per_stream, bits);
  HPX_LAUNCHED("bits");
  return HPX_OK;
}

hpx_status hpx_qam_map(int32_t order, const uint8_t* bits, int64_t num_symbols, hpx_cf32* symbols, void* stream) {
  int m;
  HPX_TRY(qam_bits_per_symbol(order, &m));
  if (num_symbols < 0) return hpx_fail(HPX_ERR_ARG, "map: negative size");
  if (num_symbols == 0) return HPX_OK;
  if (!bits || !symbols) return hpx_fail(HPX_ERR_ARG, "map: null pointer");
  k_qam_map<<<grid_for(num_symbols, 256), 256, 0, as_stream(stream)>>>(order, m, bits, num_symbols,
                                                                         reinterpret_cast<float2*>(symbols));
  HPX_LAUNCHED("map");
  return HPX_OK;
}

hpx_status hpx_qam_demap(int32_t order, const hpx_cf32* symbols, int64_t num_symbols, uint8_t* bits, void* stream) {
  QamDemapTable t;
  HPX_TRY(qam_demap_table(order, &t));
  if (num_symbols < 0) return hpx_fail(HPX_ERR_ARG, "demap: negative size");
  if (num_symbols == 0) return HPX_OK;
  if (!bits || !symbols) return hpx_fail(HPX_ERR_ARG, "demap: null pointer");
  k_qam_demap<<<grid_for(num_symbols, 256), 256, 0, as_stream(stream)>>>(
      t, reinterpret_cast<const float2*>(symbols), num_symbols, bits);
  HPX_LAUNCHED("demap");
  return HPX_OK;
}

hpx_status hpx_count_errors(const uint8_t* a, int64_t len_a, const uint8_t* b, int64_t len_b, int32_t batch,
                            uint64_t* errors, void* stream) {
  if (len_a < 0 || len_b < 0 || batch < 0) return hpx_fail(HPX_ERR_ARG, "count_errors: negative size");
  if (batch == 0) return HPX_OK;
  if (!errors) return hpx_fail(HPX_ERR_ARG, "count_errors: null output");
  if (batch > 65535) return hpx_fail(HPX_ERR_ARG, "count_errors: batch too large");
  HPX_CUDA(cudaMemsetAsync(errors, 0, sizeof(uint64_t) * batch, as_stream(stream)));
  const int64_t n = len_a > len_b ? len_a : len_b;
  if (n == 0) return HPX_OK;
  if ((len_a && !a) || (len_b && !b)) return hpx_fail(HPX_ERR_ARG, "count_errors: null input");
  dim3 grid((unsigned)((n + 255) / 256 > 256 ? 256 : (n + 255) / 256), batch);
  k_count_errors<<<grid, 256, 0, as_stream(stream)>>>(a, len_a, b, len_b,
                                                     reinterpret_cast<unsigned long long*>(errors));
  HPX_LAUNCHED("count_errors");
  return HPX_OK;
}

}  // extern "C"

// ------------------------------------------------------------------- AWGN

__global__ void k_awgn_add(float2* __restrict__ x, int num_streams, int64_t n, const float* __restrict__ power,
                           uint64_t seed, int64_t drop0) {
  const int s = blockIdx.y, b = blockIdx.z;
  const float sigma = sqrtf(0.5f * power[b]);
  if (!(sigma > 0.0f)) return;
  float2* row = x + ((int64_t)b * num_streams + s) * n;
  // complex sample k: Philox block k/2, words (0,1) for even k and (2,3) for odd k
  for (int64_t pair = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; 2 * pair < n;
       pair += (int64_t)gridDim.x * blockDim.x) {
    const uint4 w = hpx_random_block(seed, drop0 + b, (uint32_t)s, HPX_DOMAIN_NOISE, (uint32_t)pair);
    const float2 n0 = box_muller(w.x, w.y);
    const float2 n1 = box_muller(w.z, w.w);
    const int64_t k = 2 * pair;
    row[k].x += sigma * n0.x;
    row[k].y += sigma * n0.y;
    if (k + 1 < n) {
      row[k + 1].x += sigma * n1.x;
      row[k + 1].y += sigma * n1.y;
    }
  }
}

extern "C" hpx_status hpx_awgn_add(hpx_cf32* samples, int32_t batch, int32_t num_streams, int64_t num_samples,
                                   const float* noise_power, uint64_t seed, int64_t drop0, void* stream) {
  if (batch < 0 || num_streams < 0 || num_samples < 0 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "awgn: bad size");
  if (batch == 0 || num_streams == 0 || num_samples == 0) return HPX_OK;
  if (!samples || !noise_power) return hpx_fail(HPX_ERR_ARG, "awgn: null pointer");
  if (batch > 65535 || num_streams > 65535) return hpx_fail(HPX_ERR_ARG, "awgn: batch too large");
  const int64_t pairs = (num_samples + 1) / 2;
  dim3 grid((unsigned)((pairs + 255) / 256 > 1024 ? 1024 : (pairs + 255) / 256), num_streams, batch);
  k_awgn_add<<<grid, 256, 0, as_stream(stream)>>>(reinterpret_cast<float2*>(samples), num_streams, num_samples,
                                                  noise_power, seed, drop0);
  HPX_LAUNCHED("awgn");
  return HPX_OK;
}
