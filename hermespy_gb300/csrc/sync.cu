// Frame synchronization metrics: the Schmidl-Cox delay correlation
// (modem/waveforms/orthogonal/ofdm.py:217-257) and the pilot cross-correlation of
// CorrelationSynchronization (modem/waveform_correlation_synchronization.py:119-170).
//
// Both are direct sliding sums: one thread per candidate delay, the signal window
// of a 256-delay tile (and the pilot) staged in shared memory, products
// accumulated in FP32 over four interleaved partial sums and the stream
// magnitudes summed in FP64. The peak search that follows (scipy.signal.find_peaks)
// runs on the host over the FP64 metric.
#include "hpx_internal.cuh"

namespace {

constexpr int SYNC_TILE = 256;

// metric[b][0] = 0 and metric[b][1 + d] = sum_s |sum_{k<h} conj(x_s[d + k]) x_s[d + k + h]|
// for d in [0, nd), nd = n - L + 1 (L = symbol length, h = L / 2).
__global__ void __launch_bounds__(SYNC_TILE) k_schmidl_cox(const float2* __restrict__ x, int S, int64_t n, int h,
                                                           int64_t nd, double* __restrict__ metric) {
  extern __shared__ float2 win[];  // [SYNC_TILE + 2h]
  const int b = blockIdx.y;
  const int64_t d0 = (int64_t)blockIdx.x * SYNC_TILE;
  const int64_t d = d0 + threadIdx.x;
  const int span = SYNC_TILE + 2 * h;
  double total = 0.0;
  for (int s = 0; s < S; ++s) {
    const float2* xs = x + ((int64_t)b * S + s) * n;
    __syncthreads();  // previous stream's window consumed
    for (int i = threadIdx.x; i < span; i += SYNC_TILE) {
      const int64_t t = d0 + i;
      win[i] = t < n ? xs[t] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 acc[4] = {};
    const float2* a = win + threadIdx.x;
    const float2* c = a + h;
    int k = 0;
    for (; k + 4 <= h; k += 4) {
#pragma unroll
      for (int j = 0; j < 4; ++j) cfmac(acc[j], a[k + j], c[k + j]);  // conj(a) c
    }
    for (; k < h; ++k) cfmac(acc[0], a[k], c[k]);
    const double re = ((double)acc[0].x + acc[1].x) + ((double)acc[2].x + acc[3].x);
    const double im = ((double)acc[0].y + acc[1].y) + ((double)acc[2].y + acc[3].y);
    total += sqrt(re * re + im * im);
  }
  double* m = metric + (int64_t)b * (nd + 1);
  if (d < nd) m[1 + d] = total;
  if (blockIdx.x == 0 && threadIdx.x == 0) m[0] = 0.0;
}

// out[b][k] = sum_s |sum_{j<P} x_s[k - (P - 1) + j] conj(p[j])| for k in [0, n + P - 1),
// samples outside [0, n) being zero (scipy.signal.correlate(x, p, "full")).
__global__ void __launch_bounds__(SYNC_TILE) k_pilot_correlation(const float2* __restrict__ x, int S, int64_t n,
                                                                 const float2* __restrict__ pilot, int P,
                                                                 double* __restrict__ out) {
  extern __shared__ float2 sm[];
  float2* pl = sm;       // [P]
  float2* win = sm + P;  // [SYNC_TILE + P - 1]
  const int b = blockIdx.y;
  const int64_t k0 = (int64_t)blockIdx.x * SYNC_TILE;
  const int64_t nout = n + P - 1;
  const int span = SYNC_TILE + P - 1;
  for (int j = threadIdx.x; j < P; j += SYNC_TILE) pl[j] = pilot[j];
  double total = 0.0;
  for (int s = 0; s < S; ++s) {
    const float2* xs = x + ((int64_t)b * S + s) * n;
    __syncthreads();
    for (int i = threadIdx.x; i < span; i += SYNC_TILE) {
      const int64_t t = k0 - (P - 1) + i;
      win[i] = (t >= 0 && t < n) ? xs[t] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 acc[4] = {};
    const float2* a = win + threadIdx.x;
    int j = 0;
    for (; j + 4 <= P; j += 4) {
#pragma unroll
      for (int q = 0; q < 4; ++q) cfmac(acc[q], pl[j + q], a[j + q]);  // a conj(p)
    }
    for (; j < P; ++j) cfmac(acc[0], pl[j], a[j]);
    const double re = ((double)acc[0].x + acc[1].x) + ((double)acc[2].x + acc[3].x);
    const double im = ((double)acc[0].y + acc[1].y) + ((double)acc[2].y + acc[3].y);
    total += sqrt(re * re + im * im);
  }
  const int64_t k = k0 + threadIdx.x;
  if (k < nout) out[(int64_t)b * nout + k] = total;
}

hpx_status smem_attr(const void* fn, size_t bytes) {
  if (bytes > 227 * 1024) return hpx_fail(HPX_ERR_UNSUPPORTED, "sync: window of %zu bytes exceeds shared memory", bytes);
  if (bytes > 48 * 1024) HPX_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
  return HPX_OK;
}

}  // namespace

extern "C" {

hpx_status hpx_sync_schmidl_cox(const hpx_cf32* signal, int32_t batch, int32_t num_streams, int64_t num_samples,
                                int32_t symbol_length, double* metric, void* stream) {
  if (batch < 0 || num_streams < 1 || num_samples < 0) return hpx_fail(HPX_ERR_ARG, "sync_schmidl_cox: bad sizes");
  if (symbol_length < 2) return hpx_fail(HPX_ERR_ARG, "sync_schmidl_cox: symbol length below 2");
  if (batch > 65535) return hpx_fail(HPX_ERR_ARG, "sync_schmidl_cox: batch above 65535 signals per call");
  if (num_samples < symbol_length || batch == 0) return HPX_OK;  // no candidate delay
  if (!signal || !metric) return hpx_fail(HPX_ERR_ARG, "sync_schmidl_cox: null pointer");
  const int h = symbol_length / 2;
  const int64_t nd = num_samples - symbol_length + 1;
  const size_t smem = (size_t)(SYNC_TILE + 2 * h) * sizeof(float2);
  HPX_TRY(smem_attr((const void*)k_schmidl_cox, smem));
  const int64_t tiles = (nd + SYNC_TILE - 1) / SYNC_TILE;
  if (tiles > 0x7fffffff) return hpx_fail(HPX_ERR_ARG, "sync_schmidl_cox: signal too long");
  k_schmidl_cox<<<dim3((unsigned)tiles, batch), SYNC_TILE, smem, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(signal), num_streams, num_samples, h, nd, metric);
  HPX_LAUNCHED("sync_schmidl_cox");
  return HPX_OK;
}

hpx_status hpx_sync_correlation(const hpx_cf32* signal, int32_t batch, int32_t num_streams, int64_t num_samples,
                                const hpx_cf32* pilot, int32_t pilot_length, double* correlation, void* stream) {
  if (batch < 0 || num_streams < 1 || num_samples < 0) return hpx_fail(HPX_ERR_ARG, "sync_correlation: bad sizes");
  if (pilot_length < 1) return hpx_fail(HPX_ERR_ARG, "sync_correlation: empty pilot");
  if (batch > 65535) return hpx_fail(HPX_ERR_ARG, "sync_correlation: batch above 65535 signals per call");
  if (num_samples == 0 || batch == 0) return HPX_OK;
  if (!signal || !pilot || !correlation) return hpx_fail(HPX_ERR_ARG, "sync_correlation: null pointer");
  const int64_t nout = num_samples + pilot_length - 1;
  const size_t smem = (size_t)(SYNC_TILE + 2 * pilot_length - 1) * sizeof(float2);
  HPX_TRY(smem_attr((const void*)k_pilot_correlation, smem));
  const int64_t tiles = (nout + SYNC_TILE - 1) / SYNC_TILE;
  if (tiles > 0x7fffffff) return hpx_fail(HPX_ERR_ARG, "sync_correlation: signal too long");
  k_pilot_correlation<<<dim3((unsigned)tiles, batch), SYNC_TILE, smem, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(signal), num_streams, num_samples, reinterpret_cast<const float2*>(pilot),
      pilot_length, correlation);
  HPX_LAUNCHED("sync_correlation");
  return HPX_OK;
}

}  // extern "C"
