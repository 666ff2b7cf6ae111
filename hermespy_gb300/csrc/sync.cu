// Frame synchronization metrics: the Schmidl-Cox delay correlation
// (modem/waveforms/orthogonal/ofdm.py:217-257) and the pilot cross-correlation of
// CorrelationSynchronization (modem/waveform_correlation_synchronization.py:119-170).
//
// The Schmidl-Cox windows come from block-local prefix sums (one pass over the
// signal); the pilot correlation is a direct sum per lag with the pilot and the
// signal window of a 256-lag tile staged in shared memory, products accumulated
// in FP32 over four interleaved partial sums. The peak search that follows
// (scipy.signal.find_peaks) runs on the host over the FP64 metric.
#include "hpx_internal.cuh"

namespace {

constexpr int SYNC_TILE = 256;

// metric[b][0] = 0 and metric[b][1 + d] = sum_s |sum_{k<h} conj(x_s[d + k]) x_s[d + k + h]|
// for d in [0, nd), nd = n - L + 1 (L = symbol length, h = L / 2).
//
// One block covers SC_DELAYS delays of one signal. Per stream it forms the
// products c[t] = conj(x[t]) x[t + h] of its span (SC_DELAYS + h of them, x read
// once from HBM, the shifted copy from L2), turns them into an exclusive prefix
// sum in shared memory (thread-serial runs + warp shuffles + one warp over the
// warp totals) and reads every window as the difference of two prefixes. The
// prefix restarts in every block, so its magnitude (and the cancellation error of
// the difference) stays within (SC_DELAYS + h) |c| while a matching window sums to
// h |c|.
constexpr int SC_THREADS = 512;
constexpr int SC_DELAYS = 2048;

__global__ void __launch_bounds__(SC_THREADS) k_schmidl_cox(const float2* __restrict__ x, int S, int64_t n, int h,
                                                            int64_t nd, int per_thread, double* __restrict__ metric) {
  extern __shared__ float2 pre[];  // [SC_THREADS * per_thread] exclusive prefix sums
  __shared__ float2 warp_total[SC_THREADS / 32];
  const int b = blockIdx.y, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t d0 = (int64_t)blockIdx.x * SC_DELAYS;
  const int span = SC_DELAYS + h;  // products needed by the block's delays
  float mag[SC_DELAYS / SC_THREADS] = {};
  for (int s = 0; s < S; ++s) {
    const float2* xs = x + ((int64_t)b * S + s) * n;
    // products, thread-serial runs of per_thread consecutive entries
    float2 run = make_float2(0.f, 0.f);
    const int i0 = tid * per_thread;
    __syncthreads();  // previous stream's prefixes consumed
    for (int j = 0; j < per_thread; ++j) {
      const int i = i0 + j;
      const int64_t t = d0 + i;
      float2 c = make_float2(0.f, 0.f);
      if (i < span && t + h < n) cfmac(c, xs[t], xs[t + h]);
      pre[i] = run;  // exclusive within the run
      run.x += c.x;
      run.y += c.y;
    }
    // scan of the run totals: warp, then warp totals
    float2 inc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const float ux = __shfl_up_sync(0xffffffffu, inc.x, o), uy = __shfl_up_sync(0xffffffffu, inc.y, o);
      if (lane >= o) {
        inc.x += ux;
        inc.y += uy;
      }
    }
    if (lane == 31) warp_total[warp] = inc;
    __syncthreads();
    if (warp == 0) {
      float2 w = lane < SC_THREADS / 32 ? warp_total[lane] : make_float2(0.f, 0.f);
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const float ux = __shfl_up_sync(0xffffffffu, w.x, o), uy = __shfl_up_sync(0xffffffffu, w.y, o);
        if (lane >= o) {
          w.x += ux;
          w.y += uy;
        }
      }
      if (lane < SC_THREADS / 32) warp_total[lane] = w;  // inclusive over warps
    }
    __syncthreads();
    float2 base = make_float2(inc.x - run.x, inc.y - run.y);  // exclusive within the warp
    if (warp > 0) {
      base.x += warp_total[warp - 1].x;
      base.y += warp_total[warp - 1].y;
    }
    for (int j = 0; j < per_thread; ++j) {
      float2& v = pre[i0 + j];
      v.x += base.x;
      v.y += base.y;
    }
    __syncthreads();
    // windows: S(d) = pre[d - d0 + h] - pre[d - d0]
#pragma unroll
    for (int q = 0; q < SC_DELAYS / SC_THREADS; ++q) {
      const int dl = tid + q * SC_THREADS;
      const float2 hi = pre[dl + h], lo = pre[dl];
      const float re = hi.x - lo.x, im = hi.y - lo.y;
      mag[q] += sqrtf(re * re + im * im);
    }
  }
  double* m = metric + (int64_t)b * (nd + 1);
#pragma unroll
  for (int q = 0; q < SC_DELAYS / SC_THREADS; ++q) {
    const int64_t d = d0 + tid + q * SC_THREADS;
    if (d < nd) m[1 + d] = (double)mag[q];
  }
  if (blockIdx.x == 0 && tid == 0) m[0] = 0.0;
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

// Peak search of scipy.signal.find_peaks(x, height, distance) over one metric per
// block (scipy/signal/_peak_finding.py find_peaks with _local_maxima_1d and
// _select_by_peak_distance): a local maximum is a rise x[i-1] < x[i] followed by a
// plateau of equal values and a fall (the peak is the plateau's midpoint, first and
// last samples excluded); peaks below height x max(metric) are dropped (below
// `height` itself with `normalize`, see below); then, by decreasing
// height, each kept peak removes the peaks closer than `distance`. Equal heights
// are taken by decreasing index (numpy's argsort of a short priority vector is an
// insertion sort, so the later of two equal peaks comes last and is taken first).
// With `normalize` the metric is divided by its maximum first and `height` applies
// to the quotient, like the correlation routine's corr /= corr.max(). Kept peaks,
// in index order, are shifted by `offset` and, with `clip`, set to 0 below 0 and to
// clip_value above clip_max; counts[b] is their number (up to max_frames stored),
// or -1 if more than SYNC_CAND candidates passed the height test.
constexpr int SYNC_CAND = 512;
constexpr int PEAK_THREADS = 512;

__global__ void __launch_bounds__(PEAK_THREADS) k_sync_peaks(const double* __restrict__ metric, int64_t len,
                                                            int normalize, double height, int64_t distance,
                                                            int64_t offset, int clip, int64_t clip_max,
                                                            int64_t clip_value, int max_frames,
                                                            int64_t* __restrict__ starts, int32_t* __restrict__ counts) {
  __shared__ double red[PEAK_THREADS / 32];
  __shared__ int64_t cand[SYNC_CAND];
  __shared__ double cval[SYNC_CAND];
  __shared__ uint8_t keep[SYNC_CAND];
  __shared__ int ncand;
  const int b = blockIdx.x, tid = threadIdx.x;
  const double* x = metric + (int64_t)b * len;
  double mx = -INFINITY;
  for (int64_t i = tid; i < len; i += PEAK_THREADS) mx = fmax(mx, x[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if ((tid & 31) == 0) red[tid >> 5] = mx;
  if (tid == 0) ncand = 0;
  __syncthreads();
  mx = red[0];
  for (int w = 1; w < PEAK_THREADS / 32; ++w) mx = fmax(mx, red[w]);
  const double scale = normalize ? mx : 1.0;
  const double hmin = normalize ? height : height * mx;
  auto val = [&](int64_t i) { return normalize ? x[i] / scale : x[i]; };
  for (int64_t i = 1 + tid; i < len - 1; i += PEAK_THREADS) {
    const double v = val(i);
    if (!(val(i - 1) < v)) continue;
    int64_t ahead = i + 1;
    while (ahead < len - 1 && val(ahead) == v) ++ahead;
    if (!(val(ahead) < v) || !(v >= hmin)) continue;
    const int slot = atomicAdd(&ncand, 1);
    if (slot < SYNC_CAND) {
      cand[slot] = (i + ahead - 1) / 2;
      cval[slot] = v;
    }
  }
  __syncthreads();
  const int m = ncand;
  if (tid == 0) {
    if (m > SYNC_CAND) {
      counts[b] = -1;
    } else {
      // index order (insertion sort: few candidates)
      for (int a = 1; a < m; ++a) {
        const int64_t ci = cand[a];
        const double cv = cval[a];
        int j = a - 1;
        for (; j >= 0 && cand[j] > ci; --j) {
          cand[j + 1] = cand[j];
          cval[j + 1] = cval[j];
        }
        cand[j + 1] = ci;
        cval[j + 1] = cv;
      }
      for (int a = 0; a < m; ++a) keep[a] = 1;
      uint8_t done[SYNC_CAND / 8] = {};  // candidates already taken as priority
      for (int step = 0; step < m; ++step) {
        int j = -1;
        for (int a = 0; a < m; ++a) {  // highest remaining priority, later index on ties
          if (done[a >> 3] & (1u << (a & 7))) continue;
          if (j < 0 || cval[a] >= cval[j]) j = a;
        }
        done[j >> 3] |= (uint8_t)(1u << (j & 7));
        if (!keep[j]) continue;
        for (int k = j - 1; k >= 0 && cand[j] - cand[k] < distance; --k) keep[k] = 0;
        for (int k = j + 1; k < m && cand[k] - cand[j] < distance; ++k) keep[k] = 0;
      }
      int kept = 0;
      for (int a = 0; a < m; ++a) {
        if (!keep[a]) continue;
        int64_t v = cand[a] + offset;
        if (clip) {
          if (v < 0) v = 0;
          if (v > clip_max) v = clip_value;
        }
        if (kept < max_frames) starts[(int64_t)b * max_frames + kept] = v;
        ++kept;
      }
      counts[b] = kept;
    }
  }
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
  // prefix entries 0 .. SC_DELAYS + h (the last delay reads entry SC_DELAYS - 1 + h)
  const int per_thread = (SC_DELAYS + h + 1 + SC_THREADS - 1) / SC_THREADS;
  const size_t smem = (size_t)SC_THREADS * per_thread * sizeof(float2);
  HPX_TRY(smem_attr((const void*)k_schmidl_cox, smem));
  const int64_t tiles = (nd + SC_DELAYS - 1) / SC_DELAYS;
  if (tiles > 0x7fffffff) return hpx_fail(HPX_ERR_ARG, "sync_schmidl_cox: signal too long");
  k_schmidl_cox<<<dim3((unsigned)tiles, batch), SC_THREADS, smem, as_stream(stream)>>>(
      reinterpret_cast<const float2*>(signal), num_streams, num_samples, h, nd, per_thread, metric);
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

hpx_status hpx_sync_peaks(const double* metric, int32_t batch, int64_t length, int32_t normalize, double height,
                          int64_t distance, int64_t offset, int32_t clip, int64_t clip_max, int64_t clip_value,
                          int32_t max_frames, int64_t* starts, int32_t* counts, void* stream) {
  if (batch < 0 || length < 0 || max_frames < 0) return hpx_fail(HPX_ERR_ARG, "sync_peaks: bad sizes");
  if (distance < 1) return hpx_fail(HPX_ERR_ARG, "`distance` must be greater or equal to 1");
  if (batch == 0) return HPX_OK;
  if (!metric || !counts || (max_frames > 0 && !starts)) return hpx_fail(HPX_ERR_ARG, "sync_peaks: null pointer");
  k_sync_peaks<<<batch, PEAK_THREADS, 0, as_stream(stream)>>>(metric, length, normalize, height, distance, offset,
                                                              clip, clip_max, clip_value, max_frames, starts, counts);
  HPX_LAUNCHED("sync_peaks");
  return HPX_OK;
}

}  // extern "C"
