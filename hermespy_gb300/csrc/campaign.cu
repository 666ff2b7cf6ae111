// Device-resident Monte Carlo campaign over noise levels with confidence stopping.
//
// The reference's campaign (core/pymonte: Monte Carlo actors sample drops, the
// collector adds each drop's scalar artifact to its grid point) stops a grid point
// once the confidence rule of ScalarEvaluationResult.add_artifact
// (core/pymonte/scalar.py:101-125, Algorithm 1 of Bayer et al., "On non-asymptotic
// optimal stopping criteria in Monte Carlo simulations") holds:
//     std = sqrt((sum x^2 - (sum x)^2 / n) / (n - 1)),
//     confident <=> 2 (1 - Phi(sqrt(n) accuracy / std)) < confidence,  std > 0,
// evaluated every `min_samples` samples, x = the drop's bit-error rate.
// Here the per-level sums live on the GPU: each batch assigns its drops round-robin
// to the levels that are neither confident nor at their drop limit, runs them
// through hpx_link_run, adds their BERs to the level sums and re-evaluates the rule
// (at batch ends once a level holds at least `min_samples` drops). The host only
// enqueues batches and reads one integer (levels still active) every few batches.
#include "hpx_internal.cuh"

struct hpx_campaign {
  int L = 0, max_batch = 0, min_samples = 2;
  double accuracy = 0.0, confidence = 0.0, bits_per_drop = 1.0;
  int64_t max_drops = 0;
  float* d_power = nullptr;          // [L] noise power of each level
  double* d_sum = nullptr;           // [L] sum of per-drop BER
  double* d_sq = nullptr;            // [L] sum of squared per-drop BER
  unsigned long long* d_count = nullptr;   // [L] drops
  unsigned long long* d_errors = nullptr;  // [L] bit errors
  int* d_confident = nullptr;        // [L]
  int* d_active = nullptr;           // [1] levels still active after the last evaluation
  int* d_level = nullptr;            // [max_batch] level of each drop of the batch (-1: none)
  float* d_noise = nullptr;          // [max_batch]
  uint32_t* d_drop_errors = nullptr; // [max_batch]
  unsigned int* d_flags = nullptr;   // [1] HPX_DROP_* flags of drops left out of the sums
};

namespace {

__global__ void k_assign(int L, int batch, const float* __restrict__ power, const int* __restrict__ confident,
                         const unsigned long long* __restrict__ count, unsigned long long max_drops,
                         float* __restrict__ noise, int* __restrict__ level) {
  extern __shared__ int act[];  // [L] active level list
  __shared__ int n_active;
  if (threadIdx.x == 0) {
    int n = 0;
    for (int l = 0; l < L; ++l)
      if (!confident[l] && count[l] < max_drops) act[n++] = l;
    n_active = n;
  }
  __syncthreads();
  const int n = n_active;
  for (int i = threadIdx.x; i < batch; i += blockDim.x) {
    const int lv = n > 0 ? act[i % n] : -1;
    level[i] = lv;
    noise[i] = power[lv >= 0 ? lv : 0];
  }
}

// A drop whose error word carries a failure flag (HPX_DROP_TIMEOUT / NUMERIC) stays
// out of the sums; its flag goes to *flags, which ends the run with an error status.
__global__ void k_accumulate(int batch, const int* __restrict__ level, const uint32_t* __restrict__ errors,
                             double inv_bits, double* __restrict__ sum, double* __restrict__ sq,
                             unsigned long long* __restrict__ count, unsigned long long* __restrict__ errsum,
                             unsigned int* __restrict__ flags) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < batch; i += gridDim.x * blockDim.x) {
    const int lv = level[i];
    if (lv < 0) continue;
    const uint32_t f = errors[i] & ~HPX_DROP_COUNT;
    if (f) {
      atomicOr(flags, f);
      continue;
    }
    const double x = (double)errors[i] * inv_bits;
    atomicAdd(sum + lv, x);
    atomicAdd(sq + lv, x * x);
    atomicAdd(count + lv, 1ull);
    atomicAdd(errsum + lv, (unsigned long long)errors[i]);
  }
}

__global__ void k_confidence(int L, int min_samples, double accuracy, double confidence,
                             unsigned long long max_drops, const double* __restrict__ sum,
                             const double* __restrict__ sq, const unsigned long long* __restrict__ count,
                             int* __restrict__ confident, int* __restrict__ active) {
  __shared__ int n_active;
  if (threadIdx.x == 0) n_active = 0;
  __syncthreads();
  for (int l = threadIdx.x; l < L; l += blockDim.x) {
    const unsigned long long n = count[l];
    if (!confident[l] && n >= (unsigned long long)min_samples && n > 1) {
      const double s = sum[l], q = sq[l], dn = (double)n;
      const double var = (q - s * s / dn) / (dn - 1.0);
      const double sd = var > 0.0 ? sqrt(var) : 0.0;
      if (sd > 0.0) {
        const double c = 2.0 * (1.0 - normcdf(sqrt(dn) * accuracy / sd));
        if (c < confidence) confident[l] = 1;
      }
    }
    if (!confident[l] && count[l] < max_drops) atomicAdd(&n_active, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) *active = n_active;
}

void release(hpx_campaign* c) {
  if (!c) return;
  void* p[] = {c->d_power, c->d_sum, c->d_sq, c->d_count, c->d_errors, c->d_confident, c->d_active, c->d_level,
               c->d_noise, c->d_drop_errors, c->d_flags};
  for (void* q : p)
    if (q) cudaFree(q);
  delete c;
}

}  // namespace

extern "C" {

hpx_status hpx_campaign_create(int32_t num_levels, const float* noise_power, double accuracy, double confidence,
                               int32_t min_samples, int64_t max_drops_per_level, int32_t max_batch,
                               double bits_per_drop, hpx_campaign** out) {
  if (!out || !noise_power) return hpx_fail(HPX_ERR_ARG, "campaign: null argument");
  *out = nullptr;
  if (num_levels < 1 || num_levels > 4096) return hpx_fail(HPX_ERR_ARG, "campaign: 1..4096 levels");
  if (confidence > 1.0 || confidence < 0.0) return hpx_fail(HPX_ERR_ARG, "Coinfidence requirement must be between zero and one");
  if (accuracy < 0.0) return hpx_fail(HPX_ERR_ARG, "Confidence bound must be non-negative");
  if (min_samples < 2) return hpx_fail(HPX_ERR_ARG, "Minimum number of samples must be at least two");
  if (max_batch < 1 || max_batch > 65535 || max_drops_per_level < 1 || !(bits_per_drop > 0))
    return hpx_fail(HPX_ERR_ARG, "campaign: bad batch, drop limit or bits per drop");
  hpx_campaign* c = new hpx_campaign();
  c->L = num_levels;
  c->max_batch = max_batch;
  c->min_samples = min_samples;
  c->accuracy = accuracy;
  c->confidence = confidence;
  c->bits_per_drop = bits_per_drop;
  c->max_drops = max_drops_per_level;
  const size_t L = num_levels;
  cudaError_t e;
  if ((e = cudaMalloc(&c->d_power, sizeof(float) * L)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_sum, sizeof(double) * L)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_sq, sizeof(double) * L)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_count, sizeof(unsigned long long) * L)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_errors, sizeof(unsigned long long) * L)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_confident, sizeof(int) * L)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_active, sizeof(int))) != cudaSuccess ||
      (e = cudaMalloc(&c->d_level, sizeof(int) * max_batch)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_noise, sizeof(float) * max_batch)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_drop_errors, sizeof(uint32_t) * max_batch)) != cudaSuccess ||
      (e = cudaMalloc(&c->d_flags, sizeof(unsigned int))) != cudaSuccess ||
      (e = cudaMemcpy(c->d_power, noise_power, sizeof(float) * L, cudaMemcpyHostToDevice)) != cudaSuccess) {
    release(c);
    return hpx_cuda_status(e, "campaign buffers");
  }
  const hpx_status s = hpx_campaign_reset(c);
  if (s != HPX_OK) {
    release(c);
    return s;
  }
  *out = c;
  return HPX_OK;
}

hpx_status hpx_campaign_destroy(hpx_campaign* c) {
  release(c);
  return HPX_OK;
}

hpx_status hpx_campaign_reset(hpx_campaign* c) {
  if (!c) return hpx_fail(HPX_ERR_ARG, "campaign_reset: null argument");
  const size_t L = c->L;
  HPX_CUDA(cudaMemset(c->d_sum, 0, sizeof(double) * L));
  HPX_CUDA(cudaMemset(c->d_sq, 0, sizeof(double) * L));
  HPX_CUDA(cudaMemset(c->d_count, 0, sizeof(unsigned long long) * L));
  HPX_CUDA(cudaMemset(c->d_errors, 0, sizeof(unsigned long long) * L));
  HPX_CUDA(cudaMemset(c->d_confident, 0, sizeof(int) * L));
  HPX_CUDA(cudaMemset(c->d_flags, 0, sizeof(unsigned int)));
  const int all = c->L;
  HPX_CUDA(cudaMemcpy(c->d_active, &all, sizeof(int), cudaMemcpyHostToDevice));
  return HPX_OK;
}

hpx_status hpx_campaign_assign(hpx_campaign* c, int32_t batch, float* noise_power, void* stream) {
  if (!c || !noise_power) return hpx_fail(HPX_ERR_ARG, "campaign_assign: null argument");
  if (batch < 1 || batch > c->max_batch) return hpx_fail(HPX_ERR_ARG, "campaign_assign: batch must be in [1, %d]", c->max_batch);
  k_assign<<<1, 256, sizeof(int) * c->L, as_stream(stream)>>>(c->L, batch, c->d_power, c->d_confident, c->d_count,
                                                               (unsigned long long)c->max_drops, noise_power,
                                                               c->d_level);
  HPX_LAUNCHED("campaign assign");
  return HPX_OK;
}

hpx_status hpx_campaign_accumulate(hpx_campaign* c, int32_t batch, const uint32_t* errors, void* stream) {
  if (!c || !errors) return hpx_fail(HPX_ERR_ARG, "campaign_accumulate: null argument");
  if (batch < 1 || batch > c->max_batch)
    return hpx_fail(HPX_ERR_ARG, "campaign_accumulate: batch must be in [1, %d]", c->max_batch);
  cudaStream_t s = as_stream(stream);
  k_accumulate<<<(batch + 255) / 256, 256, 0, s>>>(batch, c->d_level, errors, 1.0 / c->bits_per_drop, c->d_sum, c->d_sq,
                                                   c->d_count, c->d_errors, c->d_flags);
  HPX_LAUNCHED("campaign accumulate");
  k_confidence<<<1, 256, 0, s>>>(c->L, c->min_samples, c->accuracy, c->confidence, (unsigned long long)c->max_drops,
                                 c->d_sum, c->d_sq, c->d_count, c->d_confident, c->d_active);
  HPX_LAUNCHED("campaign confidence");
  return HPX_OK;
}

hpx_status hpx_campaign_poll(hpx_campaign* c, int32_t* levels_active, void* stream) {
  if (!c || !levels_active) return hpx_fail(HPX_ERR_ARG, "campaign_poll: null argument");
  cudaStream_t s = as_stream(stream);
  int active = 0;
  unsigned int flags = 0;
  HPX_CUDA(cudaMemcpyAsync(&active, c->d_active, sizeof(int), cudaMemcpyDeviceToHost, s));
  HPX_CUDA(cudaMemcpyAsync(&flags, c->d_flags, sizeof(flags), cudaMemcpyDeviceToHost, s));
  HPX_CUDA(cudaStreamSynchronize(s));
  *levels_active = active;
  if (flags & HPX_DROP_TIMEOUT)
    return hpx_fail(HPX_ERR_TIMEOUT, "campaign: a drop's tensor-core wait ran out (left out of the sums)");
  if (flags)
    return hpx_fail(HPX_ERR_NUMERIC, "campaign: a drop's equalizer met a non-finite pivot (left out of the sums)");
  return HPX_OK;
}

hpx_status hpx_campaign_run(hpx_campaign* c, hpx_link* link, uint64_t seed, int64_t drop0, int32_t batch,
                            int32_t max_batches, int32_t check_every, int64_t* drops_run, int32_t* levels_active,
                            void* stream) {
  if (!c || !link) return hpx_fail(HPX_ERR_ARG, "campaign_run: null argument");
  if (batch < 1 || batch > c->max_batch) return hpx_fail(HPX_ERR_ARG, "campaign_run: batch must be in [1, %d]", c->max_batch);
  if (max_batches < 0 || check_every < 1 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "campaign_run: bad loop bounds");
  cudaStream_t s = as_stream(stream);
  int active = c->L;
  HPX_CUDA(cudaMemcpyAsync(&active, c->d_active, sizeof(int), cudaMemcpyDeviceToHost, s));
  HPX_CUDA(cudaStreamSynchronize(s));
  int64_t done = 0;
  unsigned int flags = 0;
  const int acc_blocks = (batch + 255) / 256;
  for (int b = 0; b < max_batches && active > 0; ++b) {
    k_assign<<<1, 256, sizeof(int) * c->L, s>>>(c->L, batch, c->d_power, c->d_confident, c->d_count,
                                                 (unsigned long long)c->max_drops, c->d_noise, c->d_level);
    HPX_LAUNCHED("campaign assign");
    HPX_TRY(hpx_link_run(link, seed, drop0 + done, batch, c->d_noise, c->d_drop_errors, stream));
    k_accumulate<<<acc_blocks, 256, 0, s>>>(batch, c->d_level, c->d_drop_errors, 1.0 / c->bits_per_drop, c->d_sum,
                                            c->d_sq, c->d_count, c->d_errors, c->d_flags);
    HPX_LAUNCHED("campaign accumulate");
    k_confidence<<<1, 256, 0, s>>>(c->L, c->min_samples, c->accuracy, c->confidence,
                                   (unsigned long long)c->max_drops, c->d_sum, c->d_sq, c->d_count, c->d_confident,
                                   c->d_active);
    HPX_LAUNCHED("campaign confidence");
    done += batch;
    if ((b + 1) % check_every == 0 || b + 1 == max_batches) {
      HPX_CUDA(cudaMemcpyAsync(&active, c->d_active, sizeof(int), cudaMemcpyDeviceToHost, s));
      HPX_CUDA(cudaMemcpyAsync(&flags, c->d_flags, sizeof(flags), cudaMemcpyDeviceToHost, s));
      HPX_CUDA(cudaStreamSynchronize(s));
      if (flags) break;
    }
  }
  if (drops_run) *drops_run = done;
  if (levels_active) *levels_active = active;
  if (flags & HPX_DROP_TIMEOUT)
    return hpx_fail(HPX_ERR_TIMEOUT, "campaign_run: a drop's tensor-core wait ran out (left out of the sums)");
  if (flags)
    return hpx_fail(HPX_ERR_NUMERIC, "campaign_run: a drop's equalizer met a non-finite pivot (left out of the sums)");
  return HPX_OK;
}

hpx_status hpx_campaign_results(const hpx_campaign* c, int64_t* drops, int64_t* errors, double* ber_sum,
                                double* ber_sq, int32_t* confident) {
  if (!c) return hpx_fail(HPX_ERR_ARG, "campaign_results: null argument");
  const size_t L = c->L;
  if (drops) HPX_CUDA(cudaMemcpy(drops, c->d_count, sizeof(int64_t) * L, cudaMemcpyDeviceToHost));
  if (errors) HPX_CUDA(cudaMemcpy(errors, c->d_errors, sizeof(int64_t) * L, cudaMemcpyDeviceToHost));
  if (ber_sum) HPX_CUDA(cudaMemcpy(ber_sum, c->d_sum, sizeof(double) * L, cudaMemcpyDeviceToHost));
  if (ber_sq) HPX_CUDA(cudaMemcpy(ber_sq, c->d_sq, sizeof(double) * L, cudaMemcpyDeviceToHost));
  if (confident) HPX_CUDA(cudaMemcpy(confident, c->d_confident, sizeof(int32_t) * L, cudaMemcpyDeviceToHost));
  return HPX_OK;
}

}  // extern "C"
