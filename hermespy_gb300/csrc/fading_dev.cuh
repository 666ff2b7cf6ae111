// Device helpers shared by the fading and detection kernels.
#pragma once

#include "hpx_internal.cuh"

struct FadingConst {
  int L, S, S1, nrx, ntx, D;
  int G;                 // distinct delays
  const int32_t* delay;  // [L]
  const int32_t* gfirst; // [G + 1] first tap of each delay group (delays are sorted)
  const int32_t* gdelay; // [G] delay of each group
  const float* amp;      // [L][2] (nlos, los)
};

static inline FadingConst fading_const(const hpx_fading* f) {
  FadingConst c;
  c.L = f->L;
  c.S = f->S;
  c.S1 = f->S1;
  c.nrx = f->nrx;
  c.ntx = f->ntx;
  c.D = f->max_delay;
  c.G = f->G;
  c.delay = f->d_delay;
  c.gfirst = f->d_group;
  c.gdelay = f->d_group ? f->d_group + f->G + 1 : nullptr;
  c.amp = f->d_amp;
  return c;
}

// Angular rate in rad/sample of a fixed-point phase increment.
__device__ __forceinline__ float fixed_rate(int64_t w) { return (float)w * 3.4061215800865545e-19f; }  // 2 pi / 2^64

// Dirichlet kernel D_N(w) = (1/N) sum_{m<N} exp(i w m) * exp(-i w (N-1)/2) = sin(N w/2) / (N sin(w/2)).
__device__ __forceinline__ float dirichlet(float w, int N) {
  const float sh = sinf(0.5f * w);
  if (fabsf(sh) < 1e-30f) return 1.0f;
  return sinf(0.5f * (float)N * w) / ((float)N * sh);
}

// Average of every tap over the N samples starting at `ws`:
//   hb[l] = (1/N) sum_{t=ws}^{ws+N-1} h_l[t]
// in closed form per sinusoid (geometric series), written to shared `hb` [L].
// `scratch` holds L*S1 float2. Must be called by all threads of the block.
__device__ __forceinline__ void tap_averages(const FadingConst& fc, const int64_t* __restrict__ W,
                                             const int64_t* __restrict__ P0, int64_t ws, int N, float2* hb,
                                             float2* scratch) {
  const int total = fc.L * fc.S1;
  for (int q = threadIdx.x; q < total; q += blockDim.x) {
    const int l = q / fc.S1, n = q - l * fc.S1;
    const int64_t w = W[q];
    // phase at the window centre: P0 + W ws + W (N-1)/2
    const uint64_t p = (uint64_t)P0[q] + (uint64_t)w * (uint64_t)ws + (uint64_t)w * (uint64_t)(N / 2 - 1) +
                       (uint64_t)(w >> 1);
    float s, c;
    __sincosf(fixed_to_angle(p), &s, &c);
    const float a = fc.amp[2 * l + (n < fc.S ? 0 : 1)] * dirichlet(fixed_rate(w), N);
    scratch[q] = make_float2(a * c, a * s);
  }
  __syncthreads();
  for (int l = threadIdx.x; l < fc.L; l += blockDim.x) {
    float2 acc = make_float2(0.f, 0.f);
    for (int n = 0; n < fc.S1; ++n) acc = cadd(acc, scratch[l * fc.S1 + n]);
    hb[l] = acc;
  }
  __syncthreads();
}

// Frequency response sum_l hb[l] exp(-2 pi i bin d_l / N) at one FFT bin, for taps
// with delays below N (longer delays fall outside the N-point transform).
__device__ __forceinline__ float2 tap_response(const FadingConst& fc, const float2* hb, const int32_t* delay_s,
                                               const float2* __restrict__ tw, int bin, int N) {
  float2 g = make_float2(0.f, 0.f);
  for (int l = 0; l < fc.L; ++l) {
    const int d = delay_s[l];
    if (d >= N) continue;
    cfma(g, hb[l], __ldg(tw + ((bin * d) & (N - 1))));
  }
  return g;
}
