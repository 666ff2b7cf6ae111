// Uneven batch: drops of different antenna counts, FFT sizes, frame lengths,
// modulation orders, channels and SNRs in ONE persistent launch.
//
// Every CTA takes whole drops from an atomic work counter (drops ordered longest
// first) and runs the complete drop on its own: fading realization, transmitter
// (Philox bits, QAM, IFFT, CP), sum-of-sinusoids propagation with AWGN, receiver
// FFT, ideal CSI, LMMSE equalization, hard demap and bit-error count, staged through
// a per-CTA scratch slot in HBM. The per-sample arithmetic of every stage is the
// homogeneous engine's (same fixed-point phases, Taylor tiles per transmit count,
// FMA order, FFT plans, ideal CSI and Cholesky), so a drop of the batch gives the
// error count the homogeneous pipeline gives for that drop. The block size, CTAs
// per SM and schedule are picked by hpx_uneven_tune (timed candidates), and the
// launch can be captured into a CUDA graph and replayed.
//
// The frame of a drop: fft_size N, U = floor(0.586 N) used data subcarriers, cyclic
// prefix N * 72 / 1024, DC suppression, num_words data words, ideal CSI. The
// channel: num_taps Rayleigh taps spaced tap_spacing seconds with power
// 10^(-decay k / 10), num_sinusoids sinusoids, sampling rate N * subcarrier_spacing.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

#include "equalize_dev.cuh"
#include "fading_dev.cuh"
#include "fft.cuh"

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr int UMAX_THREADS = 256;

struct UFrame {  // device view of one frame configuration
  int N, W, C, m, order, cp, T;
  const float2* stage_twiddle;
  const float2* twiddle;
  const int32_t* bins;
  const float2* constellation;      // MSB-first bit value order
  const float2* constellation_lsb;  // LSB-first bit value order (bit-reversed index)
};

struct UDrop {  // one drop of the batch
  int frame, nrx, ntx, L, D, K, BT;  // K: Taylor degree (-1: direct sinusoid sums), BT: propagation tile
  int taps;                          // offset into the delay / amplitude arrays
  double nlos_rate, los_rate;        // rad/sample
};

struct QamTables {
  QamDemapTable t[9];  // indexed by log2(order)
};

struct UArgs {
  const UDrop* drops;
  const UFrame* frames;
  const int32_t* delay;  // [taps]
  const float* amp;      // [taps][2] (nlos, los)
  const int32_t* order;  // schedule: drop indices, longest first
  int num_drops, S;
  unsigned int* counter;
  unsigned char* scratch;
  size_t slot_bytes, off_x, off_y, off_grid;  // per-slot layout (state at 0)
  const float* noise_power;
  uint64_t seed;
  PhiloxKeys noise_keys;  // the seed's round keys, for the AWGN of propagation
  int64_t drop0;
  uint32_t* errors;
};

__device__ __forceinline__ int column_of_bin_u(int b, int N) {  // DC suppression on
  if (b >= N / 2) return b - N / 2;
  return b == 0 ? N - 1 : b + N / 2 - 1;
}

// ------------------------------------------------------------------ stages
// Fading realization of drop `drop` (the homogeneous k_fading_params, no correlation).
__device__ void u_realize(const UDrop& d, int S, uint64_t seed, int64_t drop, int64_t* Wp, int64_t* P0, float2* Sm) {
  const int L = d.L, S1 = S + 1, nsp = d.nrx * d.ntx;
  auto word = [&](int idx) -> uint32_t {
    const uint4 r = hpx_random_block(seed, drop, 0u, HPX_DOMAIN_FADING, (uint32_t)(idx >> 2));
    return uint4_get(r, idx & 3);
  };
  auto uniform = [&](int idx) -> double { return u01_f64(word(idx)); };
  auto u01 = [](uint32_t w) { return fmaf(__uint2float_rn(w), 2.3283064365386963e-10f, 1.1641532182693481e-10f); };
  constexpr double kInv2Pi = 0.15915494309189535;
  const double inv_s = 1.0 / (double)(S > 0 ? S : 1);
  const float inv_sf = 1.0f / (float)(S > 0 ? S : 1);
  const float rate_n = (float)(d.nlos_rate * kInv2Pi), rate_l = (float)(d.los_rate * kInv2Pi);
  const bool fp32_rates = fmax(fabs(d.nlos_rate), fabs(d.los_rate)) * kInv2Pi <= kFp32RateLimit;
  for (int q = threadIdx.x; q < L * S1; q += blockDim.x) {  // the same arithmetic as k_fading_params<0>
    const int l = q / S1, n = q - l * S1;
    const uint32_t wu = n < S ? word(nsp + L + l * S + n) : word(nsp + l);
    if (fp32_rates)
      Wp[q] = n < S ? rate_to_fixed(rate_n * cospif(((float)(2 * n + 1) + 2.0f * u01(wu)) * inv_sf))
                    : rate_to_fixed(rate_l * cospif(2.0f * u01(wu)));
    else
      Wp[q] = turns_to_fixed(kInv2Pi * (n < S ? d.nlos_rate * cospi((2.0 * n + 1.0 + 2.0 * u01_f64(wu)) * inv_s)
                                              : d.los_rate * cospi(2.0 * u01_f64(wu))));
    P0[q] = phase_from_word(n < S ? word(nsp + 2 * L + L * S + l * S + n) : word(nsp + L + L * S + l));
  }
  for (int j = threadIdx.x; j < nsp; j += blockDim.x) {
    double s, c;
    sincospi(2.0 * uniform(j), &s, &c);
    Sm[j] = make_float2((float)c, (float)s);
  }
}

// Transmitter of all (stream, word) units of the drop (k_ofdm_tx, bits mode).
template <int N>
__device__ void u_tx(const UFrame& fr, int ntx, uint64_t seed, int64_t drop, float2* x, unsigned char* sm) {
  constexpr int TP = fft::Plan<N>::TP;
  constexpr int PN = fft::padded<N>();
  const int F = blockDim.x / TP, g = threadIdx.x / TP, t = threadIdx.x - g * TP;
  const int BW = staged_bit_words(fr.C, fr.m);
  float2* buf = reinterpret_cast<float2*>(sm) + g * PN;
  uint32_t* bits = reinterpret_cast<uint32_t*>(reinterpret_cast<float2*>(sm) + F * PN) + g * BW;
  const float scale = rsqrtf((float)N);
  const int units = ntx * fr.W;
  for (int base = 0; base < units; base += F) {
    const int unit = base + g;
    const bool valid = unit < units;
    const int s = valid ? unit / fr.W : 0, w = valid ? unit - s * fr.W : 0;
    const int64_t k0 = (int64_t)w * fr.C;
    const int64_t blk0 = ((k0 * fr.m) >> 5) >> 2, blk1 = (((k0 + fr.C) * fr.m - 1) >> 5) >> 2;
    if (valid)
      for (int64_t blk = blk0 + t; blk <= blk1; blk += TP) {
        const uint4 r = hpx_random_block(seed, drop, (uint32_t)s, HPX_DOMAIN_BITS, (uint32_t)blk);
        uint32_t* dst = bits + (blk - blk0) * 4;
        dst[0] = r.x;
        dst[1] = r.y;
        dst[2] = r.z;
        dst[3] = r.w;
      }
    __syncthreads();
    // data element k0 + c sits at bit c m + (k0 m) mod 128 of the staged words; the
    // LSB-first window indexes the bit-reversed constellation directly
    const int off0 = (int)((k0 * fr.m) & 127);
    const uint32_t mask = (1u << fr.m) - 1u;
    auto load = [&](int b) -> float2 {
      if (!valid) return make_float2(0.f, 0.f);
      const int c = column_of_bin_u(b, N);
      if (c >= fr.C) return make_float2(0.f, 0.f);
      const int d = c * fr.m + off0, wi = d >> 5;
      const float2 v = __ldg(fr.constellation_lsb + (__funnelshift_r(bits[wi], bits[wi + 1], d & 31) & mask));
      return cscale(v, scale);
    };
    float2* dst = x + (int64_t)s * fr.T + (int64_t)w * (N + fr.cp);
    const int P = fr.cp;
    auto store = [&](int n, float2 v) {
      if (!valid) return;
      dst[P + n] = v;
      if (n >= N - P) dst[n - (N - P)] = v;
    };
    fft::transform<N, true>(buf, t, fr.stage_twiddle, load, store);
    __syncthreads();
  }
}

// Receiver FFT of all (antenna, word) units (k_ofdm_rx).
template <int N>
__device__ void u_rx(const UFrame& fr, int nrx, int TD, const float2* y, float2* grid, unsigned char* sm) {
  constexpr int TP = fft::Plan<N>::TP;
  constexpr int PN = fft::padded<N>();
  const int F = blockDim.x / TP, g = threadIdx.x / TP, t = threadIdx.x - g * TP;
  float2* buf = reinterpret_cast<float2*>(sm) + g * PN;
  const float scale = rsqrtf((float)N);
  const int units = nrx * fr.W;
  for (int base = 0; base < units; base += F) {
    const int unit = base + g;
    const bool valid = unit < units;
    const int r = valid ? unit / fr.W : 0, w = valid ? unit - r * fr.W : 0;
    const float2* src = y + (int64_t)r * TD + (int64_t)w * (N + fr.cp) + fr.cp;
    float2* dst = grid + ((int64_t)r * fr.W + w) * fr.C;
    auto load = [&](int n) -> float2 { return valid ? src[n] : make_float2(0.f, 0.f); };
    auto store = [&](int b, float2 v) {
      const int c = column_of_bin_u(b, N);
      if (valid && c < fr.C) dst[c] = cscale(v, scale);
    };
    fft::transform<N, false>(buf, t, fr.stage_twiddle, load, store);
    __syncthreads();
  }
}

// Propagation with AWGN (k_propagate: the same tiles, Taylor terms, FMA order and
// noise streams; any transmit count up to MAXA, every thread a set of sample pairs).
template <int MAXA>
__device__ void u_propagate(const UDrop& d, const FadingConst& fc, int T, const int64_t* Wp, const int64_t* P0,
                            const float2* Sm, const int* dl, const float2* x, float2* y, float np,
                            const PhiloxKeys& nk, int64_t drop, unsigned char* sm) {
  const int L = d.L, S1 = fc.S1, D = d.D, nrx = d.nrx, ntx = d.ntx, K = d.K, BT = d.BT;
  const int XW = (BT + D + 2) & ~1;
  const int TD = T + D;
  const bool direct = K < 0;
  const int KK = direct ? 0 : K;
  float* xp = reinterpret_cast<float*>(sm);  // [ntx][4][XW]
  float2* terms = reinterpret_cast<float2*>(sm);
  const int region = direct ? 2 * ntx * XW : max(2 * ntx * XW, L * S1 * (KK + 1));
  float2* coef = reinterpret_cast<float2*>(sm) + region;  // [L][K+1]
  const float sigma = sqrtf(0.5f * np);
  for (int m0 = 0; m0 < TD; m0 += BT) {
    if (!direct) {
      const float H = 0.5f * BT;
      for (int q = threadIdx.x; q < L * S1; q += blockDim.x) {
        const int l = q / S1, n = q - l * S1;
        const int64_t tc = (int64_t)m0 - dl[l] + BT / 2;
        const uint64_t p = (uint64_t)P0[q] + (uint64_t)Wp[q] * (uint64_t)tc;
        float s, c;
        __sincosf(fixed_to_angle(p), &s, &c);
        const float a = fc.amp[2 * l + (n < fc.S ? 0 : 1)];
        const float wh = fixed_rate(Wp[q]) * H;
        float2 tt = make_float2(a * c, a * s);
        float2* dst = terms + q * (KK + 1);
        dst[0] = tt;
        for (int k = 1; k <= KK; ++k) {
          const float f = wh / (float)k;
          tt = make_float2(-tt.y * f, tt.x * f);
          dst[k] = tt;
        }
      }
      __syncthreads();
      for (int q = threadIdx.x; q < L * (KK + 1); q += blockDim.x) {
        const int l = q / (KK + 1), k = q - l * (KK + 1);
        float2 acc = make_float2(0.f, 0.f);
        for (int n = 0; n < S1; ++n) acc = cadd(acc, terms[(l * S1 + n) * (KK + 1) + k]);
        coef[q] = acc;
      }
    }
    __syncthreads();  // terms consumed: the tile may overwrite them
    for (int tx = 0; tx < ntx; ++tx) {
      const float2* xr = x + (int64_t)tx * T;
      float* pl = xp + tx * 4 * XW;
      for (int j = threadIdx.x; j <= XW; j += blockDim.x) {
        const int t = m0 - D + j;
        const float2 val = (t >= 0 && t < T) ? xr[t] : make_float2(0.f, 0.f);
        if (j < XW) {
          pl[j] = val.x;
          pl[XW + j] = val.y;
        }
        if (j > 0) {
          pl[2 * XW + j - 1] = val.x;
          pl[3 * XW + j - 1] = val.y;
        }
      }
    }
    __syncthreads();
    for (int pi = threadIdx.x; pi < BT / 2; pi += blockDim.x) {
      const int jp = 2 * pi;
      const int m = m0 + jp;
      if (m >= TD) continue;
      float2 zr[MAXA], zi[MAXA];
#pragma unroll
      for (int tx = 0; tx < MAXA; ++tx) zr[tx] = zi[tx] = make_float2(0.f, 0.f);
      float2 up[9];
      const float u0 = ((float)jp - 0.5f * BT) / (0.5f * BT);
      const float u1 = ((float)(jp + 1) - 0.5f * BT) / (0.5f * BT);
      up[0] = make_float2(1.0f, 1.0f);
#pragma unroll
      for (int k = 1; k <= 8; ++k) up[k] = make_float2(up[k - 1].x * u0, up[k - 1].y * u1);
      for (int l = 0; l < L; ++l) {
        const int dd = dl[l];
        float2 hx, hy;
        if (direct) {
          const float an = fc.amp[2 * l], al = fc.amp[2 * l + 1];
          const int64_t* Wl = Wp + l * S1;
          const int64_t* Pl = P0 + l * S1;
          float2 h0 = make_float2(0.f, 0.f), h1 = make_float2(0.f, 0.f);
          for (int side = 0; side < 2; ++side) {
            const int64_t t = (int64_t)m + side - dd;
            float2 acc = make_float2(0.f, 0.f);
            for (int n = 0; n < fc.S; ++n) {
              const uint64_t p = (uint64_t)Pl[n] + (uint64_t)Wl[n] * (uint64_t)t;
              float s, c;
              __sincosf(fixed_to_angle(p), &s, &c);
              acc.x += c;
              acc.y += s;
            }
            float2 h = make_float2(an * acc.x, an * acc.y);
            {
              const uint64_t p = (uint64_t)Pl[fc.S] + (uint64_t)Wl[fc.S] * (uint64_t)t;
              float s, c;
              __sincosf(fixed_to_angle(p), &s, &c);
              h.x += al * c;
              h.y += al * s;
            }
            if (side == 0) h0 = h;
            else h1 = h;
          }
          hx = make_float2(h0.x, h1.x);
          hy = make_float2(h0.y, h1.y);
        } else {
          const float2* cl = coef + l * (KK + 1);
          float2 ax = make_float2(cl[0].x, cl[0].x), ay = make_float2(cl[0].y, cl[0].y);
#pragma unroll
          for (int k = 1; k <= 8; ++k) {  // static indices keep up[] in registers
            if (k > KK) break;
            const float2 ck = cl[k];
            ax = __ffma2_rn(make_float2(ck.x, ck.x), up[k], ax);
            ay = __ffma2_rn(make_float2(ck.y, ck.y), up[k], ay);
          }
          hx = ax;
          hy = ay;
        }
        const int odd = (D - dd) & 1;
        const float* src = xp + 2 * odd * XW - odd;
        const int s0 = jp - dd + D;
        const float2 nhy = __fmul2_rn(hy, make_float2(-1.f, -1.f));
#pragma unroll
        for (int tx = 0; tx < MAXA; ++tx) {
          if (tx >= ntx) break;
          const float* pl = src + tx * 4 * XW + s0;
          const float2 re = *reinterpret_cast<const float2*>(pl);
          const float2 im = *reinterpret_cast<const float2*>(pl + XW);
          zr[tx] = __ffma2_rn(hx, re, zr[tx]);
          zr[tx] = __ffma2_rn(nhy, im, zr[tx]);
          zi[tx] = __ffma2_rn(hx, im, zi[tx]);
          zi[tx] = __ffma2_rn(hy, re, zi[tx]);
        }
      }
      for (int rx = 0; rx < nrx; ++rx) {
        float2 ore = make_float2(0.f, 0.f), oim = make_float2(0.f, 0.f);
#pragma unroll
        for (int tx = 0; tx < MAXA; ++tx) {
          if (tx >= ntx) break;
          const float2 sv = Sm[rx * ntx + tx];
          const float2 sr = make_float2(sv.x, sv.x), si = make_float2(sv.y, sv.y), nsi = make_float2(-sv.y, -sv.y);
          ore = __ffma2_rn(sr, zr[tx], ore);
          ore = __ffma2_rn(nsi, zi[tx], ore);
          oim = __ffma2_rn(sr, zi[tx], oim);
          oim = __ffma2_rn(si, zr[tx], oim);
        }
        if (np > 0.0f) {
          const uint4 w = hpx_random_block_k(nk, drop, (uint32_t)rx, HPX_DOMAIN_NOISE, (uint32_t)(m >> 1));
          const float2 n0 = box_muller(w.x, w.y);
          const float2 n1 = box_muller(w.z, w.w);
          ore = __ffma2_rn(make_float2(sigma, sigma), make_float2(n0.x, n1.x), ore);
          oim = __ffma2_rn(make_float2(sigma, sigma), make_float2(n0.y, n1.y), oim);
        }
        float2* yr = y + (int64_t)rx * TD;
        yr[m] = make_float2(ore.x, oim.x);
        if (m + 1 < TD) yr[m + 1] = make_float2(ore.y, oim.y);
      }
    }
    __syncthreads();
  }
}

// Ideal CSI + equalization + demap + count of one element (k_detect_ideal); `fin`
// turns false on a non-finite equalizer pivot.
template <int NRX, int NTX>
__device__ __forceinline__ unsigned int u_element(int mode, float2 g, const float2* Sm, const float2* Mg,
                                                  const float2* grid, int W, int C, int w, int c, float s2,
                                                  const QamDemapTable& qt, const uint32_t* bitsm, int BW,
                                                  int64_t wofs, int64_t k, int m, bool& fin) {
  const int out_streams = (mode == HPX_EQ_ZF && NRX == 1) ? 1 : NTX;
  float2 yv[NRX], xv[NTX];
#pragma unroll
  for (int r = 0; r < NRX; ++r) yv[r] = grid[((int64_t)r * W + w) * C + c];
  if (gram_equalizer<NRX, NTX>(mode)) {  // H = S g: the Gram from S^H S
    fin &= equalize_spatial<NRX, NTX>(mode, Sm, Mg, g, yv, s2, xv);
  } else {
    float2 H[NRX][NTX];
#pragma unroll
    for (int r = 0; r < NRX; ++r)
#pragma unroll
      for (int t = 0; t < NTX; ++t) H[r][t] = cmul(Sm[r * NTX + t], g);
    fin &= equalize_one<NRX, NTX>(mode, H, yv, s2, xv);
  }
  unsigned int e = 0;
  uint32_t dec[NTX];
  qam_decide_n<NTX>(qt, xv, out_streams, dec);
#pragma unroll
  for (int t = 0; t < NTX; ++t) {
    const uint32_t rx_v = dec[t];
    const uint32_t tx_v = extract_bits_msb(bitsm + t * BW - wofs, k * m, m);
    e += __popc(rx_v ^ tx_v);
  }
  return e;
}

template <int NRX, int MAXA>
__device__ __forceinline__ unsigned int u_element_tx(int ntx, int mode, float2 g, const float2* Sm, const float2* Mg,
                                                     const float2* grid, int W, int C, int w, int c, float s2,
                                                     const QamDemapTable& qt, const uint32_t* bitsm, int BW,
                                                     int64_t wofs, int64_t k, int m, bool& fin) {
  switch (ntx) {
    case 1: return u_element<NRX, 1>(mode, g, Sm, Mg, grid, W, C, w, c, s2, qt, bitsm, BW, wofs, k, m, fin);
    case 2: return u_element<NRX, 2>(mode, g, Sm, Mg, grid, W, C, w, c, s2, qt, bitsm, BW, wofs, k, m, fin);
    case 4:
      if constexpr (MAXA >= 4) return u_element<NRX, 4>(mode, g, Sm, Mg, grid, W, C, w, c, s2, qt, bitsm, BW, wofs, k, m, fin);
      else return 0u;
    default:
      if constexpr (MAXA >= 8) return u_element<NRX, 8>(mode, g, Sm, Mg, grid, W, C, w, c, s2, qt, bitsm, BW, wofs, k, m, fin);
      else return 0u;  // not reached: the batch's kernel covers its largest antenna count
  }
}

// The thread's share of the drop's bit errors; `fin` turns false if one of its
// elements had a non-finite equalizer pivot.
template <int MAXA>
__device__ unsigned int u_detect(const UDrop& d, const UFrame& fr, const FadingConst& fc, const int64_t* Wp,
                                 const int64_t* P0, const float2* Sm, float2* Mg, const int* dl, const float2* grid,
                                 float s2, const QamDemapTable& qt, uint64_t seed, int64_t drop, unsigned char* sm,
                                 bool& fin) {
  // M = S^H S of the drop's spatial response (visible after the first word's tap averages)
  for (int q = threadIdx.x; q < d.ntx * d.ntx; q += blockDim.x) {
    const int i = q / d.ntx, j = q - i * d.ntx;
    float2 acc = make_float2(0.f, 0.f);
    for (int r = 0; r < d.nrx; ++r) cfmac(acc, Sm[r * d.ntx + i], Sm[r * d.ntx + j]);
    Mg[q] = acc;
  }
  float2* hb = reinterpret_cast<float2*>(sm);
  float2* scratch = hb + d.L;
  uint32_t* bitsm = reinterpret_cast<uint32_t*>(scratch + d.L * fc.S1);
  const int BW = staged_bit_words(fr.C, fr.m);
  unsigned int local = 0;
  for (int w = 0; w < fr.W; ++w) {
    const int64_t k0 = (int64_t)w * fr.C;
    // bits of every stream of this word (stage_bits of the homogeneous receiver)
    const int64_t blk0 = ((k0 * fr.m) >> 5) >> 2, blk1 = (((k0 + fr.C) * fr.m - 1) >> 5) >> 2;
    const int nblk = (int)(blk1 - blk0 + 1);
    for (int q = threadIdx.x; q < nblk * d.ntx; q += blockDim.x) {
      const int s = q / nblk;
      const int64_t blk = blk0 + (q - s * nblk);
      const uint4 r = hpx_random_block(seed, drop, (uint32_t)s, HPX_DOMAIN_BITS, (uint32_t)blk);
      uint32_t* dst = bitsm + s * BW + (blk - blk0) * 4;
      dst[0] = r.x;
      dst[1] = r.y;
      dst[2] = r.z;
      dst[3] = r.w;
    }
    tap_averages(fc, Wp, P0, (int64_t)w * (fr.N + fr.cp) + fr.cp, fr.N, hb, scratch);  // ends with __syncthreads
    const int64_t wofs = blk0 * 4;
    for (int j = threadIdx.x; j < fr.C; j += blockDim.x) {
      const float2 g = tap_response(fc, hb, dl, fr.twiddle, fr.bins[j], fr.N);
      const int64_t k = k0 + j;
      switch (d.nrx) {
        case 1: local += u_element_tx<1, MAXA>(d.ntx, HPX_EQ_LMMSE, g, Sm, Mg, grid, fr.W, fr.C, w, j, s2, qt, bitsm, BW, wofs, k, fr.m, fin); break;
        case 2: local += u_element_tx<2, MAXA>(d.ntx, HPX_EQ_LMMSE, g, Sm, Mg, grid, fr.W, fr.C, w, j, s2, qt, bitsm, BW, wofs, k, fr.m, fin); break;
        case 4:
          if constexpr (MAXA >= 4) local += u_element_tx<4, MAXA>(d.ntx, HPX_EQ_LMMSE, g, Sm, Mg, grid, fr.W, fr.C, w, j, s2, qt, bitsm, BW, wofs, k, fr.m, fin);
          break;
        default:
          if constexpr (MAXA >= 8) local += u_element_tx<8, MAXA>(d.ntx, HPX_EQ_LMMSE, g, Sm, Mg, grid, fr.W, fr.C, w, j, s2, qt, bitsm, BW, wofs, k, fr.m, fin);
          break;
      }
    }
    __syncthreads();
  }
  return local;
}

// ---------------------------------------------------------- persistent kernel
// MINB = 1: registers as the largest stage needs; MINB = 2 / 3: capped so that two / three
// CTAs of 256 threads share an SM (three only without the 8 x 8 stages: 80 registers
// without spills; the autotuner measures every variant the batch can use).
template <int MINB, int MAXA>
__global__ void __launch_bounds__(UMAX_THREADS, MINB) k_uneven(UArgs a, const __grid_constant__ QamTables qts) {
  extern __shared__ float4 smem4[];
  __shared__ int s_drop;
  __shared__ unsigned int s_sum[32];
  unsigned char* base = reinterpret_cast<unsigned char*>(smem4);
  int* dl = reinterpret_cast<int*>(base);                      // [64] tap delays
  float2* Sm = reinterpret_cast<float2*>(base + 256);          // [64] spatial
  float2* Mg = Sm + 64;                                        // [64] S^H S
  unsigned char* work = base + 256 + 128 * sizeof(float2);     // stage union
  unsigned char* slot = a.scratch + (size_t)blockIdx.x * a.slot_bytes;
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned int i = atomicAdd(a.counter, 1u);
      s_drop = i < (unsigned)a.num_drops ? a.order[i] : -1;
    }
    __syncthreads();
    const int b = s_drop;
    if (b < 0) return;
    const UDrop d = a.drops[b];
    const UFrame fr = a.frames[d.frame];
    const int64_t drop = a.drop0 + b;
    const int S1 = a.S + 1;
    int64_t* Wp = reinterpret_cast<int64_t*>(slot);
    int64_t* P0 = Wp + d.L * S1;
    float2* x = reinterpret_cast<float2*>(slot + a.off_x);
    float2* y = reinterpret_cast<float2*>(slot + a.off_y);
    float2* grid = reinterpret_cast<float2*>(slot + a.off_grid);
    FadingConst fc;
    fc.L = d.L;
    fc.S = a.S;
    fc.S1 = S1;
    fc.nrx = d.nrx;
    fc.ntx = d.ntx;
    fc.D = d.D;
    fc.delay = a.delay + d.taps;
    fc.G = 0;  // delay groups are a propagate-kernel table; this kernel walks the taps
    fc.gfirst = fc.gdelay = nullptr;
    fc.amp = a.amp + 2 * d.taps;
    for (int l = threadIdx.x; l < d.L; l += blockDim.x) dl[l] = fc.delay[l];
    u_realize(d, a.S, a.seed, drop, Wp, P0, Sm);
    __syncthreads();
    switch (fr.N) {
      case 128: u_tx<128>(fr, d.ntx, a.seed, drop, x, work); break;
      case 256: u_tx<256>(fr, d.ntx, a.seed, drop, x, work); break;
      case 512: u_tx<512>(fr, d.ntx, a.seed, drop, x, work); break;
      case 1024: u_tx<1024>(fr, d.ntx, a.seed, drop, x, work); break;
      default: u_tx<2048>(fr, d.ntx, a.seed, drop, x, work); break;
    }
    const float np = a.noise_power[b];
    u_propagate<MAXA>(d, fc, fr.T, Wp, P0, Sm, dl, x, y, np, a.noise_keys, drop, work);
    switch (fr.N) {
      case 128: u_rx<128>(fr, d.nrx, fr.T + d.D, y, grid, work); break;
      case 256: u_rx<256>(fr, d.nrx, fr.T + d.D, y, grid, work); break;
      case 512: u_rx<512>(fr, d.nrx, fr.T + d.D, y, grid, work); break;
      case 1024: u_rx<1024>(fr, d.nrx, fr.T + d.D, y, grid, work); break;
      default: u_rx<2048>(fr, d.nrx, fr.T + d.D, y, grid, work); break;
    }
    bool fin = finite_f(np);  // a NaN / inf noise power is an invalid drop too
    const unsigned int e = u_detect<MAXA>(d, fr, fc, Wp, P0, Sm, Mg, dl, grid, np, qts.t[fr.m], a.seed, drop, work, fin);
    // drop total
    unsigned int v = e;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) s_sum[threadIdx.x >> 5] = v;
    const int any_bad = __syncthreads_or(!fin);
    if (threadIdx.x == 0) {
      unsigned int tot = 0;
      for (int i = 0; i < (int)(blockDim.x >> 5); ++i) tot += s_sum[i];
      a.errors[b] = any_bad ? (tot | HPX_DROP_NUMERIC) : tot;
    }
    __syncthreads();
  }
}

int taylor_degree_of(double rate_max, int BT) {  // as taylor_degree in fading.cu
  double wmax = std::fmod(rate_max, 2.0 * kPi);
  if (wmax > kPi) wmax = 2.0 * kPi - wmax;
  if (rate_max > kPi) wmax = kPi;
  const double theta = wmax * 0.5 * BT;
  const int degrees[3] = {2, 4, 8};
  for (int K : degrees) {
    double bound = 1.0;
    for (int k = 1; k <= K + 1; ++k) bound *= theta / k;
    if (bound <= 1e-7) return K;
  }
  return -1;
}

size_t round_up(size_t v) { return (v + 255) / 256 * 256; }

}  // namespace

struct hpx_uneven {
  int B = 0, S = 0;
  std::vector<hpx_frame*> frames;
  std::vector<int64_t> bits;  // data bits per drop
  std::vector<double> cost;   // schedule weights
  UDrop* d_drops = nullptr;
  UFrame* d_frames = nullptr;
  int32_t* d_delay = nullptr;
  float* d_amp = nullptr;
  int32_t* d_order = nullptr;
  unsigned int* d_counter = nullptr;
  unsigned char* d_scratch = nullptr;
  size_t slot_bytes = 0, off_x = 0, off_y = 0, off_grid = 0, smem = 0;
  int max_slots = 0;
  int threads = 256, blocks_per_sm = 1, num_sms = 1, variant = 0;
  int maxa = 8;  // largest antenna count of the batch (2, 4 or 8): selects the kernel instantiation
  QamTables qts;
  cudaGraphExec_t graph = nullptr;
  cudaGraph_t graph_def = nullptr;
};

namespace {

void uneven_release(hpx_uneven* u) {
  if (!u) return;
  if (u->graph) cudaGraphExecDestroy(u->graph);
  if (u->graph_def) cudaGraphDestroy(u->graph_def);
  for (hpx_frame* f : u->frames) hpx_frame_destroy(f);
  void* p[] = {u->d_drops, u->d_frames, u->d_delay, u->d_amp, u->d_order, u->d_counter, u->d_scratch};
  for (void* q : p)
    if (q) cudaFree(q);
  delete u;
}

// The persistent kernel for a register variant (0: registers as needed, 1: capped for two
// CTAs of 256 threads per SM) and the batch's largest antenna count: a batch without
// 8-antenna drops runs an instantiation without the 8 x 8 stages and their registers.
using UnevenKernel = void (*)(UArgs, QamTables);
UnevenKernel uneven_kernel(int variant, int maxa) {
  if (variant == 2) return maxa <= 2 ? k_uneven<3, 2> : (maxa <= 4 ? k_uneven<3, 4> : nullptr);
  if (maxa <= 2) return variant ? k_uneven<2, 2> : k_uneven<1, 2>;
  if (maxa <= 4) return variant ? k_uneven<2, 4> : k_uneven<1, 4>;
  return variant ? k_uneven<2, 8> : k_uneven<1, 8>;
}

hpx_status uneven_launch(hpx_uneven* u, uint64_t seed, int64_t drop0, const float* noise, uint32_t* errors,
                         cudaStream_t s) {
  UArgs a;
  a.drops = u->d_drops;
  a.frames = u->d_frames;
  a.delay = u->d_delay;
  a.amp = u->d_amp;
  a.order = u->d_order;
  a.num_drops = u->B;
  a.S = u->S;
  a.counter = u->d_counter;
  a.scratch = u->d_scratch;
  a.slot_bytes = u->slot_bytes;
  a.off_x = u->off_x;
  a.off_y = u->off_y;
  a.off_grid = u->off_grid;
  a.noise_power = noise;
  a.seed = seed;
  a.noise_keys = philox_keys(seed);
  a.drop0 = drop0;
  a.errors = errors;
  const int grid = std::min(u->num_sms * u->blocks_per_sm, u->max_slots);
  auto kern = uneven_kernel(u->variant, u->maxa);
  if (u->smem > 48 * 1024)  // the attribute is per kernel: set it for this batch's size
    HPX_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)u->smem));
  HPX_CUDA(cudaMemsetAsync(u->d_counter, 0, sizeof(unsigned int), s));
  kern<<<grid, u->threads, u->smem, s>>>(a, u->qts);
  HPX_LAUNCHED("uneven");
  return HPX_OK;
}

}  // namespace

extern "C" {

hpx_status hpx_uneven_create(const hpx_uneven_drop* drops, int32_t num_drops, double subcarrier_spacing,
                             double tap_spacing, int32_t num_sinusoids, int32_t max_slots, hpx_uneven** out) {
  if (!drops || !out) return hpx_fail(HPX_ERR_ARG, "uneven: null argument");
  *out = nullptr;
  if (num_drops < 1) return hpx_fail(HPX_ERR_ARG, "uneven: at least one drop");
  if (!(subcarrier_spacing > 0) || tap_spacing < 0 || num_sinusoids < 1 || max_slots < 1)
    return hpx_fail(HPX_ERR_ARG, "uneven: bad spacing, sinusoids or slot count");
  hpx_uneven* u = new hpx_uneven();
  u->B = num_drops;
  u->S = num_sinusoids;
  const int S1 = num_sinusoids + 1;
  std::vector<UDrop> hd(num_drops);
  std::vector<UFrame> hf;
  std::vector<int32_t> delays;
  std::vector<float> amps;
  std::vector<long long> frame_key;
  size_t max_state = 0, max_x = 0, max_y = 0, max_grid = 0, max_smem = 0;
  for (int i = 0; i < num_drops; ++i) {
    const hpx_uneven_drop& q = drops[i];
    const int N = q.fft_size;
    if (N < 128 || N > 2048 || (N & (N - 1))) {
      uneven_release(u);
      return hpx_fail(HPX_ERR_UNSUPPORTED, "uneven: drop %d: fft_size must be a power of two in [128, 2048]", i);
    }
    const bool ant_ok = [](int n) { return n == 1 || n == 2 || n == 4 || n == 8; }(q.num_rx) &&
                        [](int n) { return n == 1 || n == 2 || n == 4 || n == 8; }(q.num_tx);
    if (!ant_ok || q.num_words < 1 || q.num_taps < 1 || q.num_taps > 64 || q.doppler_frequency < 0) {
      uneven_release(u);
      return hpx_fail(HPX_ERR_ARG, "uneven: drop %d: antennas in {1,2,4,8}, words >= 1, taps in [1, 64]", i);
    }
    int m;
    if (qam_bits_per_symbol(q.modulation_order, &m) != HPX_OK || m < 2) {
      uneven_release(u);
      return hpx_fail(HPX_ERR_ARG, "uneven: drop %d: modulation order 4, 16, 64 or 256", i);
    }
    // frame of (N, words, order), created once
    const long long key = ((long long)N << 40) | ((long long)q.num_words << 16) | q.modulation_order;
    int fi = (int)(std::find(frame_key.begin(), frame_key.end(), key) - frame_key.begin());
    if (fi == (int)frame_key.size()) {
      const int C = (int)std::floor(0.586 * N), cp = N * 72 / 1024, W = q.num_words;
      std::vector<int32_t> prefix(W, cp);
      std::vector<int8_t> kind((size_t)W * C, HPX_RE_DATA);
      hpx_frame_desc fd{};
      fd.num_subcarriers = N;
      fd.num_words = W;
      fd.num_columns = C;
      fd.modulation_order = q.modulation_order;
      fd.dc_suppression = 1;
      fd.prefix = prefix.data();
      fd.zero_prefix = nullptr;
      fd.kind = kind.data();
      fd.pilot_comb = 0;
      hpx_frame* f = nullptr;
      const hpx_status st = hpx_frame_create(&fd, &f);
      if (st != HPX_OK) {
        uneven_release(u);
        return st;
      }
      u->frames.push_back(f);
      frame_key.push_back(key);
      UFrame v;
      v.N = N;
      v.W = W;
      v.C = C;
      v.m = m;
      v.order = q.modulation_order;
      v.cp = cp;
      v.T = f->info.samples_per_frame;
      v.stage_twiddle = f->d_stage_twiddle;
      v.twiddle = f->d_twiddle;
      v.bins = f->d_bins;
      v.constellation = f->d_constellation;
      v.constellation_lsb = f->d_constellation_lsb;
      hf.push_back(v);
      if (!u->qts.t[m].order) {
        const hpx_status s2 = qam_demap_table(q.modulation_order, &u->qts.t[m]);
        if (s2 != HPX_OK) {
          uneven_release(u);
          return s2;
        }
      }
    }
    const UFrame& fr = hf[fi];
    const double fs = (double)N * subcarrier_spacing;
    UDrop& d = hd[i];
    d.frame = fi;
    d.nrx = q.num_rx;
    d.ntx = q.num_tx;
    d.L = q.num_taps;
    d.taps = (int)delays.size();
    double maxd = 0.0;
    for (int k = 0; k < q.num_taps; ++k) {
      const double delay_s = k * tap_spacing;
      maxd = std::fmax(maxd, delay_s);
      delays.push_back((int32_t)std::nearbyint(delay_s * fs));
      const double scale = std::sqrt(std::pow(10.0, -q.tap_decay_db * k / 10.0));
      amps.push_back((float)(scale * std::sqrt(1.0 / num_sinusoids)));  // NLOS, Rice factor 0
      amps.push_back((float)(scale * 0.0));                               // LOS
    }
    d.D = (int)std::nearbyint(maxd * fs);
    d.nlos_rate = q.doppler_frequency / fs;
    d.los_rate = q.doppler_frequency / fs;
    d.BT = q.num_tx <= 4 ? 1024 : 512;  // the homogeneous tile length per transmit count
    d.K = taylor_degree_of(std::fabs(d.nlos_rate), d.BT);
    if (d.D > 4096) {
      uneven_release(u);
      return hpx_fail(HPX_ERR_UNSUPPORTED, "uneven: drop %d: delay spread above 4096 samples", i);
    }
    const size_t T = fr.T;
    max_state = std::max(max_state, (size_t)2 * d.L * S1 * sizeof(int64_t));
    max_x = std::max(max_x, (size_t)d.ntx * T * sizeof(float2));
    max_y = std::max(max_y, (size_t)d.nrx * (T + d.D) * sizeof(float2));
    max_grid = std::max(max_grid, (size_t)d.nrx * fr.W * fr.C * sizeof(float2));
    // stage shared memory (beyond the 768-byte header), for UMAX_THREADS threads
    const int TP = N == 128 ? 8 : N == 256 ? 16 : N == 512 ? 32 : N == 1024 ? 64 : 128;
    const int F = UMAX_THREADS / TP;
    const size_t fft_smem = (size_t)F * (N + N / 16) * sizeof(float2) + (size_t)F * staged_bit_words(fr.C, m) * 4;
    const int KK = d.K < 0 ? 0 : d.K;
    const int XW = (d.BT + d.D + 2) & ~1;
    const size_t region = std::max((size_t)2 * d.ntx * XW, (size_t)d.L * S1 * (KK + 1));
    const size_t prop_smem = (region + (size_t)d.L * (KK + 1)) * sizeof(float2);
    const size_t det_smem = (size_t)d.L * (1 + S1) * sizeof(float2) + (size_t)d.ntx * staged_bit_words(fr.C, m) * 4;
    max_smem = std::max({max_smem, fft_smem, prop_smem, det_smem});
    // schedule weight: samples x transmit antennas x taps + elements x Nrx x Ntx^2
    u->maxa = i == 0 ? 2 : u->maxa;
    u->maxa = std::max({u->maxa, q.num_rx, q.num_tx});
    u->cost.push_back((double)T * d.ntx * (d.L + d.nrx) + (double)fr.W * fr.C * d.nrx * d.ntx * d.ntx);
    u->bits.push_back((int64_t)fr.W * fr.C * m * d.ntx);
  }
  u->off_x = round_up(max_state);
  u->off_y = u->off_x + round_up(max_x);
  u->off_grid = u->off_y + round_up(max_y);
  u->slot_bytes = u->off_grid + round_up(max_grid);
  u->smem = 256 + 128 * sizeof(float2) + max_smem + 16;
  u->max_slots = max_slots;
  std::vector<int32_t> order(num_drops);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a2, int b2) { return u->cost[a2] > u->cost[b2]; });
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&u->num_sms, cudaDevAttrMultiProcessorCount, dev);
  cudaError_t e;
  if ((e = cudaMalloc(&u->d_drops, sizeof(UDrop) * hd.size())) != cudaSuccess ||
      (e = cudaMalloc(&u->d_frames, sizeof(UFrame) * hf.size())) != cudaSuccess ||
      (e = cudaMalloc(&u->d_delay, sizeof(int32_t) * delays.size())) != cudaSuccess ||
      (e = cudaMalloc(&u->d_amp, sizeof(float) * amps.size())) != cudaSuccess ||
      (e = cudaMalloc(&u->d_order, sizeof(int32_t) * order.size())) != cudaSuccess ||
      (e = cudaMalloc(&u->d_counter, sizeof(unsigned int))) != cudaSuccess ||
      (e = cudaMalloc(&u->d_scratch, u->slot_bytes * (size_t)max_slots)) != cudaSuccess ||
      (e = cudaMemcpy(u->d_drops, hd.data(), sizeof(UDrop) * hd.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(u->d_frames, hf.data(), sizeof(UFrame) * hf.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(u->d_delay, delays.data(), sizeof(int32_t) * delays.size(), cudaMemcpyHostToDevice)) !=
          cudaSuccess ||
      (e = cudaMemcpy(u->d_amp, amps.data(), sizeof(float) * amps.size(), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy(u->d_order, order.data(), sizeof(int32_t) * order.size(), cudaMemcpyHostToDevice)) !=
          cudaSuccess) {
    uneven_release(u);
    return hpx_cuda_status(e, "uneven tables");
  }
  if (u->smem > 48 * 1024) {
    if ((e = cudaFuncSetAttribute(uneven_kernel(0, u->maxa), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)u->smem)) != cudaSuccess ||
        (e = cudaFuncSetAttribute(uneven_kernel(1, u->maxa), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)u->smem)) != cudaSuccess ||
        (uneven_kernel(2, u->maxa) &&
         (e = cudaFuncSetAttribute(uneven_kernel(2, u->maxa), cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)u->smem)) != cudaSuccess)) {
      uneven_release(u);
      return hpx_cuda_status(e, "uneven shared memory");
    }
  }
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, uneven_kernel(0, u->maxa), u->threads, u->smem);
  u->blocks_per_sm = std::max(1, occ);
  *out = u;
  return HPX_OK;
}

hpx_status hpx_uneven_destroy(hpx_uneven* u) {
  uneven_release(u);
  return HPX_OK;
}

hpx_status hpx_uneven_bits(const hpx_uneven* u, int64_t* bits_per_drop) {
  if (!u || !bits_per_drop) return hpx_fail(HPX_ERR_ARG, "uneven_bits: null argument");
  std::copy(u->bits.begin(), u->bits.end(), bits_per_drop);
  return HPX_OK;
}

hpx_status hpx_uneven_config(hpx_uneven* u, int32_t threads, int32_t blocks_per_sm, int32_t variant) {
  if (!u) return hpx_fail(HPX_ERR_ARG, "uneven_config: null argument");
  if (threads != 128 && threads != 256) return hpx_fail(HPX_ERR_ARG, "uneven_config: 128 or 256 threads");
  if (variant < 0 || variant > 2) return hpx_fail(HPX_ERR_ARG, "uneven_config: variant 0, 1 or 2");
  if (!uneven_kernel(variant, u->maxa))
    return hpx_fail(HPX_ERR_UNSUPPORTED, "uneven_config: variant 2 needs drops of at most 4 antennas a side");
  int occ = 0;
  HPX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, uneven_kernel(variant, u->maxa), threads, u->smem));
  if (occ < 1) return hpx_fail(HPX_ERR_UNSUPPORTED, "uneven_config: %d threads do not fit one SM", threads);
  if (blocks_per_sm < 1 || blocks_per_sm > occ)
    return hpx_fail(HPX_ERR_ARG, "uneven_config: %d CTAs per SM (1..%d fit)", blocks_per_sm, occ);
  u->threads = threads;
  u->blocks_per_sm = blocks_per_sm;
  u->variant = variant;
  if (u->graph) {  // a captured graph holds the old launch shape
    cudaGraphExecDestroy(u->graph);
    cudaGraphDestroy(u->graph_def);
    u->graph = nullptr;
    u->graph_def = nullptr;
  }
  return HPX_OK;
}

hpx_status hpx_uneven_get_config(const hpx_uneven* u, int32_t threads, int32_t variant, int32_t* cur_threads,
                                 int32_t* cur_blocks_per_sm, int32_t* cur_variant, int32_t* max_fit) {
  if (!u) return hpx_fail(HPX_ERR_ARG, "uneven_get_config: null argument");
  if (cur_threads) *cur_threads = u->threads;
  if (cur_blocks_per_sm) *cur_blocks_per_sm = u->blocks_per_sm;
  if (cur_variant) *cur_variant = u->variant;
  if (max_fit) {
    int occ = 0;
    if ((threads == 128 || threads == 256) && variant >= 0 && variant <= 2 && uneven_kernel(variant, u->maxa))
      HPX_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, uneven_kernel(variant, u->maxa), threads,
                                                             u->smem));
    *max_fit = occ;
  }
  return HPX_OK;
}

hpx_status hpx_uneven_run(hpx_uneven* u, uint64_t seed, int64_t drop0, const float* noise_power, uint32_t* errors,
                          void* stream) {
  if (!u || !noise_power || !errors) return hpx_fail(HPX_ERR_ARG, "uneven_run: null argument");
  if (drop0 < 0) return hpx_fail(HPX_ERR_ARG, "uneven_run: negative drop index");
  return uneven_launch(u, seed, drop0, noise_power, errors, as_stream(stream));
}

hpx_status hpx_uneven_capture(hpx_uneven* u, uint64_t seed, int64_t drop0, const float* noise_power,
                              uint32_t* errors) {
  if (!u || !noise_power || !errors) return hpx_fail(HPX_ERR_ARG, "uneven_capture: null argument");
  if (u->graph) {
    cudaGraphExecDestroy(u->graph);
    cudaGraphDestroy(u->graph_def);
    u->graph = nullptr;
    u->graph_def = nullptr;
  }
  cudaStream_t cs;
  HPX_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) {
    cudaStreamDestroy(cs);
    return hpx_cuda_status(e, "uneven graph capture");
  }
  const hpx_status st = uneven_launch(u, seed, drop0, noise_power, errors, cs);
  cudaGraph_t g = nullptr;
  e = cudaStreamEndCapture(cs, &g);
  cudaStreamDestroy(cs);
  if (st != HPX_OK) {
    if (g) cudaGraphDestroy(g);
    return st;
  }
  if (e != cudaSuccess) return hpx_cuda_status(e, "uneven graph capture");
  cudaGraphExec_t ex = nullptr;
  e = cudaGraphInstantiate(&ex, g, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(g);
    return hpx_cuda_status(e, "uneven graph instantiate");
  }
  u->graph_def = g;
  u->graph = ex;
  return HPX_OK;
}

hpx_status hpx_uneven_replay(hpx_uneven* u, void* stream) {
  if (!u || !u->graph) return hpx_fail(HPX_ERR_ARG, "uneven_replay: no captured graph");
  HPX_CUDA(cudaGraphLaunch(u->graph, as_stream(stream)));
  return HPX_OK;
}

}  // extern "C"
