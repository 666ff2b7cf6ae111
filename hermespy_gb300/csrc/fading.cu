// Sum-of-sinusoids multipath fading: realization parameters, tap synthesis,
// channel state, ideal frequency-domain CSI and the fused propagate + AWGN kernel.
#include <cmath>

#include "fading_dev.cuh"

namespace {

constexpr double kPi = 3.14159265358979323846;

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// ---------------------------------------------------------------- parameters
// One block per drop. MODE 0: draws from the Philox stream (domain 2);
// MODE 1: explicit angles / phases / spatial response from device arrays.
// MODE 0 with `staged`: the drop's drawn words (nrx ntx + 2 L + 2 L S of them) are
// drawn once into shared memory, one Philox block per four, instead of one block per
// draw. MODE 0 forms the initial phases exactly from the drawn words and, with
// `fp32_rates` (rates within kFp32RateLimit), the rates in FP32 (cospif; see
// rate_to_fixed), so its FP64 work is the spatial response alone; MODE 1 (explicit
// angles) and faster channels stay in FP64.
template <int MODE>
__global__ void k_fading_params(FadingConst fc, double nlos_rate, double los_rate, uint64_t seed, int64_t drop0,
                                const double* __restrict__ la, const double* __restrict__ na,
                                const double* __restrict__ lp, const double* __restrict__ np_,
                                const double* __restrict__ sp_in, const double* __restrict__ rxc,
                                const double* __restrict__ txc, unsigned char* state, size_t stride, size_t off_w,
                                size_t off_p0, size_t off_sp, int staged, int fp32_rates) {
  extern __shared__ double2 sps[];  // [nrx*ntx] spatial, then [nrx*ntx] temp, then the staged words
  const int b = blockIdx.x;
  const int64_t drop = drop0 + b;
  const int L = fc.L, S = fc.S, S1 = fc.S1, nrx = fc.nrx, ntx = fc.ntx;
  const int nsp = nrx * ntx;
  unsigned char* base = state + (size_t)b * stride;
  int64_t* Wout = reinterpret_cast<int64_t*>(base + off_w);
  int64_t* Pout = reinterpret_cast<int64_t*>(base + off_p0);
  float2* Sout = reinterpret_cast<float2*>(base + off_sp);
  uint32_t* uw = reinterpret_cast<uint32_t*>(sps + 2 * nsp);
  if (MODE == 0 && staged) {
    const int num = nsp + 2 * L + 2 * L * S;
    for (int blk = threadIdx.x; blk < (num + 3) >> 2; blk += blockDim.x) {
      const uint4 r = hpx_random_block(seed, drop, 0u, HPX_DOMAIN_FADING, (uint32_t)blk);
      const uint32_t wv[4] = {r.x, r.y, r.z, r.w};
#pragma unroll
      for (int i = 0; i < 4; ++i)
        if (4 * blk + i < num) uw[4 * blk + i] = wv[i];
    }
    __syncthreads();
  }

  auto word = [&](int idx) -> uint32_t {
    if (staged) return uw[idx];
    const uint4 r = hpx_random_block(seed, drop, 0u, HPX_DOMAIN_FADING, (uint32_t)(idx >> 2));
    return uint4_get(r, idx & 3);
  };
  auto uniform = [&](int idx) -> double { return u01_f64(word(idx)); };

  // Drawn angles enter as turns: theta = -pi + 2 pi u gives (2 pi (n + 1) + theta) / S
  // = pi (2 n + 1 + 2 u) / S and phi / (2 pi) = u - 1/2: one cospif per sinusoid for its
  // rate, the phase straight from the drawn word.
  constexpr double kInv2Pi = 0.15915494309189535;
  const double inv_s = 1.0 / (double)(S > 0 ? S : 1);
  const float inv_sf = 1.0f / (float)(S > 0 ? S : 1);
  const float rate_n = (float)(nlos_rate * kInv2Pi), rate_l = (float)(los_rate * kInv2Pi);
  // (w + 1/2) 2^-32 in FP32
  auto u01 = [](uint32_t w) { return fmaf(__uint2float_rn(w), 2.3283064365386963e-10f, 1.1641532182693481e-10f); };
  for (int q = threadIdx.x; q < L * S1; q += blockDim.x) {
    const int l = q / S1, n = q - l * S1;
    if (MODE == 0) {
      const uint32_t wu = n < S ? word(nsp + L + l * S + n) : word(nsp + l);
      if (fp32_rates)
        Wout[q] = n < S ? rate_to_fixed(rate_n * cospif(((float)(2 * n + 1) + 2.0f * u01(wu)) * inv_sf))
                        : rate_to_fixed(rate_l * cospif(2.0f * u01(wu)));
      else
        Wout[q] = turns_to_fixed(kInv2Pi * (n < S ? nlos_rate * cospi((2.0 * n + 1.0 + 2.0 * u01_f64(wu)) * inv_s)
                                                  : los_rate * cospi(2.0 * u01_f64(wu))));
      Pout[q] = phase_from_word(n < S ? word(nsp + 2 * L + L * S + l * S + n) : word(nsp + L + L * S + l));
    } else {
      double omega, turns;
      if (n < S) {
        const double theta = na[((int64_t)b * L + l) * S + n];
        omega = nlos_rate * cos((2.0 * kPi * (n + 1) + theta) / (double)S);
        turns = np_[((int64_t)b * L + l) * S + n] * kInv2Pi;
      } else {
        omega = los_rate * cos(la[(int64_t)b * L + l]);
        turns = lp[(int64_t)b * L + l] * kInv2Pi;
      }
      Wout[q] = turns_to_fixed(omega * kInv2Pi);
      Pout[q] = turns_to_fixed(turns);
    }
  }
  for (int j = threadIdx.x; j < nsp; j += blockDim.x) {
    if (MODE == 0) {
      double s, c;
      sincospi(2.0 * uniform(j), &s, &c);
      sps[j] = make_double2(c, s);
    } else {
      sps[j] = make_double2(sp_in[2 * ((int64_t)b * nsp + j)], sp_in[2 * ((int64_t)b * nsp + j) + 1]);
    }
  }
  __syncthreads();
  if (rxc || txc) {
    double2* tmp = sps + nsp;
    // tmp = R_rx @ S
    for (int j = threadIdx.x; j < nsp; j += blockDim.x) {
      const int r = j / ntx, t = j - r * ntx;
      double2 acc = make_double2(0.0, 0.0);
      if (rxc) {
        for (int a = 0; a < nrx; ++a) {
          const double2 m = make_double2(rxc[2 * (r * nrx + a)], rxc[2 * (r * nrx + a) + 1]);
          const double2 v = sps[a * ntx + t];
          acc.x += m.x * v.x - m.y * v.y;
          acc.y += m.x * v.y + m.y * v.x;
        }
      } else {
        acc = sps[j];
      }
      tmp[j] = acc;
    }
    __syncthreads();
    // S = tmp @ R_tx
    for (int j = threadIdx.x; j < nsp; j += blockDim.x) {
      const int r = j / ntx, t = j - r * ntx;
      double2 acc = make_double2(0.0, 0.0);
      if (txc) {
        for (int a = 0; a < ntx; ++a) {
          const double2 m = make_double2(txc[2 * (a * ntx + t)], txc[2 * (a * ntx + t) + 1]);
          const double2 v = tmp[r * ntx + a];
          acc.x += v.x * m.x - v.y * m.y;
          acc.y += v.x * m.y + v.y * m.x;
        }
      } else {
        acc = tmp[j];
      }
      Sout[j] = make_float2((float)acc.x, (float)acc.y);
    }
  } else {
    for (int j = threadIdx.x; j < nsp; j += blockDim.x) Sout[j] = make_float2((float)sps[j].x, (float)sps[j].y);
  }
}

__global__ void k_fading_draws(int num, uint64_t seed, int64_t drop0, double* __restrict__ out) {
  const int b = blockIdx.y;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < num; i += gridDim.x * blockDim.x) {
    const uint4 r = hpx_random_block(seed, drop0 + b, 0u, HPX_DOMAIN_FADING, (uint32_t)(i >> 2));
    out[(int64_t)b * num + i] = u01_f64(uint4_get(r, i & 3));
  }
}

// ------------------------------------------------------------ direct taps
// h_l[t] = amp_nlos sum_n exp(i theta_n(t)) + amp_los exp(i theta_los(t)) with
// theta(t) = P0 + W t reduced exactly in 64-bit fixed point.
__device__ __forceinline__ float2 tap_direct(const int64_t* __restrict__ W, const int64_t* __restrict__ P0, int S,
                                             float an, float al, int64_t t) {
  float2 acc = make_float2(0.f, 0.f);
  for (int n = 0; n < S; ++n) {
    const uint64_t p = (uint64_t)P0[n] + (uint64_t)W[n] * (uint64_t)t;
    float s, c;
    __sincosf(fixed_to_angle(p), &s, &c);
    acc.x += c;
    acc.y += s;
  }
  const uint64_t p = (uint64_t)P0[S] + (uint64_t)W[S] * (uint64_t)t;
  float s, c;
  __sincosf(fixed_to_angle(p), &s, &c);
  return make_float2(an * acc.x + al * c, an * acc.y + al * s);
}

__global__ void k_fading_taps(FadingConst fc, FadingView v, int T, float2* __restrict__ taps) {
  const int b = blockIdx.z, l = blockIdx.y;
  extern __shared__ int64_t wp[];  // W[S1], P0[S1]
  const int64_t* W = v.W(b) + l * fc.S1;
  const int64_t* P = v.P0(b) + l * fc.S1;
  for (int n = threadIdx.x; n < fc.S1; n += blockDim.x) {
    wp[n] = W[n];
    wp[fc.S1 + n] = P[n];
  }
  __syncthreads();
  const float an = fc.amp[2 * l], al = fc.amp[2 * l + 1];
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x)
    taps[((int64_t)b * fc.L + l) * T + t] = tap_direct(wp, wp + fc.S1, fc.S, an, al, t);
}

__global__ void k_fading_csi(FadingConst fc, FadingView v, int T, int ntaps, float2* __restrict__ csi) {
  const int b = blockIdx.y;
  const float2* Sm = v.spatial(b);
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x) {
    for (int l = 0; l < fc.L; ++l) {
      const int d = fc.delay[l];
      if (d >= ntaps) continue;
      const float2 h = tap_direct(v.W(b) + l * fc.S1, v.P0(b) + l * fc.S1, fc.S, fc.amp[2 * l], fc.amp[2 * l + 1], t);
      for (int r = 0; r < fc.nrx; ++r)
        for (int x = 0; x < fc.ntx; ++x) {
          float2* dst = csi + ((((int64_t)b * fc.nrx + r) * fc.ntx + x) * T + t) * ntaps + d;
          *dst = cadd(*dst, cmul(Sm[r * fc.ntx + x], h));
        }
    }
  }
}

// ------------------------------------------------------------ propagation
// One block computes BT output samples [m0, m0 + BT) of all receive antennas of
// one drop. Thread t owns two sample pairs, (2t, 2t + 1) and (2t + BT/2,
// 2t + BT/2 + 1), so that lanes read consecutive 16-byte chunks of the transmit
// tile and one Philox block gives the AWGN of a pair. The taps needed by the tile,
// h_l(t) for t in [m0 - d_l, m0 + BT - d_l), are expanded per tap around the tile
// centre as a degree-K Taylor polynomial in u = (m - m0 - BT/2) / (BT/2):
//   h_l = sum_k C_lk u^k,  C_lk = (i H)^k / k! sum_n a_n w_n^k exp(i theta_n(t_c)),
// exact to |w H|^(K+1)/(K+1)! per sinusoid; u depends on the output sample only,
// so one set of powers serves every tap. Taps that round to one sample delay
// multiply the same transmit samples, so their coefficients are summed and the
// convolution runs once per distinct delay. DIRECT evaluates every sinusoid at
// every sample instead (used when the Doppler rate makes the expansion long).
// The transmit tile is staged twice, the second copy shifted by one sample, so a
// pair starting at any tap delay is one aligned 16-byte load.
// Tile length per transmit-antenna count (shared memory holds 2 NTX tile rows).
template <int NTX>
__host__ __device__ constexpr int tile_len() { return NTX <= 4 ? 1024 : (NTX <= 8 ? 512 : 256); }

__host__ __device__ constexpr int tile_width(int BT, int D) { return (BT + D + 2) & ~1; }

template <int NTX, int K, bool DIRECT, int XS = 0, int PPT = 2, int BT = tile_len<NTX>(),
          int PTHREADS = tile_len<NTX>() / (2 * PPT)>
__global__ void __launch_bounds__(PTHREADS, PPT == 1 ? 2 : 3) k_propagate(FadingConst fc, FadingView v, int T, const float2* __restrict__ x,
                                                        float2* __restrict__ y, const float* __restrict__ noise_power,
                                                        const __grid_constant__ PhiloxKeys nk, int64_t drop0) {
  extern __shared__ float4 smem4[];
  const int b = blockIdx.y;
  const int m0 = blockIdx.x * BT;
  const int L = fc.L, G = fc.G, S1 = fc.S1, D = fc.D, nrx = fc.nrx;
  const int XW = tile_width(BT, D);  // samples of a row (even)
  const int PS = XS ? XS : XW;       // row stride: a compile-time constant for short channels
  // Transmit tile as planes of real and imaginary parts, each stored twice: plane
  // (tx, q) with q = 0 re even, 1 im even, 2 re odd, 3 im odd; even copies hold
  // x[m0 - D + i], odd copies x[m0 - D + i + 1].
  float* xp = reinterpret_cast<float*>(smem4);                        // [NTX][4][PS]
  float2* terms = reinterpret_cast<float2*>(smem4);                   // [L*S1][K+1], before the tile store
  const int region = DIRECT ? 2 * NTX * PS : max(2 * NTX * PS, L * S1 * (K + 1));  // in float2
  float4* coef = reinterpret_cast<float4*>(reinterpret_cast<float2*>(smem4) + region);  // [G][K+1] (x, x, y, y)
  int64_t* wp = reinterpret_cast<int64_t*>(coef + G * (K + 1));       // [2][L*S1] (direct)
  float2* Sm = reinterpret_cast<float2*>(wp + (DIRECT ? 2 * L * S1 : 0));  // [nrx*NTX]
  int* dl = reinterpret_cast<int*>(Sm + nrx * NTX);                   // [G] group delays
  int* gf = dl + G;                                                   // [G + 1] first tap of each group
  const int tid = threadIdx.x;

  const float2* Sg = v.spatial(b);
  for (int i = tid; i < nrx * NTX; i += PTHREADS) Sm[i] = Sg[i];
  for (int g = tid; g <= G; g += PTHREADS) {
    gf[g] = fc.gfirst[g];
    if (g < G) dl[g] = fc.gdelay[g];
  }
  const int64_t* Wg = v.W(b);
  const int64_t* Pg = v.P0(b);
  // Transmit samples of the tile, fetched into registers first so that their load
  // latency overlaps the coefficient set-up (tile samples beyond PF per thread, for
  // delays above PTHREADS - 3 samples, are fetched afterwards).
  constexpr int PF = NTX <= 4 ? BT / PTHREADS + 1 : 0;  // register budget: up to 4 transmit antennas
  const float2* xb = x + (int64_t)b * NTX * T;
  float2 xpf[NTX][PF > 0 ? PF : 1];
#pragma unroll
  for (int tx = 0; tx < NTX; ++tx)
#pragma unroll
    for (int i = 0; i < PF; ++i) {
      const int j = tid + i * PTHREADS, t = m0 - D + j;
      xpf[tx][i] = (j <= XW && t >= 0 && t < T) ? __ldg(xb + (int64_t)tx * T + t) : make_float2(0.f, 0.f);
    }
  if (DIRECT) {
    for (int q = tid; q < L * S1; q += PTHREADS) {
      wp[q] = Wg[q];
      wp[L * S1 + q] = Pg[q];
    }
  } else {
    const float H = 0.5f * BT;
    for (int q = tid; q < L * S1; q += PTHREADS) {
      const int l = q / S1, n = q - l * S1;
      const int64_t tc = (int64_t)m0 - fc.delay[l] + BT / 2;
      const uint64_t p = (uint64_t)Pg[q] + (uint64_t)Wg[q] * (uint64_t)tc;
      float sn, cs;
      __sincosf(fixed_to_angle(p), &sn, &cs);
      const float a = fc.amp[2 * l + (n < fc.S ? 0 : 1)];
      const float wh = fixed_rate(Wg[q]) * H;
      float2 t = make_float2(a * cs, a * sn);
      float2* dst = terms + q * (K + 1);
      dst[0] = t;
#pragma unroll
      for (int k = 1; k <= K; ++k) {
        const float f = wh / (float)k;
        t = make_float2(-t.y * f, t.x * f);  // t *= i w H / k
        dst[k] = t;
      }
    }
    __syncthreads();
    for (int q = tid; q < G * (K + 1); q += PTHREADS) {
      const int g = q / (K + 1), k = q - g * (K + 1);
      float2 acc = make_float2(0.f, 0.f);
      for (int l = gf[g]; l < gf[g + 1]; ++l)
        for (int n = 0; n < S1; ++n) acc = cadd(acc, terms[(l * S1 + n) * (K + 1) + k]);
      coef[q] = make_float4(acc.x, acc.x, acc.y, acc.y);  // broadcast pairs for the packed FMAs
    }
  }
  __syncthreads();  // terms consumed: the tile may overwrite them
  auto put = [&](int tx, int j, float2 val) {
    float* pl = xp + tx * 4 * PS;
    if (j < XW) {
      pl[j] = val.x;
      pl[PS + j] = val.y;
    }
    if (j > 0) {
      pl[2 * PS + j - 1] = val.x;
      pl[3 * PS + j - 1] = val.y;
    }
  };
#pragma unroll
  for (int tx = 0; tx < NTX; ++tx)
#pragma unroll
    for (int i = 0; i < PF; ++i) {
      const int j = tid + i * PTHREADS;
      if (j <= XW) put(tx, j, xpf[tx][i]);
    }
  if (XW >= PF * PTHREADS) {
#pragma unroll 1
    for (int tx = 0; tx < NTX; ++tx)
      for (int j = tid + PF * PTHREADS; j <= XW; j += PTHREADS) {
        const int t = m0 - D + j;
        put(tx, j, (t >= 0 && t < T) ? __ldg(xb + (int64_t)tx * T + t) : make_float2(0.f, 0.f));
      }
  }
  __syncthreads();
  // warps whose samples all lie past the end of the received signal (last tile)
  const int TD = T + D;
  if (m0 + 2 * (tid & ~31) >= TD) return;

  // ---- convolution: z_tx[m] = sum_l h_l[m - d_l] x_tx[m - d_l], two samples per
  // packed FP32x2 FMA: zr/zi hold the real/imaginary parts of a pair of samples.
  int jp[PPT];  // tile index of each pair's first sample
#pragma unroll
  for (int pr = 0; pr < PPT; ++pr) jp[pr] = 2 * tid + pr * (BT / PPT);
  float2 zr[PPT][NTX], zi[PPT][NTX];
#pragma unroll
  for (int pr = 0; pr < PPT; ++pr)
#pragma unroll
    for (int tx = 0; tx < NTX; ++tx) zr[pr][tx] = zi[pr][tx] = make_float2(0.f, 0.f);
  float2 up[PPT][K + 1];  // powers of u for both samples of a pair
#pragma unroll
  for (int pr = 0; pr < PPT; ++pr) {
    const float u0 = ((float)jp[pr] - 0.5f * BT) / (0.5f * BT);
    const float u1 = ((float)(jp[pr] + 1) - 0.5f * BT) / (0.5f * BT);
    up[pr][0] = make_float2(1.0f, 1.0f);
#pragma unroll
    for (int k = 1; k <= K; ++k) up[pr][k] = make_float2(up[pr][k - 1].x * u0, up[pr][k - 1].y * u1);
  }
#pragma unroll 2  // two delay groups per iteration: 1.6 % faster, still 80 registers without spills
  for (int g = 0; g < G; ++g) {
    const int d = dl[g];
    float2 hx[PPT], hy[PPT];
    if (DIRECT) {
#pragma unroll
      for (int pr = 0; pr < PPT; ++pr) hx[pr] = hy[pr] = make_float2(0.f, 0.f);
      for (int l = gf[g]; l < gf[g + 1]; ++l) {
        const float an = fc.amp[2 * l], al = fc.amp[2 * l + 1];
#pragma unroll
        for (int pr = 0; pr < PPT; ++pr) {
          const float2 h0 = tap_direct(wp + l * S1, wp + L * S1 + l * S1, fc.S, an, al, (int64_t)m0 + jp[pr] - d);
          const float2 h1 = tap_direct(wp + l * S1, wp + L * S1 + l * S1, fc.S, an, al, (int64_t)m0 + jp[pr] + 1 - d);
          hx[pr] = make_float2(hx[pr].x + h0.x, hx[pr].y + h1.x);
          hy[pr] = make_float2(hy[pr].x + h0.y, hy[pr].y + h1.y);
        }
      }
    } else {
      const float4* cl = coef + g * (K + 1);
      float4 ck[K + 1];
#pragma unroll
      for (int k = 0; k <= K; ++k) ck[k] = cl[k];
#pragma unroll
      for (int pr = 0; pr < PPT; ++pr) {
        float2 ax = make_float2(ck[0].x, ck[0].y), ay = make_float2(ck[0].z, ck[0].w);
#pragma unroll
        for (int k = 1; k <= K; ++k) {
          ax = __ffma2_rn(make_float2(ck[k].x, ck[k].y), up[pr][k], ax);
          ay = __ffma2_rn(make_float2(ck[k].z, ck[k].w), up[pr][k], ay);
        }
        hx[pr] = ax;
        hy[pr] = ay;
      }
    }
    // all lanes share the parity of D - d, hence the same copy: conflict-free
    const int odd = (D - d) & 1;
    const float* src = xp + 2 * odd * PS - odd;  // plane offset of the even/odd copy, index shifted by one
#pragma unroll
    for (int pr = 0; pr < PPT; ++pr) {
      const int s0 = jp[pr] - d + D;
      const float2 nhy = __fmul2_rn(hy[pr], make_float2(-1.f, -1.f));  // one packed op
#pragma unroll
      for (int tx = 0; tx < NTX; ++tx) {
        const float* pl = src + tx * 4 * PS + s0;
        const float2 re = *reinterpret_cast<const float2*>(pl);
        const float2 im = *reinterpret_cast<const float2*>(pl + PS);
        zr[pr][tx] = __ffma2_rn(hx[pr], re, zr[pr][tx]);
        zr[pr][tx] = __ffma2_rn(nhy, im, zr[pr][tx]);
        zi[pr][tx] = __ffma2_rn(hx[pr], im, zi[pr][tx]);
        zi[pr][tx] = __ffma2_rn(hy[pr], re, zi[pr][tx]);
      }
    }
  }

  // ---- spatial mixing, AWGN, store
  const float np = noise_power ? noise_power[b] : 0.0f;
  const float sigma = sqrtf(0.5f * np);
#pragma unroll 1
  for (int rx = 0; rx < nrx; ++rx) {
    float2* yr = y + ((int64_t)b * nrx + rx) * TD;
#pragma unroll
    for (int pr = 0; pr < PPT; ++pr) {
      float2 ore = make_float2(0.f, 0.f), oim = make_float2(0.f, 0.f);
#pragma unroll
      for (int tx = 0; tx < NTX; ++tx) {
        const float2 sv = Sm[rx * NTX + tx];
        const float2 sr = make_float2(sv.x, sv.x), si = make_float2(sv.y, sv.y), nsi = make_float2(-sv.y, -sv.y);
        ore = __ffma2_rn(sr, zr[pr][tx], ore);
        ore = __ffma2_rn(nsi, zi[pr][tx], ore);
        oim = __ffma2_rn(sr, zi[pr][tx], oim);
        oim = __ffma2_rn(si, zr[pr][tx], oim);
      }
      const int m = m0 + jp[pr];
      if (noise_power && np > 0.0f) {
        // complex sample k of antenna rx: block k/2, words (0,1) for even k, (2,3) for odd k
        const uint4 w = hpx_random_block_k(nk, drop0 + b, (uint32_t)rx, HPX_DOMAIN_NOISE, (uint32_t)(m >> 1));
        const float2 n0 = box_muller(w.x, w.y);
        const float2 n1 = box_muller(w.z, w.w);
        ore = __ffma2_rn(make_float2(sigma, sigma), make_float2(n0.x, n1.x), ore);
        oim = __ffma2_rn(make_float2(sigma, sigma), make_float2(n0.y, n1.y), oim);
      }
      if (m < TD) yr[m] = make_float2(ore.x, oim.x);
      if (m + 1 < TD) yr[m + 1] = make_float2(ore.y, oim.y);
    }
  }
}

// --------------------------------------------------------- ideal CSI (API)
__global__ void k_ideal_csi(FadingConst fc, FadingView v, int N, int W, const int32_t* __restrict__ window_start,
                            const int32_t* __restrict__ bins, const float2* __restrict__ tw, int ncols,
                            float2* __restrict__ csi) {
  extern __shared__ float4 smem4[];
  float2* hb = reinterpret_cast<float2*>(smem4);
  float2* scratch = hb + fc.L;
  int* ds = reinterpret_cast<int*>(scratch + fc.L * fc.S1);
  const int b = blockIdx.y, w = blockIdx.x;
  for (int l = threadIdx.x; l < fc.L; l += blockDim.x) ds[l] = fc.delay[l];
  tap_averages(fc, v.W(b), v.P0(b), window_start[w], N, hb, scratch);
  const float2* Sm = v.spatial(b);
  for (int c = threadIdx.x; c < ncols; c += blockDim.x) {
    const float2 g = tap_response(fc, hb, ds, tw, bins[c], N);
    for (int r = 0; r < fc.nrx; ++r)
      for (int t = 0; t < fc.ntx; ++t)
        csi[((((int64_t)b * fc.nrx + r) * fc.ntx + t) * W + w) * ncols + c] = cmul(Sm[r * fc.ntx + t], g);
  }
}

void release(hpx_fading* f) {
  if (!f) return;
  if (f->d_delay) cudaFree(f->d_delay);
  if (f->d_group) cudaFree(f->d_group);
  if (f->d_amp) cudaFree(f->d_amp);
  if (f->d_rx_corr) cudaFree(f->d_rx_corr);
  if (f->d_tx_corr) cudaFree(f->d_tx_corr);
  delete f;
}

// Taylor degree for a tile half-width H = BT/2, or -1 for direct evaluation.
int taylor_degree(const hpx_fading* f, int BT) {
  const double rate = std::fmax(std::fabs(f->doppler), std::fabs(f->los_doppler)) / f->fs;  // rad/sample
  // reduce modulo 2 pi: exp(i w t) only depends on w mod 2 pi for integer t
  double wmax = std::fmod(rate, 2.0 * kPi);
  if (wmax > kPi) wmax = 2.0 * kPi - wmax;
  if (rate > kPi) wmax = kPi;  // cos() spreads the sinusoid rates over [-rate, rate]
  const double theta = wmax * 0.5 * BT;
  const int degrees[6] = {2, 3, 4, 5, 6, 8};
  for (int K : degrees) {
    double bound = 1.0;
    for (int k = 1; k <= K + 1; ++k) bound *= theta / k;
    if (bound <= 1e-7) return K;
  }
  return -1;
}

template <int NTX, int K, bool DIRECT, int XS>
hpx_status launch_propagate(const hpx_fading* f, const void* state, int B, const hpx_cf32* x, int T, hpx_cf32* y,
                            const float* np, uint64_t seed, int64_t drop0, cudaStream_t s) {
  const FadingConst fc = fading_const(f);
  const FadingView v = fading_view(f, state);
  constexpr int BT = tile_len<NTX>();
  const size_t tile = 2 * (size_t)NTX * (XS ? XS : tile_width(BT, fc.D)) * sizeof(float2);
  const size_t terms = DIRECT ? 0 : (size_t)fc.L * fc.S1 * (K + 1) * sizeof(float2);
  const size_t smem = (tile > terms ? tile : terms) + (size_t)fc.G * (K + 1) * sizeof(float4) +
                      (DIRECT ? 2 * (size_t)fc.L * fc.S1 * sizeof(int64_t) : 0) +
                      (size_t)fc.nrx * NTX * sizeof(float2) + (size_t)(2 * fc.G + 1) * sizeof(int) + 16;
  if (smem > 200 * 1024) return hpx_fail(HPX_ERR_UNSUPPORTED, "propagate: channel too long for one tile");
  // Two pairs per thread: one pair (512 threads, 62 registers, 2 CTAs/SM) took 7.4 ms and
  // four pairs (152 registers) 6.2 ms for 8 192 drops of the 4 x 4 link, against 5.5 ms.
  constexpr int PPT = 2;
  auto kern = k_propagate<NTX, K, DIRECT, XS, PPT>;
  if (smem > 48 * 1024) HPX_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  const int TD = T + fc.D;
  dim3 grid((TD + BT - 1) / BT, B);
  kern<<<grid, BT / (2 * PPT), smem, s>>>(fc, v, T, reinterpret_cast<const float2*>(x), reinterpret_cast<float2*>(y),
                                          np, philox_keys(seed), drop0);
  HPX_LAUNCHED("propagate");
  return HPX_OK;
}

// Short channels (D <= 62 samples) with up to four transmit antennas use a fixed row
// stride, so the per-antenna and per-plane offsets of the tap loop are immediates.
template <int NTX, int XS>
hpx_status dispatch_degree_xs(const hpx_fading* f, const void* state, int B, const hpx_cf32* x, int T, hpx_cf32* y,
                              const float* np, uint64_t seed, int64_t drop0, cudaStream_t s) {
  switch (taylor_degree(f, tile_len<NTX>())) {
    case 2: return launch_propagate<NTX, 2, false, XS>(f, state, B, x, T, y, np, seed, drop0, s);
    case 3: return launch_propagate<NTX, 3, false, XS>(f, state, B, x, T, y, np, seed, drop0, s);
    case 4: return launch_propagate<NTX, 4, false, XS>(f, state, B, x, T, y, np, seed, drop0, s);
    case 5: return launch_propagate<NTX, 5, false, XS>(f, state, B, x, T, y, np, seed, drop0, s);
    case 6: return launch_propagate<NTX, 6, false, XS>(f, state, B, x, T, y, np, seed, drop0, s);
    case 8: return launch_propagate<NTX, 8, false, XS>(f, state, B, x, T, y, np, seed, drop0, s);
    default: return launch_propagate<NTX, 0, true, 0>(f, state, B, x, T, y, np, seed, drop0, s);
  }
}

template <int NTX>
hpx_status dispatch_degree(const hpx_fading* f, const void* state, int B, const hpx_cf32* x, int T, hpx_cf32* y,
                           const float* np, uint64_t seed, int64_t drop0, cudaStream_t s) {
  constexpr int XS = tile_len<NTX>() + 64;
  if (NTX <= 4 && tile_width(tile_len<NTX>(), f->max_delay) <= XS)
    return dispatch_degree_xs<NTX, NTX <= 4 ? XS : 0>(f, state, B, x, T, y, np, seed, drop0, s);
  return dispatch_degree_xs<NTX, 0>(f, state, B, x, T, y, np, seed, drop0, s);
}

}  // namespace

extern "C" {

hpx_status hpx_fading_create(const hpx_fading_desc* d, hpx_fading** out) {
  if (!d || !out) return hpx_fail(HPX_ERR_ARG, "fading: null argument");
  *out = nullptr;
  const int L = d->num_taps;
  if (L < 1) return hpx_fail(HPX_ERR_ARG, "Configuration must contain at least one delay tap");
  if (!d->delays || !d->power_profile || !d->rice_factors) return hpx_fail(HPX_ERR_ARG, "fading: null profile");
  if (d->num_sinusoids < 0) return hpx_fail(HPX_ERR_ARG, "Number of sinusoids must be greater or equal to zero");
  if (d->num_rx < 1 || d->num_tx < 1 || d->num_rx > 64 || d->num_tx > 64)
    return hpx_fail(HPX_ERR_UNSUPPORTED, "fading: antenna counts must be in [1, 64]");
  if (!(d->sampling_rate > 0)) return hpx_fail(HPX_ERR_ARG, "fading: sampling rate must be positive");
  for (int l = 0; l < L; ++l) {
    if (d->delays[l] < 0) return hpx_fail(HPX_ERR_ARG, "Delays must be greater or equal to zero");
    if (d->power_profile[l] < 0) return hpx_fail(HPX_ERR_ARG, "Power profile factors must be greater or equal to zero");
    if (d->rice_factors[l] < 0) return hpx_fail(HPX_ERR_ARG, "Rice factors must be greater or equal to zero");
    if (l && d->delays[l] < d->delays[l - 1]) return hpx_fail(HPX_ERR_ARG, "fading: delays must be sorted");
  }
  if (d->num_sinusoids == 0 && !d->nlos_gains) {
    for (int l = 0; l < L; ++l)
      if (!std::isinf(d->rice_factors[l]))
        return hpx_fail(HPX_ERR_ARG, "fading: NLOS taps need at least one sinusoid");
  }
  hpx_fading* f = new hpx_fading();
  f->L = L;
  f->S = d->num_sinusoids;
  f->S1 = f->S + 1;
  f->nrx = d->num_rx;
  f->ntx = d->num_tx;
  f->fs = d->sampling_rate;
  f->doppler = d->doppler_frequency;
  f->los_doppler = d->los_doppler_frequency;
  f->gain = d->gain;
  f->h_delay.resize(L);
  f->h_amp_nlos.resize(L);
  f->h_amp_los.resize(L);
  double max_delay = 0;
  for (int l = 0; l < L; ++l) {
    f->h_delay[l] = (int32_t)std::nearbyint(d->delays[l] * d->sampling_rate);  // np.rint (half to even)
    max_delay = std::fmax(max_delay, d->delays[l]);
    const double k = d->rice_factors[l];
    const double scale = std::sqrt(d->gain * d->power_profile[l]);
    double los, nlos;
    if (std::isinf(k)) {
      los = 1.0;
      nlos = 0.0;
    } else {
      los = std::sqrt(k / (1.0 + k));
      nlos = std::sqrt(1.0 / ((1.0 + k) * f->S));
    }
    if (d->los_gains) los = d->los_gains[l];
    if (d->nlos_gains) nlos = d->nlos_gains[l];
    f->h_amp_nlos[l] = (float)(scale * nlos);
    f->h_amp_los[l] = (float)(scale * los);
  }
  f->max_delay = (int)std::nearbyint(max_delay * d->sampling_rate);  // round(): half to even
  if (f->max_delay > 4096) {
    release(f);
    return hpx_fail(HPX_ERR_UNSUPPORTED, "fading: maximum delay above 4096 samples");
  }
  const size_t n = (size_t)L * f->S1;
  f->off_w = 0;
  f->off_p0 = n * 8;
  f->off_spatial = 2 * n * 8;
  f->stride = align_up(f->off_spatial + (size_t)f->nrx * f->ntx * sizeof(float2), 256);
  std::vector<float> amp(2 * L);
  for (int l = 0; l < L; ++l) {
    amp[2 * l] = f->h_amp_nlos[l];
    amp[2 * l + 1] = f->h_amp_los[l];
  }
  // Delay groups: taps that round to one sample delay share every transmit sample, so
  // propagation sums their responses before the convolution.
  std::vector<int32_t> gfirst, gdelay;
  for (int l = 0; l < L; ++l)
    if (l == 0 || f->h_delay[l] != f->h_delay[l - 1]) {
      gfirst.push_back(l);
      gdelay.push_back(f->h_delay[l]);
    }
  f->G = (int)gdelay.size();
  gfirst.push_back(L);
  gfirst.insert(gfirst.end(), gdelay.begin(), gdelay.end());
  cudaError_t e;
  if ((e = cudaMalloc(&f->d_delay, L * sizeof(int32_t))) != cudaSuccess ||
      (e = cudaMemcpy(f->d_delay, f->h_delay.data(), L * sizeof(int32_t), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMalloc(&f->d_group, gfirst.size() * sizeof(int32_t))) != cudaSuccess ||
      (e = cudaMemcpy(f->d_group, gfirst.data(), gfirst.size() * sizeof(int32_t), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMalloc(&f->d_amp, 2 * L * sizeof(float))) != cudaSuccess ||
      (e = cudaMemcpy(f->d_amp, amp.data(), 2 * L * sizeof(float), cudaMemcpyHostToDevice)) != cudaSuccess) {
    release(f);
    return hpx_cuda_status(e, "fading tables");
  }
  if (d->rx_correlation) {
    const size_t bytes = (size_t)2 * f->nrx * f->nrx * sizeof(double);
    if ((e = cudaMalloc(&f->d_rx_corr, bytes)) != cudaSuccess ||
        (e = cudaMemcpy(f->d_rx_corr, d->rx_correlation, bytes, cudaMemcpyHostToDevice)) != cudaSuccess) {
      release(f);
      return hpx_cuda_status(e, "fading correlation");
    }
  }
  if (d->tx_correlation) {
    const size_t bytes = (size_t)2 * f->ntx * f->ntx * sizeof(double);
    if ((e = cudaMalloc(&f->d_tx_corr, bytes)) != cudaSuccess ||
        (e = cudaMemcpy(f->d_tx_corr, d->tx_correlation, bytes, cudaMemcpyHostToDevice)) != cudaSuccess) {
      release(f);
      return hpx_cuda_status(e, "fading correlation");
    }
  }
  *out = f;
  return HPX_OK;
}

hpx_status hpx_fading_destroy(hpx_fading* fading) {
  release(fading);
  return HPX_OK;
}

hpx_status hpx_fading_state_bytes(const hpx_fading* f, int32_t num_drops, int64_t* bytes) {
  if (!f || !bytes || num_drops < 0) return hpx_fail(HPX_ERR_ARG, "state_bytes: bad argument");
  *bytes = (int64_t)f->stride * num_drops;
  return HPX_OK;
}

hpx_status hpx_fading_max_delay(const hpx_fading* f, int32_t* samples) {
  if (!f || !samples) return hpx_fail(HPX_ERR_ARG, "max_delay: bad argument");
  *samples = f->max_delay;
  return HPX_OK;
}

static hpx_status launch_params(const hpx_fading* f, int mode, uint64_t seed, int64_t drop0, int B, const double* la,
                                const double* na, const double* lp, const double* np_, const double* sp, void* state,
                                void* stream) {
  if (!f || !state) return hpx_fail(HPX_ERR_ARG, "fading: null argument");
  if (B < 0 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "fading: bad drop range");
  if (B == 0) return HPX_OK;
  if (B > 2147483647) return hpx_fail(HPX_ERR_ARG, "fading: too many drops");
  const FadingConst fc = fading_const(f);
  const size_t smem0 = (size_t)2 * f->nrx * f->ntx * sizeof(double2);
  const double nlos_rate = f->doppler / f->fs, los_rate = f->los_doppler / f->fs;
  if (mode == 0) {
    const size_t draws = (size_t)f->nrx * f->ntx + 2 * (size_t)f->L + 2 * (size_t)f->L * f->S;
    const int staged = smem0 + draws * sizeof(uint32_t) <= 32 * 1024 ? 1 : 0;
    const size_t smem = smem0 + (staged ? draws * sizeof(uint32_t) : 0);
    if (smem > 48 * 1024)
      HPX_CUDA(cudaFuncSetAttribute(k_fading_params<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_fading_params<0><<<B, 128, smem, as_stream(stream)>>>(fc, nlos_rate, los_rate, seed, drop0, nullptr, nullptr,
                                                            nullptr, nullptr, nullptr, f->d_rx_corr, f->d_tx_corr,
                                                            static_cast<unsigned char*>(state), f->stride, f->off_w,
                                                            f->off_p0, f->off_spatial, staged,
                                                            std::fmax(std::fabs(nlos_rate), std::fabs(los_rate)) * 0.15915494309189535 <= kFp32RateLimit);
  } else {
    const size_t smem = smem0;
    if ((!la || !lp) || (f->S > 0 && (!na || !np_)) || !sp) return hpx_fail(HPX_ERR_ARG, "fading_load: null array");
    if (smem > 48 * 1024)
      HPX_CUDA(cudaFuncSetAttribute(k_fading_params<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    // explicit spatial responses are used as given (the caller applied any correlation)
    k_fading_params<1><<<B, 128, smem, as_stream(stream)>>>(fc, nlos_rate, los_rate, 0, 0, la, na, lp, np_, sp, nullptr,
                                                            nullptr, static_cast<unsigned char*>(state), f->stride,
                                                            f->off_w, f->off_p0, f->off_spatial, 0, 0);
  }
  HPX_LAUNCHED("fading_params");
  return HPX_OK;
}

hpx_status hpx_fading_realize(const hpx_fading* f, uint64_t seed, int64_t drop0, int32_t num_drops, void* state,
                              void* stream) {
  return launch_params(f, 0, seed, drop0, num_drops, nullptr, nullptr, nullptr, nullptr, nullptr, state, stream);
}

hpx_status hpx_fading_load(const hpx_fading* f, int32_t num_drops, const double* los_angles, const double* nlos_angles,
                           const double* los_phases, const double* nlos_phases, const double* spatial, void* state,
                           void* stream) {
  return launch_params(f, 1, 0, 0, num_drops, los_angles, nlos_angles, los_phases, nlos_phases, spatial, state, stream);
}

hpx_status hpx_fading_draws(const hpx_fading* f, uint64_t seed, int64_t drop0, int32_t B, double* uniforms,
                            void* stream) {
  if (!f || !uniforms) return hpx_fail(HPX_ERR_ARG, "draws: null argument");
  if (B < 0 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "draws: bad drop range");
  if (B == 0) return HPX_OK;
  if (B > 65535) return hpx_fail(HPX_ERR_ARG, "draws: batch too large");
  const int num = f->nrx * f->ntx + 2 * f->L * f->S1;
  dim3 grid((num + 255) / 256, B);
  k_fading_draws<<<grid, 256, 0, as_stream(stream)>>>(num, seed, drop0, uniforms);
  HPX_LAUNCHED("draws");
  return HPX_OK;
}

hpx_status hpx_fading_taps(const hpx_fading* f, const void* state, int32_t B, int32_t T, hpx_cf32* taps, void* stream) {
  if (!f || !state || !taps) return hpx_fail(HPX_ERR_ARG, "taps: null argument");
  if (B < 0 || T < 0) return hpx_fail(HPX_ERR_ARG, "taps: negative size");
  if (B == 0 || T == 0) return HPX_OK;
  if (B > 65535 || f->L > 65535) return hpx_fail(HPX_ERR_ARG, "taps: batch too large");
  dim3 grid((T + 255) / 256 > 64 ? 64 : (T + 255) / 256, f->L, B);
  k_fading_taps<<<grid, 256, 2 * f->S1 * sizeof(int64_t), as_stream(stream)>>>(
      fading_const(f), fading_view(f, state), T, reinterpret_cast<float2*>(taps));
  HPX_LAUNCHED("taps");
  return HPX_OK;
}

hpx_status hpx_fading_csi(const hpx_fading* f, const void* state, int32_t B, int32_t T, int32_t max_num_taps,
                          hpx_cf32* csi, void* stream) {
  if (!f || !state || !csi) return hpx_fail(HPX_ERR_ARG, "csi: null argument");
  if (B < 0 || T < 0 || max_num_taps < 1) return hpx_fail(HPX_ERR_ARG, "csi: bad size");
  if (B == 0 || T == 0) return HPX_OK;
  if (B > 65535) return hpx_fail(HPX_ERR_ARG, "csi: batch too large");
  const int ntaps = std::min(1 + f->max_delay, (int)max_num_taps);
  const size_t bytes = (size_t)B * f->nrx * f->ntx * T * ntaps * sizeof(float2);
  HPX_CUDA(cudaMemsetAsync(csi, 0, bytes, as_stream(stream)));
  dim3 grid((T + 255) / 256 > 256 ? 256 : (T + 255) / 256, B);
  k_fading_csi<<<grid, 256, 0, as_stream(stream)>>>(fading_const(f), fading_view(f, state), T, ntaps,
                                                    reinterpret_cast<float2*>(csi));
  HPX_LAUNCHED("csi");
  return HPX_OK;
}

hpx_status hpx_fading_propagate(const hpx_fading* f, const void* state, int32_t B, const hpx_cf32* x, int32_t T,
                                hpx_cf32* y, const float* noise_power, uint64_t seed, int64_t drop0, void* stream) {
  if (!f || !state) return hpx_fail(HPX_ERR_ARG, "propagate: null argument");
  if (B < 0 || T < 0 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "propagate: bad size");
  if (B == 0 || T + f->max_delay == 0) return HPX_OK;
  if (!x || !y) return hpx_fail(HPX_ERR_ARG, "propagate: null buffer");
  if (B > 65535) return hpx_fail(HPX_ERR_ARG, "propagate: batch above 65535 drops per call");
  cudaStream_t s = as_stream(stream);
  switch (f->ntx) {
    case 1: return dispatch_degree<1>(f, state, B, x, T, y, noise_power, seed, drop0, s);
    case 2: return dispatch_degree<2>(f, state, B, x, T, y, noise_power, seed, drop0, s);
    case 4: return dispatch_degree<4>(f, state, B, x, T, y, noise_power, seed, drop0, s);
    case 8: return dispatch_degree<8>(f, state, B, x, T, y, noise_power, seed, drop0, s);
    case 16: return dispatch_degree<16>(f, state, B, x, T, y, noise_power, seed, drop0, s);
    default:
      if (f->ntx == 3) return dispatch_degree<3>(f, state, B, x, T, y, noise_power, seed, drop0, s);
      return hpx_fail(HPX_ERR_UNSUPPORTED, "propagate: %d transmit antennas not supported (1, 2, 3, 4, 8, 16)", f->ntx);
  }
}

hpx_status hpx_fading_ideal_csi(const hpx_fading* f, const void* state, int32_t B, const hpx_frame* frame,
                                int32_t ncols, hpx_cf32* csi, void* stream) {
  if (!f || !state || !frame || !csi) return hpx_fail(HPX_ERR_ARG, "ideal_csi: null argument");
  const int N = frame->info.num_subcarriers, W = frame->info.num_words;
  if (B < 0 || ncols < 1 || ncols > N) return hpx_fail(HPX_ERR_ARG, "ideal_csi: bad size");
  if (B == 0) return HPX_OK;
  if (B > 65535) return hpx_fail(HPX_ERR_ARG, "ideal_csi: batch too large");
  const size_t smem = (size_t)f->L * sizeof(float2) * (1 + f->S1) + f->L * sizeof(int) + 16;
  dim3 grid(W, B);
  k_ideal_csi<<<grid, 256, smem, as_stream(stream)>>>(fading_const(f), fading_view(f, state), N, W,
                                                      frame->d_window_start, frame->d_bins, frame->d_twiddle, ncols,
                                                      reinterpret_cast<float2*>(csi));
  HPX_LAUNCHED("ideal_csi");
  return HPX_OK;
}

}  // extern "C"
