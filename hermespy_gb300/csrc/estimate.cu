// MIMO channel estimation from per-stream pilots (pilot comb) and channel-estimate
// error sums.
//
// The reference's least-squares estimator handles one stream only
// (modem/waveforms/orthogonal/channel.py:32-35) and the reference has no LMMSE
// channel estimator; both MIMO estimators here are engine definitions.
//
// Tap-domain LMMSE (hpx_lmmse_*), per drop b, receive antenna r and stream t:
//   1. every pilot word p of stream t: weighted LS of the U distinct tap gains,
//        g_ls[p] = (A^H A)^-1 A^H y_p,  A[k][u] = X_k exp(-2 pi i bin_k d_u / N),
//      whose error covariance is s2 (A^H A)^-1 (diagonal E[p][u] s2 kept);
//   2. every tap u: LMMSE over the words from the pilot words,
//        g[w][u] = r_u[w]^T (R_u + s2 diag(E[.][u]))^-1 g_ls[.][u],
//      R_u[p][q] = P_u rho_u(c_p - c_q), r_u[w][p] = P_u rho_u(c_w - c_p), with
//      P_u = E|g_u|^2 and rho_u(dt) = sum_l P_l (S a_n^2 J0(w_D dt) + a_los^2 J0(w_LOS dt)) / P_u
//      the Jakes correlation of the sum-of-sinusoids taps (w in rad/sample, no 2 pi:
//      channel/fading/fading.py:307-343), c_w the window start of word w;
//   3. H[w][c] = sum_u g[w][u] exp(-2 pi i bin_c d_u / N).
// Steps 1's matrices and 2's R_u, r_u depend only on frame and channel and are
// built once on the host in double precision; the noise-dependent solve of step 2
// runs per drop on the device.
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "lmmse_dev.cuh"



namespace {

constexpr int kMaxTaps = 64;

using cd = std::complex<double>;

// In-place inverse of a Hermitian positive definite n x n matrix (row-major) by
// Gauss-Jordan elimination with partial pivoting; false if singular.
bool invert(std::vector<cd>& a, int n) {
  std::vector<cd> inv(n * n, 0.0);
  for (int i = 0; i < n; ++i) inv[i * n + i] = 1.0;
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::abs(a[r * n + c]) > std::abs(a[piv * n + c])) piv = r;
    if (std::abs(a[piv * n + c]) < 1e-12) return false;
    if (piv != c)
      for (int k = 0; k < n; ++k) {
        std::swap(a[c * n + k], a[piv * n + k]);
        std::swap(inv[c * n + k], inv[piv * n + k]);
      }
    const cd d = 1.0 / a[c * n + c];
    for (int k = 0; k < n; ++k) {
      a[c * n + k] *= d;
      inv[c * n + k] *= d;
    }
    for (int r = 0; r < n; ++r) {
      if (r == c) continue;
      const cd f = a[r * n + c];
      if (f == 0.0) continue;
      for (int k = 0; k < n; ++k) {
        a[r * n + k] -= f * a[c * n + k];
        inv[r * n + k] -= f * inv[c * n + k];
      }
    }
  }
  a.swap(inv);
  return true;
}

template <typename T>
cudaError_t upload(T** dst, const std::vector<T>& src) {
  *dst = nullptr;
  if (src.empty()) return cudaSuccess;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(dst), src.size() * sizeof(T));
  if (e != cudaSuccess) return e;
  return cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
}

// One block per (rx * ntx + t, drop).
__global__ void k_tap_lmmse(int W, int N, int U, int P, int ntx, int nrx, int ccols,
                            const int32_t* __restrict__ delay, const int32_t* __restrict__ pw_word,
                            const int32_t* __restrict__ pw_count, const int32_t* __restrict__ pw_off,
                            const int32_t* __restrict__ pcol, const float2* __restrict__ G,
                            const float* __restrict__ E, const float* __restrict__ R, const float* __restrict__ rw,
                            const int32_t* __restrict__ np_stream, const int32_t* __restrict__ bins,
                            const float2* __restrict__ tw, const float2* __restrict__ grid, int gcols,
                            const float* __restrict__ noise_power, float2* __restrict__ est) {
  extern __shared__ float4 smem4[];
  const int t = blockIdx.x % ntx, r = blockIdx.x / ntx, b = blockIdx.y;
  const int np = np_stream[t];
  float2* gls = reinterpret_cast<float2*>(smem4);  // [P][U]
  float2* gt = gls + P * U;                        // [W][U]
  float* cw = reinterpret_cast<float*>(gt + W * U);  // [U][W][P]
  int* ds = reinterpret_cast<int*>(cw + U * W * P);  // [U]
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  const float s2 = noise_power ? noise_power[b] : 0.0f;
  const float2* yb = grid + ((int64_t)b * nrx + r) * W * gcols;
  for (int u = threadIdx.x; u < U; u += blockDim.x) ds[u] = delay[u];

  // 1. weighted LS tap gains of each pilot word: one warp per (p, u) dot product
  for (int q = warp; q < np * U; q += nwarps) {
    const int p = q / U, u = q - p * U;
    const int word = pw_word[t * P + p], cnt = pw_count[t * P + p], off = pw_off[t * P + p];
    const float2* grow = G + (int64_t)off * U + (int64_t)u * cnt;
    const float2* yw = yb + (int64_t)word * gcols;
    float2 acc = make_float2(0.f, 0.f);
    for (int k = lane; k < cnt; k += 32) cfma(acc, grow[k], yw[pcol[off + k]]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      acc.x += __shfl_down_sync(0xffffffffu, acc.x, o);
      acc.y += __shfl_down_sync(0xffffffffu, acc.y, o);
    }
    if (lane == 0) gls[p * U + u] = acc;
  }

  // 2. time weights of each tap: (R_u + s2 diag(E_u)) c = r_u[w] for every word
  for (int u = threadIdx.x; u < U; u += blockDim.x) {
    float m[kMaxPilotWords][kMaxPilotWords];
    for (int i = 0; i < np; ++i)
      for (int j = 0; j < np; ++j) m[i][j] = R[((size_t)u * P + i) * P + j] + (i == j ? s2 * E[(t * P + i) * U + u] : 0.f);
    // Cholesky (lower) in place; a non-positive pivot (no signal power) zeroes the tap
    bool ok = true;
    for (int j = 0; j < np && ok; ++j) {
      float d = m[j][j];
      for (int k = 0; k < j; ++k) d -= m[j][k] * m[j][k];
      if (!(d > 0.f)) {
        ok = false;
        break;
      }
      const float inv = rsqrtf(d);
      m[j][j] = inv;  // store the reciprocal pivot
      for (int i = j + 1; i < np; ++i) {
        float s = m[i][j];
        for (int k = 0; k < j; ++k) s -= m[i][k] * m[j][k];
        m[i][j] = s * inv;
      }
    }
    for (int w = 0; w < W; ++w) {
      float z[kMaxPilotWords];
      for (int i = 0; i < np; ++i) {
        float s = ok ? rw[((size_t)u * W + w) * P + i] : 0.f;
        for (int k = 0; k < i; ++k) s -= m[i][k] * z[k];
        z[i] = ok ? s * m[i][i] : 0.f;
      }
      for (int i = np - 1; i >= 0; --i) {
        float s = z[i];
        for (int k = i + 1; k < np; ++k) s -= m[k][i] * z[k];
        z[i] = ok ? s * m[i][i] : 0.f;
      }
      for (int i = 0; i < np; ++i) cw[((size_t)u * W + w) * P + i] = z[i];
    }
  }
  __syncthreads();

  // 3. tap gains of every word
  for (int q = threadIdx.x; q < W * U; q += blockDim.x) {
    const int w = q / U, u = q - w * U;
    float2 acc = make_float2(0.f, 0.f);
    for (int p = 0; p < np; ++p) {
      const float c = cw[((size_t)u * W + w) * P + p];
      const float2 g = gls[p * U + u];
      acc.x = fmaf(c, g.x, acc.x);
      acc.y = fmaf(c, g.y, acc.y);
    }
    gt[q] = acc;
  }
  __syncthreads();

  // 4. frequency response on every grid element
  float2* out = est + (((int64_t)b * nrx + r) * ntx + t) * W * ccols;
  for (int q = threadIdx.x; q < W * ccols; q += blockDim.x) {
    const int w = q / ccols, c = q - w * ccols;
    const int bin = bins[c];
    const float2* g = gt + w * U;
    float2 acc = make_float2(0.f, 0.f);
    for (int u = 0; u < U; ++u) cfma(acc, g[u], __ldg(tw + ((bin * ds[u]) & (N - 1))));
    out[q] = acc;
  }
}

// The same estimator with one block per drop for NP = Nrx * Ntx antenna pairs: the
// tap gains of all pairs stay in shared memory ([word][tap][pair]), so each twiddle
// of the final tap DFT is gathered once and used by every pair (broadcast 16-byte
// loads of two pairs' gains, NP accumulators per grid element in registers).
template <int NP>
__global__ void __launch_bounds__(256) k_tap_lmmse_drop(LmmseView e, int nrx, int ccols,
                                                        const int32_t* __restrict__ bins,
                                                        const float2* __restrict__ tw,
                                                        const float2* __restrict__ grid, int gcols,
                                                        const float* __restrict__ noise_power,
                                                        float2* __restrict__ est) {
  extern __shared__ float4 smem4[];
  const int b = blockIdx.x;
  const int W = e.W, U = e.U;
  float2* gt = reinterpret_cast<float2*>(smem4);
  float2* gls = gt + (size_t)W * U * NP;
  float* cw = reinterpret_cast<float*>(gls + NP * e.np * U);
  int* ds = reinterpret_cast<int*>(cw + (size_t)e.ntx * U * W * e.np);
  lmmse_drop_taps<NP>(e, b, nrx, grid, gcols, noise_power ? noise_power[b] : 0.0f, gt, gls, cw, ds);
  const int64_t plane = (int64_t)W * ccols;
  float2* out = est + (int64_t)b * NP * plane;
  for (int q = threadIdx.x; q < W * ccols; q += blockDim.x) {
    const int w = q / ccols, c = q - w * ccols;
    float2 acc[NP];
    lmmse_response<NP>(gt + (size_t)w * U * NP, ds, U, e.N, bins[c], tw, acc);
#pragma unroll
    for (int i = 0; i < NP; ++i) out[i * plane + (int64_t)w * ccols + c] = acc[i];
  }
}

// Per drop: sum over the frame's data elements of |est - truth|^2 and |truth|^2 for
// every (rx, tx) pair. One block per (pair, drop).
__global__ void k_csi_error(int W, int C, int ccols, int pairs, const int8_t* __restrict__ kind,
                            const float2* __restrict__ est, const float2* __restrict__ truth, double* __restrict__ err,
                            double* __restrict__ pow) {
  const int pair = blockIdx.x, b = blockIdx.y;
  const int64_t base = ((int64_t)b * pairs + pair) * W * ccols;
  float e = 0.f, p = 0.f;
  for (int q = threadIdx.x; q < W * C; q += blockDim.x) {
    if (kind[q] != HPX_RE_DATA) continue;
    const int w = q / C, c = q - w * C;
    const float2 h = truth[base + (int64_t)w * ccols + c], g = est[base + (int64_t)w * ccols + c];
    const float dx = g.x - h.x, dy = g.y - h.y;
    e = fmaf(dx, dx, fmaf(dy, dy, e));
    p = fmaf(h.x, h.x, fmaf(h.y, h.y, p));
  }
  for (int o = 16; o > 0; o >>= 1) {
    e += __shfl_down_sync(0xffffffffu, e, o);
    p += __shfl_down_sync(0xffffffffu, p, o);
  }
  __shared__ float se[32], sp[32];
  if ((threadIdx.x & 31) == 0) {
    se[threadIdx.x >> 5] = e;
    sp[threadIdx.x >> 5] = p;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double te = 0.0, tp = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) {
      te += se[i];
      tp += sp[i];
    }
    atomicAdd(err + b, te);
    atomicAdd(pow + b, tp);
  }
}

void release(hpx_lmmse* e) {
  if (!e) return;
  void* p[] = {e->d_delay, e->d_pw_word, e->d_pw_count, e->d_pw_off, e->d_pcol, e->d_G, e->d_E, e->d_R, e->d_r, e->d_np};
  for (void* q : p)
    if (q) cudaFree(q);
  lmmse_tc_release(e);
  delete e;
}

}  // namespace

extern "C" {

hpx_status hpx_lmmse_create(const hpx_frame* frame, const hpx_fading* fading, int32_t C, hpx_lmmse** out) {
  return hpx_lmmse_create_regularized(frame, fading, C, 0.0, out);
}

hpx_status hpx_lmmse_create_regularized(const hpx_frame* frame, const hpx_fading* fading, int32_t C,
                                        double ridge_noise, hpx_lmmse** out) {
  if (!frame || !fading || !out) return hpx_fail(HPX_ERR_ARG, "lmmse: null argument");
  if (!(ridge_noise >= 0.0) || !std::isfinite(ridge_noise))
    return hpx_fail(HPX_ERR_ARG, "lmmse: ridge noise variance must be finite and non-negative");
  *out = nullptr;
  const int N = frame->info.num_subcarriers, W = frame->info.num_words, FC = frame->info.num_columns;
  const int ntx = fading->ntx;
  if (C < FC || C > N) return hpx_fail(HPX_ERR_ARG, "lmmse: columns must cover the frame's resource columns");
  const int comb = frame->pilot_comb;
  if (ntx > 1 && comb < ntx)
    return hpx_fail(HPX_ERR_UNSUPPORTED, "lmmse: %d streams need a pilot comb of at least %d (frame has %d)", ntx, ntx,
                    comb);
  // distinct delays below N with their power and correlation terms
  std::vector<int> delays;
  for (int l = 0; l < fading->L; ++l) {
    const int d = fading->h_delay[l];
    if (d < N && (delays.empty() || delays.back() != d)) delays.push_back(d);  // delays are sorted
  }
  const int U = (int)delays.size();
  if (U < 1 || U > kMaxTaps) return hpx_fail(HPX_ERR_UNSUPPORTED, "lmmse: %d distinct tap delays (1..%d)", U, kMaxTaps);
  const double wn = fading->doppler / fading->fs, wl = fading->los_doppler / fading->fs;
  const double S = fading->S;
  std::vector<double> Pu(U, 0.0);
  auto rho_num = [&](int u, double dt) {
    double s = 0.0;
    for (int l = 0; l < fading->L; ++l) {
      if (fading->h_delay[l] != delays[u]) continue;
      const double an = fading->h_amp_nlos[l], al = fading->h_amp_los[l];
      s += S * an * an * j0(wn * dt) + al * al * j0(wl * dt);
    }
    return s;
  };
  for (int u = 0; u < U; ++u) Pu[u] = rho_num(u, 0.0);
  // pilots per stream and word, frame order
  std::vector<int> ref_word, ref_col;
  for (int w = 0; w < W; ++w)
    for (int c = 0; c < FC; ++c)
      if (frame->h_kind[(size_t)w * FC + c] == HPX_RE_REFERENCE) {
        ref_word.push_back(w);
        ref_col.push_back(c);
      }
  const int order = frame->info.modulation_order;
  std::vector<int32_t> pw_word(ntx * kMaxPilotWords, -1), pw_count(ntx * kMaxPilotWords, 0),
      pw_off(ntx * kMaxPilotWords, 0), np_stream(ntx, 0), pcol;
  std::vector<float2> G;
  std::vector<float> E(ntx * kMaxPilotWords * U, 0.f);
  std::vector<std::vector<int>> stream_words(ntx);
  for (int t = 0; t < ntx; ++t) {
    int np = 0;
    for (int w = 0; w < W; ++w) {
      std::vector<int> ks;
      for (size_t k = 0; k < ref_word.size(); ++k)
        if (ref_word[k] == w && (comb <= 1 || ref_col[k] % comb == t % comb)) ks.push_back((int)k);
      if (ks.empty()) continue;
      if (np == kMaxPilotWords)
        return hpx_fail(HPX_ERR_UNSUPPORTED, "lmmse: more than %d pilot words per stream", kMaxPilotWords);
      const int n = (int)ks.size();
      if (n < U)
        return hpx_fail(HPX_ERR_UNSUPPORTED, "lmmse: word %d has %d pilots of stream %d for %d tap delays", w, n, t, U);
      std::vector<cd> A((size_t)n * U);
      for (int i = 0; i < n; ++i) {
        const float2 x = qam_symbol(order, (uint32_t)(ks[i] % order));
        const int bin = frame->h_bins[ref_col[ks[i]]];
        for (int u = 0; u < U; ++u) {
          const double a = -2.0 * M_PI * (double)((int64_t)bin * delays[u] % N) / N;
          A[(size_t)i * U + u] = cd(x.x, x.y) * cd(std::cos(a), std::sin(a));
        }
      }
      std::vector<cd> AhA((size_t)U * U, 0.0);
      for (int u = 0; u < U; ++u)
        for (int v = 0; v < U; ++v) {
          cd s = 0.0;
          for (int i = 0; i < n; ++i) s += std::conj(A[(size_t)i * U + u]) * A[(size_t)i * U + v];
          AhA[(size_t)u * U + v] = s;
        }
      // plain: (A^H A)^-1 A^H, noise per tap diag((A^H A)^-1); regularized with the prior
      // profile: M = A^H A + ridge diag(1 / P_u), M^-1 A^H, noise per tap diag(M^-1 A^H A M^-1)
      std::vector<cd> AhA0;
      if (ridge_noise > 0.0) {
        AhA0 = AhA;
        for (int u = 0; u < U; ++u) AhA[(size_t)u * U + u] += ridge_noise / std::max(Pu[u], 1e-300);
      }
      if (!invert(AhA, U)) return hpx_fail(HPX_ERR_UNSUPPORTED, "lmmse: pilot geometry of word %d is singular", w);
      std::vector<double> noise_tap(U);
      for (int u = 0; u < U; ++u) {
        if (ridge_noise > 0.0) {
          cd sum = 0.0;  // (M^-1 A^H A M^-1)[u][u]
          for (int a = 0; a < U; ++a) {
            cd t = 0.0;
            for (int b = 0; b < U; ++b) t += AhA0[(size_t)a * U + b] * std::conj(AhA[(size_t)u * U + b]);
            sum += AhA[(size_t)u * U + a] * t;
          }
          noise_tap[u] = sum.real();
        } else {
          noise_tap[u] = AhA[(size_t)u * U + u].real();
        }
      }
      pw_word[t * kMaxPilotWords + np] = w;
      pw_count[t * kMaxPilotWords + np] = n;
      pw_off[t * kMaxPilotWords + np] = (int)pcol.size();
      for (int i = 0; i < n; ++i) pcol.push_back(ref_col[ks[i]]);
      const size_t g0 = G.size();
      G.resize(g0 + (size_t)U * n);
      for (int u = 0; u < U; ++u) {
        E[(t * kMaxPilotWords + np) * U + u] = (float)noise_tap[u];
        for (int i = 0; i < n; ++i) {
          cd s = 0.0;
          for (int v = 0; v < U; ++v) s += AhA[(size_t)u * U + v] * std::conj(A[(size_t)i * U + v]);
          G[g0 + (size_t)u * n + i] = make_float2((float)s.real(), (float)s.imag());
        }
      }
      stream_words[t].push_back(w);
      ++np;
    }
    if (np == 0) return hpx_fail(HPX_ERR_UNSUPPORTED, "lmmse: stream %d has no pilots", t);
    np_stream[t] = np;
  }
  // time statistics: all streams share the pilot words when they share words;
  // R and r are per tap, indexed by the stream's own pilot-word order (same order for every stream
  // under a pilot comb, whose streams use the same words)
  for (int t = 1; t < ntx; ++t)
    if (stream_words[t] != stream_words[0])
      return hpx_fail(HPX_ERR_UNSUPPORTED, "lmmse: streams must carry pilots in the same words");
  const int P = kMaxPilotWords;
  const int np = np_stream[0];
  std::vector<float> R((size_t)U * P * P, 0.f), rw((size_t)U * W * P, 0.f);
  for (int u = 0; u < U; ++u) {
    for (int i = 0; i < np; ++i)
      for (int j = 0; j < np; ++j) {
        const double dt = (double)frame->h_window_start[stream_words[0][i]] - frame->h_window_start[stream_words[0][j]];
        R[((size_t)u * P + i) * P + j] = (float)rho_num(u, dt);
      }
    for (int w = 0; w < W; ++w)
      for (int i = 0; i < np; ++i) {
        const double dt = (double)frame->h_window_start[w] - frame->h_window_start[stream_words[0][i]];
        rw[((size_t)u * W + w) * P + i] = (float)rho_num(u, dt);
      }
  }
  hpx_lmmse* e = new hpx_lmmse();
  e->frame = frame;
  e->C = C;
  e->ntx = ntx;
  e->U = U;
  e->P = P;
  e->N = N;
  e->W = W;
  e->np = np;
  std::vector<int32_t> dl(delays.begin(), delays.end());
  cudaError_t err;
  if ((err = upload(&e->d_delay, dl)) != cudaSuccess || (err = upload(&e->d_pw_word, pw_word)) != cudaSuccess ||
      (err = upload(&e->d_pw_count, pw_count)) != cudaSuccess || (err = upload(&e->d_pw_off, pw_off)) != cudaSuccess ||
      (err = upload(&e->d_pcol, pcol)) != cudaSuccess || (err = upload(&e->d_G, G)) != cudaSuccess ||
      (err = upload(&e->d_E, E)) != cudaSuccess || (err = upload(&e->d_R, R)) != cudaSuccess ||
      (err = upload(&e->d_r, rw)) != cudaSuccess || (err = upload(&e->d_np, np_stream)) != cudaSuccess) {
    release(e);
    return hpx_cuda_status(err, "lmmse tables");
  }
  if (ntx == 4 && 2 * U <= 128) {  // the 4 x 4 receiver's tensor-core path
    const hpx_status st = lmmse_tc_prepare(e, delays, G, pw_count, pw_off, pcol);
    if (st != HPX_OK) {
      release(e);
      return st;
    }
  }
  *out = e;
  return HPX_OK;
}

hpx_status hpx_lmmse_destroy(hpx_lmmse* e) {
  release(e);
  return HPX_OK;
}

hpx_status hpx_lmmse_estimate(const hpx_lmmse* e, const hpx_cf32* grid, int32_t gcols, int32_t nrx, int32_t B,
                              const float* noise_power, hpx_cf32* est, void* stream) {
  if (!e || !grid || !est) return hpx_fail(HPX_ERR_ARG, "lmmse_estimate: null argument");
  if (B < 0 || nrx < 1) return hpx_fail(HPX_ERR_ARG, "lmmse_estimate: bad batch");
  if (gcols < e->frame->info.num_columns) return hpx_fail(HPX_ERR_SHAPE, "lmmse_estimate: grid too narrow");
  if (B == 0) return HPX_OK;
  if (B > 65535) return hpx_fail(HPX_ERR_ARG, "lmmse_estimate: batch above 65535 drops per call");
  if (nrx * e->ntx > 65535) return hpx_fail(HPX_ERR_ARG, "lmmse_estimate: too many antenna pairs");
  const int NPAIRS = nrx * e->ntx;
  const size_t smem_drop = lmmse_taps_smem(e->W, e->U, e->np, e->ntx, NPAIRS);
  const bool per_drop = (NPAIRS == 1 || NPAIRS == 2 || NPAIRS == 4 || NPAIRS == 8 || NPAIRS == 16) &&
                        smem_drop <= 200 * 1024;
  if (per_drop) {
    const LmmseView v = lmmse_view(e);
    auto launch = [&](auto kern) -> hpx_status {
      if (smem_drop > 48 * 1024)
        HPX_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem_drop));
      kern<<<B, 256, smem_drop, as_stream(stream)>>>(v, nrx, e->C, e->frame->d_bins, e->frame->d_twiddle,
                                                     reinterpret_cast<const float2*>(grid), gcols, noise_power,
                                                     reinterpret_cast<float2*>(est));
      HPX_LAUNCHED("tap_lmmse");
      return HPX_OK;
    };
    switch (NPAIRS) {
      case 1: return launch(k_tap_lmmse_drop<1>);
      case 2: return launch(k_tap_lmmse_drop<2>);
      case 4: return launch(k_tap_lmmse_drop<4>);
      case 8: return launch(k_tap_lmmse_drop<8>);
      default: return launch(k_tap_lmmse_drop<16>);
    }
  }
  const size_t smem = (size_t)(e->P * e->U + e->W * e->U) * sizeof(float2) +
                      (size_t)e->U * e->W * e->P * sizeof(float) + (size_t)e->U * sizeof(int) + 16;
  if (smem > 200 * 1024) return hpx_fail(HPX_ERR_UNSUPPORTED, "lmmse_estimate: frame too long for one block");
  if (smem > 48 * 1024)
    HPX_CUDA(cudaFuncSetAttribute(k_tap_lmmse, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 g(nrx * e->ntx, B);
  k_tap_lmmse<<<g, 256, smem, as_stream(stream)>>>(
      e->W, e->N, e->U, e->P, e->ntx, nrx, e->C, e->d_delay, e->d_pw_word, e->d_pw_count, e->d_pw_off, e->d_pcol,
      e->d_G, e->d_E, e->d_R, e->d_r, e->d_np, e->frame->d_bins, e->frame->d_twiddle,
      reinterpret_cast<const float2*>(grid), gcols, noise_power, reinterpret_cast<float2*>(est));
  HPX_LAUNCHED("tap_lmmse");
  return HPX_OK;
}

hpx_status hpx_csi_error(const hpx_frame* frame, const hpx_cf32* est, const hpx_cf32* truth, int32_t ccols,
                         int32_t pairs, int32_t B, double* err, double* power, void* stream) {
  if (!frame || !est || !truth || !err || !power) return hpx_fail(HPX_ERR_ARG, "csi_error: null argument");
  if (B < 0 || pairs < 1) return hpx_fail(HPX_ERR_ARG, "csi_error: bad sizes");
  if (ccols < frame->info.num_columns) return hpx_fail(HPX_ERR_SHAPE, "csi_error: CSI narrower than the frame");
  if (B == 0) return HPX_OK;
  if (B > 65535 || pairs > 65535) return hpx_fail(HPX_ERR_ARG, "csi_error: batch too large");
  cudaStream_t s = as_stream(stream);
  HPX_CUDA(cudaMemsetAsync(err, 0, sizeof(double) * B, s));
  HPX_CUDA(cudaMemsetAsync(power, 0, sizeof(double) * B, s));
  dim3 g(pairs, B);
  k_csi_error<<<g, 256, 0, s>>>(frame->info.num_words, frame->info.num_columns, ccols, pairs, frame->d_kind,
                                reinterpret_cast<const float2*>(est), reinterpret_cast<const float2*>(truth), err,
                                power);
  HPX_LAUNCHED("csi_error");
  return HPX_OK;
}

}  // extern "C"
