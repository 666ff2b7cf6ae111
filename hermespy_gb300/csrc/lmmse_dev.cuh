// Device side of the tap-domain LMMSE channel estimator, shared by the estimate
// kernel (CSI grid output) and the fused LMMSE receiver.
#pragma once

#include "hpx_internal.cuh"

struct LmmseView {
  int W, N, U, P, ntx, np;
  const int32_t* delay;
  const int32_t* pw_word;
  const int32_t* pw_count;
  const int32_t* pw_off;
  const int32_t* pcol;
  const float2* G;
  const float* E;
  const float* R;
  const float* rw;
  const int32_t* np_stream;
};

static inline LmmseView lmmse_view(const hpx_lmmse* e) {
  return LmmseView{e->W, e->N, e->U, e->P, e->ntx, e->np, e->d_delay, e->d_pw_word, e->d_pw_count, e->d_pw_off,
                   e->d_pcol, e->d_G, e->d_E, e->d_R, e->d_r, e->d_np};
}

// Shared memory of lmmse_drop_taps: gt [W][U][NP] float2, gls [NP][np][U] float2,
// cw [ntx][U][W][np] floats, ds [U] ints (np = pilot words per stream).
__host__ __device__ inline size_t lmmse_taps_smem(int W, int U, int np, int ntx, int NP) {
  return (size_t)W * U * NP * 8 + (size_t)NP * np * U * 8 + (size_t)ntx * U * W * np * 4 + (size_t)U * 4 + 16;
}

// Per stream t and tap u the LMMSE weights of the np pilot words for every word w:
// solve (R_u + s2 diag(E_t,u)) z = r_u(w) by Cholesky, cw[t][u][w][.] = z. A tap
// without signal power (non-positive pivot) gets zero weights. NPW >= np is the
// compile-time bound of the system (exact size when np == NPW).
template <int NPW>
__device__ __forceinline__ void lmmse_word_weights(const LmmseView& e, float s2, float* cw, int np = NPW) {
  const int W = e.W, U = e.U, P = e.P, ntx = e.ntx;
  for (int q = threadIdx.x; q < ntx * U; q += blockDim.x) {
    const int t = q / U, u = q - t * U;
    float m[NPW][NPW];
#pragma unroll
    for (int i = 0; i < NPW; ++i)
#pragma unroll
      for (int j = 0; j < NPW; ++j)
        m[i][j] = (i < np && j < np)
                      ? e.R[((size_t)u * P + i) * P + j] + (i == j ? s2 * e.E[(t * P + i) * U + u] : 0.f)
                      : 0.f;
    bool ok = true;
#pragma unroll
    for (int j = 0; j < NPW; ++j) {
      if (j >= np) break;
      float d = m[j][j];
#pragma unroll
      for (int k = 0; k < j; ++k) d -= m[j][k] * m[j][k];
      if (!(d > 0.f)) ok = false;  // no signal power on this tap: its gains stay zero
      const float inv = ok ? rsqrtf(d) : 0.f;
      m[j][j] = inv;
#pragma unroll
      for (int i = j + 1; i < NPW; ++i) {
        if (i >= np) break;
        float sm = m[i][j];
#pragma unroll
        for (int k = 0; k < j; ++k) sm -= m[i][k] * m[j][k];
        m[i][j] = sm * inv;
      }
    }
    for (int w = 0; w < W; ++w) {
      float z[NPW];
#pragma unroll
      for (int i = 0; i < NPW; ++i) {
        if (i >= np) break;
        float sm = ok ? e.rw[((size_t)u * W + w) * P + i] : 0.f;
#pragma unroll
        for (int k = 0; k < i; ++k) sm -= m[i][k] * z[k];
        z[i] = ok ? sm * m[i][i] : 0.f;
      }
#pragma unroll
      for (int i = NPW - 1; i >= 0; --i) {
        if (i >= np) continue;
        float sm = z[i];
#pragma unroll
        for (int k = i + 1; k < NPW; ++k)
          if (k < np) sm -= m[k][i] * z[k];
        z[i] = ok ? sm * m[i][i] : 0.f;
      }
#pragma unroll
      for (int i = 0; i < NPW; ++i)
        if (i < np) cw[(((size_t)t * U + u) * W + w) * np + i] = z[i];
    }
  }
}

// The weights of lmmse_word_weights for the words wlist[0 .. nwl) only (-1 entries
// skipped), one thread per (stream, tap, word) system: each thread factors its own
// np x np matrix (np == NPW) and solves for its word, with the same operations as
// lmmse_word_weights, so the weights are identical. cw layout as there.
template <int NPW>
__device__ __forceinline__ void lmmse_listed_word_weights(const LmmseView& e, float s2, const int32_t* __restrict__ wlist,
                                                          int nwl, float* cw) {
  const int W = e.W, U = e.U, P = e.P;
  for (int q = threadIdx.x; q < e.ntx * U * nwl; q += blockDim.x) {
    const int tu = q / nwl, wi = q - tu * nwl, t = tu / U, u = tu - t * U;
    const int w = wlist[wi];
    if (w < 0) continue;
    float m[NPW][NPW];
#pragma unroll
    for (int i = 0; i < NPW; ++i)
#pragma unroll
      for (int j = 0; j < NPW; ++j)
        m[i][j] = e.R[((size_t)u * P + i) * P + j] + (i == j ? s2 * e.E[(t * P + i) * U + u] : 0.f);
    bool ok = true;
#pragma unroll
    for (int j = 0; j < NPW; ++j) {
      float d = m[j][j];
#pragma unroll
      for (int k = 0; k < j; ++k) d -= m[j][k] * m[j][k];
      if (!(d > 0.f)) ok = false;  // no signal power on this tap: its gains stay zero
      const float inv = ok ? rsqrtf(d) : 0.f;
      m[j][j] = inv;
#pragma unroll
      for (int i = j + 1; i < NPW; ++i) {
        float sm = m[i][j];
#pragma unroll
        for (int k = 0; k < j; ++k) sm -= m[i][k] * m[j][k];
        m[i][j] = sm * inv;
      }
    }
    float z[NPW];
#pragma unroll
    for (int i = 0; i < NPW; ++i) {
      float sm = ok ? e.rw[((size_t)u * W + w) * P + i] : 0.f;
#pragma unroll
      for (int k = 0; k < i; ++k) sm -= m[i][k] * z[k];
      z[i] = ok ? sm * m[i][i] : 0.f;
    }
#pragma unroll
    for (int i = NPW - 1; i >= 0; --i) {
      float sm = z[i];
#pragma unroll
      for (int k = i + 1; k < NPW; ++k) sm -= m[k][i] * z[k];
      z[i] = ok ? sm * m[i][i] : 0.f;
    }
#pragma unroll
    for (int i = 0; i < NPW; ++i) cw[(((size_t)t * U + u) * W + w) * NPW + i] = z[i];
  }
}

// lmmse_word_weights with register-resident systems for the usual pilot-word counts.
__device__ __forceinline__ void lmmse_word_weights_np(const LmmseView& e, float s2, float* cw) {
  switch (e.np) {
    case 1: lmmse_word_weights<1>(e, s2, cw); break;
    case 2: lmmse_word_weights<2>(e, s2, cw); break;
    case 3: lmmse_word_weights<3>(e, s2, cw); break;
    case 4: lmmse_word_weights<4>(e, s2, cw); break;
    default: lmmse_word_weights<kMaxPilotWords>(e, s2, cw, e.np); break;
  }
}

// Tap gains of every antenna pair and word of drop b into gt (pair = rx * ntx + tx),
// stored as planes: for word w and tap u, NP real parts then NP imaginary parts
// (float index (w U + u) 2 NP + {0, NP} + pair), so two pairs share each packed
// FP32x2 FMA of the response. All threads of the block:
//   1. weighted LS of the tap gains on each pilot word (one warp per dot product),
//   2. per stream and tap the LMMSE weights over the words (np x np Cholesky),
//   3. gt[w][u][pair] = sum_p weight * LS gain.
// ds receives the tap delays. Ends with __syncthreads.
template <int NP>
__device__ __forceinline__ void lmmse_drop_taps(const LmmseView& e, int b, int nrx, const float2* __restrict__ grid,
                                                int gcols, float s2, float2* gt, float2* gls, float* cw, int* ds) {
  const int W = e.W, U = e.U, P = e.P, ntx = e.ntx;
  const int np = e.np;  // every stream has the same pilot words (checked at create time)
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
  for (int u = threadIdx.x; u < U; u += blockDim.x) ds[u] = e.delay[u];
  // One warp per (stream, pilot word, pair of receive antennas): the word's received
  // pilots of both antennas stay in registers (lane holds pilots lane + 32 j, up to 160
  // per pass over the row) while the warp walks the U rows of the stream's
  // weighted-LS matrix, each row load serving both antennas. Per (antenna, tap) the
  // lane sums run over j and the warp sum is the same shuffle tree as for one antenna.
  constexpr int YR = 5;
  const int rgroups = (nrx + 1) / 2;
  for (int q = warp; q < ntx * np * rgroups; q += nwarps) {
    const int t = q / (np * rgroups), rem = q - t * np * rgroups, p = rem / rgroups;
    const int r0 = 2 * (rem - p * rgroups), nr = min(2, nrx - r0);
    const int word = e.pw_word[t * P + p], cnt = e.pw_count[t * P + p], off = e.pw_off[t * P + p];
    const float2* Gp = e.G + (int64_t)off * U;
    for (int k0 = 0; k0 < cnt; k0 += 32 * YR) {
      float2 yv[2][YR];
#pragma unroll
      for (int rr = 0; rr < 2; ++rr) {
        const float2* yw = grid + (((int64_t)b * nrx + r0 + min(rr, nr - 1)) * W + word) * gcols;
#pragma unroll
        for (int j = 0; j < YR; ++j) {
          const int k = k0 + lane + 32 * j;
          yv[rr][j] = k < cnt ? yw[e.pcol[off + k]] : make_float2(0.f, 0.f);
        }
      }
      for (int u = 0; u < U; ++u) {
        const float2* grow = Gp + (int64_t)u * cnt;
        float2 acc[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
#pragma unroll
        for (int j = 0; j < YR; ++j) {
          const int k = k0 + lane + 32 * j;
          if (k < cnt) {
            const float2 g = grow[k];
            cfma(acc[0], g, yv[0][j]);
            cfma(acc[1], g, yv[1][j]);
          }
        }
#pragma unroll
        for (int rr = 0; rr < 2; ++rr) {
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            acc[rr].x += __shfl_down_sync(0xffffffffu, acc[rr].x, o);
            acc[rr].y += __shfl_down_sync(0xffffffffu, acc[rr].y, o);
          }
        }
        if (lane == 0) {
          for (int rr = 0; rr < nr; ++rr) {
            float2* dst = gls + (((r0 + rr) * ntx + t) * np + p) * U + u;
            *dst = k0 == 0 ? acc[rr] : cadd(*dst, acc[rr]);
          }
        }
      }
    }
  }
  lmmse_word_weights_np(e, s2, cw);
  __syncthreads();
  float* gtf = reinterpret_cast<float*>(gt);
  for (int q = threadIdx.x; q < W * U * NP; q += blockDim.x) {
    const int w = q / (U * NP), rem = q - w * U * NP, u = rem / NP, pair = rem - u * NP;
    const int t = pair % ntx;
    float2 acc = make_float2(0.f, 0.f);
    for (int p = 0; p < np; ++p) {
      const float c = cw[(((size_t)t * U + u) * W + w) * np + p];
      const float2 g = gls[(pair * np + p) * U + u];
      acc.x = fmaf(c, g.x, acc.x);
      acc.y = fmaf(c, g.y, acc.y);
    }
    float* dst = gtf + ((size_t)w * U + u) * 2 * NP;
    dst[pair] = acc.x;
    dst[NP + pair] = acc.y;
  }
  __syncthreads();
}

// Channel of all NP pairs at one element: H[pair] = sum_u g_w[u][pair] tw[bin d_u],
// each twiddle gathered once; g_w points at the word's planes (see lmmse_drop_taps).
// Pairs are processed two at a time: re += gx t.x - gy t.y and im += gx t.y + gy t.x
// as packed FP32x2 FMAs with (gx, gy) of two pairs from 16-byte loads.
template <int NP>
__device__ __forceinline__ void lmmse_response(const float2* gt_w, const int* ds, int U, int N, int bin,
                                               const float2* __restrict__ tw, float2 (&acc)[NP]) {
  const float* g = reinterpret_cast<const float*>(gt_w);
  if constexpr (NP == 1) {
    acc[0] = make_float2(0.f, 0.f);
    for (int u = 0; u < U; ++u) {
      const float2 t = __ldg(tw + ((bin * ds[u]) & (N - 1)));
      cfma(acc[0], make_float2(g[2 * u], g[2 * u + 1]), t);
    }
  } else {
  constexpr int H2 = NP / 2;
  float2 re[H2], im[H2];
#pragma unroll
  for (int i = 0; i < H2; ++i) re[i] = im[i] = make_float2(0.f, 0.f);
  for (int u = 0; u < U; ++u) {
    const float2 t = __ldg(tw + ((bin * ds[u]) & (N - 1)));
    const float2 tx = make_float2(t.x, t.x), ty = make_float2(t.y, t.y), nty = make_float2(-t.y, -t.y);
    const float* gu = g + (size_t)u * 2 * NP;
    if constexpr (NP % 4 == 0) {  // 16-byte loads: the gains of four pairs at once
#pragma unroll
      for (int i = 0; i < NP / 4; ++i) {
        const float4 gx = *reinterpret_cast<const float4*>(gu + 4 * i);
        const float4 gy = *reinterpret_cast<const float4*>(gu + NP + 4 * i);
        const float2 gx0 = make_float2(gx.x, gx.y), gx1 = make_float2(gx.z, gx.w);
        const float2 gy0 = make_float2(gy.x, gy.y), gy1 = make_float2(gy.z, gy.w);
        re[2 * i] = __ffma2_rn(gx0, tx, re[2 * i]);
        re[2 * i] = __ffma2_rn(gy0, nty, re[2 * i]);
        im[2 * i] = __ffma2_rn(gx0, ty, im[2 * i]);
        im[2 * i] = __ffma2_rn(gy0, tx, im[2 * i]);
        re[2 * i + 1] = __ffma2_rn(gx1, tx, re[2 * i + 1]);
        re[2 * i + 1] = __ffma2_rn(gy1, nty, re[2 * i + 1]);
        im[2 * i + 1] = __ffma2_rn(gx1, ty, im[2 * i + 1]);
        im[2 * i + 1] = __ffma2_rn(gy1, tx, im[2 * i + 1]);
      }
    } else {
#pragma unroll
      for (int i = 0; i < H2; ++i) {
        const float2 gx = *reinterpret_cast<const float2*>(gu + 2 * i);
        const float2 gy = *reinterpret_cast<const float2*>(gu + NP + 2 * i);
        re[i] = __ffma2_rn(gx, tx, re[i]);
        re[i] = __ffma2_rn(gy, nty, re[i]);
        im[i] = __ffma2_rn(gx, ty, im[i]);
        im[i] = __ffma2_rn(gy, tx, im[i]);
      }
    }
  }
#pragma unroll
  for (int i = 0; i < H2; ++i) {
    acc[2 * i] = make_float2(re[i].x, im[i].x);
    acc[2 * i + 1] = make_float2(re[i].y, im[i].y);
  }
  }
}
