// Register-blocked Stockham FFT for one OFDM word per group of TP threads.
//
// A transform of N = R_0 R_1 ... points runs in stages; stage s has radix R_s and
// span Ns = R_0 ... R_{s-1}. Butterfly j (0 <= j < N/R_s) of a stage reads the
// R_s points j + r N/R_s, multiplies point r by exp(-+2 pi i r k / (Ns R_s)) with
// k = j mod Ns, computes a DFT of length R_s in registers and writes point r to
// (j - k) R_s + k + r Ns. Each thread of a transform owns N/TP points (one or
// more butterflies) per stage; points move between stages through shared memory
// (padded by one complex every 16 to spread banks). The first stage reads its
// points through a caller functor (device memory or generated symbols) and the
// last stage hands the natural-order results to another functor, so a transform
// touches HBM exactly once in each direction.
#pragma once

#include "hpx_internal.cuh"

namespace fft {

// cos / sin (2 pi t / 32) for any integer t, from the float32 of the float64
// values of t = 0..8 (t = 8 exact). A constant t folds to an immediate.
__host__ __device__ constexpr float cos32_base(int t) {
  return t == 0 ? 1.0f
       : t == 1 ? 0.9807852506637573f
       : t == 2 ? 0.9238795042037964f
       : t == 3 ? 0.8314695954322815f
       : t == 4 ? 0.7071067690849304f
       : t == 5 ? 0.5555702447891235f
       : t == 6 ? 0.3826834261417389f
       : t == 7 ? 0.19509032368659973f
       : 0.0f;
}
// Not recursive, so that every call inlines and folds: cos of the quarter-turn
// reduction u -> r in [0, 8] with the sign of the half-turn, sin(x) = cos(x - pi / 2).
__host__ __device__ __forceinline__ constexpr float cos32(int t) {
  const int u = t & 31;
  const int r = u <= 8 ? u : (u < 16 ? 16 - u : (u <= 24 ? u - 16 : 32 - u));
  return (u > 8 && u < 24) ? -cos32_base(r) : cos32_base(r);
}
__host__ __device__ __forceinline__ constexpr float sin32(int t) { return cos32(t - 8); }

// v * exp(-+2 pi i t / 32) with the sign of the exponent set by INV.
template <bool INV>
__device__ __forceinline__ float2 twiddle32(float2 v, int t) {
  t &= 31;
  if (t == 0) return v;
  if (t == 8) return INV ? make_float2(-v.y, v.x) : make_float2(v.y, -v.x);
  if (t == 16) return make_float2(-v.x, -v.y);
  if (t == 24) return INV ? make_float2(v.y, -v.x) : make_float2(-v.y, v.x);
  const float c = cos32(t), s = INV ? sin32(t) : -sin32(t);
  return make_float2(v.x * c - v.y * s, v.x * s + v.y * c);
}

// Complex sum and difference as packed FP32x2 adds (round to nearest, the same
// results as two scalar adds each).
__device__ __forceinline__ void dft2(float2& a, float2& b) {
  const float2 t = a;
  a = __fadd2_rn(t, b);
  b = __fadd2_rn(t, make_float2(-b.x, -b.y));
}

// In-register DFT of length R in {2, 4, 8, 16, 32}, natural order in and out.
// R > 4 splits as 4 x (R/4): DFT-4 over stride R/4, twiddles W_R^(n2 k1), DFT-(R/4)
// of contiguous groups, then the index transposition k1 + 4 k2 <- (R/4) k1 + k2.
// Every index is a compile-time constant, so the arrays stay in registers.
template <int R, bool INV>
__device__ __forceinline__ void dft(float2 (&a)[R]) {
  if constexpr (R == 2) {
    dft2(a[0], a[1]);
  } else if constexpr (R == 4) {
    dft2(a[0], a[2]);
    dft2(a[1], a[3]);
    a[3] = twiddle32<INV>(a[3], 8);
    dft2(a[0], a[1]);
    dft2(a[2], a[3]);
    const float2 t = a[1];
    a[1] = a[2];
    a[2] = t;
  } else {
    constexpr int R2 = R / 4;
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) {
      float2 q[4] = {a[n2], a[R2 + n2], a[2 * R2 + n2], a[3 * R2 + n2]};
      dft<4, INV>(q);
#pragma unroll
      for (int k1 = 0; k1 < 4; ++k1) a[k1 * R2 + n2] = twiddle32<INV>(q[k1], n2 * k1 * (32 / R));
    }
    float2 out[R];
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
      float2 g[R2];
#pragma unroll
      for (int n2 = 0; n2 < R2; ++n2) g[n2] = a[k1 * R2 + n2];
      dft<R2, INV>(g);
#pragma unroll
      for (int k2 = 0; k2 < R2; ++k2) out[k1 + 4 * k2] = g[k2];
    }
#pragma unroll
    for (int k = 0; k < R; ++k) a[k] = out[k];
  }
}

// One padding slot every 16 points: the first stage's stride-R writes of a half-warp
// (16 lanes x 8 bytes) then fall on distinct banks.
__device__ __forceinline__ int pad(int i) { return i + (i >> 4); }
template <int N>
__host__ __device__ constexpr int padded() { return N + N / 16; }

// Stage plan of an N-point transform: radices (product N), threads per transform.
template <int N>
struct Plan;
template <> struct Plan<64> { static constexpr int S = 2, TP = 8, R0 = 8, R1 = 8, R2 = 1; };
template <> struct Plan<128> { static constexpr int S = 2, TP = 8, R0 = 16, R1 = 8, R2 = 1; };
template <> struct Plan<256> { static constexpr int S = 2, TP = 16, R0 = 16, R1 = 16, R2 = 1; };
template <> struct Plan<512> { static constexpr int S = 3, TP = 32, R0 = 16, R1 = 16, R2 = 2; };
template <> struct Plan<1024> { static constexpr int S = 3, TP = 64, R0 = 16, R1 = 16, R2 = 4; };
template <> struct Plan<2048> { static constexpr int S = 3, TP = 128, R0 = 16, R1 = 16, R2 = 8; };
template <> struct Plan<4096> { static constexpr int S = 3, TP = 256, R0 = 16, R1 = 16, R2 = 16; };

template <int TP>
__device__ __forceinline__ void sync_group() {
  if (TP <= 32) __syncwarp();
  else __syncthreads();
}

// Stage twiddles: stage s with span Ns and radix R reads exp(-2 pi i r k / (Ns R))
// from entry (r Ns + k) of its table, so lanes with consecutive k load consecutive
// entries; radix 8 and 16 stages load r = 1..4 and multiply up the rest. Tables of the second and third stage are stored back to back
// (stage 2 at 0, stage 3 at R0 R1); 2 N entries cover every plan.
template <int N>
__host__ __device__ constexpr int stage_table_offset(int s) {
  return s == 1 ? 0 : Plan<N>::R0 * Plan<N>::R1;
}

// One Stockham stage with radix R for the transform whose points live in `buf`
// (padded). FIRST: inputs via load(idx); LAST: outputs via store(idx, v). `tw`
// is this stage's twiddle table.
template <int N, int TP, int R, bool INV, bool FIRST, bool LAST, typename Load, typename Store>
__device__ __forceinline__ void stage(float2* buf, int t, int Ns, const float2* __restrict__ tw, Load& load,
                                      Store& store) {
  constexpr int BPT = N / R / TP;  // butterflies per thread
  constexpr int Q = N / R;         // stride between a butterfly's points
  float2 a[BPT][R];
#pragma unroll
  for (int b = 0; b < BPT; ++b) {
    const int j = t + b * TP;
#pragma unroll
    for (int r = 0; r < R; ++r) a[b][r] = FIRST ? load(j + r * Q) : buf[pad(j + r * Q)];
  }
  if (!FIRST && !LAST) sync_group<TP>();  // every point read before the in-place writes
#pragma unroll
  for (int b = 0; b < BPT; ++b) {
    const int j = t + b * TP;
    const int k = j & (Ns - 1);
    if (Ns > 1) {
      if constexpr (R <= 4) {
#pragma unroll
        for (int r = 1; r < R; ++r) {
          float2 w = __ldg(tw + r * Ns + k);
          if (INV) w.y = -w.y;
          a[b][r] = cmul(a[b][r], w);
        }
      } else {
        // twiddles 1..4 from the table, r > 4 as w_(r-4) w_4 (at most three products
        // deep, a few 1e-7 relative): 4 loads instead of R - 1 per butterfly
        float2 wv[4];
#pragma unroll
        for (int r = 1; r <= 4; ++r) wv[r & 3] = __ldg(tw + r * Ns + k);
        const float2 w4 = wv[0];
#pragma unroll
        for (int r = 1; r < R; ++r) {
          float2 w = wv[r & 3];
          if (r > 4) {
            w = cmul(w, w4);
            wv[r & 3] = w;
          }
          if (INV) w.y = -w.y;
          a[b][r] = cmul(a[b][r], w);
        }
      }
    }
    dft<R, INV>(a[b]);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (LAST) store(base + r * Ns, a[b][r]);
      else buf[pad(base + r * Ns)] = a[b][r];
    }
  }
  if (!LAST) sync_group<TP>();
}

// Full transform of one group of TP threads (thread t of the group).
template <int N, bool INV, typename Load, typename Store>
__device__ __forceinline__ void transform(float2* buf, int t, const float2* __restrict__ tw, Load& load, Store& store) {
  using P = Plan<N>;
  if constexpr (P::S == 2) {
    stage<N, P::TP, P::R0, INV, true, false>(buf, t, 1, tw, load, store);
    stage<N, P::TP, P::R1, INV, false, true>(buf, t, P::R0, tw + stage_table_offset<N>(1), load, store);
  } else {
    stage<N, P::TP, P::R0, INV, true, false>(buf, t, 1, tw, load, store);
    stage<N, P::TP, P::R1, INV, false, false>(buf, t, P::R0, tw + stage_table_offset<N>(1), load, store);
    stage<N, P::TP, P::R2, INV, false, true>(buf, t, P::R0 * P::R1, tw + stage_table_offset<N>(2), load, store);
  }
}

}  // namespace fft
