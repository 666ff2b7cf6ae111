// Per-element linear equalizers shared by the fused receivers: Cholesky solve of
// small Hermitian systems, ZF (the reference's y / sum_tx h for one receive stream,
// pinv otherwise) and LMMSE.
#pragma once

#include "hpx_internal.cuh"

// --------------------------------------------------------------- solvers

// false for NaN and +-inf
__device__ __forceinline__ bool finite_f(float v) { return fabsf(v) < __int_as_float(0x7f800000); }

// Cholesky solve of the Hermitian positive definite A x = b (lower triangle of A
// used and overwritten). Returns false if a pivot is not positive; `fin` turns
// false if a pivot is not finite (NaN or inf inputs, as opposed to a singular but
// finite system, whose NaN solution the reference produces too).
template <int n>
__device__ __forceinline__ bool chol_solve(float2 (&A)[n][n], float2 (&b)[n], float2 (&x)[n], bool& fin) {
  bool ok = true;
  float inv[n];  // reciprocal pivots 1 / L[j][j]
#pragma unroll
  for (int j = 0; j < n; ++j) {
    float d = A[j][j].x;
#pragma unroll
    for (int k = 0; k < j; ++k) {  // d -= |A[j][k]|^2, as two fused steps
      d = fmaf(-A[j][k].x, A[j][k].x, d);
      d = fmaf(-A[j][k].y, A[j][k].y, d);
    }
    ok = ok && (d > 0.0f);
    fin = fin && finite_f(d);
    inv[j] = rsqrtf(d);
#pragma unroll
    for (int i = j + 1; i < n; ++i) {
      float2 s = A[i][j];
#pragma unroll
      for (int k = 0; k < j; ++k) {
        // s -= A[i][k] * conj(A[j][k])
        s.x = fmaf(-A[i][k].x, A[j][k].x, s.x);
        s.x = fmaf(-A[i][k].y, A[j][k].y, s.x);
        s.y = fmaf(-A[i][k].y, A[j][k].x, s.y);
        s.y = fmaf(A[i][k].x, A[j][k].y, s.y);
      }
      A[i][j] = cscale(s, inv[j]);
    }
  }
  float2 z[n];
#pragma unroll
  for (int i = 0; i < n; ++i) {
    float2 s = b[i];
#pragma unroll
    for (int k = 0; k < i; ++k) {  // s -= A[i][k] z[k]
      s.x = fmaf(-A[i][k].x, z[k].x, s.x);
      s.x = fmaf(A[i][k].y, z[k].y, s.x);
      s.y = fmaf(-A[i][k].x, z[k].y, s.y);
      s.y = fmaf(-A[i][k].y, z[k].x, s.y);
    }
    z[i] = cscale(s, inv[i]);
  }
#pragma unroll
  for (int i = n - 1; i >= 0; --i) {
    float2 s = z[i];
#pragma unroll
    for (int k = i + 1; k < n; ++k) {  // s -= conj(A[k][i]) x[k]
      s.x = fmaf(-A[k][i].x, x[k].x, s.x);
      s.x = fmaf(-A[k][i].y, x[k].y, s.x);
      s.y = fmaf(-A[k][i].x, x[k].y, s.y);
      s.y = fmaf(A[k][i].y, x[k].x, s.y);
    }
    x[i] = cscale(s, inv[i]);
  }
  return ok;
}

// Equalize one resource element: NTX outputs (ZF with a single receive antenna
// divides by sum_tx h like the reference and returns one stream, the others zero).
// Returns false if a pivot (or the ZF denominator) is not finite: the element's
// inputs held NaN or inf, which the caller reports as HPX_DROP_NUMERIC.
template <int NRX, int NTX>
__device__ __forceinline__ bool equalize_one(int mode, const float2 (&H)[NRX][NTX], const float2 (&y)[NRX], float s2,
                                             float2 (&x)[NTX]) {
  if (mode == HPX_EQ_ZF && NRX == 1) {
    float2 hs = make_float2(0.f, 0.f);
#pragma unroll
    for (int t = 0; t < NTX; ++t) hs = cadd(hs, H[0][t]);
    // complex division y / hs (numpy semantics: inf/nan for hs == 0)
    const float den = hs.x * hs.x + hs.y * hs.y;
    x[0] = make_float2((y[0].x * hs.x + y[0].y * hs.y) / den, (y[0].y * hs.x - y[0].x * hs.y) / den);
#pragma unroll
    for (int t = 1; t < NTX; ++t) x[t] = make_float2(0.f, 0.f);
    return finite_f(den);
  }
  bool fin = true;
  const float reg = mode == HPX_EQ_LMMSE ? s2 : 0.0f;
  if (mode == HPX_EQ_ZF && NRX < NTX) {
    // minimum-norm pseudo-inverse: x = H^H (H H^H)^-1 y
    float2 A[NRX][NRX], yy[NRX], w[NRX];
#pragma unroll
    for (int i = 0; i < NRX; ++i) {
      yy[i] = y[i];
#pragma unroll
      for (int j = 0; j <= i; ++j) {
        float2 acc = make_float2(0.f, 0.f);
#pragma unroll
        for (int t = 0; t < NTX; ++t) cfma(acc, H[i][t], cconj(H[j][t]));
        A[i][j] = acc;
      }
    }
    if (!chol_solve<NRX>(A, yy, w, fin)) {
#pragma unroll
      for (int t = 0; t < NTX; ++t) x[t] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
      return fin;
    }
#pragma unroll
    for (int t = 0; t < NTX; ++t) {
      float2 acc = make_float2(0.f, 0.f);
#pragma unroll
      for (int i = 0; i < NRX; ++i) cfmac(acc, H[i][t], w[i]);
      x[t] = acc;
    }
    return fin;
  }
  float2 A[NTX][NTX], b[NTX];
#pragma unroll
  for (int i = 0; i < NTX; ++i) {
    float2 mf = make_float2(0.f, 0.f);
#pragma unroll
    for (int r = 0; r < NRX; ++r) cfmac(mf, H[r][i], y[r]);
    b[i] = mf;
#pragma unroll
    for (int j = 0; j < i; ++j) {
      float2 acc = make_float2(0.f, 0.f);
#pragma unroll
      for (int r = 0; r < NRX; ++r) cfmac(acc, H[r][i], H[r][j]);  // (H^H H)[i][j] = sum_r conj(H[r][i]) H[r][j]
      A[i][j] = acc;
    }
    float d = 0.0f;  // the diagonal's real part, summed as cfmac sums it
#pragma unroll
    for (int r = 0; r < NRX; ++r) {
      d = fmaf(H[r][i].x, H[r][i].x, d);
      d = fmaf(H[r][i].y, H[r][i].y, d);
    }
    A[i][i] = make_float2(d + reg, 0.0f);
  }
  if (!chol_solve<NTX>(A, b, x, fin)) {
#pragma unroll
    for (int t = 0; t < NTX; ++t) x[t] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
  }
  return fin;
}

// Where equalize_spatial replaces equalize_one: LMMSE, whose regularized system keeps
// the rounding of a Gram formed from S^H S at the level of one formed per element. ZF
// solves the unregularized system, where near-singular elements turn that rounding
// into different decisions, so it keeps the per-element arithmetic of the staged
// receiver it is tested against bit for bit.
template <int NRX, int NTX>
__host__ __device__ constexpr bool gram_equalizer(int mode) {
  return mode == HPX_EQ_LMMSE;
}

// equalize_one for a channel H = S g: a spatial matrix S (Sm, [NRX][NTX]) fixed over the
// drop times one scalar response g per element, the ideal CSI of the fading model. Then
// H^H H = |g|^2 S^H S and H^H y = conj(g) S^H y, with M = S^H S ([NTX][NTX]) formed once
// per drop: per element the Gram is NTX (NTX + 1) / 2 scalings instead of NRX NTX^2 / 2
// complex products, and H is never formed. The same system up to rounding (LMMSE: the
// regularizer is s2).
template <int NRX, int NTX>
__device__ __forceinline__ bool equalize_spatial(int mode, const float2* __restrict__ Sm, const float2* __restrict__ M,
                                                 float2 g, const float2 (&y)[NRX], float s2, float2 (&x)[NTX]) {
  const float reg = s2;
  const float gg = fmaf(g.x, g.x, g.y * g.y);
  float2 A[NTX][NTX], b[NTX];
#pragma unroll
  for (int i = 0; i < NTX; ++i) {
    float2 mf = make_float2(0.f, 0.f);  // (S^H y)_i
#pragma unroll
    for (int r = 0; r < NRX; ++r) cfmac(mf, Sm[r * NTX + i], y[r]);
    b[i] = cmulc(g, mf);
#pragma unroll
    for (int j = 0; j < i; ++j) A[i][j] = cscale(M[i * NTX + j], gg);
    A[i][i] = make_float2(fmaf(M[i * NTX + i].x, gg, reg), 0.0f);
  }
  bool fin = true;
  if (!chol_solve<NTX>(A, b, x, fin)) {
#pragma unroll
    for (int t = 0; t < NTX; ++t) x[t] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
  }
  return fin;
}
