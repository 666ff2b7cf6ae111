// Massive-MIMO receiver: per-element Gram and matched filter on the BF16 tensor
// cores with split (3-term) products, FP32 Cholesky LMMSE / ZF, FP64 only for the
// elements whose Cholesky condition estimate exceeds 1e6, exact hard demap and
// bit-error count. No counterpart in the reference (its MIMO equalizer is a
// per-element numpy pinv, modem/waveform.py:235-250, limited to small arrays).
//
// Per resource element with H (NRX x 16) and y (NRX):
//   P = [Re H; Im H] (2 NRX x 16), Q = [Im H; -Re H], Y = [[Re y, Im y]; [Im y, -Re y]]
//   Re(H^H H) = P^T P,  Im(H^H H) = P^T Q,  H^H y = P^T Y   (K = 2 NRX real GEMMs)
// Every operand is split X = X_hi + X_lo into two BF16 numbers and each product is
// X_hi Y_hi + X_hi Y_lo + X_lo Y_hi with FP32 accumulation (mma.sync m16n8k16): the
// dropped X_lo Y_lo term is below 2^-16 of the product.
// The warp computes the Gram of two elements, then each half-warp factors one of
// them with its 16 rows in registers (lane i holds row i), solves, demaps its 16
// streams and counts errors against the regenerated Philox bits.
#include <cuda_bf16.h>

#include "fading_dev.cuh"

namespace {

constexpr int MT = 16;       // transmit streams (users)
constexpr int MWARPS = 4;
constexpr float kCondLimit = 1e6f;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void ldsm_x4_t(uint32_t addr, uint32_t& r0, uint32_t& r1, uint32_t& r2, uint32_t& r3) {
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0, %1, %2, %3}, [%4];\n"
               : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
               : "r"(addr));
}

__device__ __forceinline__ void mma16816(float (&c)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
      "{%0, %1, %2, %3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// 3-term split product accumulate: c += Ahi Bhi + Ahi Blo + Alo Bhi
__device__ __forceinline__ void mma3(float (&c)[4], const uint32_t (&ah)[4], const uint32_t (&al)[4], uint32_t bh0,
                                     uint32_t bh1, uint32_t bl0, uint32_t bl1) {
  mma16816(c, ah[0], ah[1], ah[2], ah[3], bh0, bh1);
  mma16816(c, ah[0], ah[1], ah[2], ah[3], bl0, bl1);
  mma16816(c, al[0], al[1], al[2], al[3], bh0, bh1);
}

__device__ __forceinline__ uint32_t neg2(uint32_t v) { return v ^ 0x80008000u; }

// Byte offset of element (row, col) of a [rows][16] bf16 tile whose two 16-byte
// halves swap on every other group of 4 rows (conflict-free 8-row ldmatrix).
__device__ __forceinline__ int toff(int row, int col) {
  return row * 32 + ((((col >> 3) ^ (row >> 2)) & 1) << 4) + (col & 7) * 2;
}

__device__ __forceinline__ void split_bf16(float v, __nv_bfloat16& hi, __nv_bfloat16& lo) {
  hi = __float2bfloat16_rn(v);
  lo = __float2bfloat16_rn(v - __bfloat162float(hi));
}

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 a, __nv_bfloat16 b) {
  __nv_bfloat162 t;
  t.x = a;
  t.y = b;
  uint32_t u;
  memcpy(&u, &t, sizeof(u));
  return u;
}

// Serial FP64 Cholesky solve of (G + reg I) x = b for one element whose FP32
// factorization was ill-conditioned; G (lower triangle, overwritten by L) and b
// were formed in FP64 from the element's channel.
__device__ bool solve_fp64(double2* L, const double2* b, double reg, float2* x) {
  for (int i = 0; i < MT; ++i) {
    L[i * MT + i].x += reg;
    L[i * MT + i].y = 0.0;
  }
  for (int k = 0; k < MT; ++k) {
    double d = L[k * MT + k].x;
    for (int p = 0; p < k; ++p) d -= L[k * MT + p].x * L[k * MT + p].x + L[k * MT + p].y * L[k * MT + p].y;
    if (!(d > 0.0)) return false;
    const double pk = sqrt(d);
    L[k * MT + k] = make_double2(pk, 0.0);
    for (int i = k + 1; i < MT; ++i) {
      double2 s = L[i * MT + k];
      for (int p = 0; p < k; ++p) {
        const double2 a = L[i * MT + p], c = L[k * MT + p];  // s -= a conj(c)
        s.x -= a.x * c.x + a.y * c.y;
        s.y -= a.y * c.x - a.x * c.y;
      }
      L[i * MT + k] = make_double2(s.x / pk, s.y / pk);
    }
  }
  double2 z[MT];
  for (int i = 0; i < MT; ++i) {
    double2 s = b[i];
    for (int p = 0; p < i; ++p) {
      const double2 a = L[i * MT + p];
      s.x -= a.x * z[p].x - a.y * z[p].y;
      s.y -= a.x * z[p].y + a.y * z[p].x;
    }
    z[i] = make_double2(s.x / L[i * MT + i].x, s.y / L[i * MT + i].x);
  }
  for (int i = MT - 1; i >= 0; --i) {
    double2 s = z[i];
    for (int p = i + 1; p < MT; ++p) {
      const double2 a = L[p * MT + i];  // conj(L[p][i]) * z[p]
      s.x -= a.x * z[p].x + a.y * z[p].y;
      s.y -= a.x * z[p].y - a.y * z[p].x;
    }
    z[i] = make_double2(s.x / L[i * MT + i].x, s.y / L[i * MT + i].x);
  }
  for (int i = 0; i < MT; ++i) x[i] = make_float2((float)z[i].x, (float)z[i].y);
  return true;
}

// Per-warp shared memory: [P_hi | P_lo] (reused for the FP64 Gram and matched
// filter of the two elements once the FP32 ones are formed), Y, G[2][16][17] (rows
// padded: a half-warp reading one row per lane hits distinct banks), b[2][16],
// x[2][16], Cholesky column broadcast [2][16], g[2], column[2].
template <int NRX>
struct MassiveSmem {
  static constexpr int KR = 2 * NRX;        // stacked real rows
  static constexpr int TILE = KR * 16 * 2;  // bytes of one [KR][16] bf16 tile
  static constexpr int FP64 = 2 * MT * MT * 16 + 2 * MT * 16;
  static constexpr int UNION = 2 * TILE > FP64 ? 2 * TILE : FP64;
  static constexpr int WARP_BYTES = UNION + TILE + 2 * MT * (MT + 1) * 8 + 2 * MT * 8 + 2 * MT * 8 + 2 * MT * 8 + 2 * 8 + 2 * 8;
};

// Fused ideal-CSI massive-MIMO receiver, one block (4 warps) per (word, drop).
template <int NRX>
__global__ void __launch_bounds__(MWARPS * 32, 1) k_detect_massive(
    FadingConst fc, FadingView v, int N, int W, int C, int m, const int32_t* __restrict__ window_start,
    const int32_t* __restrict__ data_offset, const int32_t* __restrict__ num_data_word,
    const int32_t* __restrict__ data_column, const int32_t* __restrict__ bins, const float2* __restrict__ tw,
    const __grid_constant__ QamDemapTable qt, int mode, const float2* __restrict__ grid, int gcols,
    const float* __restrict__ nv, uint64_t seed, int64_t drop0, uint32_t* __restrict__ errors,
    uint32_t* __restrict__ fp64_count, float2* __restrict__ equalized, int num_data) {
  using SM = MassiveSmem<NRX>;
  constexpr int KR = SM::KR, KS = KR / 16;
  extern __shared__ float4 smem4[];
  const int w = blockIdx.x, b = blockIdx.y;
  const int BW = staged_bit_words(C, m);
  unsigned char* base = reinterpret_cast<unsigned char*>(smem4);
  unsigned char* wbase = base;  // per-warp areas first (16-byte aligned)
  float2* hb = reinterpret_cast<float2*>(base + MWARPS * SM::WARP_BYTES);
  float2* scratch = hb + fc.L;
  // [NRX][16], 16-byte aligned for the float4 loads of the fill
  float2* Sm = reinterpret_cast<float2*>((reinterpret_cast<uintptr_t>(scratch + fc.L * fc.S1) + 15) & ~uintptr_t(15));
  int* ds = reinterpret_cast<int*>(Sm + NRX * MT);
  uint32_t* bitsm = reinterpret_cast<uint32_t*>(ds + fc.L + 4);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char* my = wbase + warp * SM::WARP_BYTES;
  unsigned char* Phi = my;
  unsigned char* Plo = my + SM::TILE;
  unsigned char* Yt = my + SM::UNION;
  constexpr int GS = MT + 1;                                  // padded Gram row
  float2* Gs = reinterpret_cast<float2*>(my + SM::UNION + SM::TILE);  // [2][16][17]
  float2* bs = Gs + 2 * MT * GS;                              // [2][16]
  float2* xs = bs + 2 * MT;                                   // [2][16] FP64-path results
  float2* colb = xs + 2 * MT;                                 // [2][16] column of L being broadcast
  float2* gsave = colb + 2 * MT;                              // [2] tap response of each element
  int* csave = reinterpret_cast<int*>(gsave + 2);             // [2] grid column of each element

  const int64_t k0 = data_offset[w];
  const int nd = num_data_word[w];
  for (int l = threadIdx.x; l < fc.L; l += blockDim.x) ds[l] = fc.delay[l];
  const float2* Sg = v.spatial(b);
  for (int i = threadIdx.x; i < NRX * MT; i += blockDim.x) Sm[i] = Sg[i];
  // zero the Y tiles once: only columns 0, 1 (hi) and 8, 9 (lo) change per element
  for (int i = lane; i < KR * 8; i += 32) reinterpret_cast<uint32_t*>(Yt)[i] = 0u;
  // stage the Philox bits of the 16 streams
  if (nd > 0) {
    const int64_t blk0 = ((k0 * m) >> 5) >> 2, blk1 = (((k0 + nd) * m - 1) >> 5) >> 2;
    const int nblk = (int)(blk1 - blk0 + 1);
    for (int q = threadIdx.x; q < nblk * MT; q += blockDim.x) {
      const int s = q / nblk;
      const int64_t blk = blk0 + (q - s * nblk);
      const uint4 r = hpx_random_block(seed, drop0 + b, (uint32_t)s, HPX_DOMAIN_BITS, (uint32_t)blk);
      uint32_t* dst = bitsm + s * BW + (blk - blk0) * 4;
      dst[0] = r.x;
      dst[1] = r.y;
      dst[2] = r.z;
      dst[3] = r.w;
    }
  }
  tap_averages(fc, v.W(b), v.P0(b), window_start[w], N, hb, scratch);  // ends with __syncthreads
  const int64_t wofs = (((k0 * m) >> 5) >> 2) * 4;
  const float s2 = nv ? nv[b] : 0.0f;
  const float reg = mode == HPX_EQ_LMMSE ? s2 : 0.0f;
  const uint32_t phi = smem_u32(Phi), plo = smem_u32(Plo), yt = smem_u32(Yt);
  const int j8 = lane >> 3, r8 = lane & 7;
  const int half = lane >> 4, row = lane & 15;
  unsigned int local = 0, n64 = 0;
  // a NaN / inf noise power, or an element whose solution (after the FP64 re-solve of
  // ill-conditioned elements) is not finite
  bool bad = !(fabsf(s2) < INFINITY);

  // received samples of the next element pair are loaded one iteration ahead
  constexpr int YR = (NRX + 31) / 32;
  float2 ypf[2][YR];
  int cpf[2];
  auto prefetch = [&](int jbase) {
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int j = jbase + s;
      cpf[s] = j < nd ? data_column[k0 + j] : 0;
#pragma unroll
      for (int q = 0; q < YR; ++q) {
        const int r = lane + 32 * q;
        ypf[s][q] = (j < nd && r < NRX) ? __ldg(grid + (((int64_t)b * NRX + r) * W + w) * gcols + cpf[s])
                                        : make_float2(0.f, 0.f);
      }
    }
  };
  prefetch(warp * 2);
  for (int j0 = warp * 2; j0 < nd; j0 += 2 * MWARPS) {
    float2 ycur[2][YR];
    int ccur[2];
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      ccur[s] = cpf[s];
#pragma unroll
      for (int q = 0; q < YR; ++q) ycur[s][q] = ypf[s][q];
    }
    if (j0 + 2 * MWARPS < nd) prefetch(j0 + 2 * MWARPS);
    // ---------------- Gram and matched filter of elements j0 and j0 + 1
#pragma unroll
    for (int s = 0; s < 2; ++s) {
      const int j = j0 + s;
      float2* G = Gs + s * MT * GS;
      float2* bv = bs + s * MT;
      if (j >= nd) {  // no element: an identity system keeps the half-warp's arithmetic finite
        for (int i = lane; i < MT * MT; i += 32) G[(i / MT) * GS + i % MT] = make_float2((i % (MT + 1)) == 0 ? 1.f : 0.f, 0.f);
        if (lane < MT) bv[lane] = make_float2(0.f, 0.f);
        __syncwarp();
        continue;
      }
      const int c = ccur[s];
      const float2 g = tap_response(fc, hb, ds, tw, bins[c], N);
      if (lane == 0) {
        gsave[s] = g;
        csave[s] = c;
      }
      // P tiles: rows r (Re H) and NRX + r (Im H), two columns per lane and step
      for (int e = lane; e < NRX * MT / 2; e += 32) {
        const int r = e >> 3, t = (e & 7) * 2;
        const float4 sp = *reinterpret_cast<const float4*>(Sm + r * MT + t);  // one 16-byte load, no bank conflicts
        const float2 h0 = cmul(make_float2(sp.x, sp.y), g), h1 = cmul(make_float2(sp.z, sp.w), g);
        __nv_bfloat16 a0, a1, b0, b1, c0, c1, d0, d1;
        split_bf16(h0.x, a0, a1);
        split_bf16(h1.x, b0, b1);
        split_bf16(h0.y, c0, c1);
        split_bf16(h1.y, d0, d1);
        *reinterpret_cast<uint32_t*>(Phi + toff(r, t)) = pack2(a0, b0);
        *reinterpret_cast<uint32_t*>(Plo + toff(r, t)) = pack2(a1, b1);
        *reinterpret_cast<uint32_t*>(Phi + toff(NRX + r, t)) = pack2(c0, d0);
        *reinterpret_cast<uint32_t*>(Plo + toff(NRX + r, t)) = pack2(c1, d1);
      }
      // Y tile: column 0 = [Re y; Im y], column 1 = [Im y; -Re y] (hi in 0-1, lo in 8-9)
#pragma unroll
      for (int q = 0; q < YR; ++q) {
        const int r = lane + 32 * q;
        if (r >= NRX) continue;
        const float2 yv = ycur[s][q];
        __nv_bfloat16 xr0, xr1, xi0, xi1, nr0, nr1;
        split_bf16(yv.x, xr0, xr1);
        split_bf16(yv.y, xi0, xi1);
        split_bf16(-yv.x, nr0, nr1);
        *reinterpret_cast<uint32_t*>(Yt + toff(r, 0)) = pack2(xr0, xi0);
        *reinterpret_cast<uint32_t*>(Yt + toff(r, 8)) = pack2(xr1, xi1);
        *reinterpret_cast<uint32_t*>(Yt + toff(NRX + r, 0)) = pack2(xi0, nr0);
        *reinterpret_cast<uint32_t*>(Yt + toff(NRX + r, 8)) = pack2(xi1, nr1);
      }
      __syncwarp();
      float gr[2][4] = {}, gi[2][4] = {}, by[4] = {};
#pragma unroll
      for (int ks = 0; ks < KS / 2; ++ks) {
        const int ks2 = ks + KS / 2;
        // A = P^T fragments of k-steps ks (rows of Re H) and ks2 (rows of Im H)
        uint32_t ah[2][4], al[2][4];
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          const int kk = p == 0 ? ks : ks2;
          const int rr = kk * 16 + (j8 >> 1) * 8 + r8, cc = (j8 & 1) * 8;
          ldsm_x4_t(phi + toff(rr, cc), ah[p][0], ah[p][1], ah[p][2], ah[p][3]);
          ldsm_x4_t(plo + toff(rr, cc), al[p][0], al[p][1], al[p][2], al[p][3]);
        }
        // Y fragments: matrices (hi, k lo), (hi, k hi), (lo, k lo), (lo, k hi)
        uint32_t yf[2][4];
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          const int kk = p == 0 ? ks : ks2;
          const int rr = kk * 16 + (j8 & 1) * 8 + r8, cc = (j8 >> 1) * 8;
          ldsm_x4_t(yt + toff(rr, cc), yf[p][0], yf[p][1], yf[p][2], yf[p][3]);
        }
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          // B = P fragments of the same k-step are the A fragments reordered:
          // n-tile nt, k-half kb <- A register (m-block nt, k-half kb) = index nt + 2 kb
          const int q = 1 - p;  // Q = [Im H; -Re H]: the partner k-step, negated in the lower half
#pragma unroll
          for (int nt = 0; nt < 2; ++nt) {
            mma3(gr[nt], ah[p], al[p], ah[p][nt], ah[p][nt + 2], al[p][nt], al[p][nt + 2]);
            uint32_t qh0 = ah[q][nt], qh1 = ah[q][nt + 2], ql0 = al[q][nt], ql1 = al[q][nt + 2];
            if (p == 1) {
              qh0 = neg2(qh0);
              qh1 = neg2(qh1);
              ql0 = neg2(ql0);
              ql1 = neg2(ql1);
            }
            mma3(gi[nt], ah[p], al[p], qh0, qh1, ql0, ql1);
          }
          mma3(by, ah[p], al[p], yf[p][0], yf[p][1], yf[p][2], yf[p][3]);
        }
      }
      // C fragments: rows lane/4 (+8), columns 2 (lane % 4) (+1) of each 8-column tile
      const int gm = lane >> 2, gn = (lane & 3) * 2;
#pragma unroll
      for (int nt = 0; nt < 2; ++nt)
#pragma unroll
        for (int hr = 0; hr < 2; ++hr)
#pragma unroll
          for (int e = 0; e < 2; ++e) {
            const int i = gm + hr * 8, jj = nt * 8 + gn + e;
            G[i * GS + jj] = make_float2(gr[nt][hr * 2 + e], gi[nt][hr * 2 + e]);
          }
      if ((lane & 3) == 0) {
        bv[gm] = make_float2(by[0], by[1]);
        bv[gm + 8] = make_float2(by[2], by[3]);
      }
      __syncwarp();
    }

    // ---------------- FP32 Cholesky solve, one element per half-warp (lane i: row i)
    const int jme = j0 + half;
    const bool valid = jme < nd;
    const float2* G = Gs + half * MT * GS;
    float2* col = colb + half * MT;
    float2 a[MT];
#pragma unroll
    for (int jj = 0; jj < MT; ++jj) {
      a[jj] = G[row * GS + jj];
      if (jj == row) a[jj] = make_float2(a[jj].x + reg, 0.f);  // compile-time index: a[] stays in registers
    }
    float2 bi = bs[half * MT + row];
    float pmin = INFINITY, pmax = 0.f, inv_i = 0.f;
    bool ok = true;
    // right-looking Cholesky; column k of L goes through shared memory, every loop has
    // a fixed trip count so that a[] stays in registers
#pragma unroll
    for (int k = 0; k < MT; ++k) {
      const float dkk = __shfl_sync(0xffffffffu, a[k].x, k, 16);
      ok = ok && (dkk > 0.f);
      const float ik = rsqrtf(fmaxf(dkk, 1e-30f));
      const float pk = dkk * ik;
      pmin = fminf(pmin, pk);
      pmax = fmaxf(pmax, pk);
      if (row == k) inv_i = ik;
      const float2 lik = row > k ? cscale(a[k], ik) : (row == k ? make_float2(pk, 0.f) : make_float2(0.f, 0.f));
      a[k] = lik;
      col[row] = lik;
      __syncwarp();
#pragma unroll
      for (int jj = 0; jj < MT; ++jj) {
        if (jj <= k) continue;
        const float2 ljk = col[jj];
        if (row >= jj) {  // a[jj] -= lik conj(ljk)
          a[jj].x -= lik.x * ljk.x + lik.y * ljk.y;
          a[jj].y -= lik.y * ljk.x - lik.x * ljk.y;
        }
      }
      __syncwarp();
    }
    // forward: L z = b
    float2 zi = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = 0; k < MT; ++k) {
      const float2 zl = cscale(bi, inv_i);
      const float2 zk = make_float2(__shfl_sync(0xffffffffu, zl.x, k, 16), __shfl_sync(0xffffffffu, zl.y, k, 16));
      if (row == k) zi = zk;
      if (row > k) bi = csub(bi, cmul(a[k], zk));
    }
    // backward: L^H x = z
    float2 xi = make_float2(0.f, 0.f);
#pragma unroll
    for (int k = MT - 1; k >= 0; --k) {
      float2 t = row > k ? cmulc(a[k], xi) : make_float2(0.f, 0.f);  // conj(L[row][k]) x_row
#pragma unroll
      for (int o = 8; o > 0; o >>= 1) {
        t.x += __shfl_xor_sync(0xffffffffu, t.x, o, 16);
        t.y += __shfl_xor_sync(0xffffffffu, t.y, o, 16);
      }
      if (row == k) xi = cscale(csub(zi, t), inv_i);
    }
    const bool cond_bad = !ok || pmax * pmax > kCondLimit * pmin * pmin;  // (pmax / pmin)^2 > 1e6
    const unsigned need = __ballot_sync(0xffffffffu, valid && cond_bad && row == 0);
    if (need) {
      // FP64 Gram and matched filter of the flagged elements from their channel
      // (lane i: row i), then a serial FP64 Cholesky solve on the half's first lane
      const bool mine = (need >> (16 * half)) & 1u;
      double2* G64 = reinterpret_cast<double2*>(Phi) + half * MT * MT;  // P tiles are free now
      double2* b64 = reinterpret_cast<double2*>(Phi) + 2 * MT * MT + half * MT;
      if (mine) {
        const float2 gg = gsave[half];
        const int cc = csave[half];
        double2 bacc = make_double2(0.0, 0.0);
        for (int r = 0; r < NRX; ++r) {
          const float2 hi = cmul(Sm[r * MT + row], gg);
          const float2 yv = grid[(((int64_t)b * NRX + r) * W + w) * gcols + cc];
          bacc.x += (double)hi.x * yv.x + (double)hi.y * yv.y;  // conj(h) y
          bacc.y += (double)hi.x * yv.y - (double)hi.y * yv.x;
        }
        b64[row] = bacc;
        for (int jj = 0; jj <= row; ++jj) {
          double2 acc = make_double2(0.0, 0.0);
          for (int r = 0; r < NRX; ++r) {
            const float2 hi = cmul(Sm[r * MT + row], gg), hj = cmul(Sm[r * MT + jj], gg);
            acc.x += (double)hi.x * hj.x + (double)hi.y * hj.y;  // conj(h_i) h_j
            acc.y += (double)hi.x * hj.y - (double)hi.y * hj.x;
          }
          G64[row * MT + jj] = acc;
        }
      }
      __syncwarp();
      if (mine && row == 0) {
        float2 xo[MT];
        if (!solve_fp64(G64, b64, (double)reg, xo))
          for (int i = 0; i < MT; ++i) xo[i] = make_float2(__int_as_float(0x7fc00000), __int_as_float(0x7fc00000));
        for (int i = 0; i < MT; ++i) xs[half * MT + i] = xo[i];
      }
      __syncwarp();
      if (mine) xi = xs[half * MT + row];
      n64 += (row == 0 && mine) ? 1u : 0u;
    }
    if (valid) {
      bad = bad || !(fabsf(xi.x) < INFINITY && fabsf(xi.y) < INFINITY);
      const int64_t k = k0 + jme;
      const uint32_t rx_v = qam_decide(qt, xi);
      const uint32_t tx_v = extract_bits_msb(bitsm + row * BW - wofs, k * m, m);
      local += __popc(rx_v ^ tx_v);
      if (equalized) equalized[((int64_t)b * MT + row) * num_data + k] = xi;
    }
    __syncwarp();
  }
  // block totals
  for (int o = 16; o > 0; o >>= 1) {
    local += __shfl_down_sync(0xffffffffu, local, o);
    n64 += __shfl_down_sync(0xffffffffu, n64, o);
  }
  const bool any_bad = __any_sync(0xffffffffu, bad);
  if (lane == 0) {
    if (local) atomicAdd(errors + b, local);
    if (any_bad) atomicOr(errors + b, HPX_DROP_NUMERIC);
    if (n64 && fp64_count) atomicAdd(fp64_count + b, n64);
  }
}

template <int NRX>
hpx_status launch_massive(const hpx_fading* f, const void* state, const hpx_frame* fr, int mode, const hpx_cf32* grid,
                          int gcols, const float* nv, uint64_t seed, int64_t drop0, int B, uint32_t* errors,
                          uint32_t* fp64_count, hpx_cf32* equalized, cudaStream_t s) {
  QamDemapTable qt;
  HPX_TRY(qam_demap_table(fr->info.modulation_order, &qt));
  const FadingConst fc = fading_const(f);
  const int C = fr->info.num_columns, m = fr->info.bits_per_symbol;
  const size_t smem = (size_t)MWARPS * MassiveSmem<NRX>::WARP_BYTES + (size_t)fc.L * sizeof(float2) * (1 + fc.S1) +
                      (size_t)NRX * MT * sizeof(float2) + 16 + (fc.L + 4) * sizeof(int) +
                      (size_t)MT * staged_bit_words(C, m) * 4 + 16;
  if (smem > 220 * 1024) return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_massive: frame needs %zu bytes of shared memory", smem);
  auto kern = k_detect_massive<NRX>;
  HPX_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  dim3 g(fr->info.num_words, B);
  kern<<<g, MWARPS * 32, smem, s>>>(fc, fading_view(f, state), fr->info.num_subcarriers, fr->info.num_words, C, m,
                                     fr->d_window_start, fr->d_data_offset, fr->d_num_data_word, fr->d_data_column,
                                     fr->d_bins, fr->d_twiddle, qt, mode, reinterpret_cast<const float2*>(grid), gcols,
                                     nv, seed, drop0, errors, fp64_count, reinterpret_cast<float2*>(equalized),
                                     fr->info.num_data);
  HPX_LAUNCHED("detect_massive");
  return HPX_OK;
}

}  // namespace

extern "C" hpx_status hpx_detect_massive(const hpx_fading* f, const void* state, const hpx_frame* fr, int32_t mode,
                                         const hpx_cf32* grid, int32_t gcols, const float* nv, uint64_t seed,
                                         int64_t drop0, int32_t B, uint32_t* errors, uint32_t* fp64_count,
                                         hpx_cf32* equalized, void* stream) {
  if (!f || !state || !fr || !grid || !errors) return hpx_fail(HPX_ERR_ARG, "detect_massive: null argument");
  if (mode != HPX_EQ_ZF && mode != HPX_EQ_LMMSE) return hpx_fail(HPX_ERR_ARG, "detect_massive: unknown mode");
  if (mode == HPX_EQ_LMMSE && !nv) return hpx_fail(HPX_ERR_ARG, "detect_massive: LMMSE needs noise variances");
  if (B < 0 || drop0 < 0) return hpx_fail(HPX_ERR_ARG, "detect_massive: bad drop range");
  if (gcols < fr->info.num_columns) return hpx_fail(HPX_ERR_SHAPE, "detect_massive: grid too narrow");
  if (f->ntx != MT) return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_massive: 16 transmit streams required (got %d)", f->ntx);
  if (B == 0) return HPX_OK;
  if (B > 65535) return hpx_fail(HPX_ERR_ARG, "detect_massive: batch above 65535 drops per call");
  cudaStream_t s = as_stream(stream);
  HPX_CUDA(cudaMemsetAsync(errors, 0, sizeof(uint32_t) * B, s));
  if (fp64_count) HPX_CUDA(cudaMemsetAsync(fp64_count, 0, sizeof(uint32_t) * B, s));
  switch (f->nrx) {
    case 16: return launch_massive<16>(f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, fp64_count, equalized, s);
    case 32: return launch_massive<32>(f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, fp64_count, equalized, s);
    case 64: return launch_massive<64>(f, state, fr, mode, grid, gcols, nv, seed, drop0, B, errors, fp64_count, equalized, s);
    default: return hpx_fail(HPX_ERR_UNSUPPORTED, "detect_massive: %d receive antennas not supported (16, 32, 64)", f->nrx);
  }
}
